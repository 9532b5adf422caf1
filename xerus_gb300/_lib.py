"""ctypes binding of libxtt.so (the C ABI declared in include/xtt.h).

The library is built in-tree (xerus_gb300/_build/libxtt.so). Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxtt.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "xtt.h")

c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)


class AlsOptions(ctypes.Structure):
    _fields_ = [
        ("sites", ctypes.c_int32),
        ("local_solver", ctypes.c_int32),
        ("preserve_core_position", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("num_half_sweeps", ctypes.c_int64),
        ("convergence_epsilon", ctypes.c_double),
        ("local_tolerance", ctypes.c_double),
        ("local_max_iterations", ctypes.c_int64),
        ("residual_target", ctypes.c_double),
        ("record_residuals", ctypes.c_int32),
        ("max_rank", ctypes.c_int32),
        ("svd_epsilon", ctypes.c_double),
        ("exact_environment", ctypes.c_int32),
        ("assume_spd", ctypes.c_int32),
        ("use_residual", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class AlsReport(ctypes.Structure):
    _fields_ = [
        ("energy", ctypes.c_double),
        ("residual", ctypes.c_double),
        ("half_sweeps", ctypes.c_int64),
        ("micro_steps", ctypes.c_int64),
        ("local_iterations", ctypes.c_int64),
        ("refinements", ctypes.c_int64),
        ("trace_count", ctypes.c_int64),
    ]


class BatchReport(ctypes.Structure):
    _fields_ = [
        ("milliseconds", ctypes.c_double),
        ("threads", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("ctas", ctypes.c_int32),
        ("tile", ctypes.c_int32),
    ]


class AdfOptions(ctypes.Structure):
    _fields_ = [
        ("max_iterations", ctypes.c_int64),
        ("target_residual", ctypes.c_double),
        ("min_decrease", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


VP = ctypes.c_void_p
_SIGNATURES = {
    "xtt_last_error": (ctypes.c_char_p, []),
    "xtt_version": (ctypes.c_char_p, []),
    "xtt_context_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(VP)]),
    "xtt_context_destroy": (ctypes.c_int, [VP]),
    "xtt_context_set_stream": (ctypes.c_int, [VP, VP]),
    "xtt_context_synchronize": (ctypes.c_int, [VP]),
    "xtt_context_kernel_launches": (ctypes.c_int, [VP, c_int64_p]),
    "xtt_context_profile": (ctypes.c_int, [VP, ctypes.c_int]),
    "xtt_context_profile_get": (ctypes.c_int, [VP, ctypes.c_char_p, c_int64_p, c_double_p]),
    "xtt_context_set_cg_path": (ctypes.c_int, [VP, ctypes.c_int]),
    "xtt_context_set_svd_path": (ctypes.c_int, [VP, ctypes.c_int]),
    "xtt_context_set_contraction_precision": (ctypes.c_int, [VP, ctypes.c_int]),
    "xtt_gemm_tc": (ctypes.c_int, [VP, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, VP, ctypes.c_int64, VP,
                                   ctypes.c_int64, VP, ctypes.c_int64, ctypes.c_int32]),
    "xtt_context_profile_work": (ctypes.c_int, [VP, ctypes.c_char_p, c_double_p, c_double_p]),
    "xtt_apply": (ctypes.c_int, [VP, VP, ctypes.POINTER(VP)]),
    "xtt_geometric_cg": (ctypes.c_int, [VP, VP, VP, ctypes.c_int64, ctypes.c_double, ctypes.c_int, c_double_p,
                                        c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_steepest_descent": (ctypes.c_int, [VP, VP, VP, ctypes.c_int64, ctypes.c_double, ctypes.c_int, c_double_p,
                                            c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_geometric_cg_retraction": (ctypes.c_int, [VP, VP, VP, ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                                   ctypes.c_int, c_double_p, c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_steepest_descent_retraction": (ctypes.c_int, [VP, VP, VP, ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                                       ctypes.c_int, c_double_p, c_double_p, ctypes.c_int64,
                                                       c_int64_p]),
    "xtt_iht": (ctypes.c_int, [VP, c_int64_p, c_double_p, ctypes.c_int64, ctypes.c_int64, c_double_p, c_double_p,
                               ctypes.c_int64, c_int64_p]),
    "xtt_random_rank_one": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, c_int64_p, c_double_p]),
    "xtt_entries_rank_one": (ctypes.c_int, [VP, c_double_p, ctypes.c_int64, c_double_p]),
    "xtt_adf_rank_one": (ctypes.c_int, [VP, c_double_p, c_double_p, ctypes.c_int64, ctypes.POINTER(AdfOptions),
                                        c_double_p, c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_add": (ctypes.c_int, [VP, VP, ctypes.c_double]),
    "xtt_tensor_save": (ctypes.c_int, [VP, ctypes.c_char_p]),
    "xtt_tensor_load": (ctypes.c_int, [VP, ctypes.c_char_p, ctypes.POINTER(VP)]),
    "xtt_file_encode": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, c_int64_p, c_int64_p, c_double_p, ctypes.c_int,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, c_int64_p]),
    "xtt_file_decode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_int_p, c_int64_p, c_int64_p, c_int64_p,
                                       ctypes.c_int64, c_double_p, ctypes.c_int64, c_int64_p, c_int_p, c_int64_p]),
    "xtt_als_batch": (ctypes.c_int, [VP, ctypes.c_int64, ctypes.POINTER(VP), ctypes.POINTER(VP), ctypes.POINTER(VP),
                                     ctypes.POINTER(AlsOptions), ctypes.c_int, c_double_p, c_int64_p,
                                     ctypes.POINTER(BatchReport)]),
    "xtt_tensor_create": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int64, c_int64_p, c_int64_p, ctypes.POINTER(VP)]),
    "xtt_tensor_destroy": (ctypes.c_int, [VP]),
    "xtt_tensor_copy": (ctypes.c_int, [VP, ctypes.POINTER(VP)]),
    "xtt_tensor_order": (ctypes.c_int, [VP, c_int64_p]),
    "xtt_tensor_dims": (ctypes.c_int, [VP, c_int64_p]),
    "xtt_tensor_ranks": (ctypes.c_int, [VP, c_int64_p]),
    "xtt_tensor_size": (ctypes.c_int, [VP, c_int64_p]),
    "xtt_tensor_set_cores": (ctypes.c_int, [VP, c_double_p, ctypes.c_int64]),
    "xtt_tensor_get_cores": (ctypes.c_int, [VP, c_double_p, ctypes.c_int64]),
    "xtt_tensor_assign": (ctypes.c_int, [VP, c_int64_p, c_double_p, ctypes.c_int64]),
    "xtt_tensor_get_canonical": (ctypes.c_int, [VP, c_int_p, c_int64_p]),
    "xtt_tensor_set_canonical": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int64]),
    "xtt_tensor_scale": (ctypes.c_int, [VP, ctypes.c_double]),
    "xtt_random_seed": (ctypes.c_int, [ctypes.c_uint64]),
    "xtt_tensor_random": (ctypes.c_int, [VP, ctypes.c_int64, c_int64_p, c_int64_p, ctypes.c_double, ctypes.c_double,
                                         ctypes.POINTER(VP)]),
    "xtt_random_positions": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, c_int64_p, c_int64_p]),
    "xtt_random_normal": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_int64, c_double_p]),
    "xtt_move_core": (ctypes.c_int, [VP, ctypes.c_int64, ctypes.c_int]),
    "xtt_round": (ctypes.c_int, [VP, c_int64_p, ctypes.c_double, c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_dot": (ctypes.c_int, [VP, VP, c_double_p]),
    "xtt_frob_norm": (ctypes.c_int, [VP, c_double_p]),
    "xtt_dot_noalloc": (ctypes.c_int, [ctypes.c_int64, c_int64_p, c_int64_p, VP, c_int64_p, VP, VP, VP]),
    "xtt_residual": (ctypes.c_int, [VP, VP, VP, c_double_p]),
    "xtt_entries": (ctypes.c_int, [VP, c_int64_p, ctypes.c_int64, c_double_p]),
    "xtt_als_default_options": (ctypes.c_int, [ctypes.POINTER(AlsOptions)]),
    "xtt_als": (ctypes.c_int, [VP, VP, VP, ctypes.POINTER(AlsOptions), ctypes.POINTER(AlsReport), c_double_p,
                               c_int64_p, c_double_p, ctypes.c_int64]),
    "xtt_als_energy_gradient": (ctypes.c_int, [VP, VP, VP, c_double_p, c_double_p, ctypes.c_int64]),
    "xtt_adf": (ctypes.c_int, [VP, c_int64_p, c_double_p, ctypes.c_int64, ctypes.POINTER(AdfOptions), c_double_p,
                               c_double_p, ctypes.c_int64, c_int64_p]),
    "xtt_adf_max_ranks": (ctypes.c_int, [VP, c_int64_p, c_double_p, ctypes.c_int64, c_int64_p,
                                         ctypes.POINTER(AdfOptions), c_double_p, c_double_p, c_int64_p, c_int64_p,
                                         ctypes.c_int64, c_int64_p]),
    "xtt_adf_gradient": (ctypes.c_int, [VP, c_int64_p, c_double_p, ctypes.c_int64, c_double_p, c_double_p,
                                        ctypes.c_int64]),
}

STATUS = {0: "OK", 1: "ARGUMENT", 2: "CUDA", 3: "NOT_CONVERGED", 4: "NUMERIC", 5: "TIMEOUT", 6: "CAPACITY",
          7: "NO_MEMORY"}


class XttError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"xtt error {STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def declared_functions():
    """Names of every function include/xtt.h declares."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(xtt_\w+)\s*\(", text, flags=re.M)))


def load(path=LIB_PATH):
    """Loads libxtt.so (once) and declares the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first (python -m xerus_gb300.build)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(code):
    if code != 0:
        raise XttError(code, _lib.xtt_last_error().decode())
