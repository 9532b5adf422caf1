"""xerus_gb300: the xerus Tensor-Train sweep path on a GB300, behind xerus's API.

TT tensors and operators live on the GPU (one CUDA device per Context); every
operation runs through the C ABI of libxtt.so (include/xtt.h). The names mirror
xerus's Python bindings (src/xerus/python/*.cpp): TTTensor, TTOperator,
frob_norm, TTTensor.random, move_core, round, ALS_SPD / DMRG_SPD / ASD_SPD
(ALSVariant), ADF (ADFVariant) and SinglePointMeasurementSet.

There is no CPU fallback: without the built library or a GPU, calls raise.
"""
import ctypes
import os
import sys

import numpy as np

from . import _lib as L

__all__ = ["Context", "TTTensor", "TTOperator", "frob_norm", "dot", "residual", "ALSVariant", "ALS", "ALS_SPD", "DMRG", "DMRG_SPD", "ASD",
           "ASD_SPD", "ADFVariant", "ADF", "IHT", "SinglePointMeasurementSet", "RankOneMeasurementSet", "GeometricCGVariant", "GeometricCG", "SteepestDescentVariant", "SteepestDescent", "SubmanifoldRetraction", "HOSVDRetraction", "ALSRetraction", "PerformanceData", "seed", "EPSILON",
           "XttError", "FP64", "MIXED", "als_batch", "apply", "save_to_file", "load_from_file", "file_encode", "file_decode"]

EPSILON = 8 * np.finfo(np.float64).eps  # include/xerus/basic.h:50
FP64, MIXED = 0, 1
XttError = L.XttError
INT64_MAX = np.iinfo(np.int64).max


def _i64(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int64))
    return a, a.ctypes.data_as(L.c_int64_p)


def _f64(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return a, a.ctypes.data_as(L.c_double_p)


class Context:
    """One CUDA device and stream (xtt_context)."""

    _default = None

    def __init__(self, device=0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.xtt_context_create(int(device), ctypes.byref(h)))
        self.handle = h

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def synchronize(self):
        L.check(self.lib.xtt_context_synchronize(self.handle))

    def kernel_launches(self):
        v = ctypes.c_int64()
        L.check(self.lib.xtt_context_kernel_launches(self.handle, ctypes.byref(v)))
        return v.value

    def profile(self, enable=True):
        """Starts (clears) or stops per-kernel-class CUDA-event timing."""
        L.check(self.lib.xtt_context_profile(self.handle, int(bool(enable))))

    def profile_work(self, name):
        """(bytes, flops) of algorithmic work declared by the launches of a class."""
        by, fl = ctypes.c_double(), ctypes.c_double()
        L.check(self.lib.xtt_context_profile_work(self.handle, name.encode(), ctypes.byref(by), ctypes.byref(fl)))
        return by.value, fl.value

    def set_cg_path(self, path):
        """'auto' (cluster-resident CG where the local system fits; the tensor-core
        precision form for mixed solves at ranks >= 64 or from 16384 unknowns), 'grid',
        or 'tensor' (the tensor-core precision form for every mixed solve)."""
        L.check(self.lib.xtt_context_set_cg_path(self.handle, {"auto": 0, "grid": 1, "tensor": 2}[path]))

    def set_contraction_precision(self, form):
        """Precision form of round / move_core / dot: 'fp64', 'tf32x3' (split TF32 on the
        tensor cores), 'bf16x3' (three BF16 pieces, six products) or 'tf32'. QR and SVD
        stay FP64."""
        L.check(self.lib.xtt_context_set_contraction_precision(
            self.handle, {"fp64": 0, "tf32x3": 3, "tf32": 1, "bf16x3": 6}[form]))

    def set_svd_path(self, path):
        """'auto' (QR-preconditioned Jacobi where it fits) or 'jacobi' (plain one-sided Jacobi)."""
        L.check(self.lib.xtt_context_set_svd_path(self.handle, {"auto": 0, "jacobi": 1}[path]))

    def profile_get(self, name):
        """(launches, milliseconds) of a kernel class since profiling started."""
        n, ms = ctypes.c_int64(), ctypes.c_double()
        L.check(self.lib.xtt_context_profile_get(self.handle, name.encode(), ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def set_stream(self, stream_ptr):
        L.check(self.lib.xtt_context_set_stream(self.handle, ctypes.c_void_p(stream_ptr)))

    def __del__(self):
        if getattr(self, "handle", None) and not sys.is_finalizing():
            self.lib.xtt_context_destroy(self.handle)
        self.handle = None


def seed(value=0xBAADF00D):
    """Reseeds the library's engine (xerus::misc::randomEngine.seed) and resets its normal distribution."""
    L.check(L.load().xtt_random_seed(int(value)))


class _TT:
    is_operator = False

    def __init__(self, dims=None, ranks=None, ctx=None, _handle=None):
        self.ctx = ctx or Context.default()
        self.lib = self.ctx.lib
        if _handle is not None:
            self.handle = _handle
            return
        dims = list(dims)
        if ranks is None:
            ranks = [1] * (len(dims) + 1)
        d, pd = _i64(dims)
        r, pr = _i64(ranks)
        h = ctypes.c_void_p()
        L.check(self.lib.xtt_tensor_create(self.ctx.handle, int(self.is_operator), len(dims), pd, pr, ctypes.byref(h)))
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None) and not sys.is_finalizing():
            self.lib.xtt_tensor_destroy(self.handle)
        self.handle = None

    # -- shape
    def degree(self):
        v = ctypes.c_int64()
        L.check(self.lib.xtt_tensor_order(self.handle, ctypes.byref(v)))
        return v.value

    @property
    def dimensions(self):
        d = self.degree()
        out = np.zeros(d, dtype=np.int64)
        L.check(self.lib.xtt_tensor_dims(self.handle, out.ctypes.data_as(L.c_int64_p)))
        return [int(v) for v in out]

    def all_ranks(self):
        out = np.zeros(self.degree() + 1, dtype=np.int64)
        L.check(self.lib.xtt_tensor_ranks(self.handle, out.ctypes.data_as(L.c_int64_p)))
        return [int(v) for v in out]

    def ranks(self):
        return self.all_ranks()[1:-1]

    def size(self):
        v = ctypes.c_int64()
        L.check(self.lib.xtt_tensor_size(self.handle, ctypes.byref(v)))
        return v.value

    @property
    def canonicalized(self):
        c, p = ctypes.c_int(), ctypes.c_int64()
        L.check(self.lib.xtt_tensor_get_canonical(self.handle, ctypes.byref(c), ctypes.byref(p)))
        return bool(c.value)

    @property
    def corePosition(self):
        c, p = ctypes.c_int(), ctypes.c_int64()
        L.check(self.lib.xtt_tensor_get_canonical(self.handle, ctypes.byref(c), ctypes.byref(p)))
        return p.value

    def assume_core_position(self, pos):
        L.check(self.lib.xtt_tensor_set_canonical(self.handle, 1, int(pos)))

    def set_canonical(self, canonicalized, pos=0):
        L.check(self.lib.xtt_tensor_set_canonical(self.handle, int(bool(canonicalized)), int(pos)))

    # -- data
    def get_flat(self):
        out = np.zeros(self.size())
        L.check(self.lib.xtt_tensor_get_cores(self.handle, out.ctypes.data_as(L.c_double_p), out.size))
        return out

    def set_flat(self, data, ranks=None):
        a, pa = _f64(data)
        if ranks is None:
            L.check(self.lib.xtt_tensor_set_cores(self.handle, pa, a.size))
        else:
            r, pr = _i64(ranks)
            L.check(self.lib.xtt_tensor_assign(self.handle, pr, pa, a.size))

    def _core_shape(self, k, r):
        n = self.dimensions[k]
        return (r[k], n, n, r[k + 1]) if self.is_operator else (r[k], n, r[k + 1])

    def get_cores(self):
        flat, r = self.get_flat(), self.all_ranks()
        out, off = [], 0
        for k in range(self.degree()):
            shp = self._core_shape(k, r)
            sz = int(np.prod(shp))
            out.append(flat[off:off + sz].reshape(shp).copy())
            off += sz
        return out

    def set_cores(self, cores):
        r = [1] + [int(c.shape[-1]) for c in cores]
        self.set_flat(np.concatenate([np.asarray(c, dtype=np.float64).ravel() for c in cores]), ranks=r)

    def get_component(self, k):
        return self.get_cores()[k]

    def copy(self):
        h = ctypes.c_void_p()
        L.check(self.lib.xtt_tensor_copy(self.handle, ctypes.byref(h)))
        return type(self)(ctx=self.ctx, _handle=h)

    def __imul__(self, f):
        L.check(self.lib.xtt_tensor_scale(self.handle, float(f)))
        return self

    def __itruediv__(self, f):
        return self.__imul__(1.0 / f)

    def __mul__(self, f):
        if not isinstance(f, (int, float, np.integer, np.floating)):
            return NotImplemented
        y = self.copy()
        y *= f
        return y

    __rmul__ = __mul__

    def __truediv__(self, f):
        return self * (1.0 / f)

    def __neg__(self):
        return self * -1.0

    # -- TTNetwork::operator+= / -= (src/xerus/ttNetwork.cpp:796-856)
    def __iadd__(self, other):
        if other is self:
            other = other.copy()
        L.check(self.lib.xtt_add(self.handle, other.handle, 1.0))
        return self

    def __isub__(self, other):
        if other is self:
            other = other.copy()
        L.check(self.lib.xtt_add(self.handle, other.handle, -1.0))
        return self

    def __add__(self, other):
        y = self.copy()
        y += other
        return y

    def __sub__(self, other):
        y = self.copy()
        y -= other
        return y

    # -- TTNetwork operations
    def move_core(self, position, keepRank=False):
        L.check(self.lib.xtt_move_core(self.handle, int(position), int(bool(keepRank))))

    def canonicalize_left(self):
        self.move_core(0)

    def canonicalize_right(self):
        self.move_core(self.degree() - 1)

    def round(self, arg, eps=None, spectra=False):
        """round(maxRanks: list, eps=EPSILON) | round(maxRank: int) | round(eps: float)
        (include/xerus/ttNetwork.h:352-373)."""
        d = self.degree()
        if isinstance(arg, (float, np.floating)):
            mr, e = [INT64_MAX] * (d - 1), float(arg)
        elif isinstance(arg, (int, np.integer)):
            if int(arg) <= 0:
                raise ValueError("MaxRank must be positive")
            mr, e = [int(arg)] * (d - 1), EPSILON
        else:
            mr, e = [int(v) for v in arg], EPSILON if eps is None else float(eps)
        m, pm = _i64(mr if d > 1 else [0])
        cap = sum(self.all_ranks()) * 4 + 16
        sp = np.zeros(cap)
        cnt = ctypes.c_int64()
        L.check(self.lib.xtt_round(self.handle, pm, e, sp.ctypes.data_as(L.c_double_p) if spectra else None, cap,
                                   ctypes.byref(cnt)))
        return sp[:cnt.value].copy() if spectra else None

    def frob_norm(self):
        v = ctypes.c_double()
        L.check(self.lib.xtt_frob_norm(self.handle, ctypes.byref(v)))
        return v.value


class TTTensor(_TT):
    """xerus::TTTensor on the device."""

    @staticmethod
    def random(dims, ranks, mean=0.0, stddev=1.0, ctx=None):
        """TTNetwork::random(dims, ranks, dist=N(mean, stddev)) (include/xerus/ttNetwork.h:128-169)."""
        ctx = ctx or Context.default()
        dims = list(dims)
        if isinstance(ranks, (int, np.integer)):
            ranks = [int(ranks)] * (len(dims) - 1)
        d, pd = _i64(dims)
        r, pr = _i64(list(ranks) if ranks else [1])
        h = ctypes.c_void_p()
        L.check(ctx.lib.xtt_tensor_random(ctx.handle, len(dims), pd, pr, float(mean), float(stddev), ctypes.byref(h)))
        return TTTensor(ctx=ctx, _handle=h)

    @staticmethod
    def from_cores(cores, ctx=None, canonicalized=False, core_position=0):
        dims = [int(c.shape[1]) for c in cores]
        t = TTTensor(dims, [1] + [int(c.shape[2]) for c in cores], ctx=ctx)
        t.set_cores(cores)
        t.set_canonical(canonicalized, core_position)
        return t

    def entries(self, positions):
        pos, pp = _i64(positions)
        out = np.zeros(pos.shape[0])
        L.check(self.lib.xtt_entries(self.handle, pp, pos.shape[0], out.ctypes.data_as(L.c_double_p)))
        return out


class TTOperator(_TT):
    """xerus::TTOperator on the device (cores (R_{k-1}, n, n, R_k))."""

    is_operator = True

    @staticmethod
    def from_cores(cores, ctx=None, canonicalized=False, core_position=0):
        dims = [int(c.shape[1]) for c in cores]
        t = TTOperator(dims, [1] + [int(c.shape[3]) for c in cores], ctx=ctx)
        t.set_cores(cores)
        t.set_canonical(canonicalized, core_position)
        return t

    def __matmul__(self, x):
        """A(i/2, j/2) * x(j&0) (or A * B for an operator B) as a TT; see ``apply``."""
        return apply(self, x)


def apply(A, x):
    """The TT of A x: xerus's TTStack product cast to a TTTensor (TTOperator for an
    operator x), src/xerus/ttStack.cpp:47-173; canonicalised at A's core position
    when A is canonical."""
    h = ctypes.c_void_p()
    L.check(x.lib.xtt_apply(A.handle, x.handle, ctypes.byref(h)))
    return type(x)(ctx=x.ctx, _handle=h)


def save_to_file(x, path):
    """misc::save_to_file(x, path) in xerus's binary format (include/xerus/misc/fileIO.h:103-162)."""
    L.check(x.lib.xtt_tensor_save(x.handle, os.fsencode(path)))


def load_from_file(path, ctx=None):
    """misc::load_from_file for a TTTensor or TTOperator data file; returns the device tensor."""
    ctx = ctx or Context.default()
    h = ctypes.c_void_p()
    L.check(ctx.lib.xtt_tensor_load(ctx.handle, os.fsencode(path), ctypes.byref(h)))
    # the kind is the file's header line, which the load has just validated
    with open(path, "rb") as f:
        op = f.readline().startswith(b"Xerus xerus::TTNetwork<true>")
    return (TTOperator if op else TTTensor)(ctx=ctx, _handle=h)


def file_encode(cores, is_operator=False, canonicalized=False, core_position=0):
    """Bytes of xerus's binary data file for the given cores (host only)."""
    lib = L.load()
    d = len(cores)
    dims = [int(c.shape[1]) for c in cores]
    ranks = [1] + [int(c.shape[-1]) for c in cores]
    flat = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.float64).ravel() for c in cores]))
    dv, pd = _i64(dims)
    rv, pr = _i64(ranks)
    size = ctypes.c_int64()
    L.check(lib.xtt_file_encode(int(bool(is_operator)), d, pd, pr, flat.ctypes.data_as(L.c_double_p),
                                int(bool(canonicalized)), int(core_position), None, 0, ctypes.byref(size)))
    buf = np.zeros(size.value, dtype=np.uint8)
    L.check(lib.xtt_file_encode(int(bool(is_operator)), d, pd, pr, flat.ctypes.data_as(L.c_double_p),
                                int(bool(canonicalized)), int(core_position), buf.ctypes.data_as(ctypes.c_void_p),
                                buf.size, ctypes.byref(size)))
    return buf.tobytes()


def file_decode(data):
    """(cores, is_operator, canonicalized, core_position) of a xerus binary data file's bytes (host only)."""
    lib = L.load()
    buf = np.frombuffer(bytes(data), dtype=np.uint8)
    op, order, cnt, canon, pos = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
    args = (buf.ctypes.data_as(ctypes.c_void_p), buf.size, ctypes.byref(op), ctypes.byref(order))
    L.check(lib.xtt_file_decode(*args, None, None, 0, None, 0, ctypes.byref(cnt), ctypes.byref(canon),
                                ctypes.byref(pos)))
    dims = np.zeros(order.value, dtype=np.int64)
    ranks = np.zeros(order.value + 1, dtype=np.int64)
    flat = np.zeros(cnt.value)
    L.check(lib.xtt_file_decode(*args, dims.ctypes.data_as(L.c_int64_p), ranks.ctypes.data_as(L.c_int64_p),
                                order.value, flat.ctypes.data_as(L.c_double_p), flat.size, ctypes.byref(cnt),
                                ctypes.byref(canon), ctypes.byref(pos)))
    cores, off = [], 0
    for k in range(order.value):
        shp = (ranks[k], dims[k], dims[k], ranks[k + 1]) if op.value else (ranks[k], dims[k], ranks[k + 1])
        sz = int(np.prod(shp))
        cores.append(flat[off:off + sz].reshape(shp))
        off += sz
    return cores, bool(op.value), bool(canon.value), int(pos.value)


def frob_norm(x):
    return x.frob_norm()


def dot(x, y):
    """value_t(x(i&0) * y(i&0))."""
    v = ctypes.c_double()
    L.check(x.lib.xtt_dot(x.handle, y.handle, ctypes.byref(v)))
    return v.value


def residual(A, x, b):
    """||A x - b|| / ||b|| in FP64 (no cancellation)."""
    v = ctypes.c_double()
    L.check(x.lib.xtt_residual(A.handle, x.handle, b.handle, ctypes.byref(v)))
    return v.value


class PerformanceData:
    """The parts of xerus::PerformanceData the sweep fills (include/xerus/performanceData.h)."""

    def __init__(self, active=True):
        self.active = active
        self.residuals, self.flags, self.energies = [], [], []

    def __bool__(self):
        return self.active


class ALSVariant:
    """xerus::ALSVariant (include/xerus/algorithms/als.h:37-207): SPD operators
    (assumeSPD), any operator (least squares through A^T A), or no operator
    (x approximates b)."""

    FLAG_FINISHED_HALFSWEEP = 1
    FLAG_FINISHED_FULLSWEEP = 3

    def __init__(self, sites, numHalfSweeps, localSolver, assumeSPD, useResidual=False):
        self.sites = sites
        self.numHalfSweeps = numHalfSweeps
        self.convergenceEpsilon = 1e-6
        self.useResidualForEndCriterion = useResidual
        self.preserveCorePosition = True
        self.assumeSPD = assumeSPD
        self.localSolver = localSolver  # "lapack" (exact) or "asd"
        self.precision = FP64
        self.local_tolerance = 1e-13
        self.local_max_iterations = 0
        self.residual_target = 0.0
        self.max_rank = 0
        self.svd_epsilon = 0.0
        self.exact_environment = False
        self.last_report = None

    def copy(self):
        v = ALSVariant(self.sites, self.numHalfSweeps, self.localSolver, self.assumeSPD, self.useResidualForEndCriterion)
        v.__dict__.update({k: val for k, val in self.__dict__.items() if k != "last_report"})
        return v

    def options(self, num_half_sweeps, eps, record):
        o = L.AlsOptions()
        L.check(L.load().xtt_als_default_options(ctypes.byref(o)))
        o.sites = self.sites
        o.local_solver = 1 if self.localSolver == "asd" else 0
        o.preserve_core_position = int(self.preserveCorePosition)
        o.precision = int(self.precision)
        o.num_half_sweeps = int(num_half_sweeps)
        o.convergence_epsilon = float(eps)
        o.local_tolerance = float(self.local_tolerance)
        o.local_max_iterations = int(self.local_max_iterations)
        o.residual_target = float(self.residual_target)
        o.record_residuals = int(bool(record))
        o.max_rank = int(self.max_rank)
        o.svd_epsilon = float(self.svd_epsilon)
        o.exact_environment = int(bool(self.exact_environment))
        o.assume_spd = int(bool(self.assumeSPD))
        o.use_residual = int(bool(self.useResidualForEndCriterion))
        return o

    def __call__(self, *args):
        """ALS(A, x, b[, numHalfSweeps: int | convergenceEpsilon: float][, perfData]) -> energy,
        or without an operator ALS(x, b[, ...]) minimising ||x - b|| (als.h:152-206)."""
        if len(args) >= 2 and isinstance(args[0], TTTensor):
            A, rest = None, args
        else:
            A, rest = args[0], args[1:]
        if len(rest) < 2 or len(rest) > 4:
            raise TypeError("ALSVariant(A, x, b[, numHalfSweeps | convergenceEpsilon][, perfData])")
        x, b = rest[0], rest[1]
        arg = rest[2] if len(rest) > 2 else None
        perfData = rest[3] if len(rest) > 3 else None
        if isinstance(arg, PerformanceData):
            arg, perfData = None, arg
        hs, eps = self.numHalfSweeps, self.convergenceEpsilon
        if isinstance(arg, (int, np.integer)):
            hs = int(arg)
        elif isinstance(arg, (float, np.floating)):
            eps = float(arg)
        record = bool(perfData)
        o = self.options(hs, eps, record)
        rep = L.AlsReport()
        cap = 4096
        res, flags, en = np.zeros(cap), np.zeros(cap, dtype=np.int64), np.zeros(cap)
        L.check(x.lib.xtt_als(A.handle if A is not None else None, x.handle, b.handle, ctypes.byref(o), ctypes.byref(rep),
                              res.ctypes.data_as(L.c_double_p), flags.ctypes.data_as(L.c_int64_p),
                              en.ctypes.data_as(L.c_double_p), cap))
        self.last_report = rep
        if perfData is not None and record:
            n = min(rep.micro_steps + 1, cap)
            perfData.residuals = list(res[:n])
            perfData.flags = list(flags[:n])
            perfData.energies = list(en[:rep.half_sweeps])
        return rep.energy


def als_batch(As, xs, bs, variant=None, numHalfSweeps=8, autotune=False):
    """Batched ALS_SPD: solves every (A_i, x_i, b_i) with one-site ALS in one
    persistent launch (x_i updated in place). Returns (energies, local CG
    iterations, {"milliseconds", "threads", "ctas_per_sm", "ctas", "tile"})."""
    v = (variant or ALS_SPD).copy()
    n = len(xs)
    if not (len(As) == n == len(bs)) or n == 0:
        raise ValueError("A, x and b lists must be non-empty and of equal length")
    ctx = xs[0].ctx
    o = v.options(numHalfSweeps, v.convergenceEpsilon, False)
    arr = ctypes.c_void_p * n
    pa = arr(*[t.handle for t in As])
    px = arr(*[t.handle for t in xs])
    pb = arr(*[t.handle for t in bs])
    en = np.zeros(n)
    it = np.zeros(n, dtype=np.int64)
    rep = L.BatchReport()
    L.check(ctx.lib.xtt_als_batch(ctx.handle, n, pa, px, pb, ctypes.byref(o), int(bool(autotune)),
                                  en.ctypes.data_as(L.c_double_p), it.ctypes.data_as(L.c_int64_p), ctypes.byref(rep)))
    return en, it, {"milliseconds": rep.milliseconds, "threads": rep.threads, "ctas_per_sm": rep.ctas_per_sm,
                    "tile": rep.tile,
                    "ctas": rep.ctas}


# the global variants (src/xerus/algorithms/als.cpp:556-563)
ALS = ALSVariant(1, 0, "lapack", False)
ALS_SPD = ALSVariant(1, 0, "lapack", True)
DMRG = ALSVariant(2, 0, "lapack", False)
DMRG_SPD = ALSVariant(2, 0, "lapack", True)
ASD = ALSVariant(1, 0, "asd", False)
ASD_SPD = ALSVariant(1, 0, "asd", True)


class SinglePointMeasurementSet:
    """xerus::SinglePointMeasurementSet (include/xerus/measurments.h:43-91)."""

    def __init__(self, positions=None, measuredValues=None):
        self.positions = np.zeros((0, 0), dtype=np.int64) if positions is None else np.asarray(positions, dtype=np.int64)
        self.measuredValues = np.zeros(0) if measuredValues is None else np.asarray(measuredValues, dtype=np.float64)

    @staticmethod
    def random(num, dims):
        dims = [int(v) for v in dims]
        out = np.zeros((int(num), len(dims)), dtype=np.int64)
        d, pd = _i64(dims)
        L.check(L.load().xtt_random_positions(int(num), len(dims), pd, out.ctypes.data_as(L.c_int64_p)))
        return SinglePointMeasurementSet(out, np.zeros(int(num)))

    def size(self):
        return int(self.positions.shape[0])

    def degree(self):
        return int(self.positions.shape[1]) if self.positions.ndim == 2 else 0

    def measure(self, tt):
        self.measuredValues = tt.entries(self.positions)

    def frob_norm(self):
        return float(np.sqrt(np.sum(self.measuredValues ** 2)))


# The retractions of retractions.cpp (xtt_retraction): submanifold (componentwise
# addition, SubmanifoldRetractionI / II), HOSVD (HOSVDRetractionI / II: round the sum
# back to the old ranks) and ALS (ALSRetractionI / II: two operator-free ALS half-sweeps).
SubmanifoldRetraction, HOSVDRetraction, ALSRetraction = 0, 1, 2


class GeometricCGVariant:
    """xerus::GeometricCGVariant (include/xerus/algorithms/cg.h:41-134) with the submanifold
    retraction and projective vector transport (GeometricCG): Riemannian CG on the TT
    manifold of x's ranks. Called as v(A, x, b[, numSteps | convergenceEpsilon][, perfData])
    or without an operator v(x, b, ...); returns ||b - A x||."""

    _entry = "xtt_geometric_cg_retraction"

    def __init__(self, numSteps=0, convergenceEpsilon=1e-8, assumeSymmetricPositiveDefiniteOperator=False,
                 retraction=None):
        self.numSteps = numSteps
        self.convergenceEpsilon = convergenceEpsilon
        self.assumeSymmetricPositiveDefiniteOperator = assumeSymmetricPositiveDefiniteOperator
        # SubmanifoldRetraction (default), HOSVDRetraction or ALSRetraction (retractions.h:59-88)
        self.retraction = SubmanifoldRetraction if retraction is None else retraction

    def copy(self):
        return type(self)(self.numSteps, self.convergenceEpsilon, self.assumeSymmetricPositiveDefiniteOperator,
                          self.retraction)

    def __call__(self, *args):
        if len(args) >= 2 and isinstance(args[0], TTTensor):
            A, rest = None, args
        else:
            A, rest = args[0], args[1:]
        x, b = rest[0], rest[1]
        arg = rest[2] if len(rest) > 2 else None
        perfData = rest[3] if len(rest) > 3 else None
        if isinstance(arg, PerformanceData):
            arg, perfData = None, arg
        steps, eps = self.numSteps, self.convergenceEpsilon
        if isinstance(arg, (int, np.integer)):
            steps = int(arg)
        elif isinstance(arg, (float, np.floating)):
            eps = float(arg)
        cap = max(16, steps + 2 if steps else 100000)
        trace = np.zeros(cap)
        res, cnt = ctypes.c_double(), ctypes.c_int64()
        L.check(getattr(x.lib, self._entry)(A.handle if A is not None else None, x.handle, b.handle, int(steps),
                                            float(eps), int(bool(self.assumeSymmetricPositiveDefiniteOperator)),
                                            int(self.retraction), ctypes.byref(res),
                                            trace.ctypes.data_as(L.c_double_p), cap,
                                            ctypes.byref(cnt)))
        if perfData is not None:
            perfData.residuals = list(trace[:min(cnt.value, cap)])
        return res.value


GeometricCG = GeometricCGVariant(0, 1e-8, False)


class SteepestDescentVariant(GeometricCGVariant):
    """xerus::SteepestDescentVariant (include/xerus/algorithms/steepestDescent.h) with the
    submanifold retraction (SteepestDescent); same calls as GeometricCGVariant."""

    _entry = "xtt_steepest_descent_retraction"


SteepestDescent = SteepestDescentVariant(0, 1e-8, False)


class RankOneMeasurementSet:
    """xerus::RankOneMeasurementSet (include/xerus/measurments.h:94-140): sample s is
    <x, u_1 (x) ... (x) u_d>. `positions[s][k]` is u_k of sample s; the vectors are held
    concatenated per sample in `vectors` (N x sum n_k)."""

    def __init__(self, vectors=None, measuredValues=None, dims=None):
        self.vectors = np.zeros((0, 0)) if vectors is None else np.ascontiguousarray(vectors, dtype=np.float64)
        self.dims = [int(v) for v in dims] if dims is not None else None
        self.measuredValues = np.zeros(self.vectors.shape[0]) if measuredValues is None else \
            np.asarray(measuredValues, dtype=np.float64)

    @staticmethod
    def random(num, dims_or_solution):
        """random(num, dims) or random(num, solution) (measured on the solution)."""
        sol = dims_or_solution if isinstance(dims_or_solution, _TT) else None
        dims = [int(v) for v in (sol.dimensions if sol is not None else dims_or_solution)]
        out = np.zeros((int(num), sum(dims)))
        d, pd = _i64(dims)
        L.check(L.load().xtt_random_rank_one(int(num), len(dims), pd, out.ctypes.data_as(L.c_double_p)))
        m = RankOneMeasurementSet(out, None, dims)
        if sol is not None:
            m.measure(sol)
        return m

    @property
    def positions(self):
        offs = np.cumsum([0] + self.dims)
        return [[self.vectors[s, offs[k]:offs[k + 1]] for k in range(len(self.dims))] for s in range(self.size())]

    def size(self):
        return int(self.vectors.shape[0])

    def degree(self):
        return len(self.dims) if self.dims else 0

    def measure(self, tt):
        out = np.zeros(self.size())
        L.check(tt.lib.xtt_entries_rank_one(tt.handle, self.vectors.ctypes.data_as(L.c_double_p), self.size(),
                                            out.ctypes.data_as(L.c_double_p)))
        self.measuredValues = out

    def frob_norm(self):
        return float(np.sqrt(np.sum(self.measuredValues ** 2)))


class ADFVariant:
    """xerus::ADFVariant (include/xerus/algorithms/adf.h:39-266) for single-point and
    rank-one measurement sets."""

    def __init__(self, maxIterations, targetResidualNorm, minimalResidualNormDecrease, precision=None):
        self.maxIterations = maxIterations
        self.targetResidualNorm = targetResidualNorm
        self.minimalResidualNormDecrease = minimalResidualNormDecrease
        # FP64, or MIXED: FP32 stacks and per-sample arithmetic, FP64 cores, QR and final check
        self.precision = FP64 if precision is None else precision

    def __call__(self, x, measurements, maxRanks=None, perfData=None):
        """ADFVariant::operator()(x, measurements[, maxRanks], perfData) (adf.h:248-266).
        With maxRanks, x may start at lower ranks and grows toward them (rank increases
        draw from the library's random state, see seed())."""
        if isinstance(maxRanks, PerformanceData):
            maxRanks, perfData = None, maxRanks
        val, pv = _f64(measurements.measuredValues)
        o = L.AdfOptions(int(self.maxIterations), float(self.targetResidualNorm),
                         float(self.minimalResidualNormDecrease), int(self.precision), 0)
        cap = max(16, int(self.maxIterations) + 2 if self.maxIterations else 100000)
        trace = np.zeros(cap)
        fin, cnt = ctypes.c_double(), ctypes.c_int64()
        if maxRanks is not None:
            if isinstance(measurements, RankOneMeasurementSet):
                raise NotImplementedError("maxRanks is supported for SinglePointMeasurementSet")
            d = len(x.dimensions)
            mr = [int(maxRanks)] * (d - 1) if np.isscalar(maxRanks) else [int(v) for v in maxRanks]
            if len(mr) != d - 1:
                raise ValueError("maxRanks needs one entry per inner bond")
            # every rank increase records one more point than its iterations
            cap = max(cap, 2 * cap + 2 * (d + 1))
            trace = np.zeros(cap)
            its = np.zeros(cap, dtype=np.int64)
            rks = np.zeros((cap, d - 1), dtype=np.int64)
            pos, pp = _i64(measurements.positions)
            mra, pm = _i64(mr)
            L.check(x.lib.xtt_adf_max_ranks(x.handle, pp, pv, pos.shape[0], pm, ctypes.byref(o), ctypes.byref(fin),
                                            trace.ctypes.data_as(L.c_double_p), its.ctypes.data_as(L.c_int64_p),
                                            rks.ctypes.data_as(L.c_int64_p), cap, ctypes.byref(cnt)))
            if perfData is not None:
                m = min(cnt.value, cap)
                perfData.residuals = list(trace[:m])
                perfData.iterations = list(its[:m])
                perfData.ranks = rks[:m].tolist()
            return fin.value
        if isinstance(measurements, RankOneMeasurementSet):
            vec, pu = _f64(measurements.vectors)
            L.check(x.lib.xtt_adf_rank_one(x.handle, pu, pv, vec.shape[0], ctypes.byref(o), ctypes.byref(fin),
                                           trace.ctypes.data_as(L.c_double_p), cap, ctypes.byref(cnt)))
        else:
            pos, pp = _i64(measurements.positions)
            L.check(x.lib.xtt_adf(x.handle, pp, pv, pos.shape[0], ctypes.byref(o), ctypes.byref(fin),
                                  trace.ctypes.data_as(L.c_double_p), cap, ctypes.byref(cnt)))
        if perfData is not None:
            perfData.residuals = list(trace[:min(cnt.value, cap)])
        return fin.value

    @staticmethod
    def gradient(x, measurements):
        """(0.5 ||P(x) - y||^2, [dL/dX_k]) for every core."""
        pos, pp = _i64(measurements.positions)
        val, pv = _f64(measurements.measuredValues)
        g = np.zeros(x.size())
        loss = ctypes.c_double()
        L.check(x.lib.xtt_adf_gradient(x.handle, pp, pv, pos.shape[0], ctypes.byref(loss),
                                       g.ctypes.data_as(L.c_double_p), g.size))
        return loss.value, _split(g, x)


def IHT(x, measurements, perfData=None, maxIterations=100):
    """xerus::IHT(x, measurements, perfData) (include/xerus/algorithms/iht.h:32) with an
    iteration cap (the reference runs 10^6 iterations); returns ||y - P(x)||."""
    pos, pp = _i64(measurements.positions)
    val, pv = _f64(measurements.measuredValues)
    cap = max(1, int(maxIterations))
    trace = np.zeros(cap)
    res, cnt = ctypes.c_double(), ctypes.c_int64()
    L.check(x.lib.xtt_iht(x.handle, pp, pv, pos.shape[0], int(maxIterations), ctypes.byref(res),
                          trace.ctypes.data_as(L.c_double_p), cap, ctypes.byref(cnt)))
    if perfData is not None:
        perfData.residuals = list(trace[:min(cnt.value, cap)])
    return res.value


def _split(flat, x):
    r, dims, out, off = x.all_ranks(), x.dimensions, [], 0
    for k in range(len(dims)):
        shp = (r[k], dims[k], r[k + 1])
        sz = int(np.prod(shp))
        out.append(flat[off:off + sz].reshape(shp).copy())
        off += sz
    return out


def als_energy_gradient(A, x, b):
    """(J, [dJ/dX_k]) for J(x) = <x, A x> - 2 <x, b>."""
    g = np.zeros(x.size())
    e = ctypes.c_double()
    L.check(x.lib.xtt_als_energy_gradient(A.handle, x.handle, b.handle, ctypes.byref(e),
                                          g.ctypes.data_as(L.c_double_p), g.size))
    return e.value, _split(g, x)


ADF = ADFVariant(0, 1e-8, 0.999)


def laplacian_cores(d, n, potentials=None, rank3=False, shift=0.0):
    """Cores of sum_i I x..x (L + V_i) x..x I with L = tridiag(-1, 2, -1) (n x n):
    rank 2 ([[L+V_0, I]], [[I, 0], [L+V_k, I]], [[I], [L+V]]) or, with rank3, the
    potential in its own channel ([[L+V_0, I, I]], [[I,0,0],[L,I,0],[V_k,0,I]], [[I],[L],[V]])."""
    L = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    I = np.eye(n)
    R = 3 if rank3 else 2
    cores = []
    for k in range(d):
        V = np.diag(potentials[k]) if potentials is not None else np.zeros((n, n))
        lk = L + (0 if rank3 else V) + shift * I / d
        rl, rr = (1 if k == 0 else R), (1 if k == d - 1 else R)
        c = np.zeros((rl, n, n, rr))
        if d == 1:
            c[0, :, :, 0] = L + V + shift * I
        elif k == 0:
            c[0, :, :, 0] = lk + (V if rank3 else 0)
            c[0, :, :, 1] = I
            if rank3:
                c[0, :, :, 2] = I
        elif k == d - 1:
            c[0, :, :, 0] = I
            c[1, :, :, 0] = lk
            if rank3:
                c[2, :, :, 0] = V
        else:
            c[0, :, :, 0] = I
            c[1, :, :, 0] = lk
            c[1, :, :, 1] = I
            if rank3:
                c[2, :, :, 0] = V
                c[2, :, :, 2] = I
        cores.append(c)
    return cores
