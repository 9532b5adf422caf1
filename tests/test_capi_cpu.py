"""CPU-only checks of the C ABI boundary: the library builds for sm_103a, loads,
and exports every function include/xtt.h declares (no compute calls)."""
import ctypes
import os
import shutil

import pytest

from xerus_gb300 import _lib


@pytest.fixture(scope="module")
def libpath():
    if not os.path.exists(_lib.LIB_PATH):
        if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
            pytest.skip("nvcc not available to build libxtt.so")
        from xerus_gb300 import build
        build.build()
    return _lib.LIB_PATH


def test_header_declares_the_boundary():
    names = _lib.declared_functions()
    for required in ["xtt_move_core", "xtt_round", "xtt_dot", "xtt_frob_norm", "xtt_als", "xtt_adf",
                     "xtt_adf_gradient", "xtt_als_energy_gradient", "xtt_tensor_random", "xtt_random_positions"]:
        assert required in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in _lib.declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_declared_symbol():
    assert set(_lib.declared_functions()) <= set(_lib._SIGNATURES)


def test_struct_layouts_match_header(tmp_path):
    """sizeof/offsetof of the option and report structs, compiled from the header, match ctypes."""
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    import subprocess
    structs = {"xtt_als_options": _lib.AlsOptions, "xtt_als_report": _lib.AlsReport, "xtt_adf_options": _lib.AdfOptions}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{_lib.HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for py in structs.values():
        want.append(ctypes.sizeof(py))
        want.extend(getattr(py, f).offset for f, _ in py._fields_)
    assert got == want


def test_version_and_error_without_gpu(libpath):
    lib = _lib.load(libpath)
    assert b"xtt" in lib.xtt_version()
    # argument checks run on the host and fail loudly before touching a device
    assert lib.xtt_context_create(0, None) == 1
    assert b"NULL" in lib.xtt_last_error()


def test_rank_one_random_matches_reference(libpath, golden):
    """RankOneMeasurementSet::random on the host: the reference's Gaussian vectors in its
    sort order, after a TTTensor::random draw (same engine and normal distribution)."""
    import numpy as np
    import xerus_gb300 as xg
    z = golden("adf_rankone")
    dims = [4, 5, 4, 5]
    xg.seed(0xBAADF00D)
    # the target's cores consume the first draws: 1*4*2 + 2*5*2 + 2*4*2 + 2*5*1
    burn = np.zeros(8 + 20 + 16 + 10)
    xg._lib.load().xtt_random_normal(0.0, 1.0, burn.size, burn.ctypes.data_as(xg._lib.c_double_p))
    m = xg.RankOneMeasurementSet.random(300, dims)
    np.testing.assert_array_equal(m.vectors, z["vectors"])
    assert [list(map(len, p)) for p in m.positions[:1]] == [dims]
