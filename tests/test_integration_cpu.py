"""The C++ forwarding layer of the integration guide (tests/integration/
xerus_forwarding.cpp) compiles against the reference's own headers and links
against the reference library and libxtt.so: every xerus call it makes and every
C ABI entry point it forwards to exist with the signatures used. A link check
on the CPU; it needs the xerus sources (__graft_entry__.reference_dir()) and the
reference library built from them, so it is skipped where they are absent."""
import os
import shutil
import subprocess

import pytest

from xerus_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_forwarding_layer_compiles_and_links(tmp_path):
    import __graft_entry__
    ref = __graft_entry__.reference_dir()
    if not ref:
        pytest.skip("the xerus sources are not available on this host")
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    refdir = os.path.join(ROOT, "oracle", "_ref")
    if not os.path.exists(os.path.join(refdir, "libxerus_ref.so")):
        subprocess.run(["make", "-j8", f"REF={ref}"], cwd=os.path.join(ROOT, "oracle", "ref"), check=True,
                       stdout=subprocess.DEVNULL)
    if not os.path.exists(_lib.LIB_PATH):
        from xerus_gb300 import build
        build.build()
    import scipy
    blasdir = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    blas = [f for f in os.listdir(blasdir) if f.startswith("libscipy_openblas")]
    exe = str(tmp_path / "forwarding")
    cmd = ["g++", "-std=c++14", "-O0", "-include", "cstdint", "-DXERUS_NO_FANCY_CALLSTACK", "-DXERUS_LOG_INFO",
           "-w", "-I" + os.path.join(ROOT, "oracle", "ref", "shim"), "-I" + os.path.join(ref, "include"),
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "integration", "xerus_forwarding.cpp"),
           "-o", exe, "-L" + refdir, "-lxerus_ref", _lib.LIB_PATH, os.path.join(blasdir, blas[0]),
           "-Wl,-rpath," + refdir, "-Wl,-rpath," + os.path.dirname(_lib.LIB_PATH), "-Wl,-rpath," + blasdir,
           "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # the binary loads (all shared libraries resolve) and exits without touching a GPU
    assert subprocess.run([exe], capture_output=True).returncode == 0
