"""Regenerates the golden fixtures in this folder from the xerus reference.

The reference is compiled in place by ``oracle/ref/Makefile`` (outputs under
``oracle/_ref/``, never committed) and ``oracle/_ref/golden_driver`` is run once
per case with one BLAS/OpenMP thread, so every number is reproducible. Each
case's ``.npy`` outputs are packed into ``<case>.npz`` here.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py als round  # selected cases

Needs the reference sources at $XERUS_REF and SciPy's bundled OpenBLAS; the
fixtures record the OpenBLAS build they came from.
"""
import glob
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = ["rng", "tt_random", "dot", "movecore", "round", "als", "dmrg", "adf", "adf_cfg5", "fileio", "als_nonspd", "arith", "adf_rankone", "gcg", "adf_rankinc", "qc_gap", "retractions", "iht"]


def main(argv):
    cases = argv[1:] or CASES
    ref = os.environ.get("XERUS_REF")
    if not ref:
        raise SystemExit("set XERUS_REF to the xerus source tree")
    subprocess.run(["make", "-j8", f"REF={ref}"], cwd=os.path.join(ROOT, "oracle", "ref"), check=True)
    driver = os.path.join(ROOT, "oracle", "_ref", "golden_driver")
    import scipy
    blas = scipy.show_config(mode="dicts")["Build Dependencies"]["blas"]
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    for case in cases:
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([driver, case, tmp], check=True, env=env)
            arrays = {os.path.basename(f)[:-4]: np.load(f) for f in sorted(glob.glob(os.path.join(tmp, "*.npy")))}
        arrays["_meta_openblas"] = np.array(f"{blas.get('name')} {blas.get('version')}")
        arrays["_meta_reference"] = np.array("libxerus/xerus 3.0.1, seed 0xBAADF00D, 1 thread")
        out = os.path.join(HERE, f"{case}.npz")
        np.savez_compressed(out, **arrays)
        print(f"{case}: {len(arrays)} arrays -> {os.path.relpath(out, ROOT)} ({os.path.getsize(out) // 1024} KiB)")


if __name__ == "__main__":
    main(sys.argv)
