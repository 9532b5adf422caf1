"""Times the xerus reference itself (built by this folder's Makefile into
oracle/_ref/) on this host's cores for the benchmark configurations, and writes
oracle/ref_cpu_times.json, which bench.py reports beside its own CPU legs with
the host it was measured on. The reference is compiled from its sources in
place; it is not shipped, and the GPU host, which has no copy of those sources,
does not run it.

    python oracle/ref/time_reference.py

Configurations (wall clock around the algorithm call, PerformanceData inactive):
  1: ALS_SPD d=8 n=4 Laplacian, x rank 8 for 20 half-sweeps (convergenceEpsilon 0)
     and x rank 32 for the 2 half-sweeps that reach residual 1e-8;
  2: move_core(31), round(32) and the dot product on d=32 n=4 rank-64 tensors;
  4: ALS_SPD with 8 half-sweeps on a random sample of the 4096 batch instances,
     one instance per OpenMP thread, BLAS single-threaded: instances per second;
  5: 50 ADF iterations, d=10 n=8 rank 6, 200 000 samples.
"""
import glob
import json
import os
import platform
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def run(case, threads, blas_threads=None, prepare=None):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS=str(blas_threads or threads))
    with tempfile.TemporaryDirectory() as tmp:
        if prepare:
            prepare(tmp)
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "golden_driver"), case, tmp], check=True, env=env)
        return {os.path.basename(f)[:-4]: float(np.load(f)[0]) for f in glob.glob(os.path.join(tmp, "*.npy"))}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    ref = os.environ.get("XERUS_REF")
    if not ref:
        raise SystemExit("set XERUS_REF to the xerus source tree")
    subprocess.run(["make", "-j8", f"REF={ref}"], cwd=HERE, check=True, stdout=subprocess.DEVNULL)
    import scipy
    import bench
    nproc = os.cpu_count()
    blas = scipy.show_config(mode="dicts")["Build Dependencies"]["blas"]
    out = {"host": {"cpu": cpu_model(), "machine": platform.machine(), "cores": nproc,
                    "openblas": f"{blas.get('name')} {blas.get('version')}"},
           "note": "the compiled xerus reference on this build host, not on the GPU host"}
    out["cfg1"] = {f"threads_{t}": run("time_cfg1", t) for t in (1, nproc)}
    out["cfg2"] = {f"threads_{t}": run("time_cfg2", t) for t in (1, nproc)}
    params = bench.config4_params(4096)
    rng = np.random.default_rng(41)
    sample = sorted(int(i) for i in rng.choice(len(params), 48, replace=False))

    def write_params(tmp):
        with open(os.path.join(tmp, "cfg4_params.txt"), "w") as f:
            for i in sample:
                d, n, shift, rb, rx = params[i]
                f.write(f"{d} {n} {shift!r} {rb} {rx} {bench.SEED + i}\n")

    r4 = run("time_cfg4", nproc, 1, write_params)
    r4["instances_per_s"] = r4["sample_instances"] / r4["sample_seconds"]
    r4["sample"] = f"{len(sample)} instances drawn at random from the 4096 (same shapes and seeds as the batch)"
    out["cfg4"] = {f"threads_{nproc}": r4}
    out["cfg5"] = {f"threads_{nproc}": run("time_cfg5", nproc)}
    path = os.path.join(ROOT, "oracle", "ref_cpu_times.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
