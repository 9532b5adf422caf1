"""Shared test helpers: golden-fixture readers and comparison tolerances."""
import numpy as np

from oracle import xtt_oracle as o

# FP64 parity bar against the reference for energies, residuals, norms, dot
# products, singular values and probe entries (relative).
REL_TOL = 1e-10


def tt_of(z, name, canonicalized=True, core_position=0):
    x = o.tt_from_flat([int(v) for v in z[name + "_dims"]], [int(v) for v in z[name + "_ranks"]], z[name + "_cores"])
    x.canonicalized, x.core_position = canonicalized, core_position
    return x


def op_of(z, name):
    return o.op_from_flat([int(v) for v in z[name + "_dims"]], [int(v) for v in z[name + "_ranks"]], z[name + "_cores"])


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def fnv1a(pos):
    h = 1469598103934665603
    for v in np.asarray(pos).ravel().tolist():
        h = ((h ^ int(v)) * 1099511628211) & ((1 << 64) - 1)
    return h
