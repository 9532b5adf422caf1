"""Parity of the CUDA path (through the C ABI) with the xerus reference's golden
vectors and the CPU oracle, on the GPU. Tolerances: integer results (ranks,
sample positions, random streams) bit-exact; FP64 quantities within 1e-10
relative (REL_TOL) unless a test states otherwise."""
import numpy as np
import pytest

from oracle import xtt_oracle as o
from tests.helpers import REL_TOL, fnv1a, op_of, rel_err, tt_of

pytestmark = pytest.mark.gpu

xg = pytest.importorskip("xerus_gb300")


@pytest.fixture(scope="module")
def ctx():
    from xerus_gb300 import build
    build.build()
    return xg.Context(0)


def dev_tt(ctx, x):
    return xg.TTTensor.from_cores(x.cores, ctx=ctx, canonicalized=x.canonicalized, core_position=x.core_position)


def dev_op(ctx, A):
    return xg.TTOperator.from_cores(A.cores, ctx=ctx)


def host_tt(t):
    return o.TT(t.get_cores(), t.canonicalized, t.corePosition)


# ------------------------------------------------------------------ random state (host side of the library)

def test_random_streams_match_reference(ctx, golden):
    """The engine and integer draws are bit-exact; the polar method's std::log
    comes from the platform's libm and compiler (FMA contraction), which may round
    the last bits differently on aarch64 than on the x86-64 host that wrote the
    fixtures: allow 16 ulp."""
    z = golden("rng")
    xg.seed(0xBAADF00D)
    out = np.zeros(257)
    xg._lib.load().xtt_random_normal(0.0, 1.0, 257, out.ctypes.data_as(xg._lib.c_double_p))
    np.testing.assert_array_max_ulp(out, z["rng_normal"], maxulp=16)
    xg.seed(0xBAADF00D)
    m = xg.SinglePointMeasurementSet.random(64, [2, 3, 4, 5, 7, 8, 10, 1000])
    rs = o.RandomEngine()
    assert np.array_equal(m.positions, o.random_positions(64, [2, 3, 4, 5, 7, 8, 10, 1000], rs))


def test_tt_random_and_positions(ctx, golden):
    z = golden("tt_random")
    xg.seed(0xBAADF00D)
    x = xg.TTTensor.random([3, 4, 2, 5], [2, 7, 3], ctx=ctx)
    assert [1] + x.ranks() + [1] == list(z["small_ranks_after"])
    assert rel_err(o.tt_full(host_tt(x)).ravel(), z["small_full"]) < REL_TOL
    xg.seed(0xBAADF00D)
    y = xg.TTTensor.random([4] * 8, 8, ctx=ctx)
    assert rel_err(y.entries(z["d8_probe_pos"]), z["d8_probe_val"]) < REL_TOL
    assert abs(y.frob_norm() / z["d8_norm"][0] - 1) < REL_TOL
    a = golden("adf")
    xg.seed(0xBAADF00D)
    xg.TTTensor.random([4, 5, 3, 5, 4, 3], 3, ctx=ctx)
    m = xg.SinglePointMeasurementSet.random(2000, [4, 5, 3, 5, 4, 3])
    assert np.array_equal(m.positions, a["small_positions"].astype(np.int64))


# ------------------------------------------------------------------ dot, norm, move_core, round

def test_dot_and_norm_cfg2(ctx, golden):
    z = golden("dot")
    xg.seed(0xBAADF00D)
    x = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    y = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    assert [1] + x.ranks() + [1] == list(z["cfg2_ranks_x"])
    assert abs(xg.dot(x, y) / z["cfg2_dot_xy"][0] - 1) < REL_TOL
    assert abs(x.frob_norm() / z["cfg2_norm_x"][0] - 1) < REL_TOL
    assert abs(y.frob_norm() / z["cfg2_norm_y"][0] - 1) < REL_TOL
    assert rel_err(x.entries(z["cfg2_x_probe_pos"]), z["cfg2_x_probe_val"]) < REL_TOL
    a, b = dev_tt(ctx, tt_of(z, "small_a", False)), dev_tt(ctx, tt_of(z, "small_b", False))
    assert abs(xg.dot(a, b) / z["small_dot"][0] - 1) < REL_TOL
    assert abs(a.frob_norm() / np.sqrt(o.tt_dot(tt_of(z, "small_a"), tt_of(z, "small_a"))) - 1) < REL_TOL


@pytest.mark.parametrize("tag", ["keep", "drop"])
def test_qc_rank_rule_with_clear_gap_exact(ctx, golden, tag):
    """Rank-revealing move_core on x + s w stacked in block cores (every bond rescaled by
    a diagonal, so no pivot choice is a tie): s = 1e-10 puts the w part's R_kk at
    1e-13..1e-11 R_00 (kept: far above 16 eps R_00), s = 1e-17 at or below 2.5e-16 R_00
    (dropped wherever R_00 > 0, the reference's signed rule). No decision is near the
    cutoff, so the ranks must equal the reference's exactly, in both sweep directions
    and to an inner core."""
    z = golden("qc_gap")
    zz = tt_of(z, f"{tag}_z", canonicalized=False)
    for p in (6, 0, 3):
        y = dev_tt(ctx, zz)
        y.move_core(p, False)
        assert [1] + y.ranks() + [1] == list(z[f"{tag}_qc_to{p}_ranks"])
        assert rel_err(y.entries(z[f"{tag}_qc_to{p}_probe_pos"]), z[f"{tag}_qc_to{p}_probe_val"]) < 1e-9


def test_move_core_qr_and_rank_revealing(ctx, golden):
    z = golden("movecore")
    for p in (5, 2, 0, 3):
        y = dev_tt(ctx, tt_of(z, "x"))
        y.move_core(p, True)
        assert y.canonicalized and y.corePosition == p
        assert rel_err(y.entries(z[f"qr_to{p}_probe_pos"]), z[f"qr_to{p}_probe_val"]) < REL_TOL
        assert abs(np.linalg.norm(y.get_component(p)) / z[f"qr_to{p}_corenorm"][0] - 1) < REL_TOL
        cores = y.get_cores()
        for k in range(p):  # left-orthogonal
            m = cores[k].reshape(-1, cores[k].shape[2])
            assert np.allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-12)
        for k in range(p + 1, len(cores)):  # right-orthogonal
            m = cores[k].reshape(cores[k].shape[0], -1)
            assert np.allclose(m @ m.T, np.eye(m.shape[0]), atol=1e-12)
    # rank-deficient (x + 2x in doubled ranks): the QC rank rule; ranks where the
    # reference's decision is clear (R_kk exactly at rounding level) must agree
    # with the oracle run on the same input, entries always
    zz = tt_of(z, "z", canonicalized=False)
    for p in (5, 0):
        y = dev_tt(ctx, zz)
        y.move_core(p, False)
        ref = zz.copy()
        o.move_core(ref, p, keep_rank=False)
        assert rel_err(y.entries(z[f"qc_to{p}_probe_pos"]), z[f"qc_to{p}_probe_val"]) < 1e-9
        # every rank is at least the true rank (x's ranks) and at most the representation's
        assert all(a >= b for a, b in zip(y.ranks(), tt_of(z, "x").ranks))
        assert all(a <= b for a, b in zip(y.ranks(), zz.ranks))


@pytest.mark.parametrize("mid", [128, 72, 100])
def test_move_core_keep_rank_wide_cores(ctx, mid):
    """keepRank move_core over cores with more than 64 columns (512 x mid moving right, its
    transpose moving left): the blocked Householder QR (32-column panels, the last one of
    8 columns for mid = 72; mid = 100 leaves a 4-column panel, which the cluster kernel
    does not take, so the unblocked factorisation runs). Entries against the oracle,
    cores orthonormal to rounding, ranks kept."""
    rng = np.random.default_rng(21)
    n, ranks = 8, [1, 8, 64, mid, 64, 8, 1]
    cores = [rng.standard_normal((ranks[k], n, ranks[k + 1])) / np.sqrt(ranks[k] * n) for k in range(6)]
    xh = o.TT([c.copy() for c in cores])
    pos = np.random.default_rng(4).integers(0, n, size=(64, 6))
    ref = o.tt_entries(xh, pos)
    x = xg.TTTensor.from_cores(cores, ctx=ctx)
    for p in (5, 0, 3):
        x.move_core(p, True)
        assert x.ranks() == ranks[1:-1] and x.corePosition == p
        assert rel_err(x.entries(pos), ref) < 1e-10
        cs = x.get_cores()
        for k in range(p):
            m = cs[k].reshape(-1, cs[k].shape[2])
            assert np.allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-12)
        for k in range(p + 1, len(cs)):
            m = cs[k].reshape(cs[k].shape[0], -1)
            assert np.allclose(m @ m.T, np.eye(m.shape[0]), atol=1e-12)


def test_move_core_cholesky_qr_cfg2(ctx, golden):
    """Rank-revealing move_core of the d=32, n=4, rank-64 tensor (its 256 x 64 cores take
    the Cholesky QR): ranks kept, entries and norm against the reference, cores
    orthonormal to rounding, in both directions."""
    z = golden("dot")
    xg.seed(0xBAADF00D)
    x = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    for p in (31, 0, 17):
        x.move_core(p, False)
        assert x.corePosition == p and [1] + x.ranks() + [1] == list(z["cfg2_ranks_x"])
        assert rel_err(x.entries(z["cfg2_x_probe_pos"]), z["cfg2_x_probe_val"]) < REL_TOL
        assert abs(np.linalg.norm(x.get_component(p)) / z["cfg2_norm_x"][0] - 1) < REL_TOL
        cores = x.get_cores()
        for k in range(p):
            m = cores[k].reshape(-1, cores[k].shape[2])
            assert np.allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-12)
        for k in range(p + 1, len(cores)):
            m = cores[k].reshape(cores[k].shape[0], -1)
            assert np.allclose(m @ m.T, np.eye(m.shape[0]), atol=1e-12)


def test_round_cfg2(ctx, golden):
    r = golden("round")
    xg.seed(0xBAADF00D)
    x = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    y = x.copy()
    spectra = y.round(32, spectra=True)
    assert [1] + y.ranks() + [1] == list(r["cfg2_round_ranks"])
    assert rel_err(spectra, r["cfg2_round_spectra"]) < REL_TOL
    assert abs(y.frob_norm() / r["cfg2_round_norm"][0] - 1) < REL_TOL
    assert abs(xg.dot(y, x) / r["cfg2_round_dot_x"][0] - 1) < REL_TOL
    assert rel_err(y.entries(r["cfg2_round_probe_pos"]), r["cfg2_round_probe_val"]) < REL_TOL


def test_svd_paths_agree(ctx):
    """The DMRG split through the QR-preconditioned Jacobi SVD (the default; tall
    128 x 128 and wide 64 x 128 splits at rank 16) and through plain one-sided
    Jacobi: same ranks, same energies, the same iterate to the local CG tolerance.
    Rounding through the mixed-precision Jacobi (the default) and plain Jacobi:
    same ranks, spectra and tensor to rounding."""
    out = {}
    try:
        for path in ("jacobi", "auto"):
            ctx.set_svd_path(path)
            d, n = 12, 8
            rng = np.random.default_rng(7)
            V = [rng.uniform(0.0, 1.0, n) for _ in range(d)]
            xg.seed(11)
            A = xg.TTOperator.from_cores(xg.laplacian_cores(d, n, potentials=V, rank3=True), ctx=ctx)
            b = xg.TTTensor.random([n] * d, 4, ctx=ctx)
            xd = xg.TTTensor.random([n] * d, 16, ctx=ctx)
            xd /= xd.frob_norm()
            v = xg.DMRG_SPD.copy()
            v.convergenceEpsilon = 0.0
            v.exact_environment = True
            e = v(A, xd, b, 2)
            xg.seed(0xBAADF00D)
            xr = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
            sp = np.array(xr.round(32, spectra=True))
            out[path] = (xd, e, xd.ranks(), xr, sp)
    finally:
        ctx.set_svd_path("auto")
    # rounding: the mixed-precision Jacobi (AUTO) and plain FP64 Jacobi
    assert out["auto"][3].ranks() == out["jacobi"][3].ranks()
    assert np.max(np.abs(out["auto"][4] - out["jacobi"][4]) / out["jacobi"][4]) < 1e-12
    assert (out["auto"][3] - out["jacobi"][3]).frob_norm() / out["jacobi"][3].frob_norm() < 1e-12
    assert out["auto"][2] == out["jacobi"][2]
    assert abs(out["auto"][1] / out["jacobi"][1] - 1) < 1e-10
    # the local systems' solutions reach norms ~1e7 here; rounding-level changes of
    # a core move the iterate by ~1e-8 relative, within the local CG tolerance
    xa, xj = out["auto"][0], out["jacobi"][0]
    assert (xa - xj).frob_norm() / xj.frob_norm() < 1e-6


@pytest.mark.parametrize("svd_path", ["auto", "jacobi"])
def test_dmrg_rank_growth(ctx, svd_path):
    """DMRG with rank growth (max rank 12, SVD cutoff 1e-8, exact environments) on a
    d=8, n=4 Laplacian with potential: ranks exact, energy and entries against the
    oracle, through both SVD paths (the preconditioned one drops the rows of the
    pivoted R far below the cutoff)."""
    d, n = 8, 4
    rng = np.random.default_rng(3)
    V = [rng.uniform(0.0, 1.0, n) for _ in range(d)]
    cores = xg.laplacian_cores(d, n, potentials=V, rank3=True)
    xg.seed(5)
    b = xg.TTTensor.random([n] * d, 3, ctx=ctx)
    x0 = xg.TTTensor.random([n] * d, 4, ctx=ctx)
    x0 /= x0.frob_norm()
    Ah, bh, xh = o.TTOp([np.array(c) for c in cores]), host_tt(b), host_tt(x0)
    try:
        ctx.set_svd_path(svd_path)
        A, x = xg.TTOperator.from_cores(cores, ctx=ctx), x0.copy()
        v = xg.DMRG_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.exact_environment = True
        v.max_rank = 12
        v.svd_epsilon = 1e-8
        energy = v(A, x, b, 3)
    finally:
        ctx.set_svd_path("auto")
    ref = xh.copy()
    r = o.als_spd(Ah, ref, bh, 2, 3, 0.0, exact_environment=True, max_rank=12, svd_epsilon=1e-8)
    assert x.ranks() == ref.ranks
    assert max(x.ranks()) == 12
    assert abs(energy / r.energy - 1) < 1e-10
    pos = np.random.default_rng(9).integers(0, n, size=(64, d))
    assert rel_err(x.entries(pos), o.tt_entries(ref, pos)) < 1e-8


@pytest.mark.parametrize("form,tol", [("tf32x3", 1e-4), ("bf16x3", 1e-4), ("tf32", 1e-2)])
def test_round_dot_precision_forms(ctx, golden, form, tol):
    """Precision forms of the d=32, n=4, rank-64 rounding: the contractions of move_core, round and dot
    on the tensor cores (QR and SVD FP64). Same ranks; singular values, norm and dot
    product within the form's error of the FP64 results: per contraction split TF32
    errs ~5e-7 (FP32 accumulation over K = 256), as does split BF16 (three pieces, six
    products), TF32 ~5e-4, and the 31 absorptions
    of a d=32 sweep compound them (measured 1.4e-5 and ~3e-3)."""
    r = golden("round")
    xg.seed(0xBAADF00D)
    x = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    y = xg.TTTensor.random([4] * 32, 64, 0.0, 0.125, ctx=ctx)
    d64 = xg.dot(x, y)
    try:
        ctx.set_contraction_precision(form)
        z = x.copy()
        sp = np.array(z.round(32, spectra=True))
        dt = xg.dot(x, y)
        ctx.profile(True)
        xg.dot(x, y)
        ctx.profile(False)
        assert ctx.profile_get("gemm_tc")[0] > 0  # the contractions ran on the tensor cores
    finally:
        ctx.set_contraction_precision("fp64")
    assert [1] + z.ranks() + [1] == list(r["cfg2_round_ranks"])
    assert np.max(np.abs(sp - r["cfg2_round_spectra"]) / np.abs(r["cfg2_round_spectra"])) < tol
    assert abs(z.frob_norm() / r["cfg2_round_norm"][0] - 1) < tol
    # the dot of independent tensors is far below |x| |y| (cancellation): its error is
    # measured on the scale of the accumulated products
    assert abs(dt - d64) / (x.frob_norm() * y.frob_norm()) < tol


@pytest.mark.parametrize("svd_path", ["auto", "jacobi"])
def test_round_odd_shapes(ctx, svd_path):
    """Rounding with odd bond sizes (37 x 37 bonds of a d=8, n=3 TT of rank 37)
    through the mixed-precision Jacobi (AUTO) and plain Jacobi: ranks exact,
    spectra and entries against the oracle's LAPACK-based round."""
    d, n, r = 8, 3, 37
    rng = np.random.default_rng(17)
    ranks = [1] + [min(r, n ** k, n ** (d - k)) for k in range(1, d)] + [1]
    cores = [rng.standard_normal((ranks[k], n, ranks[k + 1])) / np.sqrt(ranks[k] * n) for k in range(d)]
    xh = o.TT([c.copy() for c in cores])
    try:
        ctx.set_svd_path(svd_path)
        x = xg.TTTensor.from_cores(cores, ctx=ctx)
        sp = np.array(x.round(20, spectra=True))
    finally:
        ctx.set_svd_path("auto")
    spr = []
    o.tt_round(xh, 20, o.EPSILON, spr)
    assert x.ranks() == xh.ranks
    assert rel_err(sp, np.concatenate(spr)) < 1e-10
    pos = np.random.default_rng(3).integers(0, n, size=(50, d))
    assert rel_err(x.entries(pos), o.tt_entries(xh, pos)) < 1e-10


def _tt_with_bond_spectrum(sigma, seed):
    """d=6, n=4 TT of ranks [4, 16, 64, 16, 4] whose middle bond (cores 2 | 3) has exactly the
    singular values `sigma` (64): cores 0-2 left-orthogonal, core 3 = U diag(sigma) V^T
    (U, V orthogonal), cores 4-5 right-orthogonal. round(32) factors that bond's 64 x 64
    matrix: the product-refined SVD and the Cholesky QR of a core with condition
    sigma_max / sigma_min."""
    rng = np.random.default_rng(seed)
    n, ranks = 4, [1, 4, 16, 64, 16, 4, 1]
    cores = []
    for k in range(3):
        q, _ = np.linalg.qr(rng.standard_normal((ranks[k] * n, ranks[k + 1])))
        cores.append(q.reshape(ranks[k], n, ranks[k + 1]))
    q, _ = np.linalg.qr(rng.standard_normal((64, 64)))
    u, _ = np.linalg.qr(rng.standard_normal((64, 64)))  # non-orthogonal rows: Gram condition sigma_max^2 / sigma_min^2
    cores.append((u @ (np.asarray(sigma)[:, None] * q.T)).reshape(64, n, 16))
    for k in range(4, 6):
        q, _ = np.linalg.qr(rng.standard_normal((n * ranks[k + 1], ranks[k])))
        cores.append(q.T.reshape(ranks[k], n, ranks[k + 1]))
    return cores


@pytest.mark.parametrize("spectrum", ["separated", "duplicate", "graded", "deficient"])
def test_round_refinement_and_cholesky_qr_fallbacks(ctx, spectrum):
    """The round's fast paths against the oracle's LAPACK round on one 64 x 64 bond:
    separated singular values (product refinement, Cholesky QR); an exactly repeated pair
    (the refinement's gap test declines, Jacobi sweeps run); a 1e-6 graded spectrum (the
    FP32 start is too far off for the smallest singular vectors, so the refinement's last
    corrections stay large and it declines; the Cholesky QR's gate fails, pivoted
    Householder runs); eight exact zeros (both decline; the QC rank rule and the truncation
    drop them). Ranks exact, spectra and entries 1e-10; the rank-revealing move_core of the
    same tensor likewise."""
    rng = np.random.default_rng(5)
    sigma = np.sort(rng.uniform(0.5, 2.0, 64))[::-1]
    if spectrum == "duplicate":
        sigma[5] = sigma[4]
    elif spectrum == "graded":
        sigma = np.logspace(0, -6, 64)
    elif spectrum == "deficient":
        sigma[-8:] = 0.0
    def profiled_round(sig):
        t = xg.TTTensor.from_cores(_tt_with_bond_spectrum(sig, 11), ctx=ctx)
        ctx.profile(True)
        try:
            out = np.array(t.round(32, spectra=True))
            counts = {k: ctx.profile_get(k)[0] for k in ("svd_refine", "svd_sweeps", "qr_gram", "qr")}
        finally:
            ctx.profile(False)
        return t, out, counts

    cores = _tt_with_bond_spectrum(sigma, 11)
    xh = o.TT([c.copy() for c in cores])
    x, sp, counts = profiled_round(sigma)
    # the path each case is meant to take
    if spectrum == "separated":
        assert counts["svd_refine"] == 1 and counts["svd_sweeps"] == 0
    if spectrum in ("duplicate", "graded"):
        assert counts["svd_refine"] == 1 and counts["svd_sweeps"] == 1
    if spectrum == "graded":
        # the right-to-left move_core factors the 64 x 64 core of condition 1e6: one Householder
        # QR more than for the well-conditioned spectrum, after the same Cholesky QR attempts
        def profiled_move(sig):
            t = xg.TTTensor.from_cores(_tt_with_bond_spectrum(sig, 11), ctx=ctx)
            t.move_core(5, False)
            ctx.profile(True)
            try:
                t.move_core(0, False)
                return {k: ctx.profile_get(k)[0] for k in ("qr_gram", "qr")}
            finally:
                ctx.profile(False)
        base = profiled_move(np.sort(np.random.default_rng(5).uniform(0.5, 2.0, 64))[::-1])
        mc = profiled_move(sigma)
        assert mc["qr"] == base["qr"] + 1 and mc["qr_gram"] == base["qr_gram"] >= 1
    spr = []
    o.tt_round(xh, 32, o.EPSILON, spr)
    spr = np.concatenate(spr)
    assert x.ranks() == xh.ranks
    assert sp.shape == spr.shape and np.max(np.abs(sp - spr) / spr) < 1e-10
    pos = np.random.default_rng(3).integers(0, 4, size=(64, 6))
    assert rel_err(x.entries(pos), o.tt_entries(xh, pos)) < 1e-10
    # rank-revealing move_core, both directions. Exact zeros put R_kk at rounding level,
    # where the reference's signed rule (|R_kk| < 16 eps R_00, kept whenever LAPACK's R_00
    # is negative) depends on the gauge earlier factorisations left: there the rank must
    # lie between the true and the representation rank, as for the other exactly
    # deficient inputs; everywhere else it is exact
    y = xg.TTTensor.from_cores(cores, ctx=ctx)
    yh = o.TT([c.copy() for c in cores])
    for p in (5, 0):
        y.move_core(p, False)
        o.move_core(yh, p, keep_rank=False)
        if spectrum == "deficient":
            assert all(56 <= a <= 64 for a in y.ranks()[2:3]) and y.ranks()[:2] + y.ranks()[3:] == [4, 16, 16, 4]
        else:
            assert y.ranks() == yh.ranks
        assert rel_err(y.entries(pos), o.tt_entries(yh, pos)) < 1e-10


def test_round_eps_and_max_ranks(ctx, golden):
    r = golden("round")
    e = tt_of(r, "eps_in", canonicalized=False)
    y = dev_tt(ctx, e)
    sp = y.round(1e-6, spectra=True)
    assert [1] + y.ranks() + [1] == list(r["eps_round_ranks"])
    assert rel_err(sp, r["eps_round_spectra"]) < REL_TOL
    assert rel_err(y.entries(r["eps_round_probe_pos"]), r["eps_round_probe_val"]) < REL_TOL
    y = dev_tt(ctx, e)
    y.round([2, 5, 2, 5], 0.0)
    assert [1] + y.ranks() + [1] == list(r["maxr_round_ranks"])
    assert rel_err(y.entries(r["maxr_round_probe_pos"]), r["maxr_round_probe_val"]) < REL_TOL


# ------------------------------------------------------------------ ALS / DMRG

@pytest.mark.parametrize("tag,x0,b,hs,variant", [
    ("r8_hs20", "x0", "b", 20, "als"),
    ("r8_hs3", "x0", "b", 3, "als"),
    ("r8_asd_hs4", "x0", "b", 4, "asd"),
    ("r32_hs2", "x0_r32", "b_r32", 2, "als"),
])
def test_als_spd_matches_reference(ctx, golden, tag, x0, b, hs, variant):
    z = golden("als")
    A, bb, x = dev_op(ctx, op_of(z, "A")), dev_tt(ctx, tt_of(z, b)), dev_tt(ctx, tt_of(z, x0))
    v = (xg.ASD_SPD if variant == "asd" else xg.ALS_SPD).copy()
    v.convergenceEpsilon = 0.0
    perf = xg.PerformanceData()
    energy = v(A, x, bb, hs, perf)
    assert abs(energy / z[tag + "_energy"][0] - 1) < REL_TOL
    assert [1] + x.ranks() + [1] == list(z[tag + "_ranks"])
    assert rel_err(x.entries(z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-9
    pr = z[tag + "_perf_residual"]
    mine = np.array(perf.residuals)
    assert len(mine) == len(pr)
    keep = pr > 1e-6
    assert rel_err(mine[keep], pr[keep]) < 1e-9
    # the FP64 residual of this iterate, against the oracle on the same cores; and
    # against the reference's (dense) residual of its own iterate, which differs
    # from ours by the CG-vs-Cholesky rounding (~1e-13 in the cores): at rank 32
    # both iterates sit at the ~1e-11 noise floor of 1e-13 local solves
    r_dev = xg.residual(A, x, bb)
    r_ora = o.residual(op_of(z, "A"), host_tt(x), tt_of(z, b))
    assert abs(r_dev - r_ora) <= 1e-9 * r_ora + 1e-12
    dense = z[tag + "_dense_residual"][0]
    assert abs(r_dev - dense) <= 1e-9 * dense + 5e-11


def test_als_ragged_dims(ctx, golden):
    z = golden("als")
    A, b, x = dev_op(ctx, op_of(z, "A_rag")), dev_tt(ctx, tt_of(z, "b_rag")), dev_tt(ctx, tt_of(z, "x0_rag"))
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    energy = v(A, x, b, 6)
    assert abs(energy / z["rag_hs6_energy"][0] - 1) < REL_TOL
    assert rel_err(x.entries(z["rag_hs6_x_probe_pos"]), z["rag_hs6_x_probe_val"]) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cg_paths_agree(ctx, golden, precision):
    """The cluster-resident local CG (default where the local system fits), the
    grid-wide kernel and (mixed precision) the tensor-core form give the
    reference's energy on the rank-32 workload."""
    z = golden("als")
    out = {}
    paths = ("grid", "auto", "tensor") if precision == "mixed" else ("grid", "auto")
    try:
        for path in paths:
            ctx.set_cg_path(path)
            A, b, x = dev_op(ctx, op_of(z, "A")), dev_tt(ctx, tt_of(z, "b_r32")), dev_tt(ctx, tt_of(z, "x0_r32"))
            v = xg.ALS_SPD.copy()
            v.convergenceEpsilon = 0.0
            if precision == "mixed":
                v.precision = xg.MIXED
            out[path] = (v(A, x, b, 2), xg.residual(A, x, b))
            assert abs(out[path][0] / z["r32_hs2_energy"][0] - 1) < REL_TOL
    finally:
        ctx.set_cg_path("auto")
    # every iterate sits at the local-solve noise floor (1e-13 per local CG), far below 1e-8
    assert max(out[p][1] for p in paths) < 1e-10


def test_als_tensor_core_form_at_rank_64(ctx, golden):
    """Mixed precision at ranks >= 64 takes the tensor-core form by default (FP64
    refinement of FP32 CG with split-TF32 tcgen05 operator stages, environment pushes
    in double-float tiles): after two half-sweeps from the same start it gives the
    FP64 form's energy and iterate."""
    z = golden("als")
    out = {}
    for prec in (xg.FP64, xg.MIXED):
        A, b = dev_op(ctx, op_of(z, "A")), dev_tt(ctx, tt_of(z, "b_r32"))
        xg.seed(21)
        x = xg.TTTensor.random([4] * 8, 64, ctx=ctx)
        x /= x.frob_norm()
        v = xg.ALS_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        ctx.profile(True)
        e = v(A, x, b, 2)
        ctx.profile(False)
        out[prec] = (e, x, xg.residual(A, x, b), ctx.profile_get("cg_tc")[0], ctx.profile_get("gemm_df")[0])
    assert max(x.ranks()) == 64
    assert out[xg.MIXED][3] > 0 and out[xg.FP64][3] == 0  # the tensor-core form ran (mixed only)
    # the mixed form's environment pushes ran in double-float tiles; the FP64 form's did not
    assert out[xg.MIXED][4] > 0 and out[xg.FP64][4] == 0
    assert abs(out[xg.MIXED][0] / out[xg.FP64][0] - 1) < 1e-10
    xm, xd = out[xg.MIXED][1], out[xg.FP64][1]
    assert (xm - xd).frob_norm() / xd.frob_norm() < 1e-8
    assert out[xg.MIXED][2] < 1e-8


def test_tensor_core_form_deep_stages(ctx, golden):
    """A rank-10 operator (5 A) at x rank 64: the right-environment stage has K = 640,
    deeper than the cooperative engine tabulates, so the tensor-core form runs its
    stages as separate launches (host-driven CG); same energy as the FP64 form."""
    z = golden("als")
    A1 = dev_op(ctx, op_of(z, "A"))
    A = A1 + A1 + A1 + A1 + A1
    assert max(A.ranks()) == 10
    b = dev_tt(ctx, tt_of(z, "b_r32"))
    out = {}
    for prec in (xg.FP64, xg.MIXED):
        xg.seed(21)
        x = xg.TTTensor.random([4] * 8, 64, ctx=ctx)
        x /= x.frob_norm()
        v = xg.ALS_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        ctx.profile(True)
        e = v(A, x, b, 2)
        ctx.profile(False)
        out[prec] = (e, xg.residual(A, x, b), ctx.profile_get("gemm_tc")[0])
    assert out[xg.MIXED][2] > 0  # the separate-launch tensor-core GEMMs ran
    assert abs(out[xg.MIXED][0] / out[xg.FP64][0] - 1) < 1e-10
    assert out[xg.MIXED][1] < 1e-8


def test_als_mixed_precision_matches_fp64(ctx, golden):
    z = golden("als")
    A, b = dev_op(ctx, op_of(z, "A")), dev_tt(ctx, tt_of(z, "b_r32"))
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    v.precision = xg.MIXED
    x = dev_tt(ctx, tt_of(z, "x0_r32"))
    energy = v(A, x, b, 2)
    assert abs(energy / z["r32_hs2_energy"][0] - 1) < REL_TOL
    assert rel_err(x.entries(z["r32_hs2_x_probe_pos"]), z["r32_hs2_x_probe_val"]) < 1e-8
    assert xg.residual(A, x, b) < 1e-10


@pytest.mark.parametrize("d,n,rank,scale", [(1, 3, 1, 1.0), (2, 3, 2, 1.0), (3, 3, 2, 1.0), (4, 3, 2, 1.0),
                                             (5, 3, 2, 1e-8), (8, 4, 8, 1e-8), (4, 8, 230, 1.0)])
def test_residual_small_orders_and_meetings(ctx, d, n, rank, scale):
    """The FP64 residual's two orthogonalisation chains meet over two cores, or over one
    where the meeting's product would be large (the rank-230 case): orders 1 to 8
    against the oracle, including residuals of ~1e-8 relative (b = A x + 1e-8 r),
    where a cancellation would show."""
    rng = np.random.default_rng(1000 * d + rank)
    A = o.laplace_operator(d, n)
    xr = [1] + [rank] * (d - 1) + [1]
    x = o.TT([rng.standard_normal((xr[k], n, xr[k + 1])) / np.sqrt(n * xr[k]) for k in range(d)])
    rr = [1] + [2] * (d - 1) + [1]
    r = o.TT([rng.standard_normal((rr[k], n, rr[k + 1])) for k in range(d)])
    b = r if scale == 1.0 else o.tt_add(o.op_apply(A, x), o.tt_scale(r, scale))
    want = o.residual(A, x, b)
    got = xg.residual(dev_op(ctx, A), dev_tt(ctx, x), dev_tt(ctx, b))
    assert abs(got / want - 1) < (1e-9 if scale == 1.0 else 1e-5), (got, want)


def test_dmrg_spd(ctx, golden):
    """The reference's decreasing half-sweep contracts core k (not k+1) into the
    right environment (als.cpp:371), so after the first half-sweep its result
    depends on the sign gauge of LAPACK's singular vectors. Pinned here: the
    first half-sweep against the reference; every half-sweep against the oracle
    in the device's sign gauge; the corrected environment (gauge-invariant)
    against the oracle."""
    z = golden("dmrg")
    Ah, bh, xh = op_of(z, "A"), tt_of(z, "b"), tt_of(z, "x0")
    A, b, x = dev_op(ctx, Ah), dev_tt(ctx, bh), dev_tt(ctx, xh)
    v = xg.DMRG_SPD.copy()
    v.convergenceEpsilon = 0.0
    perf = xg.PerformanceData()
    energy = v(A, x, b, 4, perf)
    assert [1] + x.ranks() + [1] == list(z["d8_r4_hs4_ranks"])
    assert rel_err(perf.residuals[:6], z["d8_r4_hs4_perf_residual"][:6]) < 1e-10
    ref = xh.copy()
    r = o.als_spd(Ah, ref, bh, 2, 4, 0.0, track_residual=True, canonical_signs=True)
    assert abs(energy / r.energy - 1) < 1e-9
    assert rel_err(perf.residuals, r.residuals) < 1e-8
    assert rel_err(x.entries(z["d8_r4_hs4_x_probe_pos"]), o.tt_entries(ref, z["d8_r4_hs4_x_probe_pos"])) < 1e-8
    v.exact_environment = True
    x = dev_tt(ctx, xh)
    energy = v(A, x, b, 4)
    ref = xh.copy()
    r = o.als_spd(Ah, ref, bh, 2, 4, 0.0, exact_environment=True)
    assert abs(energy / r.energy - 1) < 1e-10
    assert rel_err(x.entries(z["d8_r4_hs4_x_probe_pos"]), o.tt_entries(ref, z["d8_r4_hs4_x_probe_pos"])) < 1e-9


# Non-symmetric operator (Laplacian sum + 0.6 * convection, d=6, n=4), useResidualForEndCriterion
# and the operator-free form (x of rank 3 approximates b of rank 6), against the reference.
NONSPD_RUNS = {
    # tag: (variant, half-sweeps, convergenceEpsilon 0)
    "als_hs6": ("ALS", 6, True),
    "asd_hs6": ("ASD", 6, True),
    "als_default": ("ALS", 40, False),
    "spd_useres": ("ALS_SPD", 20, False),
    "free_hs4": ("ALS", 4, True),
    "free_useres": ("ALS", 10, False),
}


@pytest.mark.parametrize("tag", list(NONSPD_RUNS))
def test_als_nonspd_and_operator_free_match_reference(ctx, golden, tag):
    """The non-symmetric sweep contracts A^T A and A^T b as TT operators of rank R^2 and
    R s (the reference contracts two copies of A in 4-leg stacks; the projections are the
    same). The reference's non-symmetric ASD step (alpha = ||g|| / ||M g||, als.cpp:86-89)
    diverges on this operator; it is reproduced as it is."""
    z = golden("als_nonspd")
    name, hs, eps0 = NONSPD_RUNS[tag]
    v = getattr(xg, name).copy()
    if eps0:
        v.convergenceEpsilon = 0.0
    v.useResidualForEndCriterion = tag.endswith("useres")
    perf = xg.PerformanceData()
    if tag.startswith("free"):
        x, b = dev_tt(ctx, tt_of(z, "y0")), dev_tt(ctx, tt_of(z, "c"))
        energy = v(x, b, hs, perf)
    else:
        A = dev_op(ctx, op_of(z, "A_spd" if tag == "spd_useres" else "A"))
        x, b = dev_tt(ctx, tt_of(z, "x0")), dev_tt(ctx, tt_of(z, "b"))
        energy = v(A, x, b, hs, perf)
    ref_e = z[tag + "_energy"][0]
    assert abs(energy / ref_e - 1) < 1e-9, (energy, ref_e)
    assert [1] + x.ranks() + [1] == list(z[tag + "_ranks"])
    pr, mine = z[tag + "_perf_residual"], np.array(perf.residuals)
    assert len(mine) == len(pr)
    assert list(perf.flags) == list(z[tag + "_perf_flags"])
    err = np.abs(mine / pr - 1)
    assert err.max() < 1e-9, (err.max(), int(err.argmax()))
    assert rel_err(x.entries(z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-8


def test_dmrg_nonspd(ctx, golden):
    """Two-site non-symmetric sweep: the first half-sweep against the reference (later
    half-sweeps depend on the singular vectors' sign gauge, as for DMRG_SPD), all three
    against the oracle in the device's gauge."""
    z = golden("als_nonspd")
    Ah, bh, xh = op_of(z, "A"), tt_of(z, "b"), tt_of(z, "x0")
    A, b, x = dev_op(ctx, Ah), dev_tt(ctx, bh), dev_tt(ctx, xh)
    v = xg.DMRG.copy()
    v.convergenceEpsilon = 0.0
    perf = xg.PerformanceData()
    energy = v(A, x, b, 3, perf)
    assert [1] + x.ranks() + [1] == list(z["dmrg_hs3_ranks"])
    assert rel_err(perf.residuals[:4], z["dmrg_hs3_perf_residual"][:4]) < 1e-9
    ref = xh.copy()
    r = o.als(Ah, ref, bh, 2, 3, 0.0, track_residual=True, canonical_signs=True, assume_spd=False)
    assert abs(energy / r.energy - 1) < 1e-9
    assert rel_err(x.entries(z["dmrg_hs3_x_probe_pos"]), o.tt_entries(ref, z["dmrg_hs3_x_probe_pos"])) < 1e-8


def test_dmrg_spd_potential_d20(ctx, golden):
    """Laplacian + potential, rank-3 operator, d=20, n=8, rank 8. The first
    half-sweep against the oracle (pinned to the reference); the corrected
    environment for two half-sweeps. The reference-environment second half-sweep
    is not pinned: its local systems reach condition numbers ~1e7 and a 1e-15
    change of one core moves its energy by ~1e-9, so it is not reproducible
    across solvers or BLAS builds to 1e-10."""
    z = golden("dmrg")
    Ah, bh, xh = op_of(z, "A_pot"), tt_of(z, "b_pot"), tt_of(z, "x0_pot")
    A, b, x = dev_op(ctx, Ah), dev_tt(ctx, bh), dev_tt(ctx, xh)
    v = xg.DMRG_SPD.copy()
    v.convergenceEpsilon = 0.0
    energy = v(A, x, b, 1)
    ref = xh.copy()
    r = o.als_spd(Ah, ref, bh, 2, 1, 0.0)
    assert abs(energy / r.energy - 1) < 1e-10
    assert rel_err(x.entries(z["pot_r8_hs2_x_probe_pos"]), o.tt_entries(ref, z["pot_r8_hs2_x_probe_pos"])) < 1e-9
    v.exact_environment = True
    x = dev_tt(ctx, xh)
    energy = v(A, x, b, 2)
    ref = xh.copy()
    r = o.als_spd(Ah, ref, bh, 2, 2, 0.0, exact_environment=True)
    assert abs(energy / r.energy - 1) < 1e-10
    assert rel_err(x.entries(z["pot_r8_hs2_x_probe_pos"]), o.tt_entries(ref, z["pot_r8_hs2_x_probe_pos"])) < 1e-9


# ------------------------------------------------------------------ ADF and adjoints

def _adf_inputs(ctx, dims, rank, n):
    xg.seed(0xBAADF00D)
    target = xg.TTTensor.random(dims, rank, ctx=ctx)
    m = xg.SinglePointMeasurementSet.random(n, dims)
    m.measure(target)
    noise = np.zeros(n)
    import ctypes
    xg._lib.load().xtt_random_normal(0.0, 1e-6, n, noise.ctypes.data_as(xg._lib.c_double_p))
    m.measuredValues = m.measuredValues + noise
    x = xg.TTTensor.random(dims, rank, ctx=ctx)
    return target, m, x


def test_adf_small(ctx, golden):
    z = golden("adf")
    _, m, x = _adf_inputs(ctx, [4, 5, 3, 5, 4, 3], 3, 2000)
    assert np.array_equal(m.positions, z["small_positions"].astype(np.int64))
    assert rel_err(m.measuredValues, z["small_values"]) < 1e-12
    perf = xg.PerformanceData()
    res = xg.ADFVariant(30, 0.0, 1.0)(x, m, perf)
    pr = z["small_perf_residual"]
    assert len(perf.residuals) == len(pr)
    assert rel_err(perf.residuals[:10], pr[:10]) < 1e-10
    assert rel_err(perf.residuals, pr) < 1e-7
    assert abs(res / z["small_final_residual"][0] - 1) < 1e-6


@pytest.mark.parametrize("tag,op,spd,steps", [("spd", "A", True, 12), ("ls", "An", False, 12), ("free", None, False, 8)])
def test_geometric_cg_matches_reference(ctx, golden, tag, op, spd, steps):
    """Riemannian CG (GeometricCG): the reference's residual after every step and its final
    iterate. The line search compares residuals, so a rounding-level difference can in
    principle pick another step length; on these cases it does not."""
    z = golden("gcg")
    A = dev_op(ctx, op_of(z, op)) if op else None
    x = dev_tt(ctx, tt_of(z, "x0"))
    b = dev_tt(ctx, tt_of(z, "b"))
    v = xg.GeometricCGVariant(0, 1e-8, spd)
    perf = xg.PerformanceData()
    res = v(A, x, b, steps, perf) if A is not None else v(x, b, steps, perf)
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-9
    assert len(perf.residuals) == len(z[tag + "_perf_residual"])
    assert rel_err(perf.residuals, z[tag + "_perf_residual"]) < 1e-9
    assert [1] + x.ranks() + [1] == list(z[tag + "_ranks"])
    assert rel_err(x.entries(z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-8


@pytest.mark.parametrize("tag,op,spd,steps", [("sd_spd", "A", True, 10), ("sd_ls", "An", False, 10),
                                              ("sd_free", None, False, 6)])
def test_steepest_descent_matches_reference(ctx, golden, tag, op, spd, steps):
    z = golden("gcg")
    A = dev_op(ctx, op_of(z, op)) if op else None
    x = dev_tt(ctx, tt_of(z, "x0"))
    b = dev_tt(ctx, tt_of(z, "b"))
    v = xg.SteepestDescentVariant(0, 1e-8, spd)
    perf = xg.PerformanceData()
    res = v(A, x, b, steps, perf) if A is not None else v(x, b, steps, perf)
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-9
    assert rel_err(perf.residuals, z[tag + "_perf_residual"]) < 1e-9
    assert rel_err(x.entries(z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-8


def test_adf_rank_increase_matches_reference(ctx, golden):
    """ADFVariant(120, 1e-10, 0.99)(x, measurements, maxRanks) from a rank-1 start
    (adf.cpp:566-604): two rank increases, each a rank-1 random TT from the library's
    random state (reseeded with 0x5EED as the reference was), scaled to 1e-6 ||x||,
    then round(maxRanks). Ranks and iteration counts exact at every recorded point;
    residuals to 1e-10 until the first increase. Each increase adds directions of size
    1e-6 ||x||, which rounding at 1e-16 ||x|| (and the platform's last bits of the
    normal draws) perturbs by ~1e-10 relative, and the later iterations amplify that:
    1e-6 from there on, the spread the reference itself shows across OpenMP thread
    counts."""
    z = golden("adf_rankinc")
    m = xg.SinglePointMeasurementSet(z["positions"], z["values"])
    x = dev_tt(ctx, tt_of(z, "x0"))
    xg.seed(0x5EED)
    perf = xg.PerformanceData()
    res = xg.ADFVariant(120, 1e-10, 0.99)(x, m, [3] * 5, perf)
    assert list(perf.iterations) == list(z["perf_iteration"])
    assert perf.ranks == z["perf_ranks"].tolist()
    r, rr = np.array(perf.residuals), z["perf_residual"]
    first = list(z["perf_ranks"][:, 0]).index(2)  # the first point after the first increase
    assert np.max(np.abs(r[:first] / rr[:first] - 1)) < 1e-10
    # relative 1e-6, or 1e-15 absolute (relative residuals of ||y|| = 1: the rounding of the
    # sum of squares over the samples) where the trajectory has fallen to ~1e-10
    assert np.all(np.abs(r - rr) <= 1e-6 * rr + 1e-15)
    assert abs(res - z["final_residual"][0]) <= 1e-6 * z["final_residual"][0] + 1e-15
    assert [1] + x.ranks() + [1] == list(z["x_final_ranks"])
    assert rel_err(x.entries(z["x_final_probe_pos"]), z["x_final_probe_val"]) < 1e-8


@pytest.mark.parametrize("alg,kind,spd", [(a, k, s) for a in ("gcg", "sd") for k in ("hosvd", "als") for s in (True, False)])
def test_hosvd_and_als_retractions_match_reference(ctx, golden, alg, kind, spd):
    """GeometricCG (type I retractions, projective vector transport) and SteepestDescent
    (type II) with the HOSVD retraction (the step added as a TT, rounded back to the old
    ranks) and the ALS retraction (two operator-free ALS half-sweeps fit x to it),
    retractions.cpp:43-69: the reference's residual after every step and its final
    iterate."""
    z = golden("retractions")
    A = dev_op(ctx, op_of(z, "A" if spd else "An"))
    x, b = dev_tt(ctx, tt_of(z, "x0")), dev_tt(ctx, tt_of(z, "b"))
    r = {"hosvd": xg.HOSVDRetraction, "als": xg.ALSRetraction}[kind]
    cls = xg.GeometricCGVariant if alg == "gcg" else xg.SteepestDescentVariant
    v = cls(0, 1e-8, spd, retraction=r)
    perf = xg.PerformanceData()
    tag = f"{alg}_{kind}_{'spd' if spd else 'ls'}"
    res = v(A, x, b, 8, perf)
    assert len(perf.residuals) == len(z[tag + "_perf_residual"])
    assert rel_err(perf.residuals, z[tag + "_perf_residual"]) < 1e-9
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-9
    assert [1] + x.ranks() + [1] == list(z[tag + "_ranks"])
    assert rel_err(x.entries(z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-8


def test_iht_matches_reference(ctx, golden):
    """IHT (iht.cpp:29-155) capped at 11 iterations: every iteration's best residual and the
    iterate after the eleventh against the reference's own run (which is stopped from its
    PerformanceData callback: it has no stopping test)."""
    z = golden("iht")
    x = dev_tt(ctx, tt_of(z, "x0"))
    m = xg.SinglePointMeasurementSet(z["positions"], z["values"])
    perf = xg.PerformanceData()
    res = xg.IHT(x, m, perf, maxIterations=11)
    assert rel_err(perf.residuals, z["perf_residual"]) < 1e-10
    assert abs(res / z["perf_residual"][-1] - 1) < 1e-10
    assert rel_err(x.entries(z["probe_pos"]), z["probe_val"][10]) < 1e-9


def test_adf_rank_one_matches_reference(ctx, golden):
    """ADF on rank-one measurements (RankOneMeasurementSet): the reference's trajectory and
    final iterate; the device measurement of the target against the reference's values."""
    z = golden("adf_rankone")
    dims = [4, 5, 4, 5]
    t = dev_tt(ctx, tt_of(z, "target"))
    m = xg.RankOneMeasurementSet(z["vectors"], None, dims)
    m.measure(t)
    assert rel_err(m.measuredValues, z["values"]) < 1e-12
    m = xg.RankOneMeasurementSet(z["vectors"], z["values"], dims)
    x = dev_tt(ctx, tt_of(z, "x0"))
    perf = xg.PerformanceData()
    res = xg.ADFVariant(25, 0.0, 1.0)(x, m, perf)
    pr = z["perf_residual"]
    assert len(perf.residuals) == len(pr)
    assert rel_err(perf.residuals[:10], pr[:10]) < 1e-10
    assert rel_err(perf.residuals, pr) < 1e-8
    assert abs(res / z["final_residual"][0] - 1) < 1e-8
    assert rel_err(x.entries(z["x_final_probe_pos"]), z["x_final_probe_val"]) < 1e-8


def test_adf_cfg5_positions_gradient_and_first_iterations(ctx, golden):
    z = golden("adf_cfg5")
    _, m, x = _adf_inputs(ctx, [8] * 10, 6, 200000)
    assert fnv1a(m.positions) == int(z["cfg5_positions_fnv1a"][0])
    assert abs(m.measuredValues.sum() / z["cfg5_values_sum"][0] - 1) < 1e-12
    x0 = host_tt(x)
    # adjoint: loss gradient vs the oracle's (all cores, no gauge)
    loss, grads = xg.ADFVariant.gradient(x, m)
    lo, go = o.adf_loss_gradient(x0, m.positions, m.measuredValues)
    assert abs(loss / lo - 1) < 1e-10
    for g, h in zip(grads, go):
        assert rel_err(g, h) < 1e-10
    perf = xg.PerformanceData()
    xg.ADFVariant(5, 0.0, 1.0)(x, m, perf)
    assert rel_err(perf.residuals, z["cfg5_perf_residual"][:5]) < 1e-9


def _cfg5_sweep_states(z, positions, values):
    """The iterates of the reference's first ADF sweep on configuration 5, x canonical at
    core k before step k, replayed by the oracle (whose projected gradients reproduce the
    reference's own, checked against the same fixture on the CPU)."""
    x = tt_of(z, "cfg5_x0")
    s = o.ADFSolver(x, positions, values, 1, 0.0, 1.0)
    o.move_core(s.x, 0, keep_rank=False)
    s.begin_iteration()
    states = []
    for k in range(s.d):
        states.append(s.x.copy())
        s.sweep_step(k)
    return states


def test_adf_cfg5_gradient_matches_reference_sweep(ctx, golden):
    """Configuration 5 (d=10, n=8, rank 6, 200 000 samples): the adjoint's gradient at
    core k, x canonical at k, equals minus the reference's projected gradient of the
    same sweep step (calculate_projected_gradient, adf.cpp:359-396; the reference's
    first-sweep values), for every k, to 1e-10."""
    z = golden("adf_cfg5")
    _, m, _ = _adf_inputs(ctx, [8] * 10, 6, 200000)
    assert fnv1a(m.positions) == int(z["cfg5_positions_fnv1a"][0])
    ref = z["cfg5_grad_sweep"]
    off = 0
    for k, xk in enumerate(_cfg5_sweep_states(z, m.positions, m.measuredValues)):
        assert xk.canonicalized and xk.core_position == k
        _, grads = xg.ADFVariant.gradient(dev_tt(ctx, xk), m)
        g = grads[k]
        want = -ref[off:off + g.size].reshape(g.shape)
        off += g.size
        assert rel_err(g, want) < REL_TOL, k
    assert off == ref.size


def test_adf_cfg5_gradient_central_differences(ctx, golden):
    """Configuration 5 itself: the adjoint's gradient of 0.5 ||P_Omega(x) - y||^2 with
    respect to 300 sampled entries spread over all ten cores against central differences
    in FP64 with h = 1e-4 (the loss is quadratic in each entry, so the difference
    quotient is exact up to the rounding of the loss). The loss is evaluated from the
    device's sampled entries, summed in FP64 on the host."""
    z = golden("adf_cfg5")
    _, m, _ = _adf_inputs(ctx, [8] * 10, 6, 200000)
    x0 = tt_of(z, "cfg5_x0")
    x = dev_tt(ctx, x0)
    loss, grads = xg.ADFVariant.gradient(x, m)
    y = m.measuredValues

    def loss_at(cores):
        t = xg.TTTensor.from_cores(cores, ctx=ctx)
        r = t.entries(m.positions) - y
        return 0.5 * float(np.dot(r, r))

    assert abs(loss_at(x0.cores) / loss - 1) < 1e-12
    rng = np.random.default_rng(29)
    h = 1e-4
    scale = max(float(np.max(np.abs(g))) for g in grads)
    worst = 0.0
    for k in range(10):
        for flat in rng.choice(x0.cores[k].size, 30, replace=False):
            idx = np.unravel_index(int(flat), x0.cores[k].shape)
            vals = []
            for sgn in (+1, -1):
                c = [cc.copy() for cc in x0.cores]
                c[k][idx] += sgn * h
                vals.append(loss_at(c))
            fd = (vals[0] - vals[1]) / (2 * h)
            worst = max(worst, abs(fd - grads[k][idx]))
    assert worst <= 1e-6 * scale, (worst, scale)


def test_adf_fp32_form_tracks_fp64(ctx, golden):
    """The FP32 form (FP32 stacks and per-sample arithmetic, FP64 cores and QR)
    follows the FP64 trajectory to FP32 accuracy over the first iterations, and its
    returned residual is the FP64 check of the returned x."""
    z = golden("adf")
    _, m, x = _adf_inputs(ctx, [4, 5, 3, 5, 4, 3], 3, 2000)
    x32 = x.copy()
    p64, p32 = xg.PerformanceData(), xg.PerformanceData()
    xg.ADFVariant(8, 0.0, 1.0)(x, m, p64)
    res32 = xg.ADFVariant(8, 0.0, 1.0, precision=xg.MIXED)(x32, m, p32)
    assert rel_err(p32.residuals[:4], p64.residuals[:4]) < 1e-4
    assert rel_err(p64.residuals[:4], z["small_perf_residual"][:4]) < 1e-10
    e = x32.entries(m.positions)
    chk = np.linalg.norm(e - m.measuredValues) / np.linalg.norm(m.measuredValues)
    assert abs(res32 / chk - 1) < 1e-10


def test_adf_gradient_central_differences(ctx):
    xg.seed(7)
    dims = [3, 4, 3, 2]
    x = xg.TTTensor.random(dims, 2, ctx=ctx)
    target = xg.TTTensor.random(dims, 2, ctx=ctx)
    m = xg.SinglePointMeasurementSet.random(40, dims)
    m.measure(target)
    loss, grads = xg.ADFVariant.gradient(x, m)
    cores = x.get_cores()
    h = 1e-4
    for k in range(len(cores)):
        fd = np.zeros_like(cores[k])
        for idx in np.ndindex(cores[k].shape):
            for sgn in (+1, -1):
                c = [cc.copy() for cc in cores]
                c[k][idx] += sgn * h
                xt = o.TT(c)
                r = o.tt_entries(xt, m.positions) - m.measuredValues
                fd[idx] += sgn * 0.5 * float(r @ r) / (2 * h)
        assert rel_err(grads[k], fd) < 1e-6


def test_als_energy_gradient(ctx, golden):
    z = golden("als")
    Ah, bh, xh = op_of(z, "A"), tt_of(z, "b"), tt_of(z, "x0")
    A, b, x = dev_op(ctx, Ah), dev_tt(ctx, bh), dev_tt(ctx, xh)
    J, grads = xg.als_energy_gradient(A, x, b)
    Ax = o.op_apply(Ah, xh)
    assert abs(J / (o.tt_dot(xh, Ax) - 2 * o.tt_dot(xh, bh)) - 1) < 1e-10
    # directional derivative along a random core perturbation
    rng = np.random.default_rng(3)
    k = 3
    dx = rng.standard_normal(xh.cores[k].shape)
    h = 1e-6
    vals = []
    for s in (+1, -1):
        c = [cc.copy() for cc in xh.cores]
        c[k] = c[k] + s * h * dx
        xt = o.TT(c)
        vals.append(o.tt_dot(xt, o.op_apply(Ah, xt)) - 2 * o.tt_dot(xt, bh))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(float(np.sum(grads[k] * dx)) / fd - 1) < 1e-6


def test_torch_autograd_adjoints(ctx):
    """The torch.autograd.Function wrappers return the device gradients; checked
    by a directional central difference in FP64 (h = 1e-4, as for ADF's check)."""
    torch = pytest.importorskip("torch")
    from xerus_gb300.autograd import adf_loss, als_energy
    xg.seed(5)
    dims = [3, 4, 3, 2, 3]
    x = xg.TTTensor.random(dims, 2, ctx=ctx)
    target = xg.TTTensor.random(dims, 2, ctx=ctx)
    m = xg.SinglePointMeasurementSet.random(60, dims)
    m.measure(target)
    cores = [torch.tensor(c, requires_grad=True) for c in x.get_cores()]
    pos, val = torch.tensor(m.positions), torch.tensor(m.measuredValues)
    loss = adf_loss(pos, val, cores)
    loss.backward()
    g = [c.grad.clone() for c in cores]
    rng = np.random.default_rng(0)
    dirs = [torch.tensor(rng.standard_normal(c.shape)) for c in cores]
    h = 1e-4
    with torch.no_grad():
        lp = adf_loss(pos, val, [c + h * d for c, d in zip(cores, dirs)])
        lm = adf_loss(pos, val, [c - h * d for c, d in zip(cores, dirs)])
    fd = float((lp - lm) / (2 * h))
    an = float(sum((gi * di).sum() for gi, di in zip(g, dirs)))
    assert abs(an / fd - 1) < 1e-6
    d3 = [3] * 5
    A = xg.TTOperator.from_cores(xg.laplacian_cores(len(d3), 3, shift=0.3), ctx=ctx)
    b = xg.TTTensor.random(d3, 2, ctx=ctx)
    x3 = xg.TTTensor.random(d3, 2, ctx=ctx)
    cores = [torch.tensor(c, requires_grad=True) for c in x3.get_cores()]
    J = als_energy(A, b, cores)
    J.backward()
    g = [c.grad.clone() for c in cores]
    dirs = [torch.tensor(rng.standard_normal(c.shape)) for c in cores]
    with torch.no_grad():
        Jp = als_energy(A, b, [c + h * d for c, d in zip(cores, dirs)])
        Jm = als_energy(A, b, [c - h * d for c, d in zip(cores, dirs)])
    fd = float((Jp - Jm) / (2 * h))
    an = float(sum((gi * di).sum() for gi, di in zip(g, dirs)))
    assert abs(an / fd - 1) < 1e-6
