"""Pins the CPU oracle (oracle/xtt_oracle.py) against golden vectors written by
the xerus reference itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import xtt_oracle as o
from tests.helpers import REL_TOL, fnv1a, op_of, rel_err, tt_of


def test_rng_streams_bit_exact(golden):
    z = golden("rng")
    rs = o.RandomEngine()
    assert np.array_equal(np.array([rs.eng() for _ in range(64)], dtype=np.uint64), z["rng_raw_u64"])
    rs.reseed()
    assert np.array_equal(rs.normal.draw(rs.eng, 257), z["rng_normal"])
    rs.reseed()
    assert np.array_equal(o.NormalDist(0.0, 0.125).draw(rs.eng, 129), z["rng_normal_sd0125"])
    rs.reseed()
    ints = [o.uniform_int(rs.eng, 0, n - 1) for n in (2, 3, 4, 5, 7, 8, 10, 1000) for _ in range(32)]
    assert np.array_equal(np.array(ints), z["rng_uniform_int"])
    rs.reseed()
    assert np.array_equal(np.array([o.uniform_real(rs.eng) for _ in range(64)]), z["rng_uniform_real"])


def test_tt_random_matches(golden):
    z = golden("tt_random")
    rs = o.RandomEngine()
    x = o.tt_random([3, 4, 2, 5], [2, 7, 3], rs)
    assert [1] + x.ranks + [1] == list(z["small_ranks_after"])
    assert rel_err(o.tt_full(x).ravel(), z["small_full"]) < REL_TOL
    rs.reseed()
    y = o.tt_random([4] * 8, 8, rs)
    assert rel_err(o.tt_entries(y, z["d8_probe_pos"]), z["d8_probe_val"]) < REL_TOL
    assert abs(o.frob_norm(y) / z["d8_norm"][0] - 1) < REL_TOL


def test_dot_and_norm_cfg2(golden):
    z = golden("dot")
    rs = o.RandomEngine()
    dist = o.NormalDist(0.0, 0.125)
    x = o.tt_random([4] * 32, 64, rs, dist)
    y = o.tt_random([4] * 32, 64, rs, dist)
    assert abs(o.tt_dot(x, y) / z["cfg2_dot_xy"][0] - 1) < REL_TOL
    assert abs(o.frob_norm(x) / z["cfg2_norm_x"][0] - 1) < REL_TOL
    assert abs(o.frob_norm(y) / z["cfg2_norm_y"][0] - 1) < REL_TOL
    assert rel_err(o.tt_entries(y, z["cfg2_y_probe_pos"]), z["cfg2_y_probe_val"]) < REL_TOL
    a, b = tt_of(z, "small_a", False), tt_of(z, "small_b", False)
    assert abs(o.tt_dot(a, b) / z["small_dot"][0] - 1) < REL_TOL
    assert abs(o.frob_norm(o.tt_add(a, b)) / z["small_sum_norm"][0] - 1) < REL_TOL


def test_move_core_and_qc_rank_rule(golden):
    z = golden("movecore")
    x = tt_of(z, "x")
    for p in (5, 2, 0, 3):
        y = x.copy()
        o.move_core(y, p, keep_rank=True)
        assert rel_err(o.tt_entries(y, z[f"qr_to{p}_probe_pos"]), z[f"qr_to{p}_probe_val"]) < REL_TOL
        assert abs(np.linalg.norm(y.cores[p]) / z[f"qr_to{p}_corenorm"][0] - 1) < REL_TOL
    zz = tt_of(z, "z", canonicalized=False)
    for p in (5, 0):
        y = zz.copy()
        o.move_core(y, p, keep_rank=False)
        assert [1] + y.ranks + [1] == list(z[f"qc_to{p}_ranks"])
        assert rel_err(o.tt_entries(y, z[f"qc_to{p}_probe_pos"]), z[f"qc_to{p}_probe_val"]) < REL_TOL


def test_round_cfg2_ranks_spectra_entries(golden):
    r, zd = golden("round"), golden("dot")
    rs = o.RandomEngine()
    x = o.tt_random([4] * 32, 64, rs, o.NormalDist(0.0, 0.125))
    y = x.copy()
    spectra = []
    o.tt_round(y, 32, o.EPSILON, spectra)
    assert [1] + y.ranks + [1] == list(r["cfg2_round_ranks"])
    assert rel_err(np.concatenate(spectra), r["cfg2_round_spectra"]) < REL_TOL
    assert abs(o.frob_norm(y) / r["cfg2_round_norm"][0] - 1) < REL_TOL
    assert abs(o.tt_dot(y, x) / r["cfg2_round_dot_x"][0] - 1) < REL_TOL
    assert rel_err(o.tt_entries(y, r["cfg2_round_probe_pos"]), r["cfg2_round_probe_val"]) < REL_TOL
    del zd


def test_round_eps_and_max_ranks(golden):
    r = golden("round")
    e = tt_of(r, "eps_in", canonicalized=False)
    e1 = e.copy()
    spectra = []
    o.tt_round(e1, [2 ** 62] * 4, 1e-6, spectra)
    assert [1] + e1.ranks + [1] == list(r["eps_round_ranks"])
    assert rel_err(np.concatenate(spectra), r["eps_round_spectra"]) < REL_TOL
    assert rel_err(o.tt_entries(e1, r["eps_round_probe_pos"]), r["eps_round_probe_val"]) < REL_TOL
    e3 = e.copy()
    o.tt_round(e3, [2, 5, 2, 5], 0.0)
    assert [1] + e3.ranks + [1] == list(r["maxr_round_ranks"])
    assert rel_err(o.tt_entries(e3, r["maxr_round_probe_pos"]), r["maxr_round_probe_val"]) < REL_TOL


@pytest.mark.parametrize("tag,x0,b,hs,solver", [
    ("r8_hs20", "x0", "b", 20, "lapack"),
    ("r8_hs3", "x0", "b", 3, "lapack"),
    ("r8_asd_hs4", "x0", "b", 4, "asd"),
    ("r32_hs2", "x0_r32", "b_r32", 2, "lapack"),
])
def test_als_spd(golden, tag, x0, b, hs, solver):
    z = golden("als")
    A, bb, x = op_of(z, "A"), tt_of(z, b), tt_of(z, x0)
    res = o.als_spd(A, x, bb, 1, hs, 0.0, solver=solver, track_residual=True)
    assert abs(res.energy / z[tag + "_energy"][0] - 1) < REL_TOL
    assert [1] + x.ranks + [1] == list(z[tag + "_ranks"])
    assert rel_err(o.tt_entries(x, z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-9
    # the reference's own residual loses accuracy below ~1e-8 (cancellation); compare above it
    pr, mine = z[tag + "_perf_residual"], np.array(res.residuals)
    assert len(pr) == len(mine)
    keep = pr > 1e-6
    assert rel_err(mine[keep], pr[keep]) < 1e-9
    dense = z[tag + "_dense_residual"][0]
    assert abs(o.residual(A, x, bb) - dense) <= 1e-9 * max(dense, 1e-3)


def test_als_ragged_dims(golden):
    z = golden("als")
    A, b, x = op_of(z, "A_rag"), tt_of(z, "b_rag"), tt_of(z, "x0_rag")
    res = o.als_spd(A, x, b, 1, 6, 0.0)
    assert abs(res.energy / z["rag_hs6_energy"][0] - 1) < REL_TOL
    assert rel_err(o.tt_entries(x, z["rag_hs6_x_probe_pos"]), z["rag_hs6_x_probe_val"]) < REL_TOL


def test_dmrg_spd_small(golden):
    z = golden("dmrg")
    A, b, x = op_of(z, "A"), tt_of(z, "b"), tt_of(z, "x0")
    res = o.als_spd(A, x, b, 2, 4, 0.0, track_residual=True)
    assert abs(res.energy / z["d8_r4_hs4_energy"][0] - 1) < REL_TOL
    assert [1] + x.ranks + [1] == list(z["d8_r4_hs4_ranks"])
    assert rel_err(o.tt_entries(x, z["d8_r4_hs4_x_probe_pos"]), z["d8_r4_hs4_x_probe_val"]) < 1e-9
    assert rel_err(res.residuals, z["d8_r4_hs4_perf_residual"]) < 1e-8


# Non-symmetric operator (Laplacian sum + 0.6 * convection), the operator-free
# form (x approximates b) and useResidualForEndCriterion, against the reference.
NONSPD_RUNS = {
    # tag: (oracle keyword arguments)
    "als_hs6": dict(num_half_sweeps=6, conv_eps=0.0, assume_spd=False),
    "asd_hs6": dict(num_half_sweeps=6, conv_eps=0.0, assume_spd=False, solver="asd"),
    "dmrg_hs3": dict(num_half_sweeps=3, conv_eps=0.0, assume_spd=False, sites=2),
    "als_default": dict(num_half_sweeps=40, assume_spd=False),
    "spd_useres": dict(num_half_sweeps=20, use_residual=True),
    "free_hs4": dict(num_half_sweeps=4, conv_eps=0.0),
    "free_useres": dict(num_half_sweeps=10, use_residual=True),
}


def nonspd_inputs(z, tag):
    """(A, x0, b) of a run in the non-SPD fixture (A None for the operator-free runs)."""
    if tag.startswith("free"):
        return None, tt_of(z, "y0"), tt_of(z, "c")
    return op_of(z, "A_spd" if tag == "spd_useres" else "A"), tt_of(z, "x0"), tt_of(z, "b")


@pytest.mark.parametrize("tag", list(NONSPD_RUNS))
def test_als_nonspd_and_operator_free(golden, tag):
    z = golden("als_nonspd")
    A, x, b = nonspd_inputs(z, tag)
    res = o.als(A, x, b, track_residual=True, **NONSPD_RUNS[tag])
    assert abs(res.energy / z[tag + "_energy"][0] - 1) < 1e-11
    assert [1] + x.ranks + [1] == list(z[tag + "_ranks"])
    assert rel_err(o.tt_entries(x, z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-12
    # the value the reference adds to PerformanceData after every micro-step
    pr = z[tag + "_perf_residual"]
    assert len(res.residuals) == len(pr)
    assert rel_err(res.residuals, pr) < 1e-12
    assert list(res.flags) == list(z[tag + "_perf_flags"])


@pytest.mark.slow
def test_dmrg_spd_potential_d20(golden):
    z = golden("dmrg")
    A, b, x = op_of(z, "A_pot"), tt_of(z, "b_pot"), tt_of(z, "x0_pot")
    res = o.als_spd(A, x, b, 2, 2, 0.0)
    assert abs(res.energy / z["pot_r8_hs2_energy"][0] - 1) < 1e-10
    assert rel_err(o.tt_entries(x, z["pot_r8_hs2_x_probe_pos"]), z["pot_r8_hs2_x_probe_val"]) < 1e-9


def _adf_inputs(dims, rank, n):
    rs = o.RandomEngine()
    target = o.tt_random(dims, rank, rs)
    pos = o.random_positions(n, dims, rs)
    vals = o.tt_entries(target, pos) + o.NormalDist(0.0, 1e-6).draw(rs.eng, n)
    x = o.tt_random(dims, rank, rs)
    return target, pos, vals, x


def test_adf_small(golden):
    z = golden("adf")
    _, pos, vals, x = _adf_inputs([4, 5, 3, 5, 4, 3], 3, 2000)
    assert np.array_equal(pos, z["small_positions"].astype(np.int64))
    assert rel_err(vals, z["small_values"]) < 1e-12
    log = []
    o.ADFSolver(x.copy(), pos, vals, 1, 0.0, 1.0).solve(first_sweep_log=log)
    assert rel_err(np.concatenate([g.ravel() for g, _ in log]), z["small_grad_sweep"]) < REL_TOL
    assert rel_err(np.concatenate([n for _, n in log]), z["small_slicenorm_sweep"]) < 1e-10
    res = o.adf(x, pos, vals, 30, 0.0, 1.0)
    # iterated ADF amplifies rounding differences (the reference's own results
    # change ~1e-6 with the OpenMP thread count): early iterations are tight
    assert rel_err(res.residuals[:10], z["small_perf_residual"][:10]) < 1e-10
    assert rel_err(res.residuals, z["small_perf_residual"]) < 1e-7


def test_adf_cfg5_positions_and_gradient(golden):
    z = golden("adf_cfg5")
    _, pos, vals, x = _adf_inputs([8] * 10, 6, 200000)
    assert fnv1a(pos) == int(z["cfg5_positions_fnv1a"][0])
    assert np.array_equal(pos[:64], z["cfg5_positions_head"].astype(np.int64))
    assert abs(vals.sum() / z["cfg5_values_sum"][0] - 1) < 1e-12
    log = []
    s = o.ADFSolver(x.copy(), pos, vals, 1, 0.0, 1.0)
    s.solve(first_sweep_log=log)
    assert rel_err(np.concatenate([g.ravel() for g, _ in log]), z["cfg5_grad_sweep"]) < REL_TOL
    assert rel_err(np.concatenate([n for _, n in log]), z["cfg5_slicenorm_sweep"]) < 1e-10


def test_adf_rank_one(golden):
    """RankOneMeasurementSet::random (Gaussian vectors, the reference's sort order) and
    ADF on rank-one measurements, against the reference run."""
    z = golden("adf_rankone")
    rs = o.RandomEngine()
    dims = [4, 5, 4, 5]
    target = o.tt_random(dims, 2, rs)
    assert np.array_equal(np.concatenate([c.ravel() for c in target.cores]), z["target_cores"])
    vec = o.rank_one_random(300, dims, rs)
    assert np.array_equal(vec, z["vectors"])
    assert rel_err(o.rank_one_measure(target, vec), z["values"]) < 1e-13
    x = tt_of(z, "x0")
    res = o.adf_rank_one(x, z["vectors"], z["values"], 25, 0.0, 1.0)
    assert rel_err(res.residuals, z["perf_residual"]) < 1e-10
    assert rel_err(o.tt_entries(x, z["x_final_probe_pos"]), z["x_final_probe_val"]) < 1e-10


@pytest.mark.parametrize("tag,op,spd,steps", [("spd", "A", True, 12), ("ls", "An", False, 12), ("free", None, False, 8)])
def test_geometric_cg(golden, tag, op, spd, steps):
    """GeometricCGVariant with the submanifold retraction and projective vector transport:
    SPD operator (gradient b - A x), least squares (A^T (b - A x)) and no operator."""
    z = golden("gcg")
    A = op_of(z, op) if op else None
    x, b = tt_of(z, "x0"), tt_of(z, "b")
    res, trace = o.geometric_cg(A, x, b, steps, 1e-8, spd)
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-12
    assert rel_err(trace, z[tag + "_perf_residual"]) < 1e-12
    assert [1] + x.ranks + [1] == list(z[tag + "_ranks"])
    assert rel_err(o.tt_entries(x, z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-12


@pytest.mark.parametrize("tag,op,spd,steps", [("sd_spd", "A", True, 10), ("sd_ls", "An", False, 10),
                                              ("sd_free", None, False, 6)])
def test_steepest_descent(golden, tag, op, spd, steps):
    """SteepestDescentVariant with SubmanifoldRetractionII."""
    z = golden("gcg")
    A = op_of(z, op) if op else None
    x, b = tt_of(z, "x0"), tt_of(z, "b")
    res, trace = o.steepest_descent(A, x, b, steps, 1e-8, spd)
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-12
    assert rel_err(trace, z[tag + "_perf_residual"]) < 1e-12
    assert rel_err(o.tt_entries(x, z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-12


def test_adf_rank_increase(golden):
    """ADFVariant(120, 1e-10, 0.99)(x, measurements, maxRanks) from a rank-1 start: two
    rank increases (1e-6-scaled rank-1 random TTs from the random state reseeded with
    0x5EED, then round(maxRanks)); ranks and iteration counts exact at every recorded
    point, residuals point by point."""
    z = golden("adf_rankinc")
    x = tt_of(z, "x0")
    rs = o.RandomEngine(0x5EED)
    res = o.adf(x, z["positions"], z["values"], 120, 1e-10, 0.99, max_ranks=[3] * 5, rs=rs)
    assert res.iteration_log == list(z["perf_iteration"])
    assert res.ranks == z["perf_ranks"].tolist()
    # Residuals point by point: to rounding through the first rank increase; each
    # increase adds directions of size 1e-6 ||x||, which rounding at 1e-16 ||x||
    # perturbs by 1e-10 relative, and the iterations after the second one amplify
    # that (the reference itself moves ~1e-6 with its OpenMP thread count).
    r, rr = np.array(res.residuals), z["perf_residual"]
    assert np.max(np.abs(r[:18] / rr[:18] - 1)) < 1e-12
    assert np.max(np.abs(r / rr - 1)) < 1e-6
    assert abs(res.residual_norm / z["final_residual"][0] - 1) < 1e-6
    assert [1] + x.ranks + [1] == list(z["x_final_ranks"])
    assert rel_err(o.tt_entries(x, z["x_final_probe_pos"]), z["x_final_probe_val"]) < 1e-9, \
        rel_err(o.tt_entries(x, z["x_final_probe_pos"]), z["x_final_probe_val"])


@pytest.mark.parametrize("tag", ["keep", "drop"])
def test_qc_rank_rule_with_clear_gap(golden, tag):
    """Rank-revealing move_core on x + s w (block cores, bonds rescaled): with s = 1e-10
    the w part is kept, with s = 1e-17 dropped where R_00 > 0; exact ranks either way."""
    z = golden("qc_gap")
    zz = tt_of(z, f"{tag}_z", canonicalized=False)
    for p in (6, 0, 3):
        y = zz.copy()
        o.move_core(y, p, keep_rank=False)
        assert [1] + y.ranks + [1] == list(z[f"{tag}_qc_to{p}_ranks"])
        assert rel_err(o.tt_entries(y, z[f"{tag}_qc_to{p}_probe_pos"]), z[f"{tag}_qc_to{p}_probe_val"]) < REL_TOL


@pytest.mark.parametrize("alg,kind,spd", [(a, k, s) for a in ("gcg", "sd") for k in ("hosvd", "als") for s in (True, False)])
def test_hosvd_and_als_retractions(golden, alg, kind, spd):
    """GeometricCG (type I retractions) and SteepestDescent (type II) with the HOSVD and ALS
    retractions (retractions.cpp:43-69) against the reference's runs: every step's residual
    and the final iterate."""
    z = golden("retractions")
    A = op_of(z, "A" if spd else "An")
    x, b = tt_of(z, "x0"), tt_of(z, "b")
    tag = f"{alg}_{kind}_{'spd' if spd else 'ls'}"
    fn = o.geometric_cg if alg == "gcg" else o.steepest_descent
    res, trace = fn(A, x, b, 8, 1e-8, spd, retraction=kind)
    assert rel_err(trace, z[tag + "_perf_residual"]) < 1e-9
    assert abs(res / z[tag + "_residual"][0] - 1) < 1e-9
    assert [1] + x.ranks + [1] == list(z[tag + "_ranks"])
    assert rel_err(o.tt_entries(x, z[tag + "_x_probe_pos"]), z[tag + "_x_probe_val"]) < 1e-8


def test_iht_matches_reference(golden):
    """IHT (iht.cpp:29-155), capped at 11 iterations: the reference's residual after every
    iteration (its PerformanceData) and the probes of its iterate after the eleventh."""
    z = golden("iht")
    x = tt_of(z, "x0")
    res, trace = o.iht(x, z["positions"], z["values"], 11)
    assert rel_err(trace, z["perf_residual"]) < 1e-12
    assert rel_err(o.tt_entries(x, z["probe_pos"]), z["probe_val"][10]) < 1e-11
