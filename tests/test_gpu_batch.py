"""Batched ALS_SPD (one persistent launch over independent instances of uneven
order, mode size and rank) against the oracle's ALS_SPD run instance by
instance (src/xerus/algorithms/als.cpp:483-553 restated): energies within 1e-10
relative, iterates within 1e-9 at probed entries."""
import numpy as np
import pytest

from oracle import xtt_oracle as o
from tests.helpers import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

xg = pytest.importorskip("xerus_gb300")


@pytest.fixture(scope="module")
def ctx():
    from xerus_gb300 import build
    build.build()
    return xg.Context(0)


def make_instances(count, seed, max_d=6, max_n=4, max_r=6):
    """Config-4-style instances at oracle-friendly sizes: Laplacian sum plus a
    shift U[0.1, 1], random rhs and start (the reference's TTTensor::random)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        d = int(rng.integers(2, max_d + 1))
        n = int(rng.integers(2, max_n + 1))
        shift = float(rng.uniform(0.1, 1.0))
        rs = o.RandomEngine(0xBA7C4 + i)
        A = o.laplace_operator(d, n, shift=shift)
        b = o.tt_random([n] * d, int(rng.integers(1, 4)), rs)
        x = o.tt_random([n] * d, int(rng.integers(2, max_r + 1)), rs)
        x = o.tt_scale(x, 1.0 / o.frob_norm(x))
        out.append((A, x, b))
    return out


def dev(ctx, inst):
    A, x, b = inst
    return (xg.TTOperator.from_cores(A.cores, ctx=ctx),
            xg.TTTensor.from_cores(x.cores, ctx=ctx, canonicalized=x.canonicalized, core_position=x.core_position),
            xg.TTTensor.from_cores(b.cores, ctx=ctx, canonicalized=b.canonicalized, core_position=b.core_position))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_als_batch_matches_oracle(ctx, precision):
    insts = make_instances(12, 4)
    devs = [dev(ctx, t) for t in insts]
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    if precision == "mixed":
        v.precision = xg.MIXED
    hs = 6
    en, it, rep = xg.als_batch([t[0] for t in devs], [t[1] for t in devs], [t[2] for t in devs], variant=v,
                               numHalfSweeps=hs)
    assert rep["ctas"] >= 1 and np.all(it > 0)
    rng = np.random.default_rng(9)
    for (A, x0, b), (_, xd, _), e in zip(insts, devs, en):
        x = x0.copy()
        ref = o.als_spd(A, x, b, 1, hs, 0.0)
        assert abs(e / ref.energy - 1) < REL_TOL
        assert xd.canonicalized and xd.corePosition == x.core_position
        pos = np.stack([rng.integers(0, n, 32) for n in x.dims], axis=1).astype(np.int64)
        assert rel_err(xd.entries(pos), o.tt_entries(x, pos)) < 1e-9


def test_als_batch_graph_replay_and_autotune(ctx):
    """A second call with the same signature replays the captured graph and gives
    the same result as the first; autotuning restores x between its trials."""
    insts = make_instances(40, 5, max_d=5, max_n=3, max_r=4)
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    runs = []
    for autotune in (True, False, False):
        devs = [dev(ctx, t) for t in insts]
        en, it, rep = xg.als_batch([t[0] for t in devs], [t[1] for t in devs], [t[2] for t in devs], variant=v,
                                   numHalfSweeps=4, autotune=autotune)
        runs.append((en, [t[1].get_flat() for t in devs], rep))
    for en, flats, rep in runs[1:]:
        assert np.array_equal(en, runs[0][0])
        for f0, f1 in zip(runs[0][1], flats):
            assert np.array_equal(f0, f1)
    assert runs[1][2]["threads"] == runs[0][2]["threads"]
    x = insts[0][1].copy()
    ref = o.als_spd(insts[0][0], x, insts[0][2], 1, 4, 0.0)
    assert abs(runs[0][0][0] / ref.energy - 1) < REL_TOL


_CFG4 = {}


def _config4_reference(ctx, hs):
    """24 instances of the benchmarked config-4 batch (d <= 16, n <= 8, start rank <= 32):
    the six with the largest local systems (up to 8192 unknowns) and 18 drawn at random,
    with the oracle's ALS_SPD result for each (its exact local solve by matrix-free CG,
    the same solution as the dense factorisation at these sizes), computed once."""
    if hs in _CFG4:
        return _CFG4[hs]
    import bench
    params = bench.config4_params(4096)

    def local_unknowns(p):
        d, n, _, _, rx = p
        rr = o.reduce_to_maximal_ranks([rx] * (d - 1), [n] * d)
        return max(rr) ** 2 * n

    order = sorted(range(len(params)), key=lambda i: -local_unknowns(params[i]))
    rng = np.random.default_rng(17)
    pick = [int(i) for i in order[:6]] + [int(i) for i in rng.choice(order[6:], 18, replace=False)]
    out = []
    for i in pick:
        A, x, b = bench.config4_instance(xg, ctx, i, params[i])
        Ah = o.TTOp(A.get_cores())
        xh = o.TT(x.get_cores(), x.canonicalized, x.corePosition)
        bh = o.TT(b.get_cores(), b.canonicalized, b.corePosition)
        x0 = xh.copy()
        ref = o.als_spd(Ah, xh, bh, 1, hs, 0.0, solver="cg")
        out.append((i, params[i], Ah, x0, bh, ref.energy, xh))
    _CFG4[hs] = out
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_als_batch_matches_oracle_at_config4_sizes(ctx, precision):
    """The benchmarked batch's own instances at their real sizes, in one batched call:
    the largest local systems (8192 unknowns in one CTA), uneven orders and ranks under
    the longest-first schedule. Each instance's energy within 1e-10 of the oracle's.
    The iterate itself is not that well determined: at start rank 32 the sweep moves
    slowly along near-flat directions, so the local solves' tolerance (1e-13 here,
    ~1e-15 in the oracle) shows up ~1e6-fold in the entries after 8 half-sweeps (the
    oracle alone moves 1e-7 between tolerances 1e-15 and 1e-13 on instance 941), while
    the energy, stationary there, does not: probed entries within 1e-6."""
    hs = 8
    cases = _config4_reference(ctx, hs)
    assert max(p[1] * max(o.reduce_to_maximal_ranks([p[4]] * (p[0] - 1), [p[1]] * p[0])) ** 2
               for _, p, *_ in cases) == 8192
    devs = [(xg.TTOperator.from_cores(Ah.cores, ctx=ctx),
             xg.TTTensor.from_cores(x0.cores, ctx=ctx, canonicalized=x0.canonicalized, core_position=x0.core_position),
             xg.TTTensor.from_cores(bh.cores, ctx=ctx, canonicalized=bh.canonicalized, core_position=bh.core_position))
            for _, _, Ah, x0, bh, _, _ in cases]
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    if precision == "mixed":
        v.precision = xg.MIXED
    en, it, rep = xg.als_batch([t[0] for t in devs], [t[1] for t in devs], [t[2] for t in devs], variant=v,
                               numHalfSweeps=hs)
    assert np.all(it > 0)
    rng = np.random.default_rng(23)
    for (i, p, _, _, _, e_ref, x_ref), (_, xd, _), e in zip(cases, devs, en):
        assert abs(e / e_ref - 1) < REL_TOL, (i, p, e, e_ref)
        pos = np.stack([rng.integers(0, n, 32) for n in x_ref.dims], axis=1).astype(np.int64)
        assert rel_err(xd.entries(pos), o.tt_entries(x_ref, pos)) < 1e-6, (i, p)
