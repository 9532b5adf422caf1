"""TT sums (TTNetwork::operator+= / -=, src/xerus/ttNetwork.cpp:796-856) and
operator products (the TTStack cast, src/xerus/ttStack.cpp:47-173) against the
reference (tests/golden/arith.npz, oracle/ref/golden_driver.cpp case_arith):
ranks exact, canonical flags exact, full tensors to 1e-12 relative. A sum with
a canonical left operand and a product with a canonical operator end in a
rank-revealing move_core, so their ranks are the reference's QC decisions."""
import numpy as np
import pytest

from oracle import xtt_oracle as o
from tests.helpers import op_of, rel_err, tt_of


def _inputs(z):
    x, y = tt_of(z, "x"), tt_of(z, "y")  # TTTensor::random: canonical at 0
    return x, y, op_of(z, "A"), op_of(z, "Ar")


def _check(z, name, full, ranks, canon):
    assert list(ranks) == list(z[name + "_ranks"]), name
    assert rel_err(full.ravel(), z[name + "_full"]) < 1e-12, name
    assert canon == (bool(z[name + "_canon"][0]), int(z[name + "_canon"][1])), name


def _apply(A, canon, x):
    y = o.op_apply(A, x)
    y.canonicalized = False
    if canon[0]:
        o.move_core(y, int(canon[1]), keep_rank=False)
    return y


def test_oracle_sums_and_products_match_reference(golden):
    z = golden("arith")
    x, y, A, Ar = _inputs(z)
    for name, t in (("sum", o.tt_add(x, y)), ("diff", o.tt_add(x, o.tt_scale(y, -1.0))),
                    ("twice", o.tt_add(x, x))):
        _check(z, name, o.tt_full(t), [1] + t.ranks + [1], (t.canonicalized, t.core_position if t.canonicalized else 0))
    assert not z["A_canon"][0] and z["Ar_canon"][0]
    ax = _apply(A, z["A_canon"], x)
    arx = _apply(Ar, z["Ar_canon"], x)
    axx = o.tt_add(ax, x)
    aarx = o.op_apply(A, o.op_apply(Ar, x))
    for name, t in (("Ax", ax), ("Arx", arx), ("Ax_plus_x", axx), ("AAr_x", aarx)):
        _check(z, name, o.tt_full(t), [1] + t.ranks + [1], (t.canonicalized, t.core_position if t.canonicalized else 0))


@pytest.mark.gpu
def test_device_sums_and_products_match_reference(golden):
    xg = pytest.importorskip("xerus_gb300")
    from xerus_gb300 import build
    build.build()
    ctx = xg.Context(0)
    z = golden("arith")
    xh, yh, Ah, Arh = _inputs(z)
    x = xg.TTTensor.from_cores(xh.cores, ctx=ctx, canonicalized=True, core_position=0)
    y = xg.TTTensor.from_cores(yh.cores, ctx=ctx, canonicalized=True, core_position=0)
    A = xg.TTOperator.from_cores(Ah.cores, ctx=ctx)
    Ar = xg.TTOperator.from_cores(Arh.cores, ctx=ctx, canonicalized=True, core_position=0)

    def full(t):
        return o.tt_full(o.TT(t.get_cores()))

    def state(t):
        return (t.canonicalized, t.corePosition if t.canonicalized else 0)

    for name, t in (("sum", x + y), ("diff", x - y), ("Ax", A @ x), ("Arx", Ar @ x), ("Ax_plus_x", (A @ x) + x),
                    ("AAr_x", (A @ Ar) @ x)):
        _check(z, name, full(t), [1] + t.ranks() + [1], state(t))
    # x + x is exactly rank-deficient: its R_kk sit at rounding level, where any two QR
    # implementations may decide differently; the tensor itself must agree
    t = x + x
    assert rel_err(full(t).ravel(), z["twice_full"]) < 1e-12
    ref = list(z["twice_ranks"])
    assert all(3 <= r <= q or r == q == 1 for r, q in zip([1] + t.ranks() + [1], ref))
    # operator-operator product: ranks R R' and not canonical (A is not)
    aa = A @ Ar
    assert [1] + aa.ranks() + [1] == [1] + list(z["AAr_ranks"]) + [1]
    assert not aa.canonicalized
    # in place: x -= y then x += y returns to x (up to rounding; x canonical: ranks via QC)
    w = x.copy()
    w -= y
    w += y
    assert rel_err(full(w).ravel(), full(x).ravel()) < 1e-12
