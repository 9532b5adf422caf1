"""CPU restatement of the xerus Tensor-Train sweep path, used ONLY as a checker.

This module is test infrastructure. It is imported by ``tests/``, by
``__graft_entry__.smoke()`` and by the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` - never by the product package ``xerus_gb300``.

It restates, in FP64 numpy/scipy on top of LAPACK, the reference's algorithms:

* RNG streams: ``std::mt19937_64``, libstdc++'s ``normal_distribution`` (Marsaglia
  polar method with one cached variate), ``uniform_int_distribution`` (Lemire's
  nearly-divisionless reduction on a 128-bit product) and
  ``uniform_real_distribution`` (``generate_canonical``), as used by
  ``src/xerus/misc/random.cpp:29-30``, ``include/xerus/tensor.h:213-220`` and
  ``src/xerus/measurments.cpp:222-248``.
* ``TTNetwork::random`` (``include/xerus/ttNetwork.h:128-155``),
  ``reduce_to_maximal_ranks`` (``src/xerus/ttNetwork.cpp:369-402``).
* ``move_core`` / ``transfer_core`` (``src/xerus/ttNetwork.cpp:581-628``,
  ``src/xerus/tensorNetwork.cpp:821-909``) with the QC/CQ rank rule of
  ``src/xerus/blasLapackWrapper.cpp:243-371`` (first k with
  ``|R[k,k]| < 16 eps R[0,0]``, compared against the SIGNED ``R[0,0]``).
* ``round`` / ``round_edge`` (``src/xerus/ttNetwork.cpp:643-684``,
  ``src/xerus/tensorNetwork.cpp:678-818``) and the SVD truncation rule of
  ``calculate_svd`` (``src/xerus/tensor.cpp:1463-1474``).
* The TT dot product / ``frob_norm`` (``src/xerus/ttNetwork.cpp:781-789``).
* ``ALSVariant::solve`` with ``lapack_solver`` / ``ASD_solver`` for SPD operators,
  1 and 2 sites (``src/xerus/algorithms/als.cpp:43-553``).
* ``ADFVariant`` for ``SinglePointMeasurementSet`` (``src/xerus/algorithms/adf.cpp``).

Parity of this restatement is pinned against golden vectors produced by the
reference itself (compiled from its own sources against SciPy's OpenBLAS 0.3.34,
see ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

EPS = np.finfo(np.float64).eps
EPSILON = 8 * EPS  # include/xerus/basic.h:50

# --------------------------------------------------------------------------- RNG

_MASK64 = (1 << 64) - 1


class MT19937_64:
    """std::mt19937_64 (the published 64-bit Mersenne Twister, MT19937-64)."""

    N, M = 312, 156

    def __init__(self, seed: int = 5489):
        self.seed(seed)

    def seed(self, seed: int) -> None:
        mt = [0] * self.N
        mt[0] = seed & _MASK64
        for i in range(1, self.N):
            mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & _MASK64
        self._mt = np.array(mt, dtype=np.uint64)
        self._idx = self.N
        self._buf = None

    def _twist(self) -> None:
        mt = self._mt
        N, M = self.N, self.M
        upper = np.uint64(0xFFFFFFFF80000000)
        lower = np.uint64(0x7FFFFFFF)
        mag = np.uint64(0xB5026F5AA96619E9)
        one = np.uint64(1)

        def step(lo, hi, nxt):
            y = (mt[lo:hi] & upper) | (mt[lo + 1:hi + 1] & lower)
            return nxt ^ (y >> one) ^ np.where((y & one) != 0, mag, np.uint64(0))

        mt[0:N - M] = step(0, N - M, mt[M:N])
        mt[N - M:N - 1] = step(N - M, N - 1, mt[0:M - 1])
        y = (mt[N - 1] & upper) | (mt[0] & lower)
        mt[N - 1] = mt[M - 1] ^ (y >> one) ^ (mag if (int(y) & 1) else np.uint64(0))
        # tempering of the whole block
        z = mt.copy()
        z ^= (z >> np.uint64(29)) & np.uint64(0x5555555555555555)
        z ^= (z << np.uint64(17)) & np.uint64(0x71D67FFFEDA60000)
        z ^= (z << np.uint64(37)) & np.uint64(0xFFF7EEE000000000)
        z ^= z >> np.uint64(43)
        self._buf = [int(v) for v in z]
        self._idx = 0

    def __call__(self) -> int:
        if self._idx >= self.N:
            self._twist()
        v = self._buf[self._idx]
        self._idx += 1
        return v


def canonical(eng: MT19937_64) -> float:
    """std::generate_canonical<double, 53>(mt19937_64): one draw / 2^64."""
    r = float(eng()) / 18446744073709551616.0
    return r if r < 1.0 else math.nextafter(1.0, 0.0)


class NormalDist:
    """libstdc++ std::normal_distribution<double> (polar method, cached variate)."""

    def __init__(self, mean: float = 0.0, stddev: float = 1.0):
        self.mean, self.stddev = mean, stddev
        self.reset()

    def reset(self) -> None:
        self._saved = None

    def __call__(self, eng: MT19937_64) -> float:
        if self._saved is not None:
            ret, self._saved = self._saved, None
        else:
            while True:
                x = 2.0 * canonical(eng) - 1.0
                y = 2.0 * canonical(eng) - 1.0
                r2 = x * x + y * y
                if not (r2 > 1.0 or r2 == 0.0):
                    break
            mult = math.sqrt(-2.0 * math.log(r2) / r2)
            self._saved = x * mult
            ret = y * mult
        return ret * self.stddev + self.mean

    def draw(self, eng: MT19937_64, count: int) -> np.ndarray:
        return np.array([self(eng) for _ in range(count)], dtype=np.float64)


def uniform_int(eng: MT19937_64, a: int, b: int) -> int:
    """libstdc++ std::uniform_int_distribution<size_t>(a, b) on a 64-bit engine."""
    rng = b - a + 1  # the engine covers [0, 2^64), rng < 2^64 here
    if rng == 0:
        return a + eng()
    prod = eng() * rng
    low = prod & _MASK64
    if low < rng:
        threshold = ((1 << 64) - rng) % rng
        while low < threshold:
            prod = eng() * rng
            low = prod & _MASK64
    return a + (prod >> 64)


def uniform_real(eng: MT19937_64, a: float = 0.0, b: float = 1.0) -> float:
    """libstdc++ std::uniform_real_distribution<double>(a, b)."""
    return canonical(eng) * (b - a) + a


class RandomEngine:
    """The reference's default random state: an engine plus the normal
    distribution object whose cached variate carries over between calls."""

    def __init__(self, seed: int = 0xBAADF00D):
        self.eng = MT19937_64(seed)
        self.normal = NormalDist()

    def reseed(self, seed: int = 0xBAADF00D) -> None:
        self.eng.seed(seed)
        self.normal.reset()


# --------------------------------------------------------------------------- TT container


@dataclass
class TT:
    """A TT tensor: cores (r_{k-1}, n_k, r_k), row-major; canonical flag and core position."""

    cores: list
    canonicalized: bool = False
    core_position: int = 0

    @property
    def d(self):
        return len(self.cores)

    @property
    def dims(self):
        return [c.shape[1] for c in self.cores]

    @property
    def ranks(self):
        return [c.shape[2] for c in self.cores[:-1]]

    def copy(self):
        return TT([c.copy() for c in self.cores], self.canonicalized, self.core_position)


@dataclass
class TTOp:
    """A TT operator: cores (R_{k-1}, n_k (row), n_k (col), R_k)."""

    cores: list

    @property
    def d(self):
        return len(self.cores)


def tt_from_flat(dims, ranks, data) -> TT:
    cores, off = [], 0
    for k, n in enumerate(dims):
        sz = ranks[k] * n * ranks[k + 1]
        cores.append(np.asarray(data[off:off + sz], dtype=np.float64).reshape(ranks[k], n, ranks[k + 1]).copy())
        off += sz
    return TT(cores)


def op_from_flat(dims, ranks, data) -> TTOp:
    cores, off = [], 0
    for k, n in enumerate(dims):
        sz = ranks[k] * n * n * ranks[k + 1]
        cores.append(np.asarray(data[off:off + sz], dtype=np.float64).reshape(ranks[k], n, n, ranks[k + 1]).copy())
        off += sz
    return TTOp(cores)


def reduce_to_maximal_ranks(ranks, dims):
    """src/xerus/ttNetwork.cpp:369-402 (TTTensor case)."""
    ranks = list(ranks)
    d = len(dims)
    cur = 1
    for i in range(d - 1):
        cur *= dims[i]
        if cur < ranks[i]:
            ranks[i] = cur
        else:
            cur = ranks[i]
    cur = 1
    for i in range(1, d):
        cur *= dims[d - i]
        if cur < ranks[d - i - 1]:
            ranks[d - i - 1] = cur
        else:
            cur = ranks[d - i - 1]
    return ranks


def tt_random(dims, ranks, rs: RandomEngine, dist: NormalDist | None = None) -> TT:
    """TTNetwork::random (include/xerus/ttNetwork.h:128-155): fill each core in
    order, row-major, one draw per entry, then move_core(0) with QC."""
    dist = dist if dist is not None else rs.normal
    if isinstance(ranks, int):
        ranks = [ranks] * (len(dims) - 1)
    r = [1] + reduce_to_maximal_ranks(ranks, dims) + [1]
    cores = []
    for k, n in enumerate(dims):
        cores.append(dist.draw(rs.eng, r[k] * n * r[k + 1]).reshape(r[k], n, r[k + 1]))
    x = TT(cores, canonicalized=True, core_position=0)
    # TTNetwork(dims) starts canonical at 0, set_component on k > 0 clears it.
    x.canonicalized = len(dims) == 1
    move_core(x, 0, keep_rank=False)
    return x


def tt_full(x: TT) -> np.ndarray:
    v = x.cores[0]
    for c in x.cores[1:]:
        v = np.tensordot(v, c, axes=([v.ndim - 1], [0]))
    return v.reshape(x.dims)


def tt_entries(x: TT, positions: np.ndarray) -> np.ndarray:
    """Entries at multi-indices (N, d), by left-to-right slice products."""
    positions = np.asarray(positions)
    v = np.ones((positions.shape[0], 1))
    for k, c in enumerate(x.cores):
        v = np.einsum("sa,sab->sb", v, c[:, positions[:, k], :].transpose(1, 0, 2))
    return v[:, 0]


def tt_dot(x: TT, y: TT) -> float:
    """Full contraction <x, y> by the left-to-right zipper."""
    m = np.ones((1, 1))
    for a, b in zip(x.cores, y.cores):
        t = np.tensordot(m, a, axes=([0], [0]))  # (s, n, r)
        m = np.tensordot(t, b, axes=([0, 1], [0, 1]))  # (r, r')
    return float(m[0, 0])


def frob_norm(x: TT) -> float:
    """src/xerus/ttNetwork.cpp:781-789: the core's norm when canonical, else sqrt(<x,x>)."""
    if x.canonicalized:
        return float(np.linalg.norm(x.cores[x.core_position]))
    return math.sqrt(tt_dot(x, x))


def tt_add(x: TT, y: TT) -> TT:
    """TTNetwork::operator+= block structure (src/xerus/ttNetwork.cpp:796-847)."""
    d = x.d
    cores = []
    for k in range(d):
        a, b = x.cores[k], y.cores[k]
        r0 = 1 if k == 0 else a.shape[0] + b.shape[0]
        r1 = 1 if k == d - 1 else a.shape[2] + b.shape[2]
        c = np.zeros((r0, a.shape[1], r1))
        c[:a.shape[0], :, :a.shape[2]] += a
        lo = 0 if k == 0 else a.shape[0]
        ro = 0 if k == d - 1 else a.shape[2]
        c[lo:lo + b.shape[0], :, ro:ro + b.shape[2]] += b
        cores.append(c)
    out = TT(cores, canonicalized=False)
    if x.canonicalized:
        move_core(out, x.core_position, keep_rank=False)
    return out


def tt_scale(x: TT, f: float) -> TT:
    y = x.copy()
    y.cores[y.core_position if y.canonicalized else 0] *= f
    return y


# --------------------------------------------------------------------------- factorisations


def qc(a: np.ndarray):
    """Rank-revealing QR with column pivoting (dgeqp3 + dorgqr),
    src/xerus/blasLapackWrapper.cpp:243-305. Returns (Q (m x rank), C (rank x n), rank)."""
    m, n = a.shape
    q, r, piv = scipy.linalg.qr(a, mode="economic", pivoting=True)
    max_rank = min(m, n)
    rank = 1
    while rank <= max_rank:
        if rank == max_rank or abs(r[rank, rank]) < 16 * EPS * r[0, 0]:
            break
        rank += 1
    c = np.zeros((rank, n))
    c[:, piv] = np.triu(r[:rank, :])
    return q[:, :rank].copy(), c, rank


def cq(a: np.ndarray):
    """A = C Q with Q row-orthonormal: the transposed QC (blasLapackWrapper.cpp:317-371)."""
    qt, ct, rank = qc(a.T)
    return ct.T.copy(), qt.T.copy(), rank


def qr(a: np.ndarray):
    q, r = np.linalg.qr(a, mode="reduced")
    return q, r


def rq(a: np.ndarray):
    m, n = a.shape
    if m <= n:
        r, q = scipy.linalg.rq(a, mode="economic")
        return r, q
    # more rows than columns: R is m x n, Q is n x n (blasLapackWrapper.cpp:455-498)
    r, q = scipy.linalg.rq(a, mode="full")
    return r[:, m - n:], q[m - n:, :] if q.shape[0] > n else q


def svd_trunc(x: np.ndarray, max_rank: int, eps: float, canonical_signs: bool = False):
    """calculate_svd (src/xerus/tensor.cpp:1424-1489): dgesdd, then the
    rank = min(rank, maxRank) cap and the first j >= 1 with S[j] <= eps*S[0].
    canonical_signs: flip each singular pair so that the largest-magnitude entry
    (first on ties) of the left vector is positive (the device's sign gauge)
    instead of keeping LAPACK's."""
    u, s, vt = np.linalg.svd(x, full_matrices=False)
    rank = len(s)
    if max_rank:
        rank = min(rank, max_rank)
    for j in range(1, rank):
        if s[j] <= eps * s[0]:
            rank = j
            break
    u, s, vt = u[:, :rank], s[:rank], vt[:rank, :]
    if canonical_signs:
        idx = np.argmax(np.abs(u), axis=0)
        f = np.where(u[idx, np.arange(rank)] < 0, -1.0, 1.0)
        u, vt = u * f[None, :], vt * f[:, None]
    return u, s, vt


# --------------------------------------------------------------------------- core movement


def transfer_core(x: TT, frm: int, to: int, allow_rank_reduction: bool) -> None:
    """src/xerus/tensorNetwork.cpp:821-909 for neighbouring TT cores."""
    f = x.cores[frm]
    r0, n, r1 = f.shape
    if to == frm + 1:
        mat = f.reshape(r0 * n, r1)
        if allow_rank_reduction:
            q, rmat, rank = qc(mat)
        else:
            q, rmat = qr(mat)
            rank = q.shape[1]
        x.cores[frm] = q.reshape(r0, n, rank)
        nxt = x.cores[to]
        x.cores[to] = np.tensordot(rmat, nxt, axes=([1], [0]))
    else:
        mat = f.reshape(r0, n * r1)
        if allow_rank_reduction:
            cmat, q, rank = cq(mat)
        else:
            cmat, q = rq(mat)
            rank = q.shape[0]
        x.cores[frm] = q.reshape(rank, n, r1)
        prv = x.cores[to]
        x.cores[to] = np.tensordot(prv, cmat, axes=([2], [0]))


def exceeds_maximal_ranks(x: TT) -> bool:
    return x.ranks != reduce_to_maximal_ranks(x.ranks, x.dims)


def move_core(x: TT, pos: int, keep_rank: bool = False) -> None:
    """TTNetwork::move_core (src/xerus/ttNetwork.cpp:581-628)."""
    d = x.d
    if x.canonicalized:
        for n in range(x.core_position, pos):
            transfer_core(x, n, n + 1, not keep_rank)
        for n in range(x.core_position, pos, -1):
            transfer_core(x, n, n - 1, not keep_rank)
    else:
        for n in range(0, pos):
            transfer_core(x, n, n + 1, not keep_rank)
        for n in range(d - 1, pos, -1):
            transfer_core(x, n, n - 1, not keep_rank)
    while exceeds_maximal_ranks(x):
        for n in range(pos, 0, -1):
            transfer_core(x, n, n - 1, not keep_rank)
        for n in range(0, d - 1):
            transfer_core(x, n, n + 1, not keep_rank)
        for n in range(d - 1, pos, -1):
            transfer_core(x, n, n - 1, not keep_rank)
    x.canonicalized = True
    x.core_position = pos


def round_edge(x: TT, frm: int, to: int, max_rank: int, eps: float, spectra=None) -> None:
    """TensorNetwork::round_edge (src/xerus/tensorNetwork.cpp:678-818) for
    from = core k+1 (bond on its left) and to = core k (bond on its right)."""
    F, T = x.cores[frm], x.cores[to]
    r, n, r1 = F.shape
    r2, n2, _ = T.shape
    if 5 * F.size * T.size >= 6 * r ** 4:
        coreA, Fq, ka = cq(F.reshape(r, n * r1))            # F = coreA Fq
        Tq, coreB, kb = qc(T.reshape(r2 * n2, r))           # T = Tq coreB
        X = coreA.T @ coreB.T                               # (ka, kb)
        U, S, Vt = svd_trunc(X, max_rank, eps)
        coreB = S[:, None] * Vt
        x.cores[frm] = (U.T @ Fq).reshape(len(S), n, r1)
        x.cores[to] = (Tq @ coreB.T).reshape(r2, n2, len(S))
    else:
        X = F.reshape(r, n * r1).T @ T.reshape(r2 * n2, r).T    # (n r1, r2 n2)
        U, S, Vt = svd_trunc(X, max_rank, eps)
        s = len(S)
        x.cores[frm] = U.reshape(n, r1, s).transpose(2, 0, 1).copy()
        x.cores[to] = (Vt.T * S[None, :]).reshape(r2, n2, s)
    if spectra is not None:
        spectra.append(S.copy())


def tt_round(x: TT, max_ranks, eps: float = EPSILON, spectra=None) -> None:
    """TTNetwork::round(maxRanks, eps) (src/xerus/ttNetwork.cpp:643-665)."""
    d = x.d
    if isinstance(max_ranks, int):
        max_ranks = [max_ranks] * (d - 1)
    init_canon, init_pos = x.canonicalized, x.core_position
    move_core(x, d - 1, keep_rank=False)
    for i in range(d - 1):
        round_edge(x, d - 1 - i, d - 2 - i, max_ranks[d - 2 - i], eps, spectra)
    x.canonicalized, x.core_position = True, 0
    if init_canon:
        move_core(x, init_pos, keep_rank=False)


def orthogonal_norm(x: TT) -> float:
    """||x|| through a left-to-right QR sweep: accurate even when the entries
    cancel (e.g. x = A y - b near a solution)."""
    y = x.copy()
    y.canonicalized = False
    for k in range(y.d - 1):
        transfer_core(y, k, k + 1, False)
    return float(np.linalg.norm(y.cores[-1]))


# --------------------------------------------------------------------------- operator application


def op_apply(A: TTOp, x: TT) -> TT:
    """The TT of A x, core by core with ranks R_k r_k."""
    cores = []
    for a, c in zip(A.cores, x.cores):
        t = np.einsum("kijl,ajb->kailb", a, c)
        K, ra, n, L, rb = t.shape
        cores.append(t.reshape(K * ra, n, L * rb))
    return TT(cores)


def residual(A: TTOp, x: TT, b: TT) -> float:
    """||A x - b|| / ||b|| in FP64 through orthogonalisation (no cancellation)."""
    diff = tt_add(op_apply(A, x), tt_scale(b, -1.0))
    return orthogonal_norm(diff) / orthogonal_norm(b)


def laplace_operator(d: int, n: int, V=None, rank3: bool = False, shift: float = 0.0) -> TTOp:
    """sum_i I x..x (L (+V_i)) x..x I, L = tridiag(-1, 2, -1); the same
    construction as the golden driver (rank 2, or rank 3 with V in its own channel)."""
    L = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    I = np.eye(n)
    R = 3 if rank3 else 2
    cores = []
    for k in range(d):
        Vk = np.diag(V[k]) if V is not None else np.zeros((n, n))
        l = L + (0 if rank3 else Vk) + shift * I / d
        rl, rr = (1 if k == 0 else R), (1 if k == d - 1 else R)
        c = np.zeros((rl, n, n, rr))
        if d == 1:
            c[0, :, :, 0] = L + Vk + shift * I
        elif k == 0:
            c[0, :, :, 0] = l + (Vk if rank3 else 0)
            c[0, :, :, 1] = I
            if rank3:
                c[0, :, :, 2] = I
        elif k == d - 1:
            c[0, :, :, 0] = I
            c[1, :, :, 0] = l
            if rank3:
                c[2, :, :, 0] = Vk
        else:
            c[0, :, :, 0] = I
            c[1, :, :, 0] = l
            c[1, :, :, 1] = I
            if rank3:
                c[2, :, :, 0] = Vk
                c[2, :, :, 2] = I
        cores.append(c)
    return TTOp(cores)


# --------------------------------------------------------------------------- ALS (SPD)

FLAG_FINISHED_HALFSWEEP = 1
FLAG_FINISHED_FULLSWEEP = 3


def _push_left_op(L, xc, ac):
    # L'(c1,c2,c3) = sum L(a1,a2,a3) x(a1,i,c1) A(a2,i,j,c2) x(a3,j,c3)   (als.cpp:184-200, 247)
    t = np.tensordot(L, xc, axes=([0], [0]))             # (k, y, i, c)
    t = np.tensordot(t, ac, axes=([0, 2], [0, 1]))       # (y, c, j, l)
    return np.tensordot(t, xc, axes=([0, 2], [0, 1]))    # (c, l, m)


def _push_right_op(R, xc, ac):
    # R'(a1,a2,a3) = sum x(a1,i,c1) A(a2,i,j,c2) x(a3,j,c3) R(c1,c2,c3)   (als.cpp:239)
    t = np.tensordot(xc, R, axes=([2], [0]))             # (x, i, l, m)
    t = np.tensordot(t, ac, axes=([1, 2], [1, 3]))       # (x, m, k, j)
    return np.tensordot(t, xc, axes=([1, 3], [2, 1]))    # (x, k, y)


def _push_left_rhs(Lb, bc, xc):
    # Lb'(c1,c2) = sum Lb(a1,a2) b(a1,i,c1) x(a2,i,c2)   (als.cpp:202-215, 250)
    t = np.tensordot(Lb, bc, axes=([0], [0]))            # (t, i, c)
    return np.tensordot(t, xc, axes=([0, 1], [0, 1]))    # (c, d)


def _push_right_rhs(Rb, bc, xc):
    # Rb'(a1,a2) = sum b(a1,i,c1) x(a2,i,c2) Rb(c1,c2)   (als.cpp:242)
    t = np.tensordot(bc, Rb, axes=([2], [0]))            # (s, i, d)
    return np.tensordot(t, xc, axes=([1, 2], [1, 2]))    # (s, t)


# non-symmetric operators: the stacks carry A^T A and A^T b (als.cpp:184-215, 392-399, 414-420)
def _push_left_op4(L, xc, ac):
    # L'(c1..c4) = sum L(a1..a4) x(a1,n1,c1) A(a2,n2,n1,c2) A(a3,n2,n3,c3) x(a4,n3,c4)
    return np.einsum("wxyz,wia,xjib,yjkc,zkd->abcd", L, xc, ac, ac, xc, optimize=True)


def _push_right_op4(R, xc, ac):
    return np.einsum("wia,xjib,yjkc,zkd,abcd->wxyz", xc, ac, ac, xc, R, optimize=True)


def _push_left_rhs3(Lb, bc, ac, xc):
    # Lb'(c1,c2,c3) = sum Lb(a1,a2,a3) b(a1,n1,c1) A(a2,n1,n2,c2) x(a3,n2,c3)
    return np.einsum("stu,sia,tijb,ujc->abc", Lb, bc, ac, xc, optimize=True)


def _push_right_rhs3(Rb, bc, ac, xc):
    return np.einsum("sia,tijb,ujc,abc->stu", bc, ac, xc, Rb, optimize=True)


def local_operator_normal(L, Acores, R):
    """construct_local_operator for a non-symmetric A (als.cpp:392-399): the
    projection of A^T A, rows (a, i.., b), columns (a', j.., b')."""
    if len(Acores) == 1:
        op = np.einsum("xkqa,kmil,qmjp,ylpb->xiyajb", L, Acores[0], Acores[0], R, optimize=True)
    else:
        a0, a1 = Acores
        op = np.einsum("rkqc,kmil,qmjp,lotu,pozv,suve->ritscjze", L, a0, a0, a1, a1, R, optimize=True)
    half = op.ndim // 2
    N = int(np.prod(op.shape[:half]))
    return op.reshape(N, N), op.shape[half:]


def local_rhs_normal(Lb, bcores, Acores, Rb):
    """construct_local_RHS for a non-symmetric A (als.cpp:414-420): projection of A^T b."""
    if len(bcores) == 1:
        return np.einsum("ska,sit,kijl,tlb->ajb", Lb, bcores[0], Acores[0], Rb, optimize=True)
    return np.einsum("ska,sit,kijl,tmu,lmzv,uvb->ajzb", Lb, bcores[0], Acores[0], bcores[1], Acores[1], Rb,
                     optimize=True)


def local_operator(L, Acores, R):
    """Dense local operator of construct_local_operator (als.cpp:383-401):
    rows (a, i_1..i_s, b), columns (a', j_1..j_s, b')."""
    if len(Acores) == 1:
        op = np.einsum("xka,kijl,ylb->xiyajb", L, Acores[0], R, optimize=True)
    else:
        op = np.einsum("xka,kijl,lmnp,ypb->ximyajnb", L, Acores[0], Acores[1], R, optimize=True)
    half = op.ndim // 2
    N = int(np.prod(op.shape[:half]))
    return op.reshape(N, N), op.shape[half:]


def local_apply(L, Acores, R, v):
    """The local operator of construct_local_operator (als.cpp:383-401) applied to a
    local vector v (a, j, b) without forming it: (x, i, y)."""
    if len(Acores) != 1:
        raise ValueError("one site only")
    t = np.tensordot(v, R, axes=([2], [2]))              # (a, j, y, l)
    t = np.tensordot(t, Acores[0], axes=([1, 3], [2, 3]))  # (a, y, k, i)
    t = np.tensordot(L, t, axes=([1, 2], [2, 0]))          # (x, y, i)
    return t.transpose(0, 2, 1)


def cg_solve(apply, rhs, tol: float = 1e-15, maxit: int | None = None):
    """Conjugate gradients on an SPD system to relative residual tol (or until the
    recomputed residual stops decreasing): the solution of the dense solve to rounding."""
    n = rhs.size
    xv = np.zeros(n)
    r = rhs.copy()
    p = r.copy()
    rr = float(r @ r)
    bb = rr
    best = rr
    since = 0
    for it in range(1, (maxit or 20 * n) + 1):
        if rr <= tol * tol * bb:
            break
        ap = apply(p)
        alpha = rr / float(p @ ap)
        xv += alpha * p
        if it % 50 == 0:
            r = rhs - apply(xv)   # refresh the recursive residual
        else:
            r -= alpha * ap
        rn = float(r @ r)
        p = r + (rn / rr) * p
        rr = rn
        if rr < 0.5 * best:
            best, since = rr, 0
        else:
            since += 1
            if since > 200:
                break
    return xv


def local_rhs(Lb, bcores, Rb):
    """construct_local_RHS (als.cpp:404-423): (a, i_1..i_s, b)."""
    if len(bcores) == 1:
        return np.einsum("sa,sit,tb->aib", Lb, bcores[0], Rb, optimize=True)
    return np.einsum("sa,sit,tju,ub->aijb", Lb, bcores[0], bcores[1], Rb, optimize=True)


def _is_symmetric(M):
    # blasLapackWrapper.cpp:500-514
    mx = max(0.0, float(M.max()))
    return np.all(np.abs(M - M.T) < 4 * mx * EPS)


def dense_solve(M, rhs):
    """xerus::solve for a square dense system (blasLapackWrapper.cpp:542-651):
    LU if not symmetric, Cholesky if the diagonal is one-signed, else LDL^T."""
    if not _is_symmetric(M):
        return scipy.linalg.solve(M, rhs)
    diag = np.diag(M)
    pos = diag[0] > 0
    onesigned = np.all(diag[1:] >= EPS) if pos else np.all(diag[1:] <= -EPS)
    if onesigned:
        try:
            c = scipy.linalg.cho_factor(M, lower=False, check_finite=False)
            return scipy.linalg.cho_solve(c, rhs, check_finite=False)
        except np.linalg.LinAlgError:
            pass
    return scipy.linalg.solve(M, rhs, assume_a="sym")


@dataclass
class ALSResult:
    energy: float
    residuals: list = field(default_factory=list)   # after every micro-step (accurate FP64)
    flags: list = field(default_factory=list)
    energies: list = field(default_factory=list)    # at the end of each half-sweep
    half_sweeps: int = 0


def als_spd(A: TTOp, x: TT, b: TT, sites: int = 1, num_half_sweeps: int = 0, conv_eps: float = 1e-6,
            solver: str = "lapack", preserve_core_position: bool = True, track_residual: bool = False,
            residual_target: float | None = None, canonical_signs: bool = False,
            exact_environment: bool = False, max_rank: int = 0, svd_epsilon: float = 0.0) -> ALSResult:
    """ALSVariant::solve for an SPD operator (ALS_SPD, DMRG_SPD, ASD_SPD); see ``als``."""
    return als(A, x, b, sites, num_half_sweeps, conv_eps, solver, preserve_core_position, track_residual,
               residual_target, canonical_signs, exact_environment, assume_spd=True, max_rank=max_rank,
               svd_epsilon=svd_epsilon)


def als(A: TTOp | None, x: TT, b: TT, sites: int = 1, num_half_sweeps: int = 0, conv_eps: float = 1e-6,
        solver: str = "lapack", preserve_core_position: bool = True, track_residual: bool = False,
        residual_target: float | None = None, canonical_signs: bool = False,
        exact_environment: bool = False, assume_spd: bool = True, use_residual: bool = False,
        max_rank: int = 0, svd_epsilon: float = 0.0) -> ALSResult:
    """ALSVariant::solve (src/xerus/algorithms/als.cpp:483-553).

    ``x`` is updated in place. ``solver`` is "lapack" (lapack_solver, als.cpp:43-71)
    or "asd" (ASD_solver, als.cpp:73-92). ``assume_spd`` False is the
    non-symmetric form (ALS, DMRG, ASD): the stacks carry A^T A and A^T b
    (als.cpp:184-215) and the energy is the residual computed from them
    (als.cpp:282-297). ``A`` None minimises ||x - b|| (the operator-free
    overloads, als.h:181-206): the local update is the projected b
    (als.cpp:540-543), the energy 0.5 |x_k|^2 - <x, b> and the residual ||x - b||
    (als.cpp:299-319). ``use_residual`` is useResidualForEndCriterion.
    With ``track_residual`` the value the reference adds to its PerformanceData
    (residual_f, als.cpp:255-320) is recorded after every micro-step.
    Two sites: the decreasing half-sweep contracts core ``cur`` into the right
    environment (als.cpp:371) as the reference does, which makes later half-
    sweeps depend on the sign gauge of the split's singular vectors;
    ``canonical_signs`` selects the device's gauge instead of LAPACK's, and
    ``exact_environment`` contracts core ``cur + 1`` (gauge-invariant).
    ``residual_target`` stops at the end of the first half-sweep whose residual
    is at or below it (a time-to-residual measurement, not a reference feature).
    ``max_rank`` > 0 (two sites) lets the split grow ranks up to that cap (and
    the bond's maximal rank) with relative cutoff ``svd_epsilon`` — the device's
    rank-growth extension; the reference keeps the ranks of x."""
    d = x.d
    free = A is None
    normal = not free and not assume_spd
    if free and sites != 1:
        raise ValueError("approximation dmrg not implemented yet")  # als.cpp:539
    target_rank = list(x.ranks)
    norm_b = frob_norm(b)
    canon_end, core_end = x.canonicalized, x.core_position
    # prepare_x_for_als (als.cpp:105-182)
    first, prod = 0, 1
    while first + 1 < d:
        nd = x.dims[first]
        newp = prod * nd
        if x.ranks[first] < newp:
            break
        comp = x.cores[first].reshape(prod * nd, x.ranks[first])
        x.cores[first + 1] = np.tensordot(comp, x.cores[first + 1], axes=([1], [0]))
        ident = np.zeros((prod, nd, newp))
        for i0 in range(prod):
            for i1 in range(nd):
                ident[i0, i1, i0 * nd + i1] = 1.0
        x.cores[first] = ident
        first += 1
        prod = newp
    last, prod = d, 1
    while last > first + sites:
        nd = x.dims[last - 1]
        newp = prod * nd
        if x.ranks[last - 2] < newp:
            break
        comp = x.cores[last - 1].reshape(x.ranks[last - 2], nd * prod)
        x.cores[last - 2] = np.tensordot(x.cores[last - 2], comp, axes=([2], [0])).reshape(
            x.cores[last - 2].shape[0], x.dims[last - 2], nd * prod)
        ident = np.zeros((newp, nd, prod))
        for i1 in range(nd):
            for i2 in range(prod):
                ident[i1 * prod + i2, i1, i2] = 1.0
        x.cores[last - 1] = ident
        last -= 1
        prod = newp
    if canon_end and core_end < first:
        x.canonicalized, x.core_position = True, first
    else:
        if canon_end and core_end >= last:
            x.canonicalized, x.core_position = True, last - 1
        move_core(x, first, keep_rank=True)

    # stack slices (localOperatorSlice / localRhsSlice, als.cpp:184-215)
    def push_op(side, E, k):
        if normal:
            return (_push_left_op4 if side == "L" else _push_right_op4)(E, x.cores[k], A.cores[k])
        return (_push_left_op if side == "L" else _push_right_op)(E, x.cores[k], A.cores[k])

    def push_rhs(side, E, k):
        if normal:
            return (_push_left_rhs3 if side == "L" else _push_right_rhs3)(E, b.cores[k], A.cores[k], x.cores[k])
        return (_push_left_rhs if side == "L" else _push_right_rhs)(E, b.cores[k], x.cores[k])

    # prepare_stacks (als.cpp:217-253)
    one_op = np.ones((1, 1, 1, 1)) if normal else np.ones((1, 1, 1))
    one_rhs = np.ones((1, 1, 1)) if normal else np.ones((1, 1))
    Lop, Rop, Lb, Rb = [one_op], [one_op], [one_rhs], [one_rhs]
    for i in range(d - 1, first + sites - 1, -1):
        if not free:
            Rop.append(push_op("R", Rop[-1], i))
        Rb.append(push_rhs("R", Rb[-1], i))
    for i in range(first):
        if not free:
            Lop.append(push_op("L", Lop[-1], i))
        Lb.append(push_rhs("L", Lb[-1], i))
    cur = first
    inc = True

    def stack_terms():
        # full contractions <x, A x> (<Ax, Ax>) and <x, b> (<b, A x>) through the current stacks
        bx = Lb[-1]
        for i in range(sites):
            bx = push_rhs("L", bx, cur + i)
        xb = float(np.sum(bx * Rb[-1]))
        if free:
            return None, xb
        xAx = Lop[-1]
        for i in range(sites):
            xAx = push_op("L", xAx, cur + i)
        return float(np.sum(xAx * Rop[-1])), xb

    def residual_f():
        if free:
            return orthogonal_norm(tt_add(x, tt_scale(b, -1.0)))
        if normal:
            xAtAx, bAx = stack_terms()
            return np.sqrt(xAtAx - 2 * bAx + norm_b ** 2) / norm_b
        return residual(A, x, b)

    def energy_f():
        if normal or use_residual:
            return residual_f()
        xAx, xb = stack_terms()
        if free:
            return 0.5 * float(np.sum(x.cores[cur] * x.cores[cur])) - xb
        return abs(0.5 * xAx - xb)  # |0.5 <x,Ax> - <x,b>| (als.cpp:265-278)

    res = ALSResult(energy=0.0)

    def record(flag):
        if track_residual:
            res.residuals.append(residual_f())
            res.flags.append(flag)

    energy, last_e, last_e2 = energy_f(), 1e101, 1e102
    record(FLAG_FINISHED_FULLSWEEP)
    # rank bounds of the growth extension (fixed at x's ranks otherwise)
    rmax = list(x.ranks)  # rmax[k]: the bond between cores k and k + 1
    if sites == 2 and max_rank > 0:
        red = reduce_to_maximal_ranks([max_rank] * (d - 1), x.dims)
        rmax = [max(r, q) for r, q in zip(x.ranks, red)]
    half = 0
    while True:
        if free:
            # x_k = the projection of b (als.cpp:540-543)
            x.cores[cur] = local_rhs(Lb[-1], b.cores[cur:cur + 1], Rb[-1])
        else:
            # local operator and rhs (als.cpp:383-423)
            if normal:
                M, shape_x = local_operator_normal(Lop[-1], A.cores[cur:cur + sites], Rop[-1])
                rhs = local_rhs_normal(Lb[-1], b.cores[cur:cur + sites], A.cores[cur:cur + sites], Rb[-1])
            elif solver == "cg":
                M = None
                rhs = local_rhs(Lb[-1], b.cores[cur:cur + sites], Rb[-1])
                shape_x = rhs.shape
            else:
                M, shape_x = local_operator(Lop[-1], A.cores[cur:cur + sites], Rop[-1])
                rhs = local_rhs(Lb[-1], b.cores[cur:cur + sites], Rb[-1])
            N = rhs.size
            rhs = rhs.reshape(N)
            if solver == "cg":
                # the exact local solve by matrix-free CG to the rounding floor, for local
                # systems too large to factor densely (the solution is the same)
                Lc, Rc, Ac = Lop[-1], Rop[-1], A.cores[cur:cur + sites]
                xv = cg_solve(lambda v: local_apply(Lc, Ac, Rc, v.reshape(shape_x)).reshape(N), rhs)
                xv = xv.reshape(shape_x)
                if sites != 1:
                    raise ValueError("the matrix-free local solve is for one site")
                x.cores[cur] = xv
            elif solver == "asd":
                xv = x.cores[cur].reshape(N)
                grad = rhs - M @ xv
                if normal:
                    # grad <- A_loc^T grad, alpha = ||grad|| / ||A_loc grad|| (als.cpp:86-89)
                    grad = M.T @ grad
                    alpha = float(np.linalg.norm(grad)) / float(np.linalg.norm(M @ grad))
                else:
                    alpha = float(grad @ grad) / float(grad @ (M @ grad))
                x.cores[cur] = (xv + alpha * grad).reshape(shape_x)
            else:
                xv = dense_solve(M, rhs).reshape(shape_x)
                if sites == 1:
                    x.cores[cur] = xv
                else:
                    a_, j1, j2, b_ = xv.shape
                    if max_rank > 0:
                        U, S, Vt = svd_trunc(xv.reshape(a_ * j1, j2 * b_), min(max_rank, rmax[cur]), svd_epsilon,
                                             canonical_signs)
                    else:
                        U, S, Vt = svd_trunc(xv.reshape(a_ * j1, j2 * b_), target_rank[cur], EPSILON, canonical_signs)
                    s = len(S)
                    # exact environment: the last split of a half-sweep leaves the singular
                    # values on the side the next half-sweep solves first, so the environment
                    # it builds from this pair stays orthonormal
                    at_end = (inc and cur == last - sites) or (not inc and cur == first)
                    if inc != (exact_environment and at_end):
                        x.cores[cur] = U.reshape(a_, j1, s)
                        x.cores[cur + 1] = (S[:, None] * Vt).reshape(s, j2, b_)
                    else:
                        x.cores[cur] = (U * S[None, :]).reshape(a_, j1, s)
                        x.cores[cur + 1] = Vt.reshape(s, j2, b_)
                    # set_component on a non-core position clears the canonical flag (ttNetwork.cpp:491)
                    if not (x.canonicalized and x.core_position == cur + 1):
                        x.canonicalized = False
        # check_for_end_of_sweep (als.cpp:426-475)
        if (not inc and cur == first) or (inc and cur == last - sites):
            half += 1
            last_e2, last_e = last_e, energy
            energy = energy_f()
            res.energies.append(energy)
            record(FLAG_FINISHED_HALFSWEEP if inc else FLAG_FINISHED_FULLSWEEP)
            done_target = residual_target is not None and residual(A, x, b) <= residual_target
            if (half == num_half_sweeps or abs(last_e - energy) < conv_eps or abs(last_e2 - energy) < conv_eps
                    or last - first <= sites or done_target):
                if canon_end and preserve_core_position:
                    move_core(x, core_end, keep_rank=True)
                res.energy, res.half_sweeps = energy, half
                return res
            inc = not inc
        else:
            record(0)
        # move_to_next_index (als.cpp:340-380)
        if inc:
            if sites == 1:
                move_core(x, cur + 1, keep_rank=True)
            if not free:
                Rop.pop()
                Lop.append(push_op("L", Lop[-1], cur))
            Rb.pop()
            Lb.append(push_rhs("L", Lb[-1], cur))
            cur += 1
        else:
            if sites == 1:
                move_core(x, cur - 1, keep_rank=True)
            kc = cur + 1 if (sites == 2 and exact_environment) else cur
            if not free:
                Lop.pop()
                Rop.append(push_op("R", Rop[-1], kc))
            Lb.pop()
            Rb.append(push_rhs("R", Rb[-1], kc))
            cur -= 1


# --------------------------------------------------------------------------- measurement sets / ADF


def random_positions(num: int, dims, rs: RandomEngine) -> np.ndarray:
    """SinglePointMeasurementSet::create_random_positions (measurments.cpp:222-248):
    per sample one uniform_int per mode, duplicates (by linear index) rejected,
    then sorted lexicographically."""
    seen = set()
    out = []
    while len(out) < num:
        idx = [uniform_int(rs.eng, 0, n - 1) for n in dims]
        lin = 0
        for i, n in zip(idx, dims):
            lin = lin * n + i
        if lin not in seen:
            seen.add(lin)
            out.append(idx)
    out.sort()
    return np.array(out, dtype=np.int64).reshape(num, len(dims))


def _num_unique(pos: np.ndarray) -> int:
    if pos.shape[1] == 0:
        return 1
    return int(np.unique(pos, axis=0).shape[0])


@dataclass
class ADFResult:
    residual_norm: float
    residuals: list = field(default_factory=list)
    iterations: int = 0
    ranks: list = field(default_factory=list)           # x's inner ranks at every recorded point
    iteration_log: list = field(default_factory=list)   # PerformanceData's iteration count per point


class ADFSolver:
    """ADFVariant::InternalSolver<SinglePointMeasurementSet> (src/xerus/algorithms/adf.cpp),
    with the per-sample stacks held as dense (N, r) arrays instead of deduplicated slots
    (deduplication shares identical values and so does not change them)."""

    def __init__(self, x: TT, positions: np.ndarray, values: np.ndarray, max_iter: int, target: float, min_dec: float):
        self.x = x
        self.pos = np.asarray(positions, dtype=np.int64)
        self.y = np.asarray(values, dtype=np.float64)
        self.N, self.d = self.pos.shape
        self.max_iter, self.target, self.min_dec = max_iter, target, min_dec
        self.norm_y = math.sqrt(float(np.sum(self.y ** 2)))
        # unique-entry counts per position decide which side evaluates (adf.cpp:295, 420)
        self.fwd_updates = [_num_unique(self.pos[:, :k + 1]) for k in range(self.d)]
        self.bwd_updates = [_num_unique(self.pos[:, k:]) for k in range(self.d)]
        self.F = {}
        self.B = {}
        self.iteration = 0
        self.residual_norm = np.finfo(np.float64).max
        self.last_residual_norm = np.finfo(np.float64).max

    def _slices(self, core, k):
        return core[:, self.pos[:, k], :].transpose(1, 0, 2)   # (N, r0, r1)

    def fstack(self, k):
        return np.ones((self.N, 1)) if k < 0 else self.F[k]

    def bstack(self, k):
        return np.ones((self.N, 1)) if k >= self.d else self.B[k]

    def update_forward(self, k, core):
        return np.einsum("sa,sab->sb", self.fstack(k - 1), self._slices(core, k))

    def update_backward(self, k, core):
        return np.einsum("sab,sb->sa", self._slices(core, k), self.bstack(k + 1))

    def calculate_residual(self, k):
        if self.fwd_updates[k] < self.bwd_updates[k]:
            self.F[k] = self.update_forward(k, self.x.cores[k])
            cur = np.einsum("sa,sa->s", self.F[k], self.bstack(k + 1))
        else:
            self.B[k] = self.update_backward(k, self.x.cores[k])
            cur = np.einsum("sa,sa->s", self.fstack(k - 1), self.B[k])
        self.res = self.y - cur

    def projected_gradient(self, k):
        c = self.x.cores[k]
        n = c.shape[1]
        outer = self.res[:, None, None] * self.fstack(k - 1)[:, :, None] * self.bstack(k + 1)[:, None, :]
        G = np.zeros((n, c.shape[0], c.shape[2]))
        np.add.at(G, self.pos[:, k], outer)
        return G.transpose(1, 0, 2).copy()   # (r0, n, r1)   (adf.cpp:395)

    def slicewise_norm(self, k, G):
        if self.fwd_updates[k] < self.bwd_updates[k]:
            tmp = self.update_forward(k, G)
            cur = np.einsum("sa,sa->s", tmp, self.bstack(k + 1))
        else:
            tmp = self.update_backward(k, G)
            cur = np.einsum("sa,sa->s", self.fstack(k - 1), tmp)
        return np.bincount(self.pos[:, k], weights=cur ** 2, minlength=G.shape[1])

    def update_x(self, k, G, norms):
        c = self.x.cores[k]
        for j in range(c.shape[1]):
            g = G[:, j, :]
            pyr = float(np.sum(g * g))
            c[:, j, :] = c[:, j, :] + (pyr / norms[j]) * g

    def sweep_step(self, k, log=None):
        if k > 0:
            self.calculate_residual(k)
        G = self.projected_gradient(k)
        norms = self.slicewise_norm(k, G)
        if log is not None:
            log.append((G.copy(), norms.copy()))
        self.update_x(k, G, norms)
        if k + 1 < self.d:
            move_core(self.x, k + 1, keep_rank=True)
            self.F[k] = self.update_forward(k, self.x.cores[k])

    def begin_iteration(self):
        move_core(self.x, 0, keep_rank=True)
        for k in range(self.d - 1, 0, -1):
            self.B[k] = self.update_backward(k, self.x.cores[k])
        self.calculate_residual(0)

    def solve_with_current_ranks(self, out: ADFResult, first_sweep_log=None) -> None:
        """solve_with_current_ranks (adf.cpp:489-542): the three earlier decrease ratios
        start at 0 on every call; iteration, residualNorm and lastResidualNorm are
        members and carry over between calls."""
        dec = [0.0, 0.0, 0.0]
        while self.max_iter == 0 or self.iteration < self.max_iter:
            self.begin_iteration()
            self.last_residual_norm = self.residual_norm
            self.residual_norm = math.sqrt(float(np.sum(self.res ** 2))) / self.norm_y
            out.residuals.append(self.residual_norm)
            out.ranks.append(list(self.x.ranks))
            out.iteration_log.append(self.iteration)
            d4 = dec[2]
            dec = [self.residual_norm / self.last_residual_norm, dec[0], dec[1]]
            if self.residual_norm < self.target or dec[0] * dec[1] * dec[2] * d4 > self.min_dec ** 4:
                break
            for k in range(self.d):
                self.sweep_step(k, first_sweep_log if self.iteration == 0 else None)
            self.iteration += 1

    def increase_ranks(self, max_ranks, rs: "RandomEngine") -> None:
        """The rank-increasing step of solve() (adf.cpp:590-599): core to 0, add a rank-1
        random TT scaled to 1e-6 ||x|| (TTTensor::random, which draws from the library's
        random state and ends with move_core(0)), round to the maximal ranks."""
        x = self.x
        move_core(x, 0, keep_rank=True)
        rnd = tt_random(x.dims, [1] * (x.d - 1), rs)
        scale = (1e-6 * frob_norm(x)) * (1.0 / frob_norm(rnd))
        y = tt_add(x, tt_scale(rnd, scale))
        tt_round(y, max_ranks)
        x.cores, x.canonicalized, x.core_position = y.cores, y.canonicalized, y.core_position
        self.F, self.B = {}, {}

    def solve(self, first_sweep_log=None, max_ranks=None, rs: "RandomEngine | None" = None) -> ADFResult:
        """solve() (adf.cpp:566-604): canonicalize_left, one run at the current ranks, then,
        with max_ranks (the ADFVariant::operator() overload taking maxRanks, adf.h:263-266),
        rank increases until the target residual, the maximal ranks or the iteration cap."""
        move_core(self.x, 0, keep_rank=False)      # canonicalize_left
        out = ADFResult(residual_norm=0.0)
        self.solve_with_current_ranks(out, first_sweep_log)
        if max_ranks is not None:
            mr = reduce_to_maximal_ranks(list(max_ranks), self.x.dims)
            while (self.residual_norm > self.target and list(self.x.ranks) != mr
                   and (self.max_iter == 0 or self.iteration < self.max_iter)):
                self.increase_ranks(mr, rs)
                self.solve_with_current_ranks(out)
        out.residual_norm = self.residual_norm
        out.iterations = self.iteration
        return out


def adf(x: TT, positions, values, max_iter: int = 0, target: float = 1e-8, min_dec: float = 0.999,
        max_ranks=None, rs: "RandomEngine | None" = None) -> ADFResult:
    """ADFVariant(max_iter, target, min_dec)(x, measurements[, maxRanks]); with max_ranks the
    rank increases draw their random TTs from rs."""
    if max_ranks is not None and rs is None:
        raise ValueError("the rank-increasing ADF needs the random state it draws from")
    return ADFSolver(x, positions, values, max_iter, target, min_dec).solve(max_ranks=max_ranks, rs=rs)


# --------------------------------------------------------------------------- rank-one measurements


def _split_vectors(vectors, dims):
    """(N, sum n_k) rows -> per mode (N, n_k) blocks."""
    out, off = [], 0
    for n in dims:
        out.append(np.asarray(vectors[:, off:off + n], dtype=np.float64))
        off += n
    return out


def rank_one_random(num: int, dims, rs: RandomEngine) -> np.ndarray:
    """RankOneMeasurementSet::create_random_positions (measurments.cpp:522-544): per sample
    and mode a Tensor::random({n}) (n draws of the stateful default normal distribution),
    then sort(true) with internal::comp (measurments.cpp:330-347, 549-...): samples ordered
    mode by mode, entry by entry, DEcreasing at the first difference."""
    dims = list(dims)
    rows = [np.concatenate([rs.normal.draw(rs.eng, n) for n in dims]) for _ in range(num)]
    rows.sort(key=lambda r: tuple(-v for v in r))
    return np.array(rows).reshape(num, sum(dims))


def rank_one_measure(x: TT, vectors) -> np.ndarray:
    """RankOneMeasurementSet::measure(TensorNetwork): <x, u_1 (x) ... (x) u_d> per sample."""
    us = _split_vectors(np.asarray(vectors), x.dims)
    v = np.ones((us[0].shape[0], 1))
    for k, c in enumerate(x.cores):
        v = np.einsum("sa,si,aib->sb", v, us[k], c, optimize=True)
    return v[:, 0]


class ADFRankOneSolver(ADFSolver):
    """ADFVariant::InternalSolver<RankOneMeasurementSet> (adf.cpp:233-288, 333-357, 405-408,
    481-487): the stacks contract each core with the sample's vector for its mode (the mixed
    component sum_i u[i] X[:, i, :]); the gradient takes every entry of the vector; the norm
    of the projected gradient is one total (position_or_zero gives slot 0); update_x takes one
    step for the whole core. Random Gaussian vectors never share prefixes, so both stack
    sides count N updates and the backward side evaluates (adf.cpp:295, 420)."""

    def __init__(self, x: TT, vectors: np.ndarray, values: np.ndarray, max_iter: int, target: float, min_dec: float):
        vectors = np.asarray(vectors, dtype=np.float64)
        self.us = _split_vectors(vectors, x.dims)
        N = vectors.shape[0]
        super().__init__(x, np.zeros((N, x.d), dtype=np.int64), values, max_iter, target, min_dec)
        self.fwd_updates = [N] * self.d
        self.bwd_updates = [N] * self.d

    def _slices(self, core, k):
        return np.einsum("si,aib->sab", self.us[k], core, optimize=True)

    def projected_gradient(self, k):
        f, b = self.fstack(k - 1), self.bstack(k + 1)
        return np.einsum("s,si,sa,sc->aic", self.res, self.us[k], f, b, optimize=True)

    def slicewise_norm(self, k, G):
        tmp = self.update_backward(k, G)
        cur = np.einsum("sa,sa->s", self.fstack(k - 1), tmp)
        out = np.zeros(G.shape[1])
        out[0] = float(np.sum(cur ** 2))
        return out

    def update_x(self, k, G, norms):
        pyr = float(np.sum(G * G))
        self.x.cores[k] = self.x.cores[k] + (pyr / float(np.sum(norms))) * G


def adf_rank_one(x: TT, vectors, values, max_iter: int = 0, target: float = 1e-8, min_dec: float = 0.999) -> ADFResult:
    return ADFRankOneSolver(x, vectors, values, max_iter, target, min_dec).solve()


def adf_loss_gradient(x: TT, positions, values):
    """Gradient of 0.5 * ||P_Omega(x) - y||^2 with respect to every core (no gauge
    condition), by the same stacks: dL/dX_k[a,i,b] = -sum_{s: i_s=i} res_s F_{k-1}[s,a] B_{k+1}[s,b]."""
    pos = np.asarray(positions, dtype=np.int64)
    y = np.asarray(values, dtype=np.float64)
    N, d = pos.shape
    F = [np.ones((N, 1))]
    for k in range(d):
        F.append(np.einsum("sa,sab->sb", F[-1], x.cores[k][:, pos[:, k], :].transpose(1, 0, 2)))
    Bk = [None] * (d + 1)
    Bk[d] = np.ones((N, 1))
    for k in range(d - 1, -1, -1):
        Bk[k] = np.einsum("sab,sb->sa", x.cores[k][:, pos[:, k], :].transpose(1, 0, 2), Bk[k + 1])
    res = y - F[d][:, 0]
    grads = []
    for k in range(d):
        c = x.cores[k]
        outer = -res[:, None, None] * F[k][:, :, None] * Bk[k + 1][:, None, :]
        G = np.zeros((c.shape[1], c.shape[0], c.shape[2]))
        np.add.at(G, pos[:, k], outer)
        grads.append(G.transpose(1, 0, 2).copy())
    return 0.5 * float(np.sum(res ** 2)), grads


# --------------------------------------------------------------------------- Riemannian CG


def pseudo_inverse(M: np.ndarray) -> np.ndarray:
    """pseudo_inverse(M, 1) (tensor.cpp:1568-1574): SVD truncated at EPSILON * S[0]
    (calculate_svd's rule), inverted singular values."""
    U, S, Vt = svd_trunc(np.asarray(M, dtype=np.float64), max(M.shape), EPSILON)
    return Vt.T @ np.diag(1.0 / S) @ U.T


def _tt_copy_at0(x: TT) -> TT:
    y = x.copy()
    move_core(y, 0, keep_rank=True)
    return y


class Tangent:
    """TTTangentVector (retractions.cpp): components shaped like the base's cores, the
    base kept canonical at position 0."""

    def __init__(self, base: TT, comps):
        self.base = base
        self.comps = comps

    def scaled(self, f: float) -> "Tangent":
        return Tangent(self.base, [f * c for c in self.comps])

    def plus(self, other: "Tangent", f: float = 1.0) -> "Tangent":
        return Tangent(self.base, [a + f * b for a, b in zip(self.comps, other.comps)])

    def dot(self, other: "Tangent") -> float:
        """TTTangentVector::scalar_product (retractions.cpp:143-155)."""
        left = np.ones((1, 1))
        out = 0.0
        d = len(self.comps)
        for i in range(d):
            out += float(np.einsum("ab,anc,bnc->", left, self.comps[i], other.comps[i], optimize=True))
            if i + 1 < d:
                u = self.base.cores[i]
                left = np.einsum("ab,anc,bnd->cd", left, u, u, optimize=True)
        return out

    def norm(self) -> float:
        return math.sqrt(self.dot(self))

    def _blocks(self, first_plus_base: bool) -> TT:
        d = len(self.comps)
        U, V = self.base.cores, self.comps
        if d == 1:
            return TT([V[0] + U[0] if first_plus_base else V[0].copy()])
        cores = []
        for i in range(d):
            r0, n, r1 = U[i].shape
            if i == 0:
                c = np.zeros((1, n, 2 * r1))
                c[:, :, :r1] = U[0]
                c[:, :, r1:] = U[0] + V[0] if first_plus_base else V[0]
            elif i + 1 < d:
                c = np.zeros((2 * r0, n, 2 * r1))
                c[:r0, :, :r1] = U[i]
                c[:r0, :, r1:] = V[i]
                c[r0:, :, r1:] = U[i]
            else:
                c = np.zeros((2 * r0, n, 1))
                c[:r0] = V[i]
                c[r0:] = U[i]
            cores.append(c)
        t = TT(cores, canonicalized=False)
        move_core(t, 0, keep_rank=False)
        return t

    def to_tt(self) -> TT:
        """TTTangentVector::operator TTTensor (retractions.cpp:186-201)."""
        return self._blocks(False)

    def added_to_base(self) -> TT:
        """TTTangentVector::added_to_base (retractions.cpp:203-219)."""
        return self._blocks(True)


def tangent_project(base: TT, direction: TT) -> Tangent:
    """TTTangentVector(base, direction) (retractions.cpp:57-103): the projection of
    `direction` onto the tangent space of the fixed-rank manifold at `base`."""
    if not (base.canonicalized and base.core_position == 0):
        raise ValueError("projection onto tangent plane is only implemented for core position 0 at the moment")
    U = _tt_copy_at0(base)
    d = U.d
    UV, UU = [np.ones((1, 1))], [np.ones((1, 1))]
    for i in range(d - 1):
        UV.append(np.einsum("ab,anc,bnd->cd", UV[-1], U.cores[i], direction.cores[i], optimize=True))
        UU.append(np.einsum("ab,anc,bnd->cd", UU[-1], U.cores[i], U.cores[i], optimize=True))
    right = np.ones((1, 1))
    comps = [None] * d
    for i in range(d - 1, -1, -1):
        u, dcore = U.cores[i], direction.cores[i]
        inv = pseudo_inverse(UU[i])
        V = np.einsum("as,sb,bnc,dc->and", inv, UV[i], dcore, right, optimize=True)
        if i != 0:
            utv = np.einsum("anc,bnc->ab", V, u, optimize=True)
            V = V - np.einsum("ab,bnc->anc", utv, u, optimize=True)
            right = np.einsum("anc,bnd,cd->ab", u, dcore, right, optimize=True)
        comps[i] = V
    return Tangent(U, comps)


def submanifold_retraction(x: TT, change: Tangent) -> None:
    """SubmanifoldRetractionI (retractions.cpp:228-236): every core plus its component,
    then move_core(0, keepRank)."""
    for i in range(x.d):
        x.cores[i] = x.cores[i] + change.comps[i]
    x.canonicalized = x.d == 1
    move_core(x, 0, keep_rank=True)


def _retract_to_ranks(x: TT, y: TT, kind: str) -> None:
    """HOSVDRetractionI / II (retractions.cpp:43-55): y.round(oldRanks); ALSRetractionI /
    II (:57-69): ALSVariant(1, 2, lapack_solver, false) without an operator fits x (ranks
    kept) to y. y is the step added as a TT (added_to_base, or x + step)."""
    old = list(x.ranks)
    if kind == "hosvd":
        tt_round(y, old)
        x.cores, x.canonicalized, x.core_position = y.cores, y.canonicalized, y.core_position
    else:
        als(None, x, y, 1, 2, 1e-6, assume_spd=False)


def retraction_i(x: TT, change: Tangent, kind: str = "submanifold") -> None:
    """Type I retractions of x at change's base along change."""
    if kind == "submanifold":
        submanifold_retraction(x, change)
    else:
        _retract_to_ranks(x, change.added_to_base(), kind)


def retraction_ii(x: TT, step: TT, kind: str = "submanifold") -> None:
    """Type II retractions of x along the TT step: SubmanifoldRetractionII projects it on
    the tangent space at x first (retractions.cpp:222-225); the others add it as a TT."""
    if kind == "submanifold":
        submanifold_retraction(x, tangent_project(x, step))
    else:
        _retract_to_ranks(x, tt_add(x, step), kind)


def _op_transpose(A: TTOp) -> TTOp:
    return TTOp([c.transpose(0, 2, 1, 3).copy() for c in A.cores])


def geometric_cg(A: TTOp | None, x: TT, b: TT, num_steps: int = 0, conv_eps: float = 1e-8,
                 assume_spd: bool = False, retraction: str = "submanifold") -> tuple[float, list]:
    """GeometricCGVariant::solve (algorithms/cg.cpp:34-120) with SubmanifoldRetractionI
    (or HOSVDRetractionI / ALSRetractionI: retraction "hosvd" / "als"),
    ProjectiveVectorTransport and line_search (steepestDescent.cpp:37-80). x is updated in
    place; returns (final residual ||b - A x||, residual after every step)."""
    norm_b = orthogonal_norm(b)
    trace = []
    state = {}

    def calc_residual():
        ax = x.copy() if A is None else op_apply(A, x)
        res = tt_add(b, tt_scale(ax, -1.0))   # b - A x; b canonical: canonicalised again
        state["res"] = res
        return orthogonal_norm(res)

    def update_gradient():
        res = state["res"]
        g = res if (assume_spd or A is None) else op_apply(_op_transpose(A), res)
        state["grad"] = tangent_project(x, g)
        state["gnorm"] = state["grad"].norm()

    def line_search(alpha, direction, derivative, residual, change=0.8):
        dir_norm = direction.norm()
        curr = alpha / change
        old = x.copy()
        retraction_i(x, direction.scaled(curr / dir_norm), retraction)
        best_res = calc_residual()
        best_alpha, best_x = curr, x.copy()
        while True:
            curr *= change
            x.cores, x.canonicalized, x.core_position = [c.copy() for c in old.cores], old.canonicalized, old.core_position
            retraction_i(x, direction.scaled(curr / dir_norm), retraction)
            new_res = calc_residual()
            if new_res < best_res:
                best_res, best_alpha, best_x = new_res, curr, x.copy()
            else:
                break
        x.cores, x.canonicalized, x.core_position = best_x.cores, best_x.canonicalized, best_x.core_position
        alpha = best_alpha
        while alpha > 1e-16 and best_res > residual - 1e-4 * alpha / dir_norm * derivative:
            alpha *= change
            x.cores, x.canonicalized, x.core_position = [c.copy() for c in old.cores], old.canonicalized, old.core_position
            retraction_i(x, direction.scaled(alpha / dir_norm), retraction)
            best_res = calc_residual()
        state["res_norm_after"] = best_res
        return alpha, best_res

    curr = calc_residual()
    last = 1e100
    trace.append(curr)
    update_gradient()
    direction = state["grad"]
    alpha = 1.0
    steps = 0
    while ((num_steps == 0 or steps < num_steps) and curr / norm_b > conv_eps
           and abs(last - curr) / norm_b > conv_eps and abs(1 - curr / last) / norm_b > conv_eps):
        steps += 1
        grad = state["grad"]
        derivative = grad.dot(direction) / direction.norm()
        if derivative <= 0:
            direction = grad
            derivative = grad.norm()
            alpha = 1.0
        alpha, curr = line_search(alpha, direction, derivative, curr)
        # as in the reference, the gradient below uses the residual TT of the last x the line
        # search evaluated, which is a rejected trial unless the Armijo loop ran
        trace.append(curr)
        old_dir = tangent_project(x, direction.to_tt())        # ProjectiveVectorTransport
        old_gnorm = state["gnorm"]
        update_gradient()
        beta = state["gnorm"] / old_gnorm
        direction = state["grad"].plus(old_dir, beta)
    return curr, trace


def steepest_descent(A: TTOp | None, x: TT, b: TT, num_steps: int = 0, conv_eps: float = 1e-8,
                     assume_spd: bool = False, retraction: str = "submanifold") -> tuple[float, list]:
    """SteepestDescentVariant::solve (algorithms/steepestDescent.cpp:83-175) with
    SubmanifoldRetractionII (retractions.cpp:222-225: project the TT step onto the tangent
    space at x, then the submanifold retraction), or HOSVDRetractionII / ALSRetractionII.
    Absolute stopping tests, step doubling and halving as in the reference; returns
    (||b - A x||, residual after every step)."""
    def residual_tt():
        ax = x.copy() if A is None else op_apply(A, x)
        return tt_add(b, tt_scale(ax, -1.0))

    res = residual_tt()
    curr, last = orthogonal_norm(res.copy()), 1e100
    trace = [curr]
    alpha, steps = 1.0, 0
    while ((num_steps == 0 or steps < num_steps) and curr > conv_eps and abs(last - curr) > conv_eps
           and abs(1 - curr / last) > conv_eps):
        steps += 1
        y = res if (A is None or assume_spd) else op_apply(_op_transpose(A), res)
        old = x.copy()
        w = tangent_project(x, y) if retraction == "submanifold" else None

        def step(f):
            if w is not None:
                submanifold_retraction(x, w.scaled(f))
            else:
                retraction_ii(x, tt_scale(y, f), retraction)

        alpha *= 2
        step(alpha)
        last = curr
        res = residual_tt()
        curr = orthogonal_norm(res.copy())
        while alpha > 1e-30 and last < curr:
            alpha /= 2
            x.cores, x.canonicalized, x.core_position = [c.copy() for c in old.cores], old.canonicalized, old.core_position
            step(alpha)
            res = residual_tt()
            curr = orthogonal_norm(res.copy())
        trace.append(curr)
    return curr, trace


# --------------------------------------------------------------------------- IHT


def iht(x: TT, positions, values, max_iter: int) -> tuple[float, list]:
    """IHT (algorithms/iht.cpp:29-155) with an iteration cap (the reference loops 10^6 times).
    Per iteration: the current entries at the samples; for beta = 1/1.1, 1, 1.1, .. (< 1.65)
    the rank-(r + N) TT largeX = x + sum_s beta alpha (y_s - cur_s) e_{pos_s} (x's cores
    plus one sparse channel per sample), then ONE ALS sweep of newX (a copy of x, moved to
    core 0) towards largeX: right stacks of (newX, largeX) from the right, then left to right
    each core set to its projection of largeX and the core moved on (keepRank). A trial
    whose residual ||y - P(newX)|| is <= the best so far (initially twice the previous
    residual) replaces x and scales alpha by its beta. As in the reference, the trials of an
    iteration after an accepted one start from (and add to) the new x, with the entries
    `cur` of the iteration's start. Returns (residual, the best residual of every iteration)."""
    pos = np.asarray(positions, dtype=np.int64)
    y = np.asarray(values, dtype=np.float64)
    N, d = pos.shape
    alpha, residual = 1.0, 1.0
    trace = []
    for _ in range(max_iter):
        cur = tt_entries(x, pos)
        best, new_alpha = residual * 2, alpha
        beta = 1 / 1.1
        while beta < 1.1 * 1.5:
            w = beta * alpha * (y - cur)
            nx = x.copy()
            move_core(nx, 0, keep_rank=True)
            # right stacks at bonds k (between cores k-1 and k): dense (newX vs x) and
            # per-sample (newX's right products at the sample), both 1 at bond d
            D = [None] * (d + 1)
            S = [None] * (d + 1)
            D[d] = np.ones((1, 1))
            S[d] = np.ones((1, N))
            for k in range(d - 1, 0, -1):
                D[k] = _iht_push_right(nx.cores[k], x.cores[k], D[k + 1])
                S[k] = np.einsum("asc,cs->as", nx.cores[k][:, pos[:, k], :], S[k + 1])
            LD = np.ones((1, 1))
            LS = None  # per-sample left products (carrying w), from core 1 on
            for k in range(d):
                dense = np.einsum("ab,bic,dc->aid", LD, x.cores[k], D[k + 1], optimize=True)
                right_s = S[k + 1]                              # (r', N)
                left_s = w[None, :] if k == 0 else LS            # (r, N)
                sparse = np.zeros_like(dense)
                outer = np.einsum("as,cs->sac", left_s, right_s)
                for s in range(N):
                    sparse[:, pos[s, k], :] += outer[s]
                nx.cores[k] = dense + sparse
                if k + 1 < d:
                    move_core(nx, k + 1, keep_rank=True)
                    LD = np.einsum("ab,aic,bid->cd", LD, nx.cores[k], x.cores[k], optimize=True)
                    LS = np.einsum("as,asc->cs", left_s, nx.cores[k][:, pos[:, k], :])
            r = math.sqrt(float(np.sum((y - tt_entries(nx, pos)) ** 2)))
            if r <= best:
                x.cores, x.canonicalized, x.core_position = nx.cores, nx.canonicalized, nx.core_position
                best, new_alpha = r, alpha * beta
            beta *= 1.1
        residual, alpha = best, new_alpha
        trace.append(best)
    return residual, trace


def _iht_push_right(u, v, D):
    """next(i1, i2) = sum u(i1, i5, i3) v(i2, i5, i4) D(i3, i4) (iht.cpp:113)."""
    t = np.tensordot(u, D, axes=([2], [0]))        # (i1, i5, i4)
    return np.tensordot(t, v, axes=([1, 2], [1, 2]))  # (i1, i2)
