// Strided batched small-GEMM tile engine. Every contraction of the sweep
// (environment pushes, the local operator, R-absorption, the dot-product
// zipper) is a short chain of these: C[b] = alpha * A[b] B[b] + beta * C[b],
// where each of the M, N and K index ranges may be split into an outer and an
// inner part with their own element strides. That lets a contraction over a
// pair of tensor modes that are not adjacent in memory run directly on the
// row-major cores, with no transposed or repacked copies.
//
// Shapes are tiny to moderate (ranks <= a few hundred), the operands live in
// L2, and on GB300 the FP64 pipe bounds the tile; a tile is 32x32 with a
// 32-deep K slab in shared memory and 2x2 outputs per thread (256 threads).
// An optional epilogue accumulates sum(C .* D) over the tile's outputs (the
// p^T A p of conjugate gradients) without another pass.
#pragma once

#include "common.cuh"

namespace xtt {

template <class T>
struct Gemm {
	int M = 0, N = 0, K = 0, batch = 1;
	int Mi = 0, Ni = 0, Ki = 0;  // inner extents of the split index ranges (0 = not split)
	const T* A = nullptr;
	long long sAb = 0, sAm = 0, sAk = 0, sAmo = 0, sAko = 0;
	const T* B = nullptr;
	long long sBb = 0, sBk = 0, sBn = 0, sBko = 0, sBno = 0;
	T* C = nullptr;
	long long sCb = 0, sCm = 0, sCn = 0, sCmo = 0, sCno = 0;
	T alpha = T(1), beta = T(0);
	const T* D = nullptr;  // optional epilogue operand, same layout as C
	// Element counts of the A, B and C buffers (host-side bounds check before any launch).
	long long lenA = -1, lenB = -1, lenC = -1;

	__host__ __device__ Gemm& lens(long long a, long long b, long long c) {
		lenA = a;
		lenB = b;
		lenC = c;
		return *this;
	}
	// Upper bounds of the largest element offset each operand can touch (strides are >= 0).
	__host__ __device__ static long long span(int ext, int inner, long long s_in, long long s_out) {
		if (ext <= 0) return 0;
		if (!inner) return (long long)(ext - 1) * s_in;
		const long long mo = (ext - 1) / inner, mi = (ext < inner ? ext : inner) - 1;
		return mo * s_out + mi * s_in;
	}
	long long max_off_A() const { return (batch - 1) * sAb + span(M, Mi, sAm, sAmo) + span(K, Ki, sAk, sAko); }
	long long max_off_B() const { return (batch - 1) * sBb + span(K, Ki, sBk, sBko) + span(N, Ni, sBn, sBno); }
	long long max_off_C() const { return (batch - 1) * sCb + span(M, Mi, sCm, sCmo) + span(N, Ni, sCn, sCno); }
	bool strides_nonnegative() const {
		return sAb >= 0 && sAm >= 0 && sAk >= 0 && sAmo >= 0 && sAko >= 0 && sBb >= 0 && sBk >= 0 && sBn >= 0 &&
		       sBko >= 0 && sBno >= 0 && sCb >= 0 && sCm >= 0 && sCn >= 0 && sCmo >= 0 && sCno >= 0;
	}

	__host__ __device__ long long tiles_m() const { return (M + 31) / 32; }
	__host__ __device__ long long tiles_n() const { return (N + 31) / 32; }
	__host__ __device__ long long tiles() const { return (long long)batch * tiles_m() * tiles_n(); }
	__host__ __device__ long long offA(int m, int k) const {
		const int mo = Mi ? m / Mi : 0, mi = Mi ? m - mo * Mi : m;
		const int ko = Ki ? k / Ki : 0, ki = Ki ? k - ko * Ki : k;
		return mo * sAmo + mi * sAm + ko * sAko + ki * sAk;
	}
	__host__ __device__ long long offB(int k, int n) const {
		const int ko = Ki ? k / Ki : 0, ki = Ki ? k - ko * Ki : k;
		const int no = Ni ? n / Ni : 0, ni = Ni ? n - no * Ni : n;
		return ko * sBko + ki * sBk + no * sBno + ni * sBn;
	}
	__host__ __device__ long long offC(int m, int n) const {
		const int mo = Mi ? m / Mi : 0, mi = Mi ? m - mo * Mi : m;
		const int no = Ni ? n / Ni : 0, ni = Ni ? n - no * Ni : n;
		return mo * sCmo + mi * sCm + no * sCno + ni * sCn;
	}
};

constexpr int kGemmThreads = 256;

template <class T>
struct GemmSmem {
	T As[32][33];  // [k][m]
	T Bs[32][33];  // [k][n]
};

// The 32 x 32 operand slabs of K range [k0, k0 + 32): thread t holds elements
// t + 256 j (j < 4) of each, fetched from global memory into registers; stored
// into the shared-memory slabs by gemm_slab_store with the same index map.
template <class T>
struct GemmSlab {
	T a[4], b[4];
};

template <class T>
__device__ __forceinline__ void gemm_slab_index(int e, bool kfast_a, bool nfast_b, int& am, int& ak, int& bn, int& bk) {
	const int hi = e >> 5, lo = e & 31;
	am = kfast_a ? hi : lo;
	ak = kfast_a ? lo : hi;
	bn = nfast_b ? lo : hi;
	bk = nfast_b ? hi : lo;
}

// (zero beyond row M, column N and K index kend)
template <class T>
__device__ __forceinline__ void gemm_slab_load(const Gemm<T>& g, const T* A, const T* B, int m0, int n0, int k0,
                                               int kend, bool a_k_fast, bool b_n_fast, GemmSlab<T>& r) {
#pragma unroll
	for (int t = 0; t < 4; ++t) {
		int am, ak, bn, bk;
		gemm_slab_index<T>(threadIdx.x + t * kGemmThreads, a_k_fast, b_n_fast, am, ak, bn, bk);
		const int gm = m0 + am, gka = k0 + ak, gn = n0 + bn, gkb = k0 + bk;
		r.a[t] = (gm < g.M && gka < kend) ? A[g.offA(gm, gka)] : T(0);
		r.b[t] = (gn < g.N && gkb < kend) ? B[g.offB(gkb, gn)] : T(0);
	}
}

// Computes output tile `tile` of g with all 256 threads of the block. Returns,
// in thread 0 only, sum over the tile of C .* D when g.D is set (else 0). The next
// K slab is fetched into registers while the current one is multiplied, so the
// global (L2) latency of a slab overlaps the arithmetic of the one before.
template <class T>
__device__ T gemm_tile(const Gemm<T>& g, long long tile, GemmSmem<T>& sm) {
	const int tid = threadIdx.x;
	const long long tn = g.tiles_n(), tm = g.tiles_m();
	const long long b = tile / (tm * tn);
	const long long rem = tile - b * tm * tn;
	const int m0 = int(rem / tn) * 32, n0 = int(rem % tn) * 32;
	const T* A = g.A + b * g.sAb;
	const T* B = g.B + b * g.sBb;
	const int tx = tid & 15, ty = tid >> 4;
	T acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;
	const bool a_k_fast = (g.sAk == 1);
	const bool b_n_fast = (g.sBn == 1) || (g.sBk != 1);
	GemmSlab<T> r;
	gemm_slab_load(g, A, B, m0, n0, 0, g.K, a_k_fast, b_n_fast, r);
	for (int k0 = 0; k0 < g.K; k0 += 32) {
#pragma unroll
		for (int t = 0; t < 4; ++t) {
			int am, ak, bn, bk;
			gemm_slab_index<T>(tid + t * kGemmThreads, a_k_fast, b_n_fast, am, ak, bn, bk);
			sm.As[ak][am] = r.a[t];
			sm.Bs[bk][bn] = r.b[t];
		}
		__syncthreads();
		if (k0 + 32 < g.K) gemm_slab_load(g, A, B, m0, n0, k0 + 32, g.K, a_k_fast, b_n_fast, r);
		const int kmax = min(32, g.K - k0);
		for (int kk = 0; kk < kmax; ++kk) {
			const T a0 = sm.As[kk][ty], a1 = sm.As[kk][ty + 16];
			const T b0 = sm.Bs[kk][tx], b1 = sm.Bs[kk][tx + 16];
			acc00 = fma(a0, b0, acc00);
			acc01 = fma(a0, b1, acc01);
			acc10 = fma(a1, b0, acc10);
			acc11 = fma(a1, b1, acc11);
		}
		__syncthreads();
	}
	T* C = g.C + b * g.sCb;
	const T* D = g.D ? g.D + b * g.sCb : nullptr;
	const T accs[2][2] = {{acc00, acc01}, {acc10, acc11}};
	T dsum = 0;
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 2; ++j) {
			const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
			if (gm < g.M && gn < g.N) {
				const long long o = g.offC(gm, gn);
				const T v = (g.beta == T(0)) ? g.alpha * accs[i][j] : g.alpha * accs[i][j] + g.beta * C[o];
				C[o] = v;
				if (D) dsum += v * D[o];
			}
		}
	if (D) {
		// fixed-order reduction over the block (deterministic)
		__shared__ T red[kGemmThreads / 32];
		dsum = warp_sum(dsum);
		if ((tid & 31) == 0) red[tid >> 5] = dsum;
		__syncthreads();
		T s = 0;
		if (tid == 0)
			for (int w = 0; w < kGemmThreads / 32; ++w) s += red[w];
		__syncthreads();
		return s;
	}
	return T(0);
}

// Square TS x TS output tile (TS = 16 or 32) over the K range [kb, ke): the
// 256 threads form a 16 x 16 grid, each accumulating (TS/16)^2 outputs into
// acc (row-major 2x2 or 1x1). No epilogue; used by the split-K launcher,
// whose CTAs of one cluster cover disjoint K ranges of the same tile.
template <class T, int TS>
struct TileSmem {
	T As[32][TS + 1];  // [k][m]
	T Bs[32][TS + 1];  // [k][n]
};

template <class T, int TS>
__device__ void gemm_tile_acc(const Gemm<T>& g, long long tile, int kb, int ke, TileSmem<T, TS>& sm,
                              T (&acc)[TS / 16][TS / 16]) {
	constexpr int R = TS / 16;
	const int tid = threadIdx.x;
	const long long tn = (g.N + TS - 1) / TS, tm = (g.M + TS - 1) / TS;
	const long long b = tile / (tm * tn);
	const long long rem = tile - b * tm * tn;
	const int m0 = int(rem / tn) * TS, n0 = int(rem % tn) * TS;
	const T* A = g.A + b * g.sAb;
	const T* B = g.B + b * g.sBb;
	const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
	for (int i = 0; i < R; ++i)
#pragma unroll
		for (int j = 0; j < R; ++j) acc[i][j] = T(0);
	const bool a_k_fast = (g.sAk == 1);
	const bool b_n_fast = (g.sBn == 1) || (g.sBk != 1);
	for (int k0 = kb; k0 < ke; k0 += 32) {
#pragma unroll
		for (int t = 0; t < TS / 8; ++t) {
			const int e = tid + t * kGemmThreads;  // e < 32 * TS
			{
				// A slab TS (m) x 32 (k): consecutive threads along k when A is k-contiguous
				const int mm = a_k_fast ? (e >> 5) : (e % TS), kk = a_k_fast ? (e & 31) : (e / TS);
				const int gm = m0 + mm, gk = k0 + kk;
				sm.As[kk][mm] = (gm < g.M && gk < ke) ? A[g.offA(gm, gk)] : T(0);
			}
			{
				const int nn = b_n_fast ? (e % TS) : (e >> 5), kk = b_n_fast ? (e / TS) : (e & 31);
				const int gn = n0 + nn, gk = k0 + kk;
				sm.Bs[kk][nn] = (gn < g.N && gk < ke) ? B[g.offB(gk, gn)] : T(0);
			}
		}
		__syncthreads();
		const int kmax = min(32, ke - k0);
		for (int kk = 0; kk < kmax; ++kk) {
			T av[R], bv[R];
#pragma unroll
			for (int i = 0; i < R; ++i) av[i] = sm.As[kk][ty + 16 * i];
#pragma unroll
			for (int j = 0; j < R; ++j) bv[j] = sm.Bs[kk][tx + 16 * j];
#pragma unroll
			for (int i = 0; i < R; ++i)
#pragma unroll
				for (int j = 0; j < R; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
		}
		__syncthreads();
	}
}

// Writes the accumulators of gemm_tile_acc through the alpha/beta epilogue.
template <class T, int TS>
__device__ void gemm_tile_store(const Gemm<T>& g, long long tile, const T (&acc)[TS / 16][TS / 16]) {
	constexpr int R = TS / 16;
	const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
	const long long tn = (g.N + TS - 1) / TS, tm = (g.M + TS - 1) / TS;
	const long long b = tile / (tm * tn);
	const long long rem = tile - b * tm * tn;
	const int m0 = int(rem / tn) * TS, n0 = int(rem % tn) * TS;
	T* C = g.C + b * g.sCb;
#pragma unroll
	for (int i = 0; i < R; ++i)
#pragma unroll
		for (int j = 0; j < R; ++j) {
			const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
			if (gm < g.M && gn < g.N) {
				const long long o = g.offC(gm, gn);
				C[o] = (g.beta == T(0)) ? g.alpha * acc[i][j] : g.alpha * acc[i][j] + g.beta * C[o];
			}
		}
}

// Processes tiles start, start+stride, ... of g (a persistent block loop);
// returns the epilogue partial sum of this block (thread 0).
template <class T>
__device__ T gemm_tiles(const Gemm<T>& g, long long start, long long stride, GemmSmem<T>& sm) {
	const long long nt = g.tiles();
	T s = 0;
	for (long long t = start; t < nt; t += stride) s += gemm_tile(g, t, sm);
	return s;
}

}  // namespace xtt
