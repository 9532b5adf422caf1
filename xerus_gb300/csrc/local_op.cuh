// The one- and two-site local operator of the SPD sweep applied to a vector
// with the right environment contracted first, so that a group of threads can
// produce any subset of the output's right-bond columns from the full input:
//   T1(a',j,k',b) = sum_b' x(a',j,b') R(b,k',b'),
//   T3(k,a',i,b)  = sum_(j,k') A(k,i,j,k') T1(a',j,k',b)   (two sites: A2 then A1),
//   y(a,i,b)      = sum_(k,a') L(a,k,a') T3(k,a',i,b).
// Used by the cluster-resident local solver (one CTA per column block) and by
// the batched persistent sweep (one CTA, all columns). Also compiled for the
// host (one thread, no barriers) so its index arithmetic can be checked on the CPU.
#pragma once

#include "common.cuh"

namespace xtt {

#ifdef __CUDA_ARCH__
#define CC_TID int(threadIdx.x)
#define CC_STRIDE int(blockDim.x)
#define CC_SYNC() __syncthreads()
#else
#define CC_TID 0
#define CC_STRIDE 1
#define CC_SYNC()
#endif

struct CcShape {
	int two = 0;
	int ra = 1, n1 = 1, n2 = 1, rb = 1, K0 = 1, K1 = 1, K2 = 1;
	int bw = 1;  // columns b per CTA (the last CTA may own fewer)
	__host__ __device__ int KL() const { return two ? K2 : K1; }
	__host__ __device__ int M1() const { return ra * n1 * n2; }  // rows (a, j[, j2]) of the full vector
	__host__ __device__ int nI() const { return n1 * n2; }
	__host__ __device__ int ldp() const { return rb + 1; }
	__host__ __device__ int ldl() const { return K0 * ra + 1; }
	__host__ __device__ int ldr() const { return rb + 1; }
	__host__ __device__ int ld3() const { return nI() * bw + 1; }
	// element counts of the shared-memory arrays (allocated for bw columns)
	__host__ __device__ size_t n_pf() const { return size_t(M1()) * ldp(); }
	__host__ __device__ size_t n_L() const { return size_t(ra) * ldl(); }
	__host__ __device__ size_t n_A1() const { return size_t(K0) * n1 * n1 * K1; }
	__host__ __device__ size_t n_A2() const { return two ? size_t(K1) * n2 * n2 * K2 : 0; }
	__host__ __device__ size_t n_R() const { return size_t(bw) * KL() * ldr(); }
	__host__ __device__ size_t n_t1() const { return size_t(M1()) * bw * KL(); }
	__host__ __device__ size_t n_t2() const { return two ? size_t(M1()) * bw * K1 : 0; }
	__host__ __device__ size_t n_t3() const { return size_t(K0) * ra * ld3(); }
	__host__ __device__ size_t n_v() const { return size_t(M1()) * bw; }
};

// Operand pointers of one local-operator application. `pf` is the full input
// vector (rows M1, leading dimension ldp); L, R and the cores may point to
// shared or global memory; the output is this CTA's slice [(a, i..)][bl].
template <class T>
struct Mv {
	const T* pf;
	int ldp;
	const T* L;
	int ldl;
	const T* A1;
	const T* A2;
	const T* R;  // row c = bl * KL + k of the CTA's columns, leading dimension ldr
	int ldr;
	T *t1, *t2, *t3;
};

// TA: output rows a per thread in the last stage (register tile TA x 1: each t3 value
// read once for TA rows); the batched sweep's autotuner picks it per batch.
template <class T, int TA = 1>
__host__ __device__ void cc_matvec(const CcShape& s, int bwl, const Mv<T>& m, T* out) {
	const int tid = CC_TID;
	const int KL = s.KL(), M1 = s.M1(), c1 = bwl * KL, ld3 = s.ld3(), c3 = s.nI() * bwl;
	// t1[rho][(bl, k)] = sum_b' pf[rho][b'] R[(bl, k)][b']: each thread one row and up to
	// four columns (four independent accumulators; one read of the row per b')
	const int ng = (c1 + 3) >> 2;
	for (int e = tid; e < M1 * ng; e += CC_STRIDE) {
		const int rho = e / ng, c0 = (e - rho * ng) * 4, cw = c1 - c0;
		const T* xp = m.pf + (size_t)rho * m.ldp;
		const T* r0 = m.R + (size_t)c0 * m.ldr;
		const T* r1 = r0 + (cw > 1 ? m.ldr : 0);  // rows past the last column repeat row c0
		const T* r2 = r0 + (cw > 2 ? 2 * m.ldr : 0);
		const T* r3 = r0 + (cw > 3 ? 3 * m.ldr : 0);
		T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
		for (int q = 0; q < s.rb; ++q) {
			const T xv = xp[q];
			a0 = fma(xv, r0[q], a0);
			a1 = fma(xv, r1[q], a1);
			a2 = fma(xv, r2[q], a2);
			a3 = fma(xv, r3[q], a3);
		}
		T* o = m.t1 + (size_t)rho * c1 + c0;
		o[0] = a0;
		if (cw > 1) o[1] = a1;
		if (cw > 2) o[2] = a2;
		if (cw > 3) o[3] = a3;
	}
	CC_SYNC();
	if (!s.two) {
		// t3[(k, a')][(i, bl)] = sum_(j, k') A1[(k, i), (j, k')] t1[(a', j)][(bl, k')]
		const int n1 = s.n1, K1 = s.K1, tot = s.K0 * s.ra * n1 * bwl;
		for (int e = tid; e < tot; e += CC_STRIDE) {
			int t = e;
			const int bl = t % bwl; t /= bwl;
			const int i = t % n1; t /= n1;
			const int ap = t % s.ra;
			const int k = t / s.ra;
			const T* ap1 = m.A1 + (size_t)(k * n1 + i) * n1 * K1;
			const T* tp = m.t1 + (size_t)ap * n1 * c1 + bl * K1;
			T acc = T(0);
			for (int j = 0; j < n1; ++j)
				for (int kp = 0; kp < K1; ++kp) acc = fma(ap1[j * K1 + kp], tp[j * c1 + kp], acc);
			m.t3[(size_t)(k * s.ra + ap) * ld3 + i * bwl + bl] = acc;
		}
	} else {
		const int n1 = s.n1, n2 = s.n2, K1 = s.K1, K2 = s.K2, c2 = bwl * K1;
		// t2[(a', j1, i2)][(bl, k1)] = sum_(j2, k2) A2[(k1, i2), (j2, k2)] t1[(a', j1, j2)][(bl, k2)]
		const int tot2 = s.ra * n1 * n2 * c2;
		for (int e = tid; e < tot2; e += CC_STRIDE) {
			int t = e;
			const int k1 = t % K1; t /= K1;
			const int bl = t % bwl; t /= bwl;
			const int i2 = t % n2; t /= n2;
			const int row = t;  // (a', j1)
			const T* a2 = m.A2 + (size_t)(k1 * n2 + i2) * n2 * K2;
			const T* tp = m.t1 + (size_t)row * n2 * c1 + bl * K2;
			T acc = T(0);
			for (int j2 = 0; j2 < n2; ++j2)
				for (int k2 = 0; k2 < K2; ++k2) acc = fma(a2[j2 * K2 + k2], tp[j2 * c1 + k2], acc);
			m.t2[((size_t)row * n2 + i2) * c2 + bl * K1 + k1] = acc;
		}
		CC_SYNC();
		// t3[(k0, a')][(i1, i2, bl)] = sum_(j1, k1) A1[(k0, i1), (j1, k1)] t2[(a', j1, i2)][(bl, k1)]
		const int tot3 = s.K0 * s.ra * n1 * n2 * bwl;
		for (int e = tid; e < tot3; e += CC_STRIDE) {
			int t = e;
			const int bl = t % bwl; t /= bwl;
			const int i2 = t % n2; t /= n2;
			const int i1 = t % n1; t /= n1;
			const int ap = t % s.ra;
			const int k0 = t / s.ra;
			const T* a1 = m.A1 + (size_t)(k0 * n1 + i1) * n1 * K1;
			const T* tp = m.t2 + ((size_t)ap * n1 * n2 + i2) * c2 + bl * K1;
			T acc = T(0);
			for (int j1 = 0; j1 < n1; ++j1)
				for (int k1 = 0; k1 < K1; ++k1) acc = fma(a1[j1 * K1 + k1], tp[(size_t)j1 * n2 * c2 + k1], acc);
			m.t3[(size_t)(k0 * s.ra + ap) * ld3 + (i1 * n2 + i2) * bwl + bl] = acc;
		}
	}
	CC_SYNC();
	// out[a][(i.., bl)] = sum_(k, a') L[a][(k, a')] t3[(k, a')][(i.., bl)]
	const int KK = s.K0 * s.ra;
	if (TA == 1) {
		for (int e = tid; e < s.ra * c3; e += CC_STRIDE) {
			const int a = e / c3, nu = e - a * c3;
			const T* lp = m.L + (size_t)a * m.ldl;
			const T* tp = m.t3 + nu;
			T acc = T(0);
			for (int kk = 0; kk < KK; ++kk) acc = fma(lp[kk], tp[(size_t)kk * ld3], acc);
			out[e] = acc;
		}
	} else {
		const int ga = (s.ra + TA - 1) / TA;
		for (int e = tid; e < ga * c3; e += CC_STRIDE) {
			const int a0 = (e / c3) * TA, nu = e - (e / c3) * c3;
			const T* lp[TA];
			T acc[TA];
			for (int i = 0; i < TA; ++i) {
				lp[i] = m.L + (size_t)(a0 + i < s.ra ? a0 + i : s.ra - 1) * m.ldl;  // rows past ra repeat the last
				acc[i] = T(0);
			}
			const T* tp = m.t3 + nu;
			for (int kk = 0; kk < KK; ++kk) {
				const T tv = tp[(size_t)kk * ld3];
				for (int i = 0; i < TA; ++i) acc[i] = fma(lp[i][kk], tv, acc[i]);
			}
			for (int i = 0; i < TA; ++i)
				if (a0 + i < s.ra) out[(size_t)(a0 + i) * c3 + nu] = acc[i];
		}
	}
	CC_SYNC();
}

}  // namespace xtt
