// Batched ALS_SPD: many independent SPD systems A_i x_i = b_i of uneven order,
// mode sizes and ranks, swept in one persistent launch.
//
// The reference solves one problem per ALSVariant::solve call
// (src/xerus/algorithms/als.cpp:483-553). Here every CTA of a persistent grid
// takes the next instance from an atomic counter (instances are ordered by
// estimated cost, longest first) and runs that instance's whole solve on its
// own: prepare_x_for_als (als.cpp:105-182), the initial orthogonalisation,
// the environment stacks (als.cpp:217-253), and the half-sweeps with local
// CG solves, move_core by Householder QR / LQ and stack pushes
// (als.cpp:340-380, 426-475), optionally restoring the core position. Every
// contraction is the same GEMM chain the single-instance driver launches,
// executed by the CTA's threads one output per thread (GB300's FP64 pipe, not
// memory, bounds these shapes); the local operator is the right-environment-
// first product shared with the cluster-resident solver. All intermediate
// data lives in the CTA's slice of one workspace (L2-resident); the launch is
// captured once as a CUDA graph (descriptor upload, counter reset, kernel) and
// replayed while the batch signature does not change. The block size and the
// number of resident CTAs per SM come from a small autotuner.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "als.cuh"
#include "blk_qr.cuh"
#include "local_op.cuh"

namespace xtt {

constexpr int kBMaxD = 16;
constexpr int kBMaxR = kBlkQrMaxCols;
constexpr int kBMaxHalfSweeps = 1024;  // bound of a launch that stops on the energy criterion

struct BInst {
	int d, first, last, canon, cpos, pad0;
	int n[kBMaxD];
	int rx[kBMaxD + 1], rA[kBMaxD + 1], rb[kBMaxD + 1];
	double* x[kBMaxD];
	const double* A[kBMaxD];
	const double* b[kBMaxD];
};

// Offsets (in doubles) inside one CTA's workspace slice.
struct BLayout {
	size_t L, R, Lb, Rb, v, bloc, q, r, p, t1, t3, s1, s2, qw, qq, qc, tg, f, total;
	size_t fL, fA, fR, fv, ft1, ft3;  // float offsets inside the f region
};

struct BArgs {
	const BInst* inst = nullptr;
	const int* order = nullptr;
	int count = 0;
	int* next = nullptr;
	double* work = nullptr;
	BLayout lay;
	int precision = 0, half_sweeps = 0, max_iter = 0, max_refine = 12, preserve = 1;
	int tile = 0;  // register tiles: 0 one output per thread, 1 GEMM 2x2 / matvec 2 rows, 2 GEMM 4x2 / matvec 4 rows
	double conv_eps = 0, tol = 1e-13;
	double* energy = nullptr;
	int* iters = nullptr;
	int* final_pos = nullptr;
	int* status = nullptr;
};

struct BShared {
	BlkQrSmem qr;
	double red[32];
	float redf[32];
	long long opoff[kBMaxD + 2], rhoff[kBMaxD + 2];
	int ibuf;
};

// ------------------------------------------------------------ block primitives

// C = alpha A B + beta C over the whole CTA, a TM x TN register tile of outputs per
// thread (each loaded A value used TN times, each B value TM times).
template <class T, int TM, int TN>
__device__ void blk_gemm_tiled(const Gemm<T>& g) {
	if (g.M > 0 && g.N > 0 && g.batch > 0) {
		const int tm = (g.M + TM - 1) / TM, tn = (g.N + TN - 1) / TN;
		const long long total = (long long)g.batch * tm * tn;
		const int Ki = g.Ki ? g.Ki : (g.K > 0 ? g.K : 1);
		for (long long e = threadIdx.x; e < total; e += blockDim.x) {
			const int n0 = int(e % tn) * TN;
			const long long t = e / tn;
			const int m0 = int(t % tm) * TM;
			const long long bb = t / tm;
			const T* Ap[TM];
			const T* Bp[TN];
#pragma unroll
			for (int i = 0; i < TM; ++i) Ap[i] = g.A + bb * g.sAb + g.offA(min(m0 + i, g.M - 1), 0);
#pragma unroll
			for (int j = 0; j < TN; ++j) Bp[j] = g.B + bb * g.sBb + g.offB(0, min(n0 + j, g.N - 1));
			T acc[TM][TN];
#pragma unroll
			for (int i = 0; i < TM; ++i)
#pragma unroll
				for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
			for (int ko = 0, k0 = 0; k0 < g.K; ++ko, k0 += Ki) {
				const int kl = min(Ki, g.K - k0);
				for (int ki = 0; ki < kl; ++ki) {
					T av[TM], bv[TN];
#pragma unroll
					for (int i = 0; i < TM; ++i) av[i] = Ap[i][ko * g.sAko + ki * g.sAk];
#pragma unroll
					for (int j = 0; j < TN; ++j) bv[j] = Bp[j][ko * g.sBko + ki * g.sBk];
#pragma unroll
					for (int i = 0; i < TM; ++i)
#pragma unroll
						for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
				}
			}
#pragma unroll
			for (int i = 0; i < TM; ++i)
#pragma unroll
				for (int j = 0; j < TN; ++j)
					if (m0 + i < g.M && n0 + j < g.N) {
						T* C = g.C + bb * g.sCb + g.offC(m0 + i, n0 + j);
						*C = (g.beta == T(0)) ? g.alpha * acc[i][j] : g.alpha * acc[i][j] + g.beta * *C;
					}
		}
	}
	__syncthreads();
}

// C = alpha A B + beta C over the whole CTA, one output per thread.
template <class T>
__device__ void blk_gemm(const Gemm<T>& g, int tile = 0) {
	if (tile == 1) {
		blk_gemm_tiled<T, 2, 2>(g);
		return;
	}
	if (tile == 2) {
		blk_gemm_tiled<T, 4, 2>(g);
		return;
	}
	if (g.M > 0 && g.N > 0 && g.batch > 0) {
		const long long total = (long long)g.batch * g.M * g.N;
		const int Ki = g.Ki ? g.Ki : (g.K > 0 ? g.K : 1);
		for (long long e = threadIdx.x; e < total; e += blockDim.x) {
			const int nn = int(e % g.N);
			const long long t = e / g.N;
			const int m = int(t % g.M);
			const long long bb = t / g.M;
			const T* Ap = g.A + bb * g.sAb + g.offA(m, 0);
			const T* Bp = g.B + bb * g.sBb + g.offB(0, nn);
			T acc = T(0);
			for (int ko = 0, k0 = 0; k0 < g.K; ++ko, k0 += Ki) {
				const int kl = min(Ki, g.K - k0);
				const T* ap = Ap + ko * g.sAko;
				const T* bp = Bp + ko * g.sBko;
				for (int ki = 0; ki < kl; ++ki) acc = fma(ap[ki * g.sAk], bp[ki * g.sBk], acc);
			}
			T* C = g.C + bb * g.sCb + g.offC(m, nn);
			*C = (g.beta == T(0)) ? g.alpha * acc : g.alpha * acc + g.beta * *C;
		}
	}
	__syncthreads();
}

__device__ void blk_chain(int tile, const GemmChain& ch) {
	for (int i = 0; i < ch.ns; ++i) blk_gemm(ch.g[i], tile);
}

template <class D, class S>
__device__ void blk_copy(D* dst, const S* src, long long n) {
	for (long long e = threadIdx.x; e < n; e += blockDim.x) dst[e] = D(src[e]);
	__syncthreads();
}

// ------------------------------------------------------------ one instance

struct BInstance {
	const BArgs& a;
	const BInst& I;
	double* ws;
	BShared& sh;
	int iters = 0;
	bool fp32_stalled = false;  // once set, this instance's remaining solves run in FP64

	__device__ double* Lop(int k) const { return ws + a.lay.L + sh.opoff[k]; }
	__device__ double* Rop(int k) const { return ws + a.lay.R + sh.opoff[k]; }
	__device__ double* Lb(int k) const { return ws + a.lay.Lb + sh.rhoff[k]; }
	__device__ double* Rb(int k) const { return ws + a.lay.Rb + sh.rhoff[k]; }
	__device__ long long csize(int k) const { return (long long)I.rx[k] * I.n[k] * I.rx[k + 1]; }

	__device__ void push_left(int k) {
		blk_chain(a.tile, plan_push_left_op(Lop(k), I.x[k], I.A[k], Lop(k + 1), ws + a.lay.s1, ws + a.lay.s2, I.rx[k], I.rA[k],
		                            I.n[k], I.rx[k + 1], I.rA[k + 1]));
		blk_chain(a.tile, plan_push_left_rhs(Lb(k), I.b[k], I.x[k], Lb(k + 1), ws + a.lay.s1, I.rb[k], I.rx[k], I.n[k],
		                             I.rb[k + 1], I.rx[k + 1]));
	}
	__device__ void push_right(int k) {
		blk_chain(a.tile, plan_push_right_op(Rop(k + 1), I.x[k], I.A[k], Rop(k), ws + a.lay.s1, ws + a.lay.s2, I.rx[k],
		                             I.rA[k], I.n[k], I.rx[k + 1], I.rA[k + 1]));
		blk_chain(a.tile, plan_push_right_rhs(Rb(k + 1), I.b[k], I.x[k], Rb(k), ws + a.lay.s1, I.rb[k], I.rx[k], I.n[k],
		                              I.rb[k + 1], I.rx[k + 1]));
	}
	// core k -> Q, R absorbed into core k+1 (move_core to the right, keepRank)
	__device__ void move_right(int k) {
		const int m = I.rx[k] * I.n[k], nc = I.rx[k + 1];
		double *Q = ws + a.lay.qq, *C = ws + a.lay.qc, *T = ws + a.lay.tg;
		blk_qr(I.x[k], nc, m, nc, 0, ws + a.lay.qw, C, Q, true, sh.qr);
		Gemm<double> g;  // T = C (nc x nc) * core_{k+1} (nc x n r2)
		const int n2r2 = I.n[k + 1] * I.rx[k + 2];
		g.M = nc; g.N = n2r2; g.K = nc;
		g.A = C; g.sAm = nc; g.sAk = 1;
		g.B = I.x[k + 1]; g.sBk = n2r2; g.sBn = 1;
		g.C = T; g.sCm = n2r2; g.sCn = 1;
		blk_gemm(g, a.tile);
		blk_copy(I.x[k + 1], T, (long long)nc * n2r2);
		blk_copy(I.x[k], Q, (long long)m * nc);
	}
	// core k -> Q (rows orthonormal), L absorbed into core k-1 (move_core to the left, keepRank)
	__device__ void move_left(int k) {
		const int m = I.rx[k], nc = I.n[k] * I.rx[k + 1];
		double *Q = ws + a.lay.qq, *C = ws + a.lay.qc, *T = ws + a.lay.tg;
		blk_qr(I.x[k], nc, m, nc, 1, ws + a.lay.qw, C, Q, true, sh.qr);
		Gemm<double> g;  // T = core_{k-1} (r n x m) * C (m x m)
		const int rn = I.rx[k - 1] * I.n[k - 1];
		g.M = rn; g.N = m; g.K = m;
		g.A = I.x[k - 1]; g.sAm = m; g.sAk = 1;
		g.B = C; g.sBk = m; g.sBn = 1;
		g.C = T; g.sCm = m; g.sCn = 1;
		blk_gemm(g, a.tile);
		blk_copy(I.x[k - 1], T, (long long)rn * m);
		blk_copy(I.x[k], Q, (long long)m * nc);
	}
	__device__ void identity_core(double* core, int p0, int n, int p1, int right) {
		const long long total = (long long)p0 * n * p1;
		for (long long e = threadIdx.x; e < total; e += blockDim.x) {
			const long long i2 = e % p1, i1 = (e / p1) % n, i0 = e / ((long long)p1 * n);
			core[e] = right ? (i0 == i1 * p1 + i2 ? 1.0 : 0.0) : (i0 * n + i1 == i2 ? 1.0 : 0.0);
		}
		__syncthreads();
	}
	__device__ CcShape shape(int k) const {
		CcShape s;
		s.two = 0;
		s.ra = I.rx[k];
		s.n1 = I.n[k];
		s.n2 = 1;
		s.rb = I.rx[k + 1];
		s.K0 = I.rA[k];
		s.K1 = I.rA[k + 1];
		s.K2 = 1;
		s.bw = s.rb;
		return s;
	}
	template <class T>
	__device__ Mv<T> mv(const CcShape& s, const T* pf, const T* L, const T* A, const T* R, T* t1, T* t3) const {
		return Mv<T>{pf, s.rb, L, s.K0 * s.ra, A, nullptr, R, s.rb, t1, t1, t3};
	}
	// the local operator with the batch's register tile (rows per thread of the last stage)
	template <class T>
	__device__ void apply(const CcShape& s, const Mv<T>& m, T* out) const {
		if (a.tile == 1) cc_matvec<T, 2>(s, s.rb, m, out);
		else if (a.tile == 2) cc_matvec<T, 4>(s, s.rb, m, out);
		else cc_matvec<T, 1>(s, s.rb, m, out);
	}
	__device__ double dot(const double* x, const double* y, long long n) {
		double l = 0;
		for (long long e = threadIdx.x; e < n; e += blockDim.x) l = fma(x[e], y[e], l);
		return block_sum(l, sh.red);
	}
	// |0.5 <v, M v> - <v, b_loc>| for the core at k  (als.cpp:265-278)
	__device__ double energy(int k) {
		const CcShape s = shape(k);
		const long long n = (long long)s.ra * s.n1 * s.rb;
		double* v = ws + a.lay.v;
		blk_copy(v, I.x[k], n);
		apply(s, mv<double>(s, v, Lop(k), I.A[k], Rop(k + 1), ws + a.lay.t1, ws + a.lay.t3), ws + a.lay.q);
		const double vq = dot(v, ws + a.lay.q, n), vb = dot(v, ws + a.lay.bloc, n);
		return fabs(0.5 * vq - vb);
	}
	__device__ void rhs(int k) {
		blk_chain(a.tile, plan_local_rhs1(Lb(k), I.b[k], Rb(k + 1), ws + a.lay.bloc, ws + a.lay.s1, I.rx[k], I.rx[k + 1],
		                          I.rb[k], I.rb[k + 1], I.n[k]));
	}
	// FP64 CG on M v = b_loc from the current v.
	__device__ void cg64(int k) {
		const CcShape s = shape(k);
		const long long n = (long long)s.ra * s.n1 * s.rb;
		double *x = ws + a.lay.v, *b = ws + a.lay.bloc, *q = ws + a.lay.q, *r = ws + a.lay.r, *p = ws + a.lay.p;
		const Mv<double> mx = mv<double>(s, x, Lop(k), I.A[k], Rop(k + 1), ws + a.lay.t1, ws + a.lay.t3);
		const Mv<double> mp = mv<double>(s, p, Lop(k), I.A[k], Rop(k + 1), ws + a.lay.t1, ws + a.lay.t3);
		apply(s, mx, q);
		double rl = 0, bl = 0;
		for (long long e = threadIdx.x; e < n; e += blockDim.x) {
			const double v = b[e] - q[e];
			r[e] = v;
			p[e] = v;
			rl = fma(v, v, rl);
			bl = fma(b[e], b[e], bl);
		}
		double rr = block_sum(rl, sh.red);
		const double bb = block_sum(bl, sh.red);
		const int maxit = a.max_iter > 0 ? a.max_iter : int(min(10 * n + 100, (long long)1 << 30));
		const double tol2 = a.tol * a.tol * bb;
		int it = 0;
		CgFloor floor_check;
		while (bb > 0 && rr > tol2 && it < maxit) {
			apply(s, mp, q);
			const double pAp = dot(p, q, n);
			// the test and the division once per CTA (FP64 pipe), broadcast through shared memory
			__shared__ double s_ab[2];
			__shared__ int s_good;
			if (threadIdx.x == 0) {
				s_good = pAp > 0.0 && isfinite(pAp);
				s_ab[0] = s_good ? rr / pAp : 0.0;
			}
			__syncthreads();
			if (!s_good) {
				if (threadIdx.x == 0 && cg_breakdown_is_error(rr, bb)) record_status(a.status, DEV_BREAKDOWN);
				break;
			}
			const double alpha = s_ab[0];
			double l = 0;
			for (long long e = threadIdx.x; e < n; e += blockDim.x) {
				x[e] = fma(alpha, p[e], x[e]);
				const double v = fma(-alpha, q[e], r[e]);
				r[e] = v;
				l = fma(v, v, l);
			}
			const double rrn = block_sum(l, sh.red);
			if (threadIdx.x == 0) s_ab[1] = rrn / rr;
			__syncthreads();
			const double beta = s_ab[1];
			rr = rrn;
			for (long long e = threadIdx.x; e < n; e += blockDim.x) p[e] = fma(beta, p[e], r[e]);
			__syncthreads();
			++it;
			if (floor_check.stalled(rr, it)) break;
		}
		if (bb == 0) blk_copy(x, b, n);  // b_loc = 0: x = 0
		iters += it;
	}
	// Mixed: FP32 CG corrections on FP32 copies of the operands, FP64 residuals.
	// returns false when the FP32 corrections stalled (the FP64 CG finished the solve)
	__device__ bool cg_mixed(int k) {
		const CcShape s = shape(k);
		const long long n = (long long)s.ra * s.n1 * s.rb;
		double *x = ws + a.lay.v, *b = ws + a.lay.bloc, *q = ws + a.lay.q;
		float* f = reinterpret_cast<float*>(ws + a.lay.f);
		float *Lf = f + a.lay.fL, *Af = f + a.lay.fA, *Rf = f + a.lay.fR, *fv = f + a.lay.fv;
		float *xf = fv, *rf = fv + n, *pf = fv + 2 * n, *qf = fv + 3 * n, *bf = fv + 4 * n;
		blk_copy(Lf, Lop(k), (long long)s.ra * s.K0 * s.ra);
		blk_copy(Af, I.A[k], (long long)s.K0 * s.n1 * s.n1 * s.K1);
		blk_copy(Rf, Rop(k + 1), (long long)s.rb * s.K1 * s.rb);
		const Mv<double> m64 = mv<double>(s, x, Lop(k), I.A[k], Rop(k + 1), ws + a.lay.t1, ws + a.lay.t3);
		const Mv<float> m32 = mv<float>(s, pf, Lf, Af, Rf, f + a.lay.ft1, f + a.lay.ft3);
		const double bb = dot(b, b, n);
		const int maxit = a.max_iter > 0 ? a.max_iter : int(min(10 * n + 100, (long long)1 << 30));
		bool reached = bb == 0;
		double rr_prev = 0, nr_prev = 0;
		for (int ref = 0; ref <= a.max_refine && bb > 0; ++ref) {
			apply(s, m64, q);
			double l = 0;
			for (long long e = threadIdx.x; e < n; e += blockDim.x) {
				const double v = b[e] - q[e];
				q[e] = v;
				l = fma(v, v, l);
			}
			const double rr64 = block_sum(l, sh.red);
			if (ref > 0 && !(rr64 < rr_prev)) {
				// the FP32 correction did not help: take it back, FP64 CG finishes below
				for (long long e = threadIdx.x; e < n; e += blockDim.x) x[e] = fma(-nr_prev, double(xf[e]), x[e]);
				__syncthreads();
				break;
			}
			if (rr64 <= a.tol * a.tol * bb) {
				reached = true;
				break;
			}
			if (ref == a.max_refine) break;
			const double nr = sqrt(rr64), inr = 1.0 / nr;
			rr_prev = rr64;
			nr_prev = nr;
			float bl = 0;
			for (long long e = threadIdx.x; e < n; e += blockDim.x) {
				const float v = float(q[e] * inr);
				bf[e] = v;
				xf[e] = 0.f;
				rf[e] = v;
				pf[e] = v;
				bl = fmaf(v, v, bl);
			}
			const float bbf = block_sum(bl, sh.redf);
			float rr = bbf;
			// FP32 inner tolerance 1e-6, or half of the reduction the FP64 target still needs
			const double itol = fmin(0.5, fmax(1e-6, 0.5 * a.tol * sqrt(bb) / nr));
			const float tol2 = float(itol * itol) * bbf;
			int it = 0;
			while (rr > tol2 && it < maxit) {
				apply(s, m32, qf);
				float lq = 0;
				for (long long e = threadIdx.x; e < n; e += blockDim.x) lq = fmaf(pf[e], qf[e], lq);
				const float pAp = block_sum(lq, sh.redf);
				if (!(pAp > 0.f) || !isfinite(pAp)) break;
				const float alpha = rr / pAp;
				float lr = 0;
				for (long long e = threadIdx.x; e < n; e += blockDim.x) {
					xf[e] = fmaf(alpha, pf[e], xf[e]);
					const float v = fmaf(-alpha, qf[e], rf[e]);
					rf[e] = v;
					lr = fmaf(v, v, lr);
				}
				const float rrn = block_sum(lr, sh.redf);
				const float beta = rrn / rr;
				rr = rrn;
				for (long long e = threadIdx.x; e < n; e += blockDim.x) pf[e] = fmaf(beta, pf[e], rf[e]);
				__syncthreads();
				++it;
			}
			for (long long e = threadIdx.x; e < n; e += blockDim.x) x[e] = fma(nr, double(xf[e]), x[e]);
			__syncthreads();
			iters += it;
		}
		if (!reached) cg64(k);  // from the best mixed iterate
		if (bb == 0) blk_copy(x, b, n);
		return reached;
	}

	__device__ void solve(int id) {
		const int d = I.d, first = I.first, last = I.last;
		if (threadIdx.x == 0) {
			sh.opoff[0] = 0;
			sh.rhoff[0] = 0;
			for (int k = 0; k <= d; ++k) {
				sh.opoff[k + 1] = sh.opoff[k] + (long long)I.rx[k] * I.rA[k] * I.rx[k];
				sh.rhoff[k + 1] = sh.rhoff[k] + (long long)I.rb[k] * I.rx[k];
			}
		}
		__syncthreads();
		// prepare_x_for_als (als.cpp:105-182): fully determined outer cores become identity reshapes
		{
			long long prod = 1;
			for (int f = 0; f < first; ++f) {
				const int nd = I.n[f], newp = int(prod * nd), rk = I.rx[f + 1], n2 = I.n[f + 1], r2 = I.rx[f + 2];
				Gemm<double> g;
				g.M = newp; g.N = n2 * r2; g.K = rk;
				g.A = I.x[f]; g.sAm = rk; g.sAk = 1;
				g.B = I.x[f + 1]; g.sBk = n2 * r2; g.sBn = 1;
				g.C = ws + a.lay.tg; g.sCm = n2 * r2; g.sCn = 1;
				blk_gemm(g, a.tile);
				blk_copy(I.x[f + 1], ws + a.lay.tg, (long long)newp * n2 * r2);
				identity_core(I.x[f], int(prod), nd, newp, 0);
				prod = newp;
			}
			prod = 1;
			for (int l = d; l > last; --l) {
				const int nd = I.n[l - 1], newp = int(prod * nd), rk = I.rx[l - 1], r0 = I.rx[l - 2], n0 = I.n[l - 2];
				Gemm<double> g;
				g.M = r0 * n0; g.N = newp; g.K = rk;
				g.A = I.x[l - 2]; g.sAm = rk; g.sAk = 1;
				g.B = I.x[l - 1]; g.sBk = newp; g.sBn = 1;
				g.C = ws + a.lay.tg; g.sCm = newp; g.sCn = 1;
				blk_gemm(g, a.tile);
				blk_copy(I.x[l - 2], ws + a.lay.tg, (long long)r0 * n0 * newp);
				identity_core(I.x[l - 1], newp, nd, int(prod), 1);
				prod = newp;
			}
		}
		// move_core(first, keepRank): the core ends at `first`
		if (I.canon && I.cpos < first) {
		} else if (I.canon) {
			const int from = I.cpos >= last ? last - 1 : I.cpos;
			for (int k = from; k > first; --k) move_left(k);
		} else {
			for (int k = 0; k < first; ++k) move_right(k);
			for (int k = d - 1; k > first; --k) move_left(k);
		}
		// stacks (als.cpp:217-253)
		if (threadIdx.x == 0) {
			Lop(0)[0] = 1.0;
			Rop(d)[0] = 1.0;
			Lb(0)[0] = 1.0;
			Rb(d)[0] = 1.0;
		}
		__syncthreads();
		for (int i = d - 1; i > first; --i) push_right(i);
		for (int i = 0; i < first; ++i) push_left(i);
		// half-sweeps (als.cpp:426-475, 340-380)
		int cur = first, half = 0;
		bool inc = true;
		rhs(cur);
		double e = energy(cur), last_e = 1e101, last_e2 = 1e102;
		const int max_half = a.half_sweeps > 0 ? a.half_sweeps : kBMaxHalfSweeps;
		while (true) {
			rhs(cur);
			blk_copy(ws + a.lay.v, I.x[cur], csize(cur));
			if (a.precision == XTT_PRECISION_FP64 || fp32_stalled) cg64(cur);
			else fp32_stalled = !cg_mixed(cur);
			blk_copy(I.x[cur], ws + a.lay.v, csize(cur));
			if ((!inc && cur == first) || (inc && cur == last - 1)) {
				++half;
				last_e2 = last_e;
				last_e = e;
				e = energy(cur);
				if (half == max_half || fabs(last_e - e) < a.conv_eps || fabs(last_e2 - e) < a.conv_eps ||
				    last - first <= 1)
					break;
				inc = !inc;
			}
			if (inc) {
				move_right(cur);
				push_left(cur);
				++cur;
			} else {
				move_left(cur);
				push_right(cur);
				--cur;
			}
		}
		if (I.canon && a.preserve) {
			for (; cur < I.cpos; ++cur) move_right(cur);
			for (; cur > I.cpos; --cur) move_left(cur);
		}
		if (threadIdx.x == 0) {
			a.energy[id] = e;
			a.iters[id] = iters;
			a.final_pos[id] = cur;
		}
		__syncthreads();
	}
};

__global__ void __launch_bounds__(512) k_als_batch(BArgs a) {
	__shared__ BShared sh;
	__shared__ BInst I;
	double* ws = a.work + (size_t)blockIdx.x * a.lay.total;
	while (true) {
		if (threadIdx.x == 0) sh.ibuf = atomicAdd(a.next, 1);
		__syncthreads();
		const int i = sh.ibuf;
		__syncthreads();
		if (i >= a.count) break;
		const int id = a.order[i];
		{
			const int* src = reinterpret_cast<const int*>(a.inst + id);
			int* dst = reinterpret_cast<int*>(&I);
			for (int e = threadIdx.x; e < int(sizeof(BInst) / sizeof(int)); e += blockDim.x) dst[e] = src[e];
		}
		__syncthreads();
		BInstance inst{a, I, ws, sh};
		inst.solve(id);
	}
}

// ------------------------------------------------------------ host side

namespace {

struct Sizes {
	size_t L = 1, R = 1, dim = 1, t1 = 1, t3 = 1, s1 = 1, s2 = 1, core = 1, fL = 1, fA = 1, fR = 1;
};

void grow(size_t& v, size_t w) { v = std::max(v, w); }

}  // namespace

struct BatchPlan {
	std::vector<BInst> inst;
	std::vector<int> order;
	BLayout lay;
};

static BLayout make_layout(const Sizes& z) {
	BLayout l;
	size_t o = 0;
	auto take = [&](size_t n) {
		const size_t at = o;
		o += (n + 3) & ~size_t(3);
		return at;
	};
	l.L = take(z.L);
	l.R = take(z.L);
	l.Lb = take(z.R);
	l.Rb = take(z.R);
	l.v = take(z.dim);
	l.bloc = take(z.dim);
	l.q = take(z.dim);
	l.r = take(z.dim);
	l.p = take(z.dim);
	l.t1 = take(z.t1);
	l.t3 = take(z.t3);
	l.s1 = take(z.s1);
	l.s2 = take(z.s2);
	l.qw = take(z.core);
	l.qq = take(z.core);
	l.qc = take(z.core);
	l.tg = take(z.core);
	// float region
	size_t fo = 0;
	auto ftake = [&](size_t n) {
		const size_t at = fo;
		fo += (n + 3) & ~size_t(3);
		return at;
	};
	l.fL = ftake(z.fL);
	l.fA = ftake(z.fA);
	l.fR = ftake(z.fR);
	l.fv = ftake(5 * z.dim);
	l.ft1 = ftake(z.t1);
	l.ft3 = ftake(z.t3);
	l.f = take((fo + 1) / 2);
	l.total = (o + 31) & ~size_t(31);
	return l;
}

// Copies every instance's x cores to (to_buf) or from a packed buffer.
__global__ void k_batch_x_copy(const BInst* inst, const long long* off, int count, double* buf, int to_buf) {
	for (int i = blockIdx.x; i < count; i += gridDim.x) {
		const BInst& I = inst[i];
		long long o = off[i];
		for (int k = 0; k < I.d; ++k) {
			const long long n = (long long)I.rx[k] * I.n[k] * I.rx[k + 1];
			for (long long e = threadIdx.x; e < n; e += blockDim.x) {
				if (to_buf) buf[o + e] = I.x[k][e];
				else I.x[k][e] = buf[o + e];
			}
			o += n;
		}
	}
}

static unsigned long long mix(unsigned long long h, unsigned long long v) {
	h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
	return h;
}

static BatchResult run_batch(Context& c, const std::vector<BInst>& inst, const std::vector<int>& order,
                             const BLayout& lay, const AlsOptions& o, bool autotune) {
	const int count = int(inst.size());
	// device descriptors and results, and their pinned staging (same byte layout)
	const size_t o_inst = 0, o_order = o_inst + count * sizeof(BInst);
	const size_t o_energy = (o_order + count * sizeof(int) + 15) & ~size_t(15);
	const size_t o_iters = o_energy + count * sizeof(double), o_pos = o_iters + count * sizeof(int);
	const size_t o_next = (o_pos + count * sizeof(int) + 15) & ~size_t(15), o_off = o_next + 16;
	const size_t meta_bytes = o_off + size_t(count) * sizeof(long long);
	char* dm = c.scratch<char>(S_BATCH_META, meta_bytes);
	if (c.batch_host_bytes < meta_bytes) {
		if (c.batch_host) {
			XTT_CUDA(cudaStreamSynchronize(c.stream));
			XTT_CUDA(cudaFreeHost(c.batch_host));
			c.batch_host = nullptr;
		}
		XTT_CUDA(cudaMallocHost(&c.batch_host, meta_bytes));
		c.batch_host_bytes = meta_bytes;
		c.batch_key = 0;
	}
	char* hm = static_cast<char*>(c.batch_host);
	std::memcpy(hm + o_inst, inst.data(), count * sizeof(BInst));
	std::memcpy(hm + o_order, order.data(), count * sizeof(int));
	BArgs a;
	a.inst = reinterpret_cast<const BInst*>(dm + o_inst);
	a.order = reinterpret_cast<const int*>(dm + o_order);
	a.count = count;
	a.next = reinterpret_cast<int*>(dm + o_next);
	a.lay = lay;
	a.precision = o.precision;
	a.half_sweeps = int(std::min<int64_t>(o.num_half_sweeps, kBMaxHalfSweeps));
	a.max_iter = int(std::min<int64_t>(o.local_max_iterations, 1 << 30));
	a.preserve = o.preserve_core_position ? 1 : 0;
	a.conv_eps = o.convergence_epsilon;
	a.tol = o.local_tolerance;
	a.energy = reinterpret_cast<double*>(dm + o_energy);
	a.iters = reinterpret_cast<int*>(dm + o_iters);
	a.final_pos = reinterpret_cast<int*>(dm + o_pos);
	a.status = c.d_status;
	// signature of the launch shape (the autotuner's cache key)
	unsigned long long sig = mix(0, (unsigned long long)count);
	sig = mix(sig, lay.total);
	sig = mix(sig, (unsigned long long)o.precision);
	for (const BInst& I : inst) {
		sig = mix(sig, (unsigned long long)I.d);
		for (int k = 0; k < I.d; ++k) sig = mix(sig, (unsigned long long)(I.n[k] * 4096 + I.rx[k + 1] * 64 + I.rA[k + 1]));
	}
	int threads = 256, per_sm = 1, tile = 0;
	bool have = false;
	for (auto& t : c.batch_tuned)
		if (t.sig == sig) {
			threads = t.threads;
			per_sm = t.per_sm;
			tile = t.tile;
			have = true;
		}
	XTT_CUDA(cudaMemcpyAsync(dm, hm, o_energy, cudaMemcpyHostToDevice, c.stream));
	cudaEvent_t e0, e1;
	XTT_CUDA(cudaEventCreate(&e0));
	XTT_CUDA(cudaEventCreate(&e1));
	if (autotune && !have) {
		// time each launch shape on the real batch, restoring x between trials
		long long tot = 0;
		std::vector<long long> off(count);
		for (int i = 0; i < count; ++i) {
			off[i] = tot;
			for (int k = 0; k < inst[i].d; ++k) tot += (long long)inst[i].rx[k] * inst[i].n[k] * inst[i].rx[k + 1];
		}
		std::memcpy(hm + o_off, off.data(), count * sizeof(long long));
		XTT_CUDA(cudaMemcpyAsync(dm + o_off, hm + o_off, count * sizeof(long long), cudaMemcpyHostToDevice, c.stream));
		double* bk = c.scratch<double>(S_BATCH_BACKUP, size_t(tot));
		const long long* doff = reinterpret_cast<const long long*>(dm + o_off);
		k_batch_x_copy<<<std::min(count, 4 * c.num_sms), 256, 0, c.stream>>>(a.inst, doff, count, bk, 1);
		XTT_CUDA(cudaGetLastError());
		double best = 1e300;
		auto trial = [&](int th, int ps, int tl) {
			const int G = std::max(1, std::min(count, ps * c.num_sms));
			a.work = c.scratch<double>(S_BATCH_WORK, size_t(G) * lay.total);
			a.tile = tl;
			XTT_CUDA(cudaMemsetAsync(a.next, 0, sizeof(int), c.stream));
			XTT_CUDA(cudaEventRecord(e0, c.stream));
			k_als_batch<<<G, th, 0, c.stream>>>(a);
			XTT_CUDA(cudaGetLastError());
			XTT_CUDA(cudaEventRecord(e1, c.stream));
			k_batch_x_copy<<<std::min(count, 4 * c.num_sms), 256, 0, c.stream>>>(a.inst, doff, count, bk, 0);
			c.count_launch(2);
			XTT_CUDA(cudaEventSynchronize(e1));
			float ms = 0;
			XTT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			if (ms < best) {
				best = ms;
				threads = th;
				per_sm = ps;
				tile = tl;
			}
		};
		// launch shapes (threads x resident CTAs per SM) with one output per thread, then the
		// register tile shapes of the GEMMs and the local operator at the fastest launch shape
		for (int th : {128, 256, 512}) {
			int occ = 0;
			XTT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_als_batch, th, 0));
			for (int ps : {1, 2, 4})
				if (ps <= occ) trial(th, ps, 0);
		}
		const int th_best = threads, ps_best = per_sm;
		for (int tl : {1, 2}) trial(th_best, ps_best, tl);
		c.sync();
		c.batch_tuned.push_back({sig, threads, per_sm, tile});
	}
	a.tile = tile;
	const int G = std::max(1, std::min(count, per_sm * c.num_sms));
	a.work = c.scratch<double>(S_BATCH_WORK, size_t(G) * lay.total);
	// the whole batched sweep as one CUDA graph: descriptor upload, counter reset, kernel, results
	unsigned long long key = mix(sig, (unsigned long long)(uintptr_t)a.work);
	key = mix(key, (unsigned long long)(uintptr_t)dm);
	key = mix(key, (unsigned long long)(uintptr_t)hm);
	key = mix(key, (unsigned long long)(threads * 64 + per_sm * 4 + tile));
	key = mix(key, (unsigned long long)(a.half_sweeps * 7 + a.max_iter * 13 + a.preserve));
	unsigned long long eb;
	std::memcpy(&eb, &a.conv_eps, 8);
	key = mix(key, eb);
	std::memcpy(&eb, &a.tol, 8);
	key = mix(key, eb);
	if (key != c.batch_key || !c.batch_exec) {
		if (c.batch_exec) {
			XTT_CUDA(cudaGraphExecDestroy(c.batch_exec));
			c.batch_exec = nullptr;
		}
		cudaGraph_t graph;
		XTT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
		cudaMemcpyAsync(dm, hm, o_energy, cudaMemcpyHostToDevice, c.stream);
		cudaMemsetAsync(a.next, 0, sizeof(int), c.stream);
		k_als_batch<<<G, threads, 0, c.stream>>>(a);
		cudaMemcpyAsync(hm + o_energy, dm + o_energy, o_next - o_energy, cudaMemcpyDeviceToHost, c.stream);
		XTT_CUDA(cudaStreamEndCapture(c.stream, &graph));
		XTT_CUDA(cudaGraphInstantiate(&c.batch_exec, graph, 0));
		XTT_CUDA(cudaGraphDestroy(graph));
		c.batch_key = key;
	}
	XTT_CUDA(cudaEventRecord(e0, c.stream));
	XTT_CUDA(cudaGraphLaunch(c.batch_exec, c.stream));
	XTT_CUDA(cudaEventRecord(e1, c.stream));
	c.count_launch();
	c.sync();
	float ms = 0;
	XTT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	BatchResult r;
	r.ms = ms;
	r.threads = threads;
	r.ctas_per_sm = per_sm;
	r.ctas = G;
	r.tile = tile;
	r.energy.assign(reinterpret_cast<double*>(hm + o_energy), reinterpret_cast<double*>(hm + o_energy) + count);
	r.iterations.assign(reinterpret_cast<int*>(hm + o_iters), reinterpret_cast<int*>(hm + o_iters) + count);
	r.final_pos.assign(reinterpret_cast<int*>(hm + o_pos), reinterpret_cast<int*>(hm + o_pos) + count);
	return r;
}

BatchResult als_batch(Context& c, const std::vector<const Tensor*>& A, const std::vector<Tensor*>& x,
                      const std::vector<const Tensor*>& b, const AlsOptions& o, bool autotune) {
	const int count = int(x.size());
	XTT_REQUIRE(count > 0 && A.size() == x.size() && b.size() == x.size(), "batch: A, x and b lists differ in length");
	XTT_REQUIRE(o.sites == 1 && o.local_solver == 0, "batch: one-site ALS with exact local solves only");
	XTT_REQUIRE(o.num_half_sweeps > 0 || o.convergence_epsilon > 0, "batch: give num_half_sweeps or an epsilon");
	std::vector<BInst> inst(count);
	std::vector<double> cost(count);
	Sizes z;
	for (int i = 0; i < count; ++i) {
		const Tensor &Ai = *A[i], &xi = *x[i], &bi = *b[i];
		XTT_REQUIRE(Ai.ctx == &c && xi.ctx == &c && bi.ctx == &c, "batch: all tensors must live on the context");
		XTT_REQUIRE(Ai.op && !xi.op && !bi.op, "batch: needs TT operators, TT tensors x and b");
		const int d = xi.d;
		XTT_REQUIRE(d >= 1 && d <= kBMaxD, "batch: order must be 1..16");
		XTT_REQUIRE(xi.dims == bi.dims && Ai.dims == xi.dims && Ai.d == d, "batch: dimensions of A, x and b differ");
		BInst& I = inst[i];
		std::memset(&I, 0, sizeof(I));
		I.d = d;
		for (int k = 0; k <= d; ++k) {
			I.rx[k] = int(xi.ranks[k]);
			I.rA[k] = int(Ai.ranks[k]);
			I.rb[k] = int(bi.ranks[k]);
			XTT_REQUIRE(I.rx[k] <= kBMaxR, "batch: TT ranks of x must be <= 64");
		}
		for (int k = 0; k < d; ++k) {
			I.n[k] = int(xi.dims[k]);
			I.x[k] = xi.core[k];
			I.A[k] = Ai.core[k];
			I.b[k] = bi.core[k];
			XTT_REQUIRE(xi.ranks[k + 1] <= xi.ranks[k] * xi.dims[k] && xi.ranks[k] <= xi.dims[k] * xi.ranks[k + 1],
			            "batch: x must have maximal-reduced ranks (reduce_to_maximal_ranks)");
		}
		// prepare_x_for_als: pruned outer cores (same rule as the single-instance driver)
		int first = 0;
		long long prod = 1;
		while (first + 1 < d) {
			const long long newp = prod * xi.dims[first];
			if (xi.ranks[first + 1] < newp) break;
			++first;
			prod = newp;
		}
		int last = d;
		prod = 1;
		while (last > first + 1) {
			const long long newp = prod * xi.dims[last - 1];
			if (xi.ranks[last - 1] < newp) break;
			--last;
			prod = newp;
		}
		I.first = first;
		I.last = last;
		I.canon = xi.canonicalized ? 1 : 0;
		I.cpos = int(xi.core_position);
		double cst = 0;
		size_t L = 0, R = 0;
		for (int k = 0; k <= d; ++k) {
			L += size_t(I.rx[k]) * I.rA[k] * I.rx[k];
			R += size_t(I.rb[k]) * I.rx[k];
		}
		grow(z.L, L);
		grow(z.R, R);
		for (int k = 0; k < d; ++k) {
			const size_t ra = I.rx[k], rb = I.rx[k + 1], n = I.n[k], K0 = I.rA[k], K1 = I.rA[k + 1];
			const size_t s0 = I.rb[k], s1 = I.rb[k + 1];
			const size_t dim = ra * n * rb;
			grow(z.dim, dim);
			grow(z.t1, ra * n * rb * K1);
			grow(z.t3, K0 * ra * (n * rb + 1));
			grow(z.s1, std::max({K0 * ra * n * rb, ra * n * rb * K1, ra * n * s1, ra * n * s0}));
			grow(z.s2, std::max(ra * rb * n * K1, ra * K0 * n * rb));
			grow(z.core, std::max({dim, ra * ra, rb * rb}));
			if (k + 1 < d) grow(z.core, size_t(I.rx[k + 1]) * I.n[k + 1] * I.rx[k + 2]);
			grow(z.fL, ra * K0 * ra);
			grow(z.fA, K0 * n * n * K1);
			grow(z.fR, rb * K1 * rb);
			cost[i] += double(dim) * double(ra * K0 + n * K0 * K1 + K1 * rb);
		}
		(void)cst;
	}
	std::vector<int> order(count);
	std::iota(order.begin(), order.end(), 0);
	std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return cost[p] > cost[q]; });
	const BLayout lay = make_layout(z);
	BatchResult r = run_batch(c, inst, order, lay, o, autotune);
	for (int i = 0; i < count; ++i) {
		x[i]->canonicalized = true;
		x[i]->core_position = r.final_pos[i];
	}
	return r;
}

}  // namespace xtt
