// Cluster-resident local solver of the ALS / DMRG sweep: a whole conjugate-
// gradient solve of the local SPD system (src/xerus/algorithms/als.cpp:43-71
// solves the same system densely) in one thread-block cluster of up to 16
// CTAs, with every operand on chip.
//
// Partition. The local vector x(a, i[, i2], b) is split over the CTAs by its
// last (right-bond) index b. Contracting the right environment first,
//   T1(a',j,k',b) = sum_b' x(a',j,b') R(b,k',b'),
//   T2(k,a',i,b)  = sum_(j,k') A(k,i,j,k') T1(a',j,k',b),
//   y(a,i,b)      = sum_(k,a') L(a,k,a') T2(k,a',i,b),
// every stage produces only the columns b the CTA owns, so the only data a CTA
// needs from the others is the full input vector. After each update of the
// search direction every CTA pushes its slice into all CTAs' shared memory
// (remote stores do not stall the issuing warp), and one hardware cluster
// barrier later each CTA holds the whole vector. Dot products are pushed the
// same way (one partial per CTA) and summed in rank order, so every CTA takes
// bit-identical, uniform decisions. Three cluster barriers per CG iteration
// (the push of p, p^T M p, r^T r).
//
// Precision. FP64 form: everything in double. Mixed form: the CG runs in FP32
// on FP32 copies of L, A and R converted on load; each correction is checked
// against an FP64 residual b - M x computed from the FP64 operands, and the
// solve stops on the FP64 residual (iterative refinement).
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include <cooperative_groups.h>

#include "als.cuh"
#include "local_op.cuh"

namespace xtt {

namespace cgx = cooperative_groups;

constexpr int kCcThreads = 256;

constexpr int kCcMaxCluster = 16;
constexpr size_t kCcSmemMax = 220 * 1024;

// Byte offsets of the shared-memory regions; `w` is the compute type's size,
// `mixed` adds the FP64 refinement buffers.
struct CcLayout {
	size_t pf, L, A1, A2, R, t1, t2, t3, v, r64, red, total;
};

static size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

static CcLayout cc_layout(const CcShape& s, bool mixed) {
	const size_t w = mixed ? sizeof(float) : sizeof(double);
	CcLayout l;
	size_t o = 0;
	l.red = o;  // reduction slots: 6 arrays of 16 doubles
	o = align16(o + 6 * kCcMaxCluster * sizeof(double));
	l.pf = o;  // the gathered vector: FP32 p or, in the mixed form, the FP64 iterate
	o = align16(o + s.n_pf() * (mixed ? sizeof(double) : w));
	l.L = o;
	o = align16(o + s.n_L() * w);
	l.A1 = o;
	o = align16(o + s.n_A1() * w);
	l.A2 = o;
	o = align16(o + s.n_A2() * w);
	l.R = o;
	o = align16(o + s.n_R() * w);
	// temporaries: in the mixed form the FP64 refinement reuses them as doubles
	const size_t tw = mixed ? sizeof(double) : w;
	l.t1 = o;
	o = align16(o + s.n_t1() * tw);
	l.t2 = o;
	o = align16(o + s.n_t2() * tw);
	l.t3 = o;
	o = align16(o + s.n_t3() * tw);
	l.v = o;  // x, r, p, q, b slices
	o = align16(o + 5 * s.n_v() * w);
	l.r64 = o;
	if (mixed) o = align16(o + s.n_v() * sizeof(double));
	l.total = o;
	return l;
}

struct CcArgs {
	CcShape s;
	CcLayout lay;
	int P = 1;
	const double *L = nullptr, *A1 = nullptr, *A2 = nullptr, *R = nullptr, *b = nullptr;
	double* x = nullptr;  // initial guess in, solution out (global, row-major (a, i[, i2], b))
	double tol = 0;       // FP64 relative residual target
	int max_iter = 0;     // per CG
	int max_refine = 0;   // mixed form
	float inner_tol = 1e-6f;
	int* status = nullptr;
	int* out_i = nullptr;
	double* out_d = nullptr;
	int* flag = nullptr;        // mixed form: 1 when the FP64 target was not reached, else 0
	int* sticky = nullptr;      // mixed form: set once FP32 corrections stalled; later solves skip them
	const int* gate = nullptr;  // FP64 form: run only if *gate != 0 (polish after a mixed solve)
};

// Every CTA writes its slice v[(rho, bl)] into column b0 + bl of the gathered
// vector of every CTA of the cluster (including itself).
template <class T>
__device__ void cc_push(T* pf, const T* v, int M1, int bwl, int b0, int ldp, int P) {
	cgx::cluster_group cl = cgx::this_cluster();
	T* dst[kCcMaxCluster];
#pragma unroll
	for (int q = 0; q < kCcMaxCluster; ++q) dst[q] = cl.map_shared_rank(pf, q < P ? q : 0);
	const int n = M1 * bwl;
	for (int e = threadIdx.x; e < n; e += blockDim.x) {
		const int rho = e / bwl, bl = e - rho * bwl;
		const size_t off = (size_t)rho * ldp + b0 + bl;
		const T val = v[e];
#pragma unroll
		for (int q = 0; q < kCcMaxCluster; ++q)
			if (q < P) dst[q][off] = val;
	}
}

// Sums over the cluster of N values per CTA (`mine`, equal in all threads):
// partials are pushed into slots[N rank + i] of every CTA, then summed in rank
// order by thread 0 and broadcast, so every CTA gets bit-identical totals. A
// slot array may be reused by the next call only after another cluster barrier.
template <class T, int N>
__device__ void cc_total(const T (&mine)[N], T* slots, T* bcast, int me, int P, T (&tot)[N]) {
	cgx::cluster_group cl = cgx::this_cluster();
	if ((int)threadIdx.x < P) {
		T* d = cl.map_shared_rank(slots, (int)threadIdx.x);
#pragma unroll
		for (int i = 0; i < N; ++i) d[N * me + i] = mine[i];
	}
	cl.sync();
	if (threadIdx.x == 0) {
#pragma unroll
		for (int i = 0; i < N; ++i) {
			T s = T(0);
			for (int p = 0; p < P; ++p) s += slots[N * p + i];
			bcast[i] = s;
		}
	}
	__syncthreads();
#pragma unroll
	for (int i = 0; i < N; ++i) tot[i] = bcast[i];
}

template <class T>
__device__ T cc_total(T mine, T* slots, T* bcast, int me, int P) {
	const T m1[1] = {mine};
	T t1[1];
	cc_total<T, 1>(m1, slots, bcast, me, P, t1);
	return t1[0];
}

template <class T>
__host__ __device__ void cc_load_operands(const CcArgs& a, int b0, int bwl, T* Ls, T* A1s, T* A2s, T* Rs) {
	const CcShape& s = a.s;
	const int tid = CC_TID, KK = s.K0 * s.ra, ldl = s.ldl(), KL = s.KL(), ldr = s.ldr();
	for (int e = tid; e < s.ra * KK; e += CC_STRIDE) {
		const int r = e / KK, c = e - r * KK;
		Ls[(size_t)r * ldl + c] = T(a.L[e]);
	}
	for (int e = tid; e < (int)s.n_A1(); e += CC_STRIDE) A1s[e] = T(a.A1[e]);
	for (int e = tid; e < (int)s.n_A2(); e += CC_STRIDE) A2s[e] = T(a.A2[e]);
	const double* Rg = a.R + (size_t)b0 * KL * s.rb;
	for (int e = tid; e < bwl * KL * s.rb; e += CC_STRIDE) {
		const int r = e / s.rb, c = e - r * s.rb;
		Rs[(size_t)r * ldr + c] = T(Rg[e]);
	}
}

// CG on this CTA's slices (x, r, p, q, b of length M1 * bwl) for M v = b:
// from x (zero_guess: x = 0), to ||r|| <= tol ||b|| or max_iter iterations.
// Returns the iteration count; rel receives ||r|| / ||b|| of the recursion.
// p^T M p is formed directly each iteration (not by a recurrence), which keeps
// the breakdown test meaningful down to the 1e-13 tolerances of the FP64 form.
template <class T>
__device__ int cc_cg(const CcShape& s, int me, int P, int b0, int bwl, const Mv<T>& m, T* pf, T* x, T* r, T* p, T* q,
                     const T* b, bool zero_guess, double tol, int max_iter, T* slots, T* bcast, int* status,
                     double& rel) {
	const int tid = threadIdx.x, n = s.M1() * bwl, M1 = s.M1(), ldp = s.ldp();
	__shared__ T sc[32];
	__shared__ T s_ab[2];
	__shared__ bool s_ok;
	if (zero_guess) {
		for (int e = tid; e < n; e += blockDim.x) {
			x[e] = T(0);
			r[e] = b[e];
			p[e] = b[e];
		}
		__syncthreads();
	} else {
		cc_push(pf, x, M1, bwl, b0, ldp, P);
		cgx::this_cluster().sync();
		cc_matvec(s, bwl, m, q);
		for (int e = tid; e < n; e += blockDim.x) {
			const T v = b[e] - q[e];
			r[e] = v;
			p[e] = v;
		}
		__syncthreads();
	}
	T rl = 0, bl = 0;
	for (int e = tid; e < n; e += blockDim.x) {
		rl = fma(r[e], r[e], rl);
		bl = fma(b[e], b[e], bl);
	}
	rl = block_sum(rl, sc);
	bl = block_sum(bl, sc);
	T tot[2];
	{
		const T mine[2] = {bl, rl};
		cc_total<T, 2>(mine, slots, bcast, me, P, tot);
	}
	const T bb = tot[0];
	T rr = tot[1];
	if (bb == T(0)) {
		for (int e = tid; e < n; e += blockDim.x) x[e] = T(0);
		__syncthreads();
		rel = 0;
		return 0;
	}
	const T tol2 = T(tol * tol) * bb;
	T* s_pap = slots + 2 * kCcMaxCluster;
	T* s_rr = slots + 3 * kCcMaxCluster;
	int it = 0;
	CgFloor floor_check;
	while (rr > tol2 && it < max_iter) {
		cc_push(pf, p, M1, bwl, b0, ldp, P);
		cgx::this_cluster().sync();
		cc_matvec(s, bwl, m, q);
		T l = 0;
		for (int e = tid; e < n; e += blockDim.x) l = fma(p[e], q[e], l);
		const T pAp = cc_total(block_sum(l, sc), s_pap, bcast, me, P);
		T alpha;
		bool ok;
		if (sizeof(T) == 8) {
			// FP64: the test and the division once per CTA (redundant copies in every thread
			// would queue on GB300's FP64 pipe), broadcast through shared memory
			if (tid == 0) {
				const bool good = pAp > T(0) && isfinite(double(pAp));
				s_ab[0] = good ? rr / pAp : T(0);
				s_ok = good;
			}
			__syncthreads();
			alpha = s_ab[0];
			ok = s_ok;
		} else {
			ok = pAp > T(0) && isfinite(double(pAp));
			alpha = ok ? rr / pAp : T(0);
		}
		if (!ok) {
			// an FP32 correction solve just stops: the FP64 refinement around it decides
			if (sizeof(T) == 8 && tid == 0 && me == 0 && cg_breakdown_is_error(double(rr), double(bb)))
				record_status(status, DEV_BREAKDOWN);
			break;
		}
		l = 0;
		for (int e = tid; e < n; e += blockDim.x) {
			x[e] = fma(alpha, p[e], x[e]);
			const T v = fma(-alpha, q[e], r[e]);
			r[e] = v;
			l = fma(v, v, l);
		}
		const T rrn = cc_total(block_sum(l, sc), s_rr, bcast, me, P);
		T beta;
		if (sizeof(T) == 8) {
			if (tid == 0) s_ab[1] = rrn / rr;
			__syncthreads();
			beta = s_ab[1];
		} else {
			beta = rrn / rr;
		}
		rr = rrn;
		for (int e = tid; e < n; e += blockDim.x) p[e] = fma(beta, p[e], r[e]);
		__syncthreads();
		++it;
		if (floor_check.stalled(double(rr), it)) break;  // identical in every CTA
	}
	rel = sqrt(double(rr) / double(bb));
	return it;
}

template <class T>
struct CcView {
	T *pf, *L, *A1, *A2, *R, *t1, *t2, *t3, *x, *r, *p, *q, *b;
	__device__ CcView(unsigned char* sm, const CcShape& s, const CcLayout& l) {
		pf = reinterpret_cast<T*>(sm + l.pf);
		L = reinterpret_cast<T*>(sm + l.L);
		A1 = reinterpret_cast<T*>(sm + l.A1);
		A2 = reinterpret_cast<T*>(sm + l.A2);
		R = reinterpret_cast<T*>(sm + l.R);
		t1 = reinterpret_cast<T*>(sm + l.t1);
		t2 = reinterpret_cast<T*>(sm + l.t2);
		t3 = reinterpret_cast<T*>(sm + l.t3);
		T* v = reinterpret_cast<T*>(sm + l.v);
		const size_t nv = s.n_v();
		x = v;
		r = v + nv;
		p = v + 2 * nv;
		q = v + 3 * nv;
		b = v + 4 * nv;
	}
	__device__ Mv<T> mv(const CcShape& s) const {
		return Mv<T>{pf, s.ldp(), L, s.ldl(), A1, A2, R, s.ldr(), t1, t2, t3};
	}
};

// FP64 form.
__global__ void __launch_bounds__(kCcThreads, 1) k_cg_cluster_f64(CcArgs a) {
	if (a.gate && __ldcg(a.gate) == 0) return;  // uniform: every CTA reads the same flag
	extern __shared__ __align__(16) unsigned char smem[];
	cgx::cluster_group cl = cgx::this_cluster();
	const CcShape& s = a.s;
	const int P = a.P, me = int(cl.block_rank()), b0 = me * s.bw, bwl = min(s.bw, s.rb - b0);
	const int M1 = s.M1(), n = M1 * bwl, tid = threadIdx.x;
	CcView<double> v(smem, s, a.lay);
	double* slots = reinterpret_cast<double*>(smem + a.lay.red);
	__shared__ double bcast[4];
	cc_load_operands(a, b0, bwl, v.L, v.A1, v.A2, v.R);
	for (int e = tid; e < n; e += kCcThreads) {
		const int rho = e / bwl, bl = e - rho * bwl;
		v.x[e] = a.x[(size_t)rho * s.rb + b0 + bl];
		v.b[e] = a.b[(size_t)rho * s.rb + b0 + bl];
	}
	__syncthreads();
	double rel = 0;
	const int it = cc_cg<double>(s, me, P, b0, bwl, v.mv(s), v.pf, v.x, v.r, v.p, v.q, v.b, false, a.tol,
	                             a.max_iter, slots, bcast, a.status, rel);
	for (int e = tid; e < n; e += kCcThreads) {
		const int rho = e / bwl, bl = e - rho * bwl;
		a.x[(size_t)rho * s.rb + b0 + bl] = v.x[e];
	}
	if (me == 0 && tid == 0) {  // counters accumulate over a sweep; the host reads them once
		a.out_i[0] += it;
		a.out_d[0] = rel;
	}
	cl.sync();  // no CTA exits while another may still store into its shared memory
}

// Mixed form: FP32 CG corrections, FP64 residuals and iterate.
__global__ void __launch_bounds__(kCcThreads, 1) k_cg_cluster_mixed(CcArgs a) {
	if (a.sticky && __ldcg(a.sticky) != 0) {  // an earlier solve of this sweep showed FP32 does not help
		if (blockIdx.x == 0 && threadIdx.x == 0) *a.flag = 1;
		return;
	}
	extern __shared__ __align__(16) unsigned char smem[];
	cgx::cluster_group cl = cgx::this_cluster();
	const CcShape& s = a.s;
	const int P = a.P, me = int(cl.block_rank()), b0 = me * s.bw, bwl = min(s.bw, s.rb - b0);
	const int M1 = s.M1(), n = M1 * bwl, tid = threadIdx.x, ldp = s.ldp();
	CcView<float> v(smem, s, a.lay);
	double* xf64 = reinterpret_cast<double*>(smem + a.lay.pf);  // gathered FP64 iterate (same region as pf)
	double* r64 = reinterpret_cast<double*>(smem + a.lay.r64);
	double* dslots = reinterpret_cast<double*>(smem + a.lay.red);
	float* fslots = reinterpret_cast<float*>(dslots + 2 * kCcMaxCluster);
	__shared__ double dbc[4];
	__shared__ float fbc[4];
	__shared__ double dsc[32];
	cc_load_operands(a, b0, bwl, v.L, v.A1, v.A2, v.R);
	// FP64 operands straight from global memory (read-only during the launch)
	const Mv<double> m64{xf64, ldp, a.L, s.K0 * s.ra, a.A1, a.A2, a.R + (size_t)b0 * s.KL() * s.rb, s.rb,
	                     reinterpret_cast<double*>(smem + a.lay.t1), reinterpret_cast<double*>(smem + a.lay.t2),
	                     reinterpret_cast<double*>(smem + a.lay.t3)};
	double bl = 0;
	for (int e = tid; e < n; e += kCcThreads) {
		const int rho = e / bwl, b = e - rho * bwl;
		const double bv = a.b[(size_t)rho * s.rb + b0 + b];
		bl = fma(bv, bv, bl);
	}
	const double bb = cc_total(block_sum(bl, dsc), dslots, dbc, me, P);
	int iters = 0, refs = 0;
	double rel = 0, rr_prev = 0, nr_prev = 0;
	bool reached = false;
	for (int ref = 0; ref <= a.max_refine; ++ref) {
		// r64 = b - M x (FP64), x gathered from global memory (L1 bypassed: other CTAs wrote it)
		for (int e = tid; e < M1 * s.rb; e += kCcThreads) {
			const int rho = e / s.rb, c = e - rho * s.rb;
			xf64[(size_t)rho * ldp + c] = __ldcg(a.x + e);
		}
		__syncthreads();
		cc_matvec(s, bwl, m64, r64);
		double l = 0;
		for (int e = tid; e < n; e += kCcThreads) {
			const int rho = e / bwl, b = e - rho * bwl;
			const double rv = a.b[(size_t)rho * s.rb + b0 + b] - r64[e];
			r64[e] = rv;
			l = fma(rv, rv, l);
		}
		const double rr = cc_total(block_sum(l, dsc), dslots + kCcMaxCluster, dbc, me, P);
		if (ref > 0 && !(rr < rr_prev)) {
			// the FP32 correction did not help (FP32 CG past its precision on this system):
			// take it back and leave the rest to the FP64 polish
			for (int e = tid; e < n; e += kCcThreads) {
				const int rho = e / bwl, b = e - rho * bwl;
				double* xp = a.x + (size_t)rho * s.rb + b0 + b;
				*xp = fma(-nr_prev, double(v.x[e]), *xp);
			}
			rel = bb > 0 ? sqrt(rr_prev / bb) : 0.0;
			break;
		}
		rel = bb > 0 ? sqrt(rr / bb) : 0.0;
		if (rr <= a.tol * a.tol * bb) {
			reached = true;
			break;
		}
		if (ref == a.max_refine) break;
		const double nr = sqrt(rr), inr = 1.0 / nr;
		rr_prev = rr;
		nr_prev = nr;
		for (int e = tid; e < n; e += kCcThreads) v.b[e] = float(r64[e] * inr);
		__syncthreads();  // the FP32 CG below overwrites the region that held the FP64 iterate
		double irel = 0;
		// the correction solve need not reduce its residual below half of what the target
		// still asks for (fewer FP32 iterations on the last correction)
		const double itol = fmin(0.5, fmax(double(a.inner_tol), 0.5 * a.tol * sqrt(bb) / nr));
		iters += cc_cg<float>(s, me, P, b0, bwl, v.mv(s), v.pf, v.x, v.r, v.p, v.q, v.b, true, itol, a.max_iter,
		                      fslots, fbc, a.status, irel);
		for (int e = tid; e < n; e += kCcThreads) {
			const int rho = e / bwl, b = e - rho * bwl;
			double* xp = a.x + (size_t)rho * s.rb + b0 + b;
			*xp = fma(nr, double(v.x[e]), *xp);
		}
		++refs;
		cl.sync();  // every CTA's new slice of x is in global memory before the next residual
	}
	if (me == 0 && tid == 0) {
		a.out_i[0] += iters;
		a.out_i[1] += refs;
		a.out_d[0] = rel;
		const int failed = (reached || bb == 0.0) ? 0 : 1;
		if (a.flag) *a.flag = failed;
		if (failed && a.sticky) *a.sticky = 1;
	}
	cl.sync();
}

// Launch geometry and the shared-memory plan; false when the system does not
// fit one cluster (the caller then uses the grid-wide solver).
static bool cc_plan(const LocalShape& ls, bool mixed, CcArgs& a) {
	CcShape s;
	s.two = ls.sites == 2 ? 1 : 0;
	s.ra = ls.ra;
	s.n1 = ls.n1;
	s.n2 = ls.sites == 2 ? ls.n2 : 1;
	s.rb = ls.rb;
	s.K0 = ls.K0;
	s.K1 = ls.K1;
	s.K2 = ls.sites == 2 ? ls.K2 : 1;
	int P = std::min(kCcMaxCluster, s.rb);
	s.bw = (s.rb + P - 1) / P;
	P = (s.rb + s.bw - 1) / s.bw;
	const CcLayout l = cc_layout(s, mixed);
	if (l.total > kCcSmemMax) return false;
	a.s = s;
	a.lay = l;
	a.P = P;
	return true;
}

template <class K>
static bool cc_launch(K kernel, const CcArgs& a, cudaStream_t st) {
	// function attributes and occupancy are per device: the caches are keyed by it
	static std::mutex mu;
	static std::map<std::tuple<int, const void*, int, size_t>, bool> ok_cache;
	static std::map<std::pair<int, const void*>, size_t> smem_set;
	int dev = 0;
	XTT_CUDA(cudaGetDevice(&dev));
	const auto key = std::make_tuple(dev, (const void*)kernel, a.P, a.lay.total);
	std::lock_guard<std::mutex> g(mu);
	size_t& cur = smem_set[std::make_pair(dev, (const void*)kernel)];
	if (cur < a.lay.total) {
		if (cur == 0) XTT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
		XTT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(a.lay.total)));
		cur = a.lay.total;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(a.P);
	cfg.blockDim = dim3(kCcThreads);
	cfg.dynamicSmemBytes = a.lay.total;
	cfg.stream = st;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = a.P;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	auto it = ok_cache.find(key);
	if (it == ok_cache.end()) {
		int clusters = 0;
		const bool ok = cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) == cudaSuccess && clusters > 0;
		cudaGetLastError();
		it = ok_cache.emplace(key, ok).first;
	}
	if (!it->second) return false;
	XTT_CUDA(cudaLaunchKernelEx(&cfg, kernel, a));
	return true;
}

bool cluster_local_solve(Context& c, const LocalShape& ls, const double* L, const double* A1, const double* A2,
                         const double* R, const double* b, double* x, double tol, int max_iter, int precision,
                         int* flag, const int* gate) {
	const bool mixed = precision != XTT_PRECISION_FP64;
	CcArgs a;
	if (!cc_plan(ls, mixed, a)) return false;
	a.L = L;
	a.A1 = A1;
	a.A2 = ls.sites == 2 ? A2 : nullptr;
	a.R = R;
	a.b = b;
	a.x = x;
	a.tol = tol;
	a.max_iter = max_iter;
	a.max_refine = 12;
	a.inner_tol = 1e-6f;
	a.status = c.d_status;
	a.out_i = c.d_ints + 8;
	a.out_d = c.d_dbl + 8;
	a.flag = flag;
	a.sticky = flag ? c.d_ints + 11 : nullptr;
	a.gate = gate;
	bool launched;
	{
		ProfScope ps(c, mixed ? "cg_mixed" : "cg_fp64");
		launched = mixed ? cc_launch(k_cg_cluster_mixed, a, c.stream) : cc_launch(k_cg_cluster_f64, a, c.stream);
	}
	if (launched) c.count_launch();
	return launched;
}

}  // namespace xtt
