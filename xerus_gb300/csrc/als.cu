// ALS / DMRG sweep engine for SPD operators (src/xerus/algorithms/als.cpp).
//
// The reference assembles the local operator densely and factors it with
// LAPACK (lapack_solver, als.cpp:43-71: O((r n r)^3) per step). Here the local
// operator is never formed: it is applied as a chain of strided GEMMs on the
// resident environment stacks, inside one persistent cooperative kernel that
// runs the whole conjugate-gradient solve (bounded grid barriers between the
// stages, deterministic fixed-order reductions). The mixed form runs the CG
// in FP32 on FP32 copies of the environments and corrects it against FP64
// residuals (iterative refinement) in the same launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include <cooperative_groups.h>

#include "als.cuh"
#include "df.cuh"
#include "tc_tiles.cuh"

namespace xtt {

// ------------------------------------------------------------ GEMM plans

void local_matvec(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                  const double* R, const double* x, double* y) {
	double* t1 = c.scratch<double>(S_ALS_FIRST + 20, matvec_tmp_elems(s, 0));
	double* t2 = c.scratch<double>(S_ALS_FIRST + 21, matvec_tmp_elems(s, 1));
	double* t3 = c.scratch<double>(S_ALS_FIRST + 22, matvec_tmp_elems(s, 2));
	MatvecPlan<double> p = make_matvec_plan<double>(s, L, A1, A2, R, t1, t2, t3);
	p.g[0].B = x;
	p.g[p.ns - 1].C = y;
	for (int i = 0; i < p.ns; ++i) gemm(c, p.g[i]);
}

// ------------------------------------------------------------ persistent CG
//
// One launch runs a whole local solve. The CG body is written against a
// "group" of CTAs that provides its rank/size, a barrier and a sum over the
// group: GridGroup is a cooperative launch over many SMs with a bounded
// software barrier (large local systems), ClusterGroup is one thread-block
// cluster of up to 16 CTAs with the hardware cluster barrier and sums through
// distributed shared memory (local systems up to kClusterMaxN unknowns, where
// the software grid barrier dominated the iteration time).

constexpr long long kClusterMaxN = 65536;
constexpr int kCgClusterMax = 16;

struct GridGroup {
	static constexpr bool kCluster = false;
	GridBarrier bar;
	double* partial;  // 2 * gridDim doubles
	int turn = 0;
	__device__ int rank() const { return blockIdx.x; }
	__device__ int size() const { return gridDim.x; }
	__device__ bool sync() { return grid_sync(bar); }
	// sum over the group of one value per CTA (thread 0's), identical in every CTA
	__device__ double total(double mine, bool& ok) {
		__shared__ double sc[32];
		double* slot = partial + (turn ^= 1) * gridDim.x;
		if (threadIdx.x == 0) slot[blockIdx.x] = mine;
		ok = grid_sync(bar);
		double t = 0;
		for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += slot[i];
		return block_sum(t, sc);
	}
	__device__ void record(int code) { record_status(bar.status, code); }
};

struct ClusterGroup {
	static constexpr bool kCluster = true;
	int* status;
	int turn = 0;
	__device__ int rank() const { return int(cooperative_groups::this_cluster().block_rank()); }
	__device__ int size() const { return int(cooperative_groups::this_cluster().num_blocks()); }
	__device__ bool sync() {
		cooperative_groups::this_cluster().sync();
		return true;
	}
	// two alternating slots: a slot is rewritten only after the barrier that follows its reads
	__device__ double total(double mine, bool& ok) {
		namespace cg = cooperative_groups;
		__shared__ double slot[2];
		const int t = (turn ^= 1);
		if (threadIdx.x == 0) slot[t] = mine;
		cg::cluster_group cl = cg::this_cluster();
		cl.sync();
		double s = 0;
		for (int p = 0; p < (int)cl.num_blocks(); ++p) s += cl.map_shared_rank(slot, p)[t];
		ok = true;
		return s;
	}
	__device__ void record(int code) { record_status(status, code); }
};

template <class T>
struct CgParams {
	MatvecPlan<T> plan;
	T *x, *r, *p, *q;
	const T* b;
	long long n;
	int max_iter;
	double tol;
	int zero_guess;
	const int* gate = nullptr;  // run only if *gate != 0 (FP64 polish after a mixed solve)
};

struct CgOut {
	int iterations, refinements;
	double rel_residual;
};

// Tile engines of the persistent solvers: CUDA-core tiles (FP64 / FP32) or the
// tensor-core engine (tc::TcEngine, FP32 stages).
template <class T>
struct CoreTiles {
	GemmSmem<T>* sm;
	template <class Grp>
	__device__ T tiles(const Gemm<T>& g, Grp& grp) { return gemm_tiles(g, grp.rank(), grp.size(), *sm); }
};

// Double-float tiles (df.cuh) for the refinement's residual updates r -= ||r|| M d and
// the mixed sweeps' environment pushes: FP64 operands split on load into FP32 pairs in
// shared memory, ~13 FP32 instructions per product, where GB300's FP64 pipe retires one
// DFMA in the time of ~64 FFMAs. Sums of 384 products come out within ~1e-15 of
// sum |a b| (mean; FP64: ~2e-16).
struct DfSmem {
	float2 As[32][33];  // [k][m]: (hi, lo)
	float2 Bs[32][33];  // [k][n]
};

// Output tile `tile` of g (32 x 32, 2 x 2 outputs per thread, as gemm_tile; no epilogue
// sum) over the K range [kb, ke) (ke <= 0: all of K).
__device__ void gemm_tile_df(const Gemm<double>& g, long long tile, DfSmem& sm, int kb = 0, int ke = 0) {
	const int tid = threadIdx.x;
	const long long tn = g.tiles_n(), tm = g.tiles_m();
	const long long b = tile / (tm * tn);
	const long long rem = tile - b * tm * tn;
	const int m0 = int(rem / tn) * 32, n0 = int(rem % tn) * 32;
	const double* A = g.A + b * g.sAb;
	const double* B = g.B + b * g.sBb;
	const int tx = tid & 15, ty = tid >> 4;
	float s[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, c[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
	const bool a_k_fast = (g.sAk == 1);
	const bool b_n_fast = (g.sBn == 1) || (g.sBk != 1);
	// the next K slab is fetched into registers while the current one is multiplied
	const int kend = ke > 0 ? min(ke, g.K) : g.K;  // the loads zero-fill beyond it
	GemmSlab<double> r;
	gemm_slab_load(g, A, B, m0, n0, kb, kend, a_k_fast, b_n_fast, r);
	for (int k0 = kb; k0 < kend; k0 += 32) {
#pragma unroll
		for (int t = 0; t < 4; ++t) {
			int am, ak, bn, bk;
			gemm_slab_index<double>(tid + t * kGemmThreads, a_k_fast, b_n_fast, am, ak, bn, bk);
			sm.As[ak][am] = df_split(r.a[t]);
			sm.Bs[bk][bn] = df_split(r.b[t]);
		}
		__syncthreads();
		if (k0 + 32 < kend) gemm_slab_load(g, A, B, m0, n0, k0 + 32, kend, a_k_fast, b_n_fast, r);
		const int kmax = min(32, kend - k0);
#pragma unroll 4
		for (int kk = 0; kk < kmax; ++kk) {
			const float2 a0 = sm.As[kk][ty], a1 = sm.As[kk][ty + 16];
			const float2 b0 = sm.Bs[kk][tx], b1 = sm.Bs[kk][tx + 16];
			df_fma(a0, b0, s[0][0], c[0][0]);
			df_fma(a0, b1, s[0][1], c[0][1]);
			df_fma(a1, b0, s[1][0], c[1][0]);
			df_fma(a1, b1, s[1][1], c[1][1]);
			if ((kk & 3) == 3) {  // every fourth product (accuracy ~1e-15 of sum |a b| at K = 384)
				df_renorm(s[0][0], c[0][0]);
				df_renorm(s[0][1], c[0][1]);
				df_renorm(s[1][0], c[1][0]);
				df_renorm(s[1][1], c[1][1]);
			}
		}
		__syncthreads();
	}
	double* C = g.C + b * g.sCb;
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 2; ++j) {
			const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
			if (gm < g.M && gn < g.N) {
				const long long o = g.offC(gm, gn);
				const double acc = double(s[i][j]) + double(c[i][j]);
				C[o] = (g.beta == 0.0) ? g.alpha * acc : g.alpha * acc + g.beta * C[o];
			}
		}
}

struct DfTiles {
	DfSmem* sm;
	template <class Grp>
	__device__ double tiles(const Gemm<double>& g, Grp& grp) {
		const long long nt = g.tiles();
		for (long long t = grp.rank(); t < nt; t += grp.size()) gemm_tile_df(g, t, *sm);
		return 0.0;
	}
};

__global__ void __launch_bounds__(kGemmThreads) k_gemm_df(Gemm<double> g) {
	__shared__ DfSmem sm;
	const long long nt = g.tiles();
	for (long long t = blockIdx.x; t < nt; t += gridDim.x) gemm_tile_df(g, t, sm);
}

// Split K: CTA (tile, part) writes the part's products (alpha 1, beta 0) into C's layout at
// part_base + part * span; k_gemm_df_sum adds the parts in order and applies alpha, beta.
__global__ void __launch_bounds__(kGemmThreads) k_gemm_df_split(Gemm<double> g, int kchunk, double* part_base,
                                                                 long long span) {
	__shared__ DfSmem sm;
	const long long nt = g.tiles();
	const int part = int(blockIdx.x / nt);
	Gemm<double> gp = g;
	gp.C = part_base + part * span;
	gp.alpha = 1.0;
	gp.beta = 0.0;
	gemm_tile_df(gp, blockIdx.x % nt, sm, part * kchunk, (part + 1) * kchunk);
}

__global__ void k_gemm_df_sum(Gemm<double> g, int S, const double* part_base, long long span) {
	const long long mn = (long long)g.M * g.N, total = (long long)g.batch * mn;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
	     e += (long long)gridDim.x * blockDim.x) {
		const long long b = e / mn, r = e - b * mn;
		const int m = int(r / g.N), n = int(r - (long long)m * g.N);
		const long long o = b * g.sCb + g.offC(m, n);
		double acc = 0.0;
		for (int s = 0; s < S; ++s) acc += part_base[s * span + o];
		g.C[o] = g.beta == 0.0 ? g.alpha * acc : g.alpha * acc + g.beta * g.C[o];
	}
}

void gemm_df(Context& c, const Gemm<double>& g) {
	check_gemm(g);
	const long long nt = g.tiles();
	if (nt == 0) return;
	// split K when the tiles leave SMs idle: at least two 32-deep slabs per part
	int S = 1;
	if (nt < c.num_sms && g.K >= 128) {
		S = int(std::min<long long>(8, (3 * c.num_sms / 2 + nt - 1) / nt));
		S = std::max(1, std::min(S, g.K / 64));
	}
	if (S == 1) {
		k_gemm_df<<<unsigned(std::min<long long>(nt, 4LL * c.num_sms)), kGemmThreads, 0, c.stream>>>(g);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		return;
	}
	const int kchunk = ((g.K + S - 1) / S + 31) / 32 * 32;
	S = (g.K + kchunk - 1) / kchunk;
	const long long span = g.max_off_C() + 1;
	// a buffer per stream: the sweeps' operator and rhs pushes run on the two streams at once
	double* part = c.scratch<double>(c.stream == c.aux ? S_ALS_FIRST + 13 : S_ALS_FIRST + 12, size_t(S) * size_t(span));
	k_gemm_df_split<<<unsigned(nt * S), kGemmThreads, 0, c.stream>>>(g, kchunk, part, span);
	const long long total = (long long)g.batch * g.M * g.N;
	k_gemm_df_sum<<<unsigned(std::min<long long>((total + 255) / 256, 8LL * c.num_sms)), 256, 0, c.stream>>>(g, S, part,
	                                                                                                    span);
	XTT_CUDA(cudaGetLastError());
	c.count_launch(2);
}

template <class T, class Grp, class E>
__device__ bool matvec_dev(const MatvecPlan<T>& plan, const T* in, T* out, const T* dotv, E& eng, Grp& grp,
                           T& blk_dot) {
	for (int s = 0; s < plan.ns; ++s) {
		Gemm<T> g = plan.g[s];
		if (s == 0) g.B = in;
		if (s == plan.ns - 1) {
			g.C = out;
			g.D = dotv;
		}
		const T part = eng.tiles(g, grp);
		if (s == plan.ns - 1) blk_dot = part;
		else if (!grp.sync()) return false;
	}
	return true;
}

template <class T, class Grp, class E>
__device__ CgOut cg_body(const CgParams<T>& a, E& sm, Grp& grp, double tol = -1.0) {  // tol < 0: a.tol
	__shared__ double sc[32];
	CgOut out{0, 0, 0.0};
	const long long gt = grp.rank() * (long long)blockDim.x + threadIdx.x;
	const long long gs = (long long)grp.size() * blockDim.x;
	bool ok = true;
	T dummy;
	if (!a.zero_guess) {
		if (!matvec_dev(a.plan, a.x, a.q, (const T*)nullptr, sm, grp, dummy)) return out;
		if (!grp.sync()) return out;
		for (long long i = gt; i < a.n; i += gs) {
			const T ri = a.b[i] - a.q[i];
			a.r[i] = ri;
			a.p[i] = ri;
		}
	} else {
		for (long long i = gt; i < a.n; i += gs) {
			a.x[i] = T(0);
			a.r[i] = a.b[i];
			a.p[i] = a.b[i];
		}
	}
	double rl = 0, bl = 0;
	for (long long i = gt; i < a.n; i += gs) {
		rl += double(a.r[i]) * double(a.r[i]);
		bl += double(a.b[i]) * double(a.b[i]);
	}
	rl = block_sum(rl, sc);
	bl = block_sum(bl, sc);
	double rr = grp.total(rl, ok);
	if (!ok) return out;
	const double bb = grp.total(bl, ok);
	if (!ok) return out;
	if (bb == 0.0) {
		for (long long i = gt; i < a.n; i += gs) a.x[i] = T(0);
		return out;
	}
	const double tl = tol < 0 ? a.tol : tol;
	const double tol2 = tl * tl * bb;
	int it = 0;
	CgFloor floor_check;
	while (rr > tol2 && it < a.max_iter) {
		T blk = 0;
		if (!matvec_dev(a.plan, a.p, a.q, a.p, sm, grp, blk)) return out;
		const double pAp = grp.total(double(blk), ok);
		if (!ok) return out;
		// the test and the division once per CTA (in every thread they would queue on the
		// FP64 pipe), broadcast through shared memory
		__shared__ double s_ab[2];
		__shared__ int s_good;
		if (threadIdx.x == 0) {
			s_good = pAp > 0.0 && isfinite(pAp);
			s_ab[0] = s_good ? rr / pAp : 0.0;
		}
		__syncthreads();
		if (!s_good) {
			// an FP32 correction solve just stops: the FP64 refinement around it decides
			if (sizeof(T) == 8 && cg_breakdown_is_error(rr, bb)) grp.record(DEV_BREAKDOWN);
			break;
		}
		const double alpha = s_ab[0];
		double l = 0;
		for (long long i = gt; i < a.n; i += gs) {
			a.x[i] += T(alpha) * a.p[i];
			const T ri = a.r[i] - T(alpha) * a.q[i];
			a.r[i] = ri;
			l += double(ri) * double(ri);
		}
		l = block_sum(l, sc);
		const double rrn = grp.total(l, ok);
		if (!ok) return out;
		if (threadIdx.x == 0) s_ab[1] = rrn / rr;
		__syncthreads();
		const double beta = s_ab[1];
		rr = rrn;
		for (long long i = gt; i < a.n; i += gs) a.p[i] = a.r[i] + T(beta) * a.p[i];
		if (!grp.sync()) return out;
		++it;
		if (floor_check.stalled(rr, it)) break;  // identical in every CTA
	}
	out.iterations = it;
	out.rel_residual = sqrt(rr / bb);
	return out;
}

template <class T, class Grp>
__global__ void __launch_bounds__(kGemmThreads, Grp::kCluster ? 1 : 2) k_cg(CgParams<T> a, Grp grp, int* out_i, double* out_d) {
	if (a.gate && __ldcg(a.gate) == 0) return;  // uniform: every block reads the same flag
	__shared__ GemmSmem<T> sm;
	CoreTiles<T> eng{&sm};
	const CgOut o = cg_body(a, eng, grp);
	if (grp.rank() == 0 && threadIdx.x == 0) {  // counters accumulate over a sweep
		out_i[0] += o.iterations;
		out_d[0] = o.rel_residual;
	}
	if (Grp::kCluster) grp.sync();
}

// Mixed precision (iterative refinement): the residual r = b - M x is formed in FP64,
// each correction M d = r / ||r|| is solved by CG in FP32, x += ||r|| d, and r is then
// updated as r -= ||r|| M d with M d in double-float arithmetic (DfTiles). An update's
// error is ~2^-47 ||M|| ||d|| ||r||: relative to the residual it corrects, not to ||b||,
// so the updated residual follows the true one to FP64 level at a fraction of an FP64
// operator application. An update whose residual norm would take the summed norms of
// the double-float updates past the drift budget (their sum times 2^-47, times an
// allowance of 1024 for ||M|| ||d||, at most half the target) runs with FP64 products
// instead, so from a poor start the first, large correction is exact and the small
// ones that follow are cheap; the updated residual then stays within half the target
// of the true one, and meeting the target with it is meeting it.
struct MixedParams {
	MatvecPlan<double> p64;
	CgParams<float> inner;   // inner.b = rhs32, inner.x = d
	double *x, *q64, *r64;   // q64: operator products; r64: the residual
	const double* b;
	long long n;
	double tol;
	int max_refine;
	int* flag;               // 1 when the FP64 target was not reached, else 0
	int* sticky;             // set once FP32 corrections stalled; later solves skip them
	int* status = nullptr;   // device status (the tensor-core engine's bounded waits)
	float* part = nullptr;   // the tensor-core engine's split-K partials
	int* arrivals = nullptr; // and its per-tile arrival counters (zeroed before the launch)
};

// r = b - M x in FP64 (r64), returns ||r||^2 (identical in every CTA); false on a barrier timeout.
template <class Grp, class E64>
__device__ bool fp64_residual(const MixedParams& a, E64& e64, Grp& grp, double* sc, double& rr) {
	const long long gt = grp.rank() * (long long)blockDim.x + threadIdx.x;
	const long long gs = (long long)grp.size() * blockDim.x;
	double dummy;
	if (!matvec_dev(a.p64, a.x, a.q64, (const double*)nullptr, e64, grp, dummy) || !grp.sync()) return false;
	double l = 0;
	for (long long i = gt; i < a.n; i += gs) {
		const double ri = a.b[i] - a.q64[i];
		a.r64[i] = ri;
		l += ri * ri;
	}
	bool ok = true;
	rr = grp.total(block_sum(l, sc), ok);
	return ok;
}

template <class Grp, class E64, class E32, class EDF>
__device__ void mixed_body(const MixedParams& a, E64& e64, E32& e32, EDF& edf, Grp& grp, int* out_i, double* out_d) {
	__shared__ double sc[32];
	const long long gt = grp.rank() * (long long)blockDim.x + threadIdx.x;
	const long long gs = (long long)grp.size() * blockDim.x;
	bool ok = true;
	double bl = 0;
	for (long long i = gt; i < a.n; i += gs) bl += a.b[i] * a.b[i];
	const double bb = grp.total(block_sum(bl, sc), ok);
	const double tol2 = a.tol * a.tol * bb;
	// drift allowance of the double-float updates (see above): 2^-47 * 1024 = 2^-37
	const double drift_limit = 0.5 * a.tol * sqrt(bb) * 137438953472.0;  // 2^37
	int iters = 0, refs = 0;
	double rel = 0, rr = 0, drift = 0;  // drift: sum of the residual norms updated in double-float
	bool reached = false;
	ok = ok && fp64_residual(a, e64, grp, sc, rr);
	for (int ref = 0; ok; ++ref) {
		rel = bb > 0 ? sqrt(rr / bb) : 0.0;
		if (rr <= tol2) {  // drift <= drift_limit (the update rule below keeps it there)
			reached = true;
			break;
		}
		if (ref >= a.max_refine) break;
		const double nr = sqrt(rr), inr = 1.0 / nr;
		for (long long i = gt; i < a.n; i += gs) const_cast<float*>(a.inner.b)[i] = float(a.r64[i] * inr);
		if (!grp.sync()) break;
		// the correction solve need not reduce its residual below half of what the target
		// still asks for (fewer FP32 iterations on the last correction)
		const double itol = fmin(0.5, fmax(a.inner.tol, 0.5 * a.tol * sqrt(bb) / nr));
		const CgOut o = cg_body(a.inner, e32, grp, itol);
		iters += o.iterations;
		for (long long i = gt; i < a.n; i += gs) {
			const double di = double(a.inner.x[i]);
			a.x[i] += nr * di;
			a.q64[i] = di;
		}
		++refs;
		// a large correction (||r|| still a sizeable part of ||b||, as from a poor start) is
		// applied with FP64 products, which add no drift; the others in double-float
		const bool df = !(drift + nr > drift_limit);
		double dummy;
		if (!grp.sync()) break;
		if (!(df ? matvec_dev(a.p64, a.q64, a.q64, (const double*)nullptr, edf, grp, dummy)
		         : matvec_dev(a.p64, a.q64, a.q64, (const double*)nullptr, e64, grp, dummy)) ||
		    !grp.sync())
			break;
		double l = 0;
		for (long long i = gt; i < a.n; i += gs) {
			const double ri = a.r64[i] - nr * a.q64[i];
			a.r64[i] = ri;
			l += ri * ri;
		}
		const double rn = grp.total(block_sum(l, sc), ok);
		if (!ok) break;
		if (!(rn < rr)) {
			// the FP32 correction did not help: take it back, the FP64 polish finishes
			for (long long i = gt; i < a.n; i += gs) a.x[i] -= nr * double(a.inner.x[i]);
			break;
		}
		if (df) drift += nr;
		rr = rn;
	}
	if (grp.rank() == 0 && threadIdx.x == 0) {
		out_i[0] += iters;
		out_i[1] += refs;
		out_d[0] = rel;
		const int failed = (reached || bb == 0.0) ? 0 : 1;
		if (a.flag) *a.flag = failed;
		if (failed && a.sticky) *a.sticky = 1;
	}
}

template <class Grp>
__global__ void __launch_bounds__(kGemmThreads, Grp::kCluster ? 1 : 2) k_cg_mixed(MixedParams a, Grp grp, int* out_i, double* out_d) {
	if (a.sticky && __ldcg(a.sticky) != 0) {  // an earlier solve of this sweep showed FP32 does not help
		if (blockIdx.x == 0 && threadIdx.x == 0) *a.flag = 1;
		return;
	}
	__shared__ union U {
		GemmSmem<double> d;
		GemmSmem<float> f;
		DfSmem df;
		__device__ U() {}
	} sm;
	CoreTiles<double> e64{&sm.d};
	CoreTiles<float> e32{&sm.f};
	DfTiles edf{&sm.df};
	mixed_body(a, e64, e32, edf, grp, out_i, out_d);
	if (Grp::kCluster) grp.sync();
}

// The same solve with the FP32 CG's operator stages on the tensor cores: every CTA
// holds kPN tensor-memory columns and two mbarriers for the whole launch.
__global__ void __launch_bounds__(kGemmThreads) k_cg_mixed_tc(MixedParams a, GridGroup grp, int* out_i, double* out_d) {
	if (a.sticky && __ldcg(a.sticky) != 0) {
		if (blockIdx.x == 0 && threadIdx.x == 0) *a.flag = 1;
		return;
	}
	extern __shared__ __align__(1024) unsigned char tc_dyn[];
	__shared__ union U {
		GemmSmem<double> d;
		DfSmem df;
		__device__ U() {}
	} sm64;
	__shared__ __align__(8) uint64_t bars[2];
	__shared__ uint32_t s_tmem;
	__shared__ int s_ok, s_last, s_fix;
	__shared__ float fred[32];
	const int warp = threadIdx.x >> 5;
	if (warp == 0) tc::tmem_alloc(&s_tmem, tc::kPN);
	if (threadIdx.x == 0) {
		tc::mbar_init(&bars[0], 1);
		tc::mbar_init(&bars[1], 1);
		tc::mbar_fence_init();
		s_ok = 1;
		s_last = -1;
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	tc::TcEngine e32{tc_dyn, bars, &s_ok, &s_last, fred, s_tmem, 0u, a.status, a.part, a.arrivals, &s_fix};
	CoreTiles<double> e64{&sm64.d};
	DfTiles edf{&sm64.df};
	mixed_body(a, e64, e32, edf, grp, out_i, out_d);
	__syncthreads();
	// a wait gave up: wait (bounded) once more for the MMAs in flight before freeing TMEM
	if (threadIdx.x == 0 && !s_ok && s_last >= 0) tc::mbar_wait(&bars[s_last & 1], uint32_t((s_last >> 1) & 1));
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::fence_after_sync();
		tc::tmem_dealloc(s_tmem, tc::kPN);
	}
}

template <class F>
static int coop_grid(F kernel, Context& c, long long work_blocks) {
	int occ = 0;
	XTT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kGemmThreads, 0));
	const long long maxg = (long long)std::max(1, occ) * c.num_sms;
	return int(std::max<long long>(1, std::min<long long>(maxg, work_blocks)));
}

// Launches `kernel` as one cluster of P CTAs if the device can schedule it; returns false otherwise.
template <class K, class... Args>
static bool launch_cluster(K kernel, int P, cudaStream_t s, Args... args) {
	func_attr_once(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(P);
	cfg.blockDim = dim3(kGemmThreads);
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = P;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	int clusters = 0;
	if (cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) != cudaSuccess || clusters < 1) {
		cudaGetLastError();
		return false;
	}
	XTT_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
	return true;
}

__global__ void k_to_float(float* out, const double* in, size_t n) {
	for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
		out[i] = float(in[i]);
}

static void to_float(Context& c, float* out, const double* in, size_t n) {
	if (!n) return;
	k_to_float<<<unsigned(std::min<size_t>((n + 255) / 256, 2048)), 256, 0, c.stream>>>(out, in, n);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}


// ------------------------------------------------------------ tensor-core mixed solve
//
// The precision form of the local solve for large local systems (a rank of 64 or
// more at the site): iterative refinement against the FP64 residual r = b - M x,
// whose correction M d = r / ||r|| is solved by CG in FP32 vectors with every
// operator stage on the tensor cores (split TF32, FP32-level products, FP32
// accumulation). The host drives the iterations; the CG scalars stay on the
// device (sums over fixed per-block partials, so every run adds in the same order),
// and the host reads the residual every kTcCheck iterations.

constexpr int kTcVecThreads = 256;
constexpr int kTcCheck = 4;

__device__ double sum_partials(const double* part, int G, double* red) {
	double s = 0;
	for (int i = threadIdx.x; i < G; i += blockDim.x) s += part[i];
	return block_sum(s, red);
}

// part[block] = sum a . b
__global__ void __launch_bounds__(kTcVecThreads) k_tdot(const float* a, const float* b, long long n, double* part) {
	__shared__ double red[32];
	double s = 0;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		s = fma(double(a[i]), double(b[i]), s);
	s = block_sum(s, red);
	if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// alpha = rr / (p . q); x += alpha p; r -= alpha q; part2[block] = sum r_new . r_new
__global__ void __launch_bounds__(kTcVecThreads) k_tcg_step1(float* x, float* r, const float* p, const float* q,
                                                              long long n, const double* part_pq, int G,
                                                              const double* rr, double* part2, int* status) {
	__shared__ double red[32];
	__shared__ float s_alpha;
	const double pq = sum_partials(part_pq, G, red);
	if (threadIdx.x == 0) {
		const bool good = pq > 0.0 && isfinite(pq);
		// p = 0 after an exact solve is not a breakdown; p^T M p <= 0 otherwise is
		if (!good && blockIdx.x == 0 && !(pq == 0.0 && *rr == 0.0)) record_status(status, DEV_BREAKDOWN);
		s_alpha = good ? float(*rr / pq) : 0.f;
	}
	__syncthreads();
	const float alpha = s_alpha;
	double s = 0;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
		x[i] = fmaf(alpha, p[i], x[i]);
		const float rv = fmaf(-alpha, q[i], r[i]);
		r[i] = rv;
		s = fma(double(rv), double(rv), s);
	}
	s = block_sum(s, red);
	if (threadIdx.x == 0) part2[blockIdx.x] = s;
}

// rr_new = sum part2; p = r + (rr_new / rr) p; rr_out = rr_new (another slot than rr)
__global__ void __launch_bounds__(kTcVecThreads) k_tcg_step2(float* p, const float* r, long long n,
                                                              const double* part2, int G, const double* rr,
                                                              double* rr_out) {
	__shared__ double red[32];
	const double rn = sum_partials(part2, G, red);
	const float beta = *rr > 0.0 ? float(rn / *rr) : 0.f;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		p[i] = fmaf(beta, p[i], r[i]);
	if (blockIdx.x == 0 && threadIdx.x == 0) *rr_out = rn;
}

// r = b - q (FP64), part[block] = sum r . r
__global__ void __launch_bounds__(kTcVecThreads) k_tres(double* r, const double* b, const double* q, long long n,
                                                         double* part) {
	__shared__ double red[32];
	double s = 0;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
		const double v = b[i] - q[i];
		r[i] = v;
		s = fma(v, v, s);
	}
	s = block_sum(s, red);
	if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kTcVecThreads) k_tsum_partials(const double* part, int G, double* out) {
	__shared__ double red[32];
	const double s = sum_partials(part, G, red);
	if (threadIdx.x == 0) *out = s;
}

// CG start: r = p = f32(r64 * inr), x = 0
__global__ void k_tcg_init(float* x, float* r, float* p, const double* r64, double inr, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
		const float v = float(r64[i] * inr);
		r[i] = v;
		p[i] = v;
		x[i] = 0.f;
	}
}

// x64 += f * d
__global__ void k_tcg_apply(double* x, const float* d, double f, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		x[i] = fma(f, double(d[i]), x[i]);
}

__global__ void k_add_counters(int* out, int iters, int refs) {
	out[0] += iters;
	out[1] += refs;
}

// Whether the tensor-core precision form takes this local system.
static bool use_tc_solve(const Context& c, const LocalShape& s, int precision) {
	if (precision != XTT_PRECISION_MIXED) return false;
	if (c.cg_path == XTT_CG_PATH_TENSOR) return true;
	// measured: the cluster-resident CG wins at 4096 unknowns (rank-32 one-site ALS), the
	// tensor-core form from 16384 (two-site DMRG at rank 16) and at ranks >= 64
	return c.cg_path == XTT_CG_PATH_AUTO && (std::max(s.ra, s.rb) >= 64 || s.dim() >= 16384);
}

// Returns false when the refinement stalled (x then holds its best iterate and
// the caller finishes in FP64).
static bool tc_mixed_solve(Context& c, const LocalShape& s, const MatvecPlan<double>& p64, const MatvecPlan<float>& p32,
                           const double* b, double* x, double tol, int max_iter, double bb) {
	const long long n = s.dim();
	const int G = int(std::max<long long>(1, std::min<long long>(2ll * c.num_sms, (n + kTcVecThreads - 1) / kTcVecThreads)));
	double* part = c.scratch<double>(S_ALS_FIRST + 26, 2 * size_t(G));
	double* part2 = part + G;
	double* r64 = c.scratch<double>(S_ALS_FIRST + 23, size_t(n));
	double* q64 = c.scratch<double>(S_ALS_FIRST + 25, size_t(n));
	float* v = c.scratch<float>(S_ALS_FIRST + 31, 4 * size_t(n));
	float *dx = v, *r = v + n, *p = v + 2 * n, *q = v + 3 * n;
	double* sc = c.d_dbl + 40;  // [0], [1]: ping-pong rr; [2]: FP64 residual norm^2
	MatvecPlan<double> m64 = p64;
	m64.g[0].B = x;
	m64.g[m64.ns - 1].C = q64;
	MatvecPlan<float> m32 = p32;
	m32.g[0].B = p;
	m32.g[m32.ns - 1].C = q;
	const unsigned VB = unsigned(G);
	auto read_dbl = [&](double* d) {
		XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 40, d, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		return c.h_dbl[40];
	};
	const double inner_tol = 1e-5;
	int iters = 0, refs = 0;
	double rr_prev = 0, nr_prev = 0;
	bool ok = false;
	for (int ref = 0; ref <= 12; ++ref) {
		{
			ProfScope ps(c, "cg_fp64");
			for (int i = 0; i < m64.ns; ++i) gemm(c, m64.g[i]);
			k_tres<<<VB, kTcVecThreads, 0, c.stream>>>(r64, b, q64, n, part);
			k_tsum_partials<<<1, kTcVecThreads, 0, c.stream>>>(part, G, sc + 2);
			c.count_launch(2);
			XTT_CUDA(cudaGetLastError());
		}
		const double rr = read_dbl(sc + 2);
		if (ref > 0 && !(rr < rr_prev)) {
			// the correction did not help: take it back, leave the rest to FP64 CG
			k_tcg_apply<<<VB, kTcVecThreads, 0, c.stream>>>(x, dx, -nr_prev, n);
			c.count_launch();
			break;
		}
		if (rr <= tol * tol * bb) {
			ok = true;
			break;
		}
		if (ref == 12) break;
		const double nr = std::sqrt(rr);
		rr_prev = rr;
		nr_prev = nr;
		ProfScope ps(c, "cg_tc");
		k_tcg_init<<<VB, kTcVecThreads, 0, c.stream>>>(dx, r, p, r64, 1.0 / nr, n);
		k_tdot<<<VB, kTcVecThreads, 0, c.stream>>>(r, r, n, part2);
		k_tsum_partials<<<1, kTcVecThreads, 0, c.stream>>>(part2, G, sc + 0);
		c.count_launch(3);
		int it = 0;
		while (it < max_iter) {
			for (int j = 0; j < kTcCheck && it < max_iter; ++j, ++it) {
				for (int i = 0; i < m32.ns; ++i) gemm_tc(c, m32.g[i], 3);
				double* rr_in = sc + (it & 1);
				double* rr_out = sc + ((it + 1) & 1);
				k_tdot<<<VB, kTcVecThreads, 0, c.stream>>>(p, q, n, part);
				k_tcg_step1<<<VB, kTcVecThreads, 0, c.stream>>>(dx, r, p, q, n, part, G, rr_in, part2, c.d_status);
				k_tcg_step2<<<VB, kTcVecThreads, 0, c.stream>>>(p, r, n, part2, G, rr_in, rr_out);
				c.count_launch(3);
				XTT_CUDA(cudaGetLastError());
			}
			const double rin = read_dbl(sc + (it & 1));  // the normalised start has |r| = 1
			if (!(rin > inner_tol * inner_tol)) break;
		}
		iters += it;
		k_tcg_apply<<<VB, kTcVecThreads, 0, c.stream>>>(x, dx, nr, n);
		c.count_launch();
		++refs;
	}
	k_add_counters<<<1, 1, 0, c.stream>>>(c.d_ints + 8, iters, refs);
	c.count_launch();
	XTT_CUDA(cudaGetLastError());
	return ok;
}

CgResult local_solve(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                     const double* R, const double* b, double* x, double tol, int max_iter, int precision) {
	const long long n = s.dim();
	double* t1 = c.scratch<double>(S_ALS_FIRST + 20, matvec_tmp_elems(s, 0));
	double* t2 = c.scratch<double>(S_ALS_FIRST + 21, matvec_tmp_elems(s, 1));
	double* t3 = c.scratch<double>(S_ALS_FIRST + 22, matvec_tmp_elems(s, 2));
	MatvecPlan<double> p64 = make_matvec_plan<double>(s, L, A1, A2, R, t1, t2, t3);
	{
		MatvecPlan<double> chk = p64;  // validate with the vectors the kernel substitutes
		chk.g[0].B = b;
		chk.g[chk.ns - 1].C = x;
		for (int i = 0; i < chk.ns; ++i) check_gemm(chk.g[i]);
	}
	CgResult res;  // counters are read lazily by the driver (ctx d_ints[8..9], d_dbl[8])
	long long work = (n + kGemmThreads - 1) / kGemmThreads;
	for (int i = 0; i < p64.ns; ++i) work = std::max(work, p64.g[i].tiles());
	const bool use_cluster = n <= kClusterMaxN && c.cg_path != XTT_CG_PATH_GRID;
	const int P = int(std::max<long long>(2, std::min<long long>(kCgClusterMax, work)));
	int* oi = c.d_ints + 8;
	double* od = c.d_dbl + 8;
	int* flag = c.d_ints + 10;  // mixed solve: 1 when its FP64 target was not reached
	ClusterGroup cgrp{c.d_status, 0};
	// FP64 CG from the current x; with `gate`, only when *gate != 0 (checked on the device)
	auto fp64_solve = [&](const int* gate) {
		if (c.cg_path != XTT_CG_PATH_GRID &&
		    cluster_local_solve(c, s, L, A1, A2, R, b, x, tol, max_iter, XTT_PRECISION_FP64, nullptr, gate))
			return;
		CgParams<double> a;
		a.plan = p64;
		a.x = x;
		a.r = c.scratch<double>(S_ALS_FIRST + 23, n);
		a.p = c.scratch<double>(S_ALS_FIRST + 24, n);
		a.q = c.scratch<double>(S_ALS_FIRST + 25, n);
		a.b = b;
		a.n = n;
		a.max_iter = max_iter;
		a.tol = tol;
		a.zero_guess = 0;
		a.gate = gate;
		ProfScope ps(c, "cg_fp64");
		if (!(use_cluster && launch_cluster(k_cg<double, ClusterGroup>, P, c.stream, a, cgrp, oi, od))) {
			const int G = coop_grid(k_cg<double, GridGroup>, c, work);
			GridGroup g{GridBarrier{c.d_barrier, c.d_barrier + 1, c.d_status}, c.scratch<double>(S_ALS_FIRST + 26, 2 * size_t(G)), 0};
			void* args[] = {&a, &g, &oi, &od};
			XTT_CUDA(cudaLaunchCooperativeKernel((void*)k_cg<double, GridGroup>, dim3(G), dim3(kGemmThreads), args, 0, c.stream));
		}
		c.count_launch();
	};
	if (precision == XTT_PRECISION_FP64) {
		fp64_solve(nullptr);
		return res;
	}
	if (use_tc_solve(c, s, precision)) {
		// FP32 copies of the environments and operator cores, the FP32 operator on the tensor cores
		const size_t nL = size_t(s.ra) * s.K0 * s.ra, nA1 = size_t(s.K0) * s.n1 * s.n1 * s.K1;
		const size_t nA2 = s.sites == 2 ? size_t(s.K1) * s.n2 * s.n2 * s.K2 : 0;
		const size_t nR = size_t(s.rb) * (s.sites == 2 ? s.K2 : s.K1) * s.rb;
		float* f = c.scratch<float>(S_ALS_FIRST + 27, nL + nA1 + nA2 + nR + 4);
		to_float(c, f, L, nL);
		to_float(c, f + nL, A1, nA1);
		if (nA2) to_float(c, f + nL + nA1, A2, nA2);
		to_float(c, f + nL + nA1 + nA2, R, nR);
		float* u1 = c.scratch<float>(S_ALS_FIRST + 28, matvec_tmp_elems(s, 0));
		float* u2 = c.scratch<float>(S_ALS_FIRST + 29, matvec_tmp_elems(s, 1));
		float* u3 = c.scratch<float>(S_ALS_FIRST + 30, matvec_tmp_elems(s, 2));
		const MatvecPlan<float> p32 =
		    make_matvec_plan<float>(s, f, f + nL, nA2 ? f + nL + nA1 : nullptr, f + nL + nA1 + nA2, u1, u2, u3);
		bool persistent = true;  // the engine tabulates K offsets for at most 512 per stage, < 2^31 outputs
		for (int i = 0; i < p32.ns; ++i)
			persistent = persistent && p32.g[i].K <= tc::kPMaxChunks * tc::kTileK && tc::stage_fits(p32.g[i]);
		if (persistent) {
			// one cooperative launch: FP64 refinement, FP32 CG with tensor-core operator stages
			MixedParams m;
			m.p64 = p64;
			m.inner.plan = p32;
			float* v = c.scratch<float>(S_ALS_FIRST + 31, 5 * size_t(n));
			m.inner.x = v;
			m.inner.r = v + n;
			m.inner.p = v + 2 * n;
			m.inner.q = v + 3 * n;
			m.inner.b = v + 4 * n;
			m.inner.n = n;
			m.inner.max_iter = max_iter;
			m.inner.tol = 1e-5;  // split-TF32 products: FP32-level
			m.inner.zero_guess = 1;
			m.x = x;
			m.q64 = c.scratch<double>(S_ALS_FIRST + 25, n);
			m.r64 = c.scratch<double>(S_ALS_FIRST + 23, n);
			m.b = b;
			m.n = n;
			m.tol = tol;
			m.max_refine = 12;
			m.flag = flag;
			m.sticky = c.d_ints + 11;
			m.status = c.d_status;
			const int smem = tc::kPSmem + 1024;
			func_attr_once(k_cg_mixed_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
			int occ = 0;
			XTT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cg_mixed_tc, kGemmThreads, smem));
			const int G = std::max(1, occ) * c.num_sms;
			long long part_elems = 1;
			int split_tiles = 1;
			for (int i = 0; i < p32.ns; ++i) {
				part_elems = std::max(part_elems, tc::split_k_partials(p32.g[i], G));
				split_tiles = std::max(split_tiles, tc::split_k_tiles(p32.g[i], G));
			}
			m.part = c.scratch<float>(S_ALS_FIRST + 9, size_t(part_elems));
			m.arrivals = c.scratch<int>(S_ALS_FIRST + 10, size_t(split_tiles));
			XTT_CUDA(cudaMemsetAsync(m.arrivals, 0, sizeof(int) * size_t(split_tiles), c.stream));
			GridGroup g{GridBarrier{c.d_barrier, c.d_barrier + 1, c.d_status}, c.scratch<double>(S_ALS_FIRST + 26, 2 * size_t(G)), 0};
			void* args[] = {&m, &g, &oi, &od};
			{
				ProfScope ps(c, "cg_tc");
				XTT_CUDA(cudaLaunchCooperativeKernel((void*)k_cg_mixed_tc, dim3(G), dim3(kGemmThreads), args, smem, c.stream));
			}
			c.count_launch();
			fp64_solve(flag);  // FP64 polish, a no-op unless the mixed solve fell short
			return res;
		}
		dot_async(c, b, b, size_t(n), 12);
		XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 12, c.d_dbl + 12, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		const double bb = c.h_dbl[12];
		if (bb == 0.0 || !tc_mixed_solve(c, s, p64, p32, b, x, tol, max_iter, bb)) fp64_solve(nullptr);
		return res;
	}
	if (c.cg_path != XTT_CG_PATH_GRID && c.cg_path != XTT_CG_PATH_TENSOR &&
	    cluster_local_solve(c, s, L, A1, A2, R, b, x, tol, max_iter, precision, flag, nullptr)) {
		fp64_solve(flag);  // FP64 polish, a no-op unless the mixed solve fell short
		return res;
	}
	{
		// FP32 copies of the environments and operator cores
		const size_t nL = size_t(s.ra) * s.K0 * s.ra, nA1 = size_t(s.K0) * s.n1 * s.n1 * s.K1;
		const size_t nA2 = s.sites == 2 ? size_t(s.K1) * s.n2 * s.n2 * s.K2 : 0;
		const size_t nR = size_t(s.rb) * (s.sites == 2 ? s.K2 : s.K1) * s.rb;
		float* f = c.scratch<float>(S_ALS_FIRST + 27, nL + nA1 + nA2 + nR + 4);
		to_float(c, f, L, nL);
		to_float(c, f + nL, A1, nA1);
		if (nA2) to_float(c, f + nL + nA1, A2, nA2);
		to_float(c, f + nL + nA1 + nA2, R, nR);
		float* u1 = c.scratch<float>(S_ALS_FIRST + 28, matvec_tmp_elems(s, 0));
		float* u2 = c.scratch<float>(S_ALS_FIRST + 29, matvec_tmp_elems(s, 1));
		float* u3 = c.scratch<float>(S_ALS_FIRST + 30, matvec_tmp_elems(s, 2));
		MixedParams m;
		m.p64 = p64;
		m.inner.plan = make_matvec_plan<float>(s, f, f + nL, nA2 ? f + nL + nA1 : nullptr, f + nL + nA1 + nA2, u1, u2, u3);
		{
			MatvecPlan<float> chk = m.inner.plan;
			chk.g[0].B = u1;  // any non-null vector of length n: lengths come from lens()
			chk.g[chk.ns - 1].C = u1;
			for (int i = 0; i < chk.ns; ++i) check_gemm(chk.g[i]);
		}
		float* v = c.scratch<float>(S_ALS_FIRST + 31, 5 * size_t(n));
		m.inner.x = v;
		m.inner.r = v + n;
		m.inner.p = v + 2 * n;
		m.inner.q = v + 3 * n;
		m.inner.b = v + 4 * n;
		m.inner.n = n;
		m.inner.max_iter = max_iter;
		m.inner.tol = 1e-6;
		m.inner.zero_guess = 1;
		m.x = x;
		m.q64 = c.scratch<double>(S_ALS_FIRST + 25, n);
		m.r64 = c.scratch<double>(S_ALS_FIRST + 23, n);
		m.b = b;
		m.n = n;
		m.tol = tol;
		m.max_refine = 12;
		m.flag = flag;
		m.sticky = c.d_ints + 11;
		{
			ProfScope ps(c, "cg_mixed");
			if (!(use_cluster && launch_cluster(k_cg_mixed<ClusterGroup>, P, c.stream, m, cgrp, oi, od))) {
				const int G = coop_grid(k_cg_mixed<GridGroup>, c, work);
				GridGroup g{GridBarrier{c.d_barrier, c.d_barrier + 1, c.d_status}, c.scratch<double>(S_ALS_FIRST + 26, 2 * size_t(G)), 0};
				void* args[] = {&m, &g, &oi, &od};
				XTT_CUDA(cudaLaunchCooperativeKernel((void*)k_cg_mixed<GridGroup>, dim3(G), dim3(kGemmThreads), args, 0, c.stream));
			}
			c.count_launch();
		}
		fp64_solve(flag);  // FP64 polish, a no-op unless the mixed solve fell short
	}
	return res;
}

// ------------------------------------------------------------ environment pushes

static void run_plan(Context& c, const GemmChain& p) {
	for (int i = 0; i < p.ns; ++i) gemm(c, p.g[i]);
}

static void push_left_op(Context& c, const double* L, const double* x, const double* A, double* out, long long r,
                         long long K, long long n, long long r1, long long K1) {
	double* s1 = c.scratch<double>(S_ALS_FIRST + 16, size_t(K * r * n * r1));
	double* s2 = c.scratch<double>(S_ALS_FIRST + 17, size_t(r * r1 * n * K1));
	run_plan(c, plan_push_left_op(L, x, A, out, s1, s2, r, K, n, r1, K1));
}

static void push_right_op(Context& c, const double* R, const double* x, const double* A, double* out, long long r,
                          long long K, long long n, long long r1, long long K1) {
	double* s1 = c.scratch<double>(S_ALS_FIRST + 16, size_t(r * n * r1 * K1));
	double* s2 = c.scratch<double>(S_ALS_FIRST + 17, size_t(r * K * n * r1));
	run_plan(c, plan_push_right_op(R, x, A, out, s1, s2, r, K, n, r1, K1));
}

static void push_left_rhs(Context& c, const double* Lb, const double* bc, const double* x, double* out, long long s,
                          long long r, long long n, long long s1, long long r1) {
	double* t = c.scratch<double>(S_ALS_FIRST + 18, size_t(r * n * s1));
	run_plan(c, plan_push_left_rhs(Lb, bc, x, out, t, s, r, n, s1, r1));
}

static void push_right_rhs(Context& c, const double* Rb, const double* bc, const double* x, double* out, long long s,
                           long long r, long long n, long long s1, long long r1) {
	double* t = c.scratch<double>(S_ALS_FIRST + 18, size_t(r * n * s1));
	run_plan(c, plan_push_right_rhs(Rb, bc, x, out, t, s, r, n, s1, r1));
}

// b_loc(a, i.., b) = sum Lb(s0,a) b_k(s0,i,s1) [b_k+1(s1,i2,s2)] Rb(s_last,b)   (als.cpp:404-423)
static void local_rhs(Context& c, int sites, const double* Lb, const double* b1, const double* b2, const double* Rb,
                      double* out, long long ra, long long rb, long long s0, long long s1, long long s2, long long n1,
                      long long n2) {
	double* t1 = c.scratch<double>(S_ALS_FIRST + 18, size_t(ra * n1 * s1));
	Gemm<double> w1;
	w1.M = int(ra); w1.N = int(n1 * s1); w1.K = int(s0);
	w1.A = Lb; w1.sAm = 1; w1.sAk = ra;
	w1.B = b1; w1.sBk = n1 * s1; w1.sBn = 1;
	w1.C = t1; w1.sCm = n1 * s1; w1.sCn = 1;
	w1.lens(s0 * ra, s0 * n1 * s1, ra * n1 * s1);
	gemm(c, w1);
	const double* last = t1;
	long long rows = ra * n1, sl = s1;
	if (sites == 2) {
		double* t2 = c.scratch<double>(S_ALS_FIRST + 19, size_t(ra * n1 * n2 * s2));
		Gemm<double> w2;
		w2.M = int(ra * n1); w2.N = int(n2 * s2); w2.K = int(s1);
		w2.A = t1; w2.sAm = s1; w2.sAk = 1;
		w2.B = b2; w2.sBk = n2 * s2; w2.sBn = 1;
		w2.C = t2; w2.sCm = n2 * s2; w2.sCn = 1;
		w2.lens(ra * n1 * s1, s1 * n2 * s2, ra * n1 * n2 * s2);
		gemm(c, w2);
		last = t2;
		rows = ra * n1 * n2;
		sl = s2;
	}
	Gemm<double> w3;
	w3.M = int(rows); w3.N = int(rb); w3.K = int(sl);
	w3.A = last; w3.sAm = sl; w3.sAk = 1;
	w3.B = Rb; w3.sBk = rb; w3.sBn = 1;
	w3.C = out; w3.sCm = rb; w3.sCn = 1;
	w3.lens(rows * sl, sl * rb, rows * rb);
	gemm(c, w3);
}

// ------------------------------------------------------------ small kernels

__global__ void k_identity_core(double* core, long long p0, long long n, long long p1, int right) {
	const long long total = p0 * n * p1;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		const long long i2 = e % p1, i1 = (e / p1) % n, i0 = e / (p1 * n);
		core[e] = right ? (i0 == i1 * p1 + i2 ? 1.0 : 0.0) : (i0 * n + i1 == i2 ? 1.0 : 0.0);
	}
}

// v += (d_dbl[s0] / d_dbl[s1]) g     (ASD step, alpha = <g,g>/<g,Mg>)
__global__ void k_asd_step(double* v, const double* g, long long n, const double* dd, int s0, int s1) {
	const double alpha = dd[s0] / dd[s1];
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		v[i] += alpha * g[i];
}

__global__ void k_sub(double* out, const double* a, const double* b, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		out[i] = a[i] - b[i];
}

// v += (||g|| / ||M g||) g: the non-symmetric ASD step (als.cpp:86-89), squared norms in dd
__global__ void k_asd_step_normal(double* v, const double* g, long long n, const double* dd, int s0, int s1) {
	const double alpha = sqrt(dd[s0]) / sqrt(dd[s1]);
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		v[i] += alpha * g[i];
}

enum AlsMode { kSpd = 0, kNormal = 1, kFree = 2 };

// e = 0.5 <v, M v> - <v, b_loc> (M v = v without an operator). SPD: |e| (als.cpp:265-278);
// non-symmetric: sqrt(<Ax, Ax> - 2 <b, Ax> + ||b||^2) / ||b|| = sqrt(2 e + ||b||^2) / ||b||
// (als.cpp:282-296), clamped at 0 where rounding makes the radicand negative; free: e (als.cpp:306-318).
__global__ void k_energy(double* out, const double* dd, int sxq, int sxb, int mode, double nb) {
	const double e = 0.5 * dd[sxq] - dd[sxb];
	out[0] = mode == kSpd ? fabs(e) : mode == kNormal ? sqrt(fmax(0.0, 2.0 * e + nb * nb)) / nb : e;
}

// One core of A^T A as a TT operator of rank K^2 (the product the non-symmetric local operator
// contracts, als.cpp:392-399): B((p q), i, j, (p' q')) = sum_m A(p, m, i, p') A(q, m, j, q').
__global__ void k_normal_op_core(double* B, const double* A, int K, int L, int n) {
	const long long total = (long long)K * K * n * n * L * L;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		long long t = e;
		const int q2 = int(t % L); t /= L;
		const int p2 = int(t % L); t /= L;
		const int j = int(t % n); t /= n;
		const int i = int(t % n); t /= n;
		const int q = int(t % K);
		const int p = int(t / K);
		double acc = 0;
		for (int m = 0; m < n; ++m)
			acc = fma(A[((size_t(p) * n + m) * n + i) * L + p2], A[((size_t(q) * n + m) * n + j) * L + q2], acc);
		B[e] = acc;
	}
}

// One core of A^T b as a TT of rank s K (the non-symmetric local right-hand side, als.cpp:414-420):
// C((s p), j, (s' p')) = sum_i b(s, i, s') A(p, i, j, p').
__global__ void k_normal_rhs_core(double* C, const double* b, const double* A, int Q0, int Q1, int K, int L, int n) {
	const long long total = (long long)Q0 * K * n * Q1 * L;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		long long t = e;
		const int p2 = int(t % L); t /= L;
		const int s2 = int(t % Q1); t /= Q1;
		const int j = int(t % n); t /= n;
		const int p = int(t % K);
		const int s0 = int(t / K);
		double acc = 0;
		for (int i = 0; i < n; ++i)
			acc = fma(b[(size_t(s0) * n + i) * Q1 + s2], A[((size_t(p) * n + i) * n + j) * L + p2], acc);
		C[e] = acc;
	}
}

static unsigned blocks_for(long long n) { return unsigned(std::max<long long>(1, std::min<long long>((n + 255) / 256, 2048))); }

// ------------------------------------------------------------ the sweep

namespace {

struct Stacks {
	std::vector<double*> Lop, Rop, Lb, Rb;
};

// A and b are what the sweep contracts: the SPD operator and b; A^T A and A^T b for a
// non-symmetric operator; without an operator, a rank-1 placeholder whose cores are never read.
struct AlsState {
	Context& c;
	const Tensor& A;
	Tensor& x;
	const Tensor& b;
	const AlsOptions& o;
	int d, S, mode;
	double nb;  // ||b|| of the caller's b
	Stacks st;
	double *v, *bloc, *q, *grad, *q2;
	AlsState(Context& cc, const Tensor& AA, Tensor& xx, const Tensor& bb, const AlsOptions& oo, int md, double norm_b)
	    : c(cc), A(AA), x(xx), b(bb), o(oo), d(xx.d), S(oo.sites), mode(md), nb(norm_b) {}

	LocalShape shape(int cur) const {
		LocalShape s;
		s.sites = S;
		s.ra = int(x.ranks[cur]);
		s.rb = int(x.ranks[cur + S]);
		s.n1 = int(x.dims[cur]);
		s.n2 = S == 2 ? int(x.dims[cur + 1]) : 1;
		s.K0 = int(A.ranks[cur]);
		s.K1 = int(A.ranks[cur + 1]);
		s.K2 = S == 2 ? int(A.ranks[cur + 2]) : 1;
		return s;
	}
	// the operator and rhs pushes are independent (separate scratch): rhs on the aux stream;
	// with `df` (the mixed form) their large GEMMs run in double-float tiles
	bool df = false;
	void push_left(int k) {
		DfGemmScope dfs(c, df);
		c.fork();
		{
			OnAux aux(c);
			push_left_rhs(c, st.Lb[k], b.core[k], x.core[k], st.Lb[k + 1], b.ranks[k], x.ranks[k], x.dims[k],
			              b.ranks[k + 1], x.ranks[k + 1]);
		}
		if (mode != kFree)
			push_left_op(c, st.Lop[k], x.core[k], A.core[k], st.Lop[k + 1], x.ranks[k], A.ranks[k], x.dims[k],
			             x.ranks[k + 1], A.ranks[k + 1]);
		c.join();
	}
	// right environment of bond `slot` from bond slot+1 and core kc
	void push_right(int slot, int kc) {
		XTT_REQUIRE(kc == slot || (x.ranks[kc + 1] == x.ranks[slot + 1] && A.ranks[kc + 1] == A.ranks[slot + 1] &&
		                           b.ranks[kc + 1] == b.ranks[slot + 1] && x.ranks[kc] == x.ranks[slot] &&
		                           A.ranks[kc] == A.ranks[slot] && b.ranks[kc] == b.ranks[slot] &&
		                           x.dims[kc] == x.dims[slot]),
		            "index dimensions do not coincide (the two-site decreasing sweep contracts core k into the right "
		            "environment of bond k+2, which needs equal neighbouring ranks)");
		DfGemmScope dfs(c, df);
		c.fork();
		{
			OnAux aux(c);
			push_right_rhs(c, st.Rb[slot + 1], b.core[kc], x.core[kc], st.Rb[slot], b.ranks[kc], x.ranks[kc],
			               x.dims[kc], b.ranks[kc + 1], x.ranks[kc + 1]);
		}
		if (mode != kFree)
			push_right_op(c, st.Rop[slot + 1], x.core[kc], A.core[kc], st.Rop[slot], x.ranks[kc], A.ranks[kc],
			              x.dims[kc], x.ranks[kc + 1], A.ranks[kc + 1]);
		c.join();
	}
	// v <- current local block (core cur, or core cur * core cur+1)
	void gather_block(int cur) {
		const LocalShape s = shape(cur);
		if (S == 1) {
			copy_d2d(c, v, x.core[cur], size_t(s.dim()));
		} else {
			const long long ra = x.ranks[cur], m = x.ranks[cur + 1], n1 = x.dims[cur], n2 = x.dims[cur + 1],
			                rb = x.ranks[cur + 2];
			Gemm<double> g;
			g.M = int(ra * n1); g.N = int(n2 * rb); g.K = int(m);
			g.A = x.core[cur]; g.sAm = m; g.sAk = 1;
			g.B = x.core[cur + 1]; g.sBk = n2 * rb; g.sBn = 1;
			g.C = v; g.sCm = n2 * rb; g.sCn = 1;
			g.lens(ra * n1 * m, m * n2 * rb, ra * n1 * n2 * rb);
			gemm(c, g);
		}
	}
	void rhs(int cur) {
		const LocalShape s = shape(cur);
		local_rhs(c, S, st.Lb[cur], b.core[cur], S == 2 ? b.core[cur + 1] : nullptr, st.Rb[cur + S], bloc, s.ra, s.rb,
		          b.ranks[cur], b.ranks[cur + 1], S == 2 ? b.ranks[cur + 2] : 1, s.n1, s.n2);
	}
	const double* A2(int cur) const { return S == 2 ? A.core[cur + 1] : nullptr; }
	// energy_f from the stacks with v, b_loc current (als.cpp:255-320, see k_energy)
	double energy(int cur) {
		const LocalShape s = shape(cur);
		if (mode == kFree) {
			dot_async(c, v, v, size_t(s.dim()), 4);
		} else {
			local_matvec(c, s, st.Lop[cur], A.core[cur], A2(cur), st.Rop[cur + S], v, q);
			dot_async(c, v, q, size_t(s.dim()), 4);
		}
		dot_async(c, v, bloc, size_t(s.dim()), 5);
		k_energy<<<1, 1, 0, c.stream>>>(c.d_dbl + 6, c.d_dbl, 4, 5, mode, nb);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 6, c.d_dbl + 6, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		return c.h_dbl[6];
	}
};

}  // namespace

// The sweep's operator and right-hand side for a non-symmetric A: A^T A and A^T b core by core.
static void normal_equations(Context& c, const Tensor& A, const Tensor& b, std::unique_ptr<Tensor>& B,
                             std::unique_ptr<Tensor>& C) {
	const int d = A.d;
	std::vector<int64_t> rB(d + 1), rC(d + 1);
	for (int k = 0; k <= d; ++k) {
		rB[k] = A.ranks[k] * A.ranks[k];
		rC[k] = b.ranks[k] * A.ranks[k];
	}
	B.reset(new Tensor(&c, true, d, A.dims.data(), rB.data()));
	C.reset(new Tensor(&c, false, d, A.dims.data(), rC.data()));
	for (int k = 0; k < d; ++k) {
		const int K = int(A.ranks[k]), L = int(A.ranks[k + 1]), n = int(A.dims[k]);
		k_normal_op_core<<<blocks_for((long long)B->core_size(k)), 256, 0, c.stream>>>(B->core[k], A.core[k], K, L, n);
		k_normal_rhs_core<<<blocks_for((long long)C->core_size(k)), 256, 0, c.stream>>>(
		    C->core[k], b.core[k], A.core[k], int(b.ranks[k]), int(b.ranks[k + 1]), K, L, n);
		c.count_launch(2);
	}
	XTT_CUDA(cudaGetLastError());
}

AlsReport als(const Tensor* Ap, Tensor& x, const Tensor& b, const AlsOptions& o) {
	// ALSVariant::solve, src/xerus/algorithms/als.cpp:483-553
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op && !b.op && (!Ap || Ap->op), "ALS needs a TT operator, a TT tensor x and a TT tensor b");
	XTT_REQUIRE(x.d > 0 && x.dims == b.dims && (!Ap || (Ap->dims == x.dims && Ap->d == x.d)),
	            "dimensions of A, x and b must match");
	XTT_REQUIRE(o.sites == 1 || o.sites == 2, "sites must be 1 or 2");
	XTT_REQUIRE(!(o.local_solver == 1 && o.sites != 1), "ASD only defined for single site alternation");
	XTT_REQUIRE(Ap || o.sites == 1, "approximation dmrg not implemented yet");  // als.cpp:539
	XTT_REQUIRE(o.sites <= x.d, "more sites than components");
	const int d = x.d, S = o.sites;
	const int mode = !Ap ? kFree : o.assume_spd ? kSpd : kNormal;
	// the operator and right-hand side the sweep contracts
	std::unique_ptr<Tensor> Bn, Cn;
	if (mode == kNormal) normal_equations(c, *Ap, b, Bn, Cn);
	if (mode == kFree) {
		const std::vector<int64_t> ones(d + 1, 1);
		Bn.reset(new Tensor(&c, true, d, x.dims.data(), ones.data()));
	}
	const Tensor& A = mode == kSpd ? *Ap : *Bn;
	const Tensor& bw = mode == kNormal ? *Cn : b;
	const double norm_b = mode == kNormal ? frob_norm(b) : 0.0;
	AlsReport rep;
	std::vector<int64_t> target(x.ranks.begin() + 1, x.ranks.end() - 1);
	const bool canon_end = x.canonicalized;
	const int64_t core_end = x.core_position;

	// prepare_x_for_als (als.cpp:105-182)
	int first = 0;
	int64_t prod = 1;
	while (first + 1 < d) {
		const int64_t nd = x.dims[first], newp = prod * nd;
		if (x.ranks[first + 1] < newp) break;
		const int64_t rk = x.ranks[first + 1], n2 = x.dims[first + 1], r2 = x.ranks[first + 2];
		double* T = c.scratch<double>(S_GEMM_A, size_t(newp * n2 * r2));
		Gemm<double> g;  // core_{f+1} <- reshape(core_f, newp x rk) * core_{f+1}
		g.M = int(newp); g.N = int(n2 * r2); g.K = int(rk);
		g.A = x.core[first]; g.sAm = rk; g.sAk = 1;
		g.B = x.core[first + 1]; g.sBk = n2 * r2; g.sBn = 1;
		g.C = T; g.sCm = n2 * r2; g.sCn = 1;
		g.lens((long long)x.core_size(first), (long long)x.core_size(first + 1), newp * n2 * r2);
		gemm(c, g);
		x.reshape_core(first + 1, newp, r2);
		copy_d2d(c, x.core[first + 1], T, size_t(newp * n2 * r2));
		x.reshape_core(first, prod, newp);
		k_identity_core<<<blocks_for(prod * nd * newp), 256, 0, c.stream>>>(x.core[first], prod, nd, newp, 0);
		c.count_launch();
		++first;
		prod = newp;
	}
	int last = d;
	prod = 1;
	while (last > first + S) {
		const int64_t nd = x.dims[last - 1], newp = prod * nd;
		if (x.ranks[last - 1] < newp) break;
		const int64_t rk = x.ranks[last - 1], r0 = x.ranks[last - 2], n0 = x.dims[last - 2];
		double* T = c.scratch<double>(S_GEMM_A, size_t(r0 * n0 * newp));
		Gemm<double> g;  // core_{l-2} <- core_{l-2} * reshape(core_{l-1}, rk x newp)
		g.M = int(r0 * n0); g.N = int(newp); g.K = int(rk);
		g.A = x.core[last - 2]; g.sAm = rk; g.sAk = 1;
		g.B = x.core[last - 1]; g.sBk = newp; g.sBn = 1;
		g.C = T; g.sCm = newp; g.sCn = 1;
		g.lens((long long)x.core_size(last - 2), (long long)x.core_size(last - 1), r0 * n0 * newp);
		gemm(c, g);
		x.reshape_core(last - 2, r0, newp);
		copy_d2d(c, x.core[last - 2], T, size_t(r0 * n0 * newp));
		x.reshape_core(last - 1, newp, prod);
		k_identity_core<<<blocks_for(newp * nd * prod), 256, 0, c.stream>>>(x.core[last - 1], newp, nd, prod, 1);
		c.count_launch();
		--last;
		prod = newp;
	}
	XTT_CUDA(cudaGetLastError());
	if (canon_end && core_end < first) {
		x.canonicalized = true;
		x.core_position = first;
	} else {
		if (canon_end && core_end >= last) {
			x.canonicalized = true;
			x.core_position = last - 1;
		}
		move_core(x, first, true);
	}

	// rank bounds (ranks only change in DMRG with rank growth)
	std::vector<int64_t> rmax(x.ranks);
	if (S == 2 && o.max_rank > 0) {
		std::vector<int64_t> nn(x.dims), inner(d - 1, o.max_rank);
		auto red = reduce_to_maximal_ranks(inner, nn);
		for (int k = 1; k < d; ++k) rmax[k] = std::max(x.ranks[k], red[k - 1]);
	}
	AlsState s(c, A, x, bw, o, mode, norm_b);
	// the mixed form's environments from double-float GEMMs (~1e-15 of sum |a b|): its local
	// problems are solved to the FP64 target for these environments
	s.df = o.precision != XTT_PRECISION_FP64;
	// stacks: one buffer per family, a slot per bond 0..d
	{
		std::vector<size_t> oop(d + 2, 0), orh(d + 2, 0);
		for (int k = 0; k <= d; ++k) {
			oop[k + 1] = oop[k] + (mode == kFree ? 1 : size_t(rmax[k] * A.ranks[k] * rmax[k]));
			orh[k + 1] = orh[k] + size_t(bw.ranks[k] * rmax[k]);
		}
		double* L = c.scratch<double>(S_ALS_FIRST + 0, oop[d + 1]);
		double* R = c.scratch<double>(S_ALS_FIRST + 1, oop[d + 1]);
		double* Lb = c.scratch<double>(S_ALS_FIRST + 2, orh[d + 1]);
		double* Rb = c.scratch<double>(S_ALS_FIRST + 3, orh[d + 1]);
		for (int k = 0; k <= d; ++k) {
			s.st.Lop.push_back(L + oop[k]);
			s.st.Rop.push_back(R + oop[k]);
			s.st.Lb.push_back(Lb + orh[k]);
			s.st.Rb.push_back(Rb + orh[k]);
		}
		fill(c, s.st.Lop[0], 1.0, 1);
		fill(c, s.st.Rop[d], 1.0, 1);
		fill(c, s.st.Lb[0], 1.0, 1);
		fill(c, s.st.Rb[d], 1.0, 1);
		long long maxdim = 1;
		for (int k = 0; k + S <= d; ++k) {
			long long dim = rmax[k] * rmax[k + S] * x.dims[k] * (S == 2 ? x.dims[k + 1] : 1);
			maxdim = std::max(maxdim, dim);
		}
		s.v = c.scratch<double>(S_ALS_FIRST + 4, maxdim);
		s.bloc = c.scratch<double>(S_ALS_FIRST + 5, maxdim);
		s.q = c.scratch<double>(S_ALS_FIRST + 6, maxdim);
		s.grad = c.scratch<double>(S_ALS_FIRST + 7, maxdim);
		s.q2 = mode == kNormal && o.local_solver == 1 ? c.scratch<double>(S_ALS_FIRST + 8, maxdim) : nullptr;
	}
	for (int i = d - 1; i > first + S - 1; --i) s.push_right(i, i);
	for (int i = 0; i < first; ++i) s.push_left(i);

	int cur = first;
	bool inc = true;
	const int max_it_opt = int(std::min<int64_t>(o.local_max_iterations, int64_t(1) << 30));
	// FP64 residual of the caller's problem: ||A x - b|| / ||b||, or ||x - b|| / ||b|| without an operator
	auto true_residual = [&] { return residual(Ap, x, b); };
	// what the reference adds to PerformanceData (residual_f, als.cpp:255-320): the relative
	// residual (here also for a non-symmetric A, which the reference evaluates from its stacks as
	// sqrt(<Ax,Ax> - 2<b,Ax> + ||b||^2) / ||b||), or ||x - b|| without an operator
	double nb_free = -1;
	auto trace_value = [&] {
		const double r = true_residual();
		if (mode != kFree) return r;
		if (nb_free < 0) nb_free = frob_norm(b);
		return r * nb_free;
	};
	auto record = [&](int64_t flag) {
		if (o.record_residuals) {
			rep.residuals.push_back(trace_value());
			rep.flags.push_back(flag);
		}
	};
	// energy_f (als.cpp:255-320): with useResidualForEndCriterion the residual (a non-symmetric
	// operator always uses its stack residual)
	auto energy_f = [&](int k) {
		if (o.use_residual && mode != kNormal) return trace_value();
		s.gather_block(k);
		return s.energy(k);
	};
	s.rhs(cur);
	double energy = energy_f(cur), last_e = 1e101, last_e2 = 1e102;
	record(3);
	int half = 0;
	// CG counters of this solve, the mixed solves' flag and the sticky FP64 switch
	XTT_CUDA(cudaMemsetAsync(c.d_ints + 8, 0, 4 * sizeof(int), c.stream));
	while (true) {
		const LocalShape sh = s.shape(cur);
		const long long n = sh.dim();
		s.rhs(cur);
		s.gather_block(cur);
		if (mode == kFree) {
			// x_k = the projected b (als.cpp:540-543)
			copy_d2d(c, s.v, s.bloc, size_t(n));
		} else if (o.local_solver == 1 && mode == kNormal) {
			// ASD_solver for a non-symmetric A (als.cpp:80-89): g = M^T (b_loc - M v) with M = the
			// local A^T A (symmetric), v += (||g|| / ||M g||) g
			local_matvec(c, sh, s.st.Lop[cur], A.core[cur], nullptr, s.st.Rop[cur + 1], s.v, s.q);
			k_sub<<<blocks_for(n), 256, 0, c.stream>>>(s.grad, s.bloc, s.q, n);
			c.count_launch();
			local_matvec(c, sh, s.st.Lop[cur], A.core[cur], nullptr, s.st.Rop[cur + 1], s.grad, s.q);
			local_matvec(c, sh, s.st.Lop[cur], A.core[cur], nullptr, s.st.Rop[cur + 1], s.q, s.q2);
			dot_async(c, s.q, s.q, size_t(n), 10);
			dot_async(c, s.q2, s.q2, size_t(n), 11);
			k_asd_step_normal<<<blocks_for(n), 256, 0, c.stream>>>(s.v, s.q, n, c.d_dbl, 10, 11);
			c.count_launch();
			XTT_CUDA(cudaGetLastError());
		} else if (o.local_solver == 1) {
			// ASD_solver (als.cpp:73-92): one exact line-search gradient step
			local_matvec(c, sh, s.st.Lop[cur], A.core[cur], nullptr, s.st.Rop[cur + 1], s.v, s.q);
			k_sub<<<blocks_for(n), 256, 0, c.stream>>>(s.grad, s.bloc, s.q, n);
			c.count_launch();
			local_matvec(c, sh, s.st.Lop[cur], A.core[cur], nullptr, s.st.Rop[cur + 1], s.grad, s.q);
			dot_async(c, s.grad, s.grad, size_t(n), 10);
			dot_async(c, s.grad, s.q, size_t(n), 11);
			k_asd_step<<<blocks_for(n), 256, 0, c.stream>>>(s.v, s.grad, n, c.d_dbl, 10, 11);
			c.count_launch();
			XTT_CUDA(cudaGetLastError());
		} else {
			const int max_it = max_it_opt > 0 ? max_it_opt : int(std::min<long long>(10 * n + 100, 1 << 30));
			local_solve(c, sh, s.st.Lop[cur], A.core[cur], s.A2(cur), s.st.Rop[cur + S], s.bloc, s.v, o.local_tolerance,
			            max_it, o.precision);
		}
		if (S == 1) {
			copy_d2d(c, x.core[cur], s.v, size_t(n));
		} else {
			// split by truncated SVD (als.cpp:51-70): increasing keeps U left, decreasing keeps Vt right
			const long long ra = sh.ra, rb = sh.rb, n1 = sh.n1, n2 = sh.n2;
			const bool grow = o.max_rank > 0;
			const int mr = grow ? int(std::min<int64_t>(o.max_rank, rmax[cur + 1])) : int(target[cur]);
			const double eps = grow ? o.svd_epsilon : 8 * 2.220446049250313e-16;
			SvdArgs a;
			const int m = int(ra * n1), nn = int(n2 * rb), q = std::min(m, nn);
			double* U = c.scratch<double>(S_SVD_U, size_t(m) * q);
			double* Sv = c.scratch<double>(S_SVD_S, size_t(q));
			double* Vt = c.scratch<double>(S_SVD_VT, size_t(q) * nn);
			a.X = s.v; a.ldx = nn; a.m = m; a.n = nn; a.max_rank = mr; a.eps = eps;
			a.U = U; a.S = Sv; a.Vt = Vt; a.rank_out = c.d_ints + 1; a.status = c.d_status;
			run_svd(c, a, true);
			const int rk = c.read_int(1);
			XTT_REQUIRE(rk <= rmax[cur + 1], "DMRG split rank exceeds the stack capacity");
			// exact environment: the last split of a half-sweep leaves S on the side the next
			// half-sweep solves first, so the environment it builds from this pair stays
			// orthonormal (otherwise its local systems inherit cond(S)^2)
			const bool at_end = (inc && cur == last - S) || (!inc && cur == first);
			if (inc != (o.exact_environment && at_end)) {
				x.reshape_core(cur, ra, rk);
				copy_d2d(c, x.core[cur], U, size_t(m) * rk);
				scale_rows(c, Vt, Sv, rk, nn);
				x.reshape_core(cur + 1, rk, rb);
				copy_d2d(c, x.core[cur + 1], Vt, size_t(rk) * nn);
			} else {
				scale_cols(c, U, Sv, m, rk);
				x.reshape_core(cur, ra, rk);
				copy_d2d(c, x.core[cur], U, size_t(m) * rk);
				x.reshape_core(cur + 1, rk, rb);
				copy_d2d(c, x.core[cur + 1], Vt, size_t(rk) * nn);
			}
			x.canonicalized = false;  // set_component on a second position (ttNetwork.cpp:491)
		}
		++rep.micro_steps;
		// check_for_end_of_sweep (als.cpp:426-475)
		if ((!inc && cur == first) || (inc && cur == last - S)) {
			++half;
			last_e2 = last_e;
			last_e = energy;
			energy = energy_f(cur);
			rep.energies.push_back(energy);
			record(inc ? 1 : 3);
			bool target_met = false;
			if (o.residual_target > 0) {
				rep.residual = true_residual();
				target_met = rep.residual <= o.residual_target;
			}
			if (half == o.num_half_sweeps || std::fabs(last_e - energy) < o.convergence_epsilon ||
			    std::fabs(last_e2 - energy) < o.convergence_epsilon || last - first <= S || target_met) {
				if (canon_end && o.preserve_core_position) move_core(x, core_end, true);
				break;
			}
			inc = !inc;
		} else {
			record(0);
		}
		// move_to_next_index (als.cpp:340-380)
		if (inc) {
			if (S == 1) move_core(x, cur + 1, true);
			s.push_left(cur);
			++cur;
		} else {
			if (S == 1) move_core(x, cur - 1, true);
			const int kc = (S == 2 && o.exact_environment) ? cur + 1 : cur;
			s.push_right(cur + S - 1, kc);
			--cur;
		}
	}
	rep.energy = energy;
	rep.half_sweeps = half;
	if (o.record_residuals && !rep.residuals.empty())
		rep.residual = mode == kFree ? rep.residuals.back() / nb_free : rep.residuals.back();
	XTT_CUDA(cudaMemcpyAsync(c.h_ints + 8, c.d_ints + 8, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	rep.local_iterations = c.h_ints[8];
	rep.refinements = c.h_ints[9];
	return rep;
}

// ------------------------------------------------------------ ALS energy gradient

double als_energy_gradient(const Tensor& A, const Tensor& x, const Tensor& b, std::vector<double>& grad) {
	Context& c = *x.ctx;
	XTT_REQUIRE(A.op && !x.op && !b.op && x.dims == b.dims && A.dims == x.dims, "dimensions of A, x and b must match");
	const int d = x.d;
	AlsOptions o;
	AlsState s(c, A, const_cast<Tensor&>(x), b, o, kSpd, 0.0);
	std::vector<size_t> oop(d + 2, 0), orh(d + 2, 0);
	for (int k = 0; k <= d; ++k) {
		oop[k + 1] = oop[k] + size_t(x.ranks[k] * A.ranks[k] * x.ranks[k]);
		orh[k + 1] = orh[k] + size_t(b.ranks[k] * x.ranks[k]);
	}
	double* L = c.scratch<double>(S_ALS_FIRST + 0, oop[d + 1]);
	double* R = c.scratch<double>(S_ALS_FIRST + 1, oop[d + 1]);
	double* Lb = c.scratch<double>(S_ALS_FIRST + 2, orh[d + 1]);
	double* Rb = c.scratch<double>(S_ALS_FIRST + 3, orh[d + 1]);
	for (int k = 0; k <= d; ++k) {
		s.st.Lop.push_back(L + oop[k]);
		s.st.Rop.push_back(R + oop[k]);
		s.st.Lb.push_back(Lb + orh[k]);
		s.st.Rb.push_back(Rb + orh[k]);
	}
	fill(c, s.st.Lop[0], 1.0, 1);
	fill(c, s.st.Rop[d], 1.0, 1);
	fill(c, s.st.Lb[0], 1.0, 1);
	fill(c, s.st.Rb[d], 1.0, 1);
	for (int k = 0; k < d; ++k) s.push_left(k);
	for (int k = d - 1; k >= 0; --k) s.push_right(k, k);
	long long maxdim = 1;
	for (int k = 0; k < d; ++k) maxdim = std::max<long long>(maxdim, x.core_size(k));
	s.v = c.scratch<double>(S_ALS_FIRST + 4, maxdim);
	s.bloc = c.scratch<double>(S_ALS_FIRST + 5, maxdim);
	s.q = c.scratch<double>(S_ALS_FIRST + 6, maxdim);
	grad.assign(x.total_size(), 0.0);
	size_t off = 0;
	double J = 0;
	for (int k = 0; k < d; ++k) {
		s.rhs(k);
		const LocalShape sh = s.shape(k);
		local_matvec(c, sh, s.st.Lop[k], A.core[k], nullptr, s.st.Rop[k + 1], x.core[k], s.q);
		const long long n = sh.dim();
		if (k == 0) {
			dot_async(c, x.core[0], s.q, size_t(n), 12);
			dot_async(c, x.core[0], s.bloc, size_t(n), 13);
		}
		// grad_k = 2 (M x_k - b_loc)
		k_sub<<<blocks_for(n), 256, 0, c.stream>>>(s.v, s.q, s.bloc, n);
		c.count_launch();
		scale(c, s.v, 2.0, size_t(n));
		XTT_CUDA(cudaMemcpyAsync(grad.data() + off, s.v, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		off += size_t(n);
	}
	XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 12, c.d_dbl + 12, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	J = c.h_dbl[12] - 2.0 * c.h_dbl[13];
	return J;
}

}  // namespace xtt
