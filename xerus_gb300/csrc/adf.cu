// ADF tensor completion for single-point measurement sets
// (src/xerus/algorithms/adf.cpp, include/xerus/algorithms/adf.h) on the device.
//
// The reference keeps, per sample, a forward stack F_k (contraction of cores
// 0..k at the sample's indices) and a backward stack B_k (cores k..d-1),
// deduplicated over shared prefixes/suffixes (adf.cpp:102-191), and updates
// them with one tiny GEMV per unique entry under OpenMP. Here every stack
// level is one dense array of r x N doubles stored mode-major (entry a of
// sample s at a*N + s) so that consecutive threads touch consecutive samples;
// a level update is one pass over the samples (HBM-bound). Deduplication only
// shares identical arithmetic, so dropping it changes no value.
//
// Per core position k the sweep needs (adf.cpp:524-539):
//   res_s   = y_s - F_{k-1}[s]^T X_k[:, i_s, :] B_{k+1}[s]          (calculate_residual)
//   G[:,i,:] = sum_{s: i_s = i} res_s F_{k-1}[s] (x) B_{k+1}[s]       (calculate_projected_gradient)
//   nrm_i   = sum_{s: i_s = i} (F_{k-1}[s]^T G[:, i_s, :] B_{k+1}[s])^2 (calculate_slicewise_norm_A_projGrad)
//   X_k[:, i, :] += (||G_i||^2 / nrm_i) G_i                           (update_x)
// The gradient and slice norms are reduced deterministically: each warp (each
// thread, for the slice norms) accumulates its contiguous chunk of samples in a
// fixed order, each block sums its warps (threads) in a fixed order, and the
// per-block partials are summed in a fixed order by a second kernel.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "als.cuh"
#include "engine.cuh"

namespace xtt {

constexpr int kAdfMaxR = 8;        // fast path: ranks <= 8
constexpr int kAdfMaxSlices = 16;  // fast path: mode sizes <= 16
constexpr int kAdfPairsPerLane = 2;  // r0 * r1 <= 64

// One core position of the sweep. S is the type of the stacks and of the
// per-sample arithmetic (double; float in the FP32 form); the core is FP64.
template <class S>
struct AdfLevelT {
	const int* pos;     // indices of this mode, N ints
	const S* F;         // F_{k-1}: r0 x N (nullptr: the constant 1)
	const S* B;         // B_{k+1}: r1 x N (nullptr: the constant 1)
	const double* X;    // core (r0, n, r1)
	int r0, n, r1;
	long long N;
};
using AdfLevel = AdfLevelT<double>;

// res_s (optional write), and per-block partials of G (r0, n, r1) and of sum res^2.
// mode 0: res_s = y_s - <F, X_i B>; mode 1: res_s given in `res` (read only).
// Each warp walks its chunk of samples 32 at a time: lane s stages its sample's
// index, res_s F[s] (premultiplied) and B[s] in the warp's shared memory (one
// row per rank index, lanes contiguous: conflict-free), then the lanes own the
// (a, c) pairs and add res_j F_j[a] B_j[c] into slice i_j of the warp's gradient
// accumulator, sample by sample in order: one multiply-add per pair and sample.
// The block's warps are summed in a fixed order at the end (deterministic).
constexpr int kAdfResThreads = 128;
constexpr int kAdfResWarps = kAdfResThreads / 32;

template <class S>
struct AdfResSmem {
	// offsets (elements of S) into the dynamic shared memory
	int P, n, r0, r1;
	__host__ __device__ int xs() const { return 0; }
	__host__ __device__ int g(int w) const { return r0 * n * r1 + w * n * P; }
	__host__ __device__ int rf(int w) const { return g(kAdfResWarps) + w * (r0 + r1) * 33; }
	__host__ __device__ int bb(int w) const { return rf(w) + r0 * 33; }
	__host__ __device__ int total() const { return rf(kAdfResWarps); }
};

template <class S>
__global__ void __launch_bounds__(kAdfResThreads) k_adf_res_grad(AdfLevelT<S> L, const S* y, S* res, int mode,
                                                                  double* gpart, double* rrpart, long long chunk) {
	extern __shared__ __align__(16) unsigned char adf_raw[];
	S* sm = reinterpret_cast<S*>(adf_raw);
	__shared__ int Iw[kAdfResWarps][32];
	__shared__ double rrw[kAdfResWarps];
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	const int r0 = L.r0, n = L.n, r1 = L.r1, P = r0 * r1;
	AdfResSmem<S> lay{P, n, r0, r1};
	S* Xs = sm + lay.xs();
	S* G = sm + lay.g(wib);
	S* RF = sm + lay.rf(wib);
	S* BB = sm + lay.bb(wib);
	for (int e = threadIdx.x; e < r0 * n * r1; e += blockDim.x) Xs[e] = S(L.X[e]);
	for (int e = lane; e < n * P; e += 32) G[e] = S(0);
	__syncthreads();
	int pa[kAdfPairsPerLane], pc[kAdfPairsPerLane];
#pragma unroll
	for (int t = 0; t < kAdfPairsPerLane; ++t) {
		const int p = lane + 32 * t;
		pa[t] = p < P ? p / r1 : 0;
		pc[t] = p < P ? p - pa[t] * r1 : 0;
	}
	double rr = 0.0;
	const long long s0 = ((long long)blockIdx.x * kAdfResWarps + wib) * chunk, s1 = min(L.N, s0 + chunk);
	for (long long base = s0; base < s1; base += 32) {
		const long long s = base + lane;
		if (s < s1) {
			const int idx = L.pos[s];
			S f[kAdfMaxR], b[kAdfMaxR];
#pragma unroll
			for (int a = 0; a < kAdfMaxR; ++a) f[a] = a < r0 ? (L.F ? L.F[a * L.N + s] : S(1)) : S(0);
#pragma unroll
			for (int c = 0; c < kAdfMaxR; ++c) b[c] = c < r1 ? (L.B ? L.B[c * L.N + s] : S(1)) : S(0);
			S rs;
			if (mode == 0) {
				S v = S(0);
#pragma unroll
				for (int a = 0; a < kAdfMaxR; ++a) {
					if (a >= r0) break;
					S t = S(0);
					const S* xr = Xs + (a * n + idx) * r1;
#pragma unroll
					for (int c = 0; c < kAdfMaxR; ++c)
						if (c < r1) t = fma(xr[c], b[c], t);
					v = fma(f[a], t, v);
				}
				rs = y[s] - v;
				res[s] = rs;
			} else {
				rs = res[s];
			}
			rr += double(rs) * double(rs);
#pragma unroll
			for (int a = 0; a < kAdfMaxR; ++a)
				if (a < r0) RF[a * 33 + lane] = rs * f[a];
#pragma unroll
			for (int c = 0; c < kAdfMaxR; ++c)
				if (c < r1) BB[c * 33 + lane] = b[c];
			Iw[wib][lane] = idx;
		}
		__syncwarp();
		const int cnt = int((s1 - base) < 32 ? (s1 - base) : 32);
		for (int j = 0; j < cnt; ++j) {
			S* gi = G + Iw[wib][j] * P;
#pragma unroll
			for (int t = 0; t < kAdfPairsPerLane; ++t) {
				const int p = lane + 32 * t;
				if (p < P) gi[p] = fma(RF[pa[t] * 33 + j], BB[pc[t] * 33 + j], gi[p]);
			}
		}
		__syncwarp();
	}
	rr = warp_sum(rr);
	if (lane == 0) rrw[wib] = rr;
	__syncthreads();
	// the block's partial: its warps' accumulators in warp order, stored (r0, n, r1)
	double* gp = gpart + (long long)blockIdx.x * r0 * n * r1;
	for (int e = threadIdx.x; e < n * P; e += blockDim.x) {
		double t = 0;
		for (int q = 0; q < kAdfResWarps; ++q) t += double(sm[lay.g(q) + e]);
		const int i = e / P, p = e - i * P, a = p / r1, c = p - a * r1;
		gp[(a * n + i) * r1 + c] = t;
	}
	if (threadIdx.x == 0 && rrpart) {
		double t = 0;
		for (int q = 0; q < kAdfResWarps; ++q) t += rrw[q];
		rrpart[blockIdx.x] = t;
	}
}

// Generic (slow) path for shapes beyond the fast path: residual per sample,
// then one thread per gradient entry summing over all samples in order.
__global__ void k_adf_res_generic(AdfLevel L, const double* y, double* res) {
	for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < L.N; s += (long long)gridDim.x * blockDim.x) {
		const int idx = L.pos[s];
		double v = 0.0;
		for (int a = 0; a < L.r0; ++a) {
			double t = 0.0;
			for (int c = 0; c < L.r1; ++c) t += L.X[(a * L.n + idx) * L.r1 + c] * (L.B ? L.B[c * L.N + s] : 1.0);
			v += (L.F ? L.F[a * L.N + s] : 1.0) * t;
		}
		res[s] = y[s] - v;
	}
}

__global__ void k_adf_grad_generic(AdfLevel L, const double* res, double* G) {
	const int total = L.r0 * L.n * L.r1;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
		const int c = e % L.r1, i = (e / L.r1) % L.n, a = e / (L.r1 * L.n);
		double s = 0.0;
		for (long long q = 0; q < L.N; ++q)
			if (L.pos[q] == i) s += res[q] * (L.F ? L.F[a * L.N + q] : 1.0) * (L.B ? L.B[c * L.N + q] : 1.0);
		G[e] = s;
	}
}

// out[e] = scale * sum over `parts` partial arrays of length len: one block per
// element, threads take the partials in a fixed stride, then a fixed-order
// block reduction (deterministic).
__global__ void k_sum_parts(const double* part, long long parts, int len, double* out, double scale) {
	__shared__ double sc[32];
	for (int e = blockIdx.x; e < len; e += gridDim.x) {
		double s = 0.0;
		for (long long p = threadIdx.x; p < parts; p += blockDim.x) s += part[p * len + e];
		s = block_sum(s, sc);
		if (threadIdx.x == 0) out[e] = scale * s;
	}
}

static void sum_parts(Context& c, const double* part, long long parts, int len, double* out, double scale) {
	k_sum_parts<<<unsigned(std::min(len, 4096)), 128, 0, c.stream>>>(part, parts, len, out, scale);
	c.count_launch();
}

// slice norms: nrm_i = sum_{s: i_s = i} (F[s]^T G[:, i_s, :] B[s])^2, per-block partials
// (n values). Every thread walks its samples with a per-thread accumulator per slice in
// shared memory (its own column: conflict-free); the block sums them in thread order.
constexpr int kAdfNormThreads = 256;

template <class S>
__global__ void __launch_bounds__(kAdfNormThreads) k_adf_slicenorm(AdfLevelT<S> L, const double* G, double* npart,
                                                                    long long chunk) {
	__shared__ S Gs[kAdfMaxR * kAdfMaxSlices * kAdfMaxR];
	__shared__ S Acc[kAdfMaxSlices][kAdfNormThreads];
	const int r0 = L.r0, n = L.n, r1 = L.r1, tid = threadIdx.x;
	for (int e = tid; e < r0 * n * r1; e += blockDim.x) Gs[e] = S(G[e]);
	for (int i = 0; i < n; ++i) Acc[i][tid] = S(0);
	__syncthreads();
	const long long s0 = (long long)blockIdx.x * chunk, s1 = min(L.N, s0 + chunk);
	for (long long s = s0 + tid; s < s1; s += blockDim.x) {
		const int idx = L.pos[s];
		S f[kAdfMaxR], b[kAdfMaxR];
#pragma unroll
		for (int a = 0; a < kAdfMaxR; ++a) f[a] = a < r0 ? (L.F ? L.F[a * L.N + s] : S(1)) : S(0);
#pragma unroll
		for (int c = 0; c < kAdfMaxR; ++c) b[c] = c < r1 ? (L.B ? L.B[c * L.N + s] : S(1)) : S(0);
		S v = S(0);
#pragma unroll
		for (int a = 0; a < kAdfMaxR; ++a) {
			if (a >= r0) break;
			S t = S(0);
			const S* gr = Gs + (a * n + idx) * r1;
#pragma unroll
			for (int c = 0; c < kAdfMaxR; ++c)
				if (c < r1) t = fma(gr[c], b[c], t);
			v = fma(f[a], t, v);
		}
		Acc[idx][tid] = fma(v, v, Acc[idx][tid]);
	}
	__syncthreads();
	// per slice: the block's threads in order (one warp per slice, lanes strided, then a fixed tree)
	const int lane = tid & 31, warp = tid >> 5;
	for (int i = warp; i < n; i += kAdfNormThreads / 32) {
		double t = 0;
		for (int q = lane; q < kAdfNormThreads; q += 32) t += double(Acc[i][q]);
		t = warp_sum(t);
		if (lane == 0) npart[(long long)blockIdx.x * n + i] = t;
	}
}

__global__ void k_adf_slicenorm_generic(AdfLevel L, const double* G, double* nrm) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += gridDim.x * blockDim.x) {
		double s = 0.0;
		for (long long q = 0; q < L.N; ++q) {
			if (L.pos[q] != i) continue;
			double v = 0.0;
			for (int a = 0; a < L.r0; ++a) {
				double t = 0.0;
				for (int c = 0; c < L.r1; ++c) t += G[(a * L.n + i) * L.r1 + c] * (L.B ? L.B[c * L.N + q] : 1.0);
				v += (L.F ? L.F[a * L.N + q] : 1.0) * t;
			}
			s += v * v;
		}
		nrm[i] = s;
	}
}

// X[:, j, :] += (||G_j||^2 / nrm_j) G_j   (update_x, adf.cpp:468-478); one block
// update_x (adf.cpp:468-478): X[:, j, :] += (||G_j||^2 / nrm_j) G_j, one warp per slice j
// (the slices' reductions and divisions are independent chains: on GB300 a dependent FP64
// operation costs ~64 cycles and a division ~370, so slices in sequence would add up).
__global__ void k_adf_update(double* X, const double* G, const double* nrm, int r0, int n, int r1) {
	const int lane = threadIdx.x & 31;
	for (int j = threadIdx.x >> 5; j < n; j += blockDim.x >> 5) {
		double s = 0.0;
		for (int e = lane; e < r0 * r1; e += 32) {
			const int a = e / r1, c = e % r1;
			const double g = G[(a * n + j) * r1 + c];
			s = fma(g, g, s);
		}
		const double step = warp_sum(s) / nrm[j];
		for (int e = lane; e < r0 * r1; e += 32) {
			const int a = e / r1, c = e % r1;
			X[(a * n + j) * r1 + c] = fma(step, G[(a * n + j) * r1 + c], X[(a * n + j) * r1 + c]);
		}
	}
}

static void adf_update(Context& c, double* X, const double* G, const double* nrm, int r0, int n, int r1) {
	const int warps = std::min(32, std::max(1, n));
	k_adf_update<<<1, 32 * warps, 0, c.stream>>>(X, G, nrm, r0, n, r1);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

// F_k[b][s] = sum_a F_{k-1}[a][s] X[a, i_s, b]
template <class S>
__global__ void k_adf_forward(const int* pos, const S* Fp, const double* X, S* Fo, int r0, int n, int r1,
                              long long N) {
	extern __shared__ __align__(16) unsigned char xs_raw[];
	S* Xs = reinterpret_cast<S*>(xs_raw);
	for (int e = threadIdx.x; e < r0 * n * r1; e += blockDim.x) Xs[e] = S(X[e]);
	__syncthreads();
	for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
		const int idx = pos[s];
		for (int b = 0; b < r1; ++b) {
			S v = S(0);
			for (int a = 0; a < r0; ++a) v += (Fp ? Fp[a * N + s] : S(1)) * Xs[(a * n + idx) * r1 + b];
			Fo[b * N + s] = v;
		}
	}
}

// B_k[a][s] = sum_b X[a, i_s, b] B_{k+1}[b][s]
template <class S>
__global__ void k_adf_backward(const int* pos, const S* Bn, const double* X, S* Bo, int r0, int n, int r1,
                               long long N) {
	extern __shared__ __align__(16) unsigned char xs_raw[];
	S* Xs = reinterpret_cast<S*>(xs_raw);
	for (int e = threadIdx.x; e < r0 * n * r1; e += blockDim.x) Xs[e] = S(X[e]);
	__syncthreads();
	for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
		const int idx = pos[s];
		for (int a = 0; a < r0; ++a) {
			S v = S(0);
			for (int b = 0; b < r1; ++b) v += Xs[(a * n + idx) * r1 + b] * (Bn ? Bn[b * N + s] : S(1));
			Bo[a * N + s] = v;
		}
	}
}

__global__ void k_to_f32(float* out, const double* in, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		out[i] = float(in[i]);
}

namespace {

struct AdfData {
	Context& c;
	Tensor& x;
	int d;
	long long N;
	int* pos = nullptr;  // d x N (mode-major)
	double* y = nullptr;
	double* res = nullptr;
	std::vector<double*> F, B;  // F[k]: r_{k+1} x N ; B[k]: r_k x N
	// FP32 form: stacks, samples and residuals in single precision
	bool f32 = false;
	float *y32 = nullptr, *res32 = nullptr;
	std::vector<float*> F32, B32;
	double *gpart = nullptr, *npart = nullptr, *rrpart = nullptr, *G = nullptr, *nrm = nullptr, *rr = nullptr;
	long long chunk = 0, res_blocks = 0, norm_chunk = 0, norm_blocks = 0;
	bool fast = true;

	AdfData(Context& cc, Tensor& xx, const int64_t* positions, const double* values, long long n, bool want_f32 = false)
	    : c(cc), x(xx), d(xx.d), N(n) {
		std::vector<int> hp(size_t(d) * N);
		for (long long s = 0; s < N; ++s)
			for (int k = 0; k < d; ++k) {
				const int64_t v = positions[s * d + k];
				XTT_REQUIRE(v >= 0 && v < x.dims[k], "measurement position out of range");
				hp[size_t(k) * N + s] = int(v);
			}
		pos = c.scratch<int>(S_ADF_FIRST + 0, hp.size());
		y = c.scratch<double>(S_ADF_FIRST + 1, N);
		res = c.scratch<double>(S_ADF_FIRST + 2, N);
		XTT_CUDA(cudaMemcpyAsync(pos, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
		XTT_CUDA(cudaMemcpyAsync(y, values, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
		int64_t maxr = 1, maxn = 1;
		for (int k = 0; k <= d; ++k) maxr = std::max(maxr, x.ranks[k]);
		for (int k = 0; k < d; ++k) maxn = std::max(maxn, x.dims[k]);
		fast = maxr <= kAdfMaxR && maxn <= kAdfMaxSlices && maxr * maxr <= 32 * kAdfPairsPerLane;
		f32 = want_f32 && fast;
		size_t fo = 0, bo = 0;
		for (int k = 0; k < d; ++k) {
			fo += size_t(x.ranks[k + 1]) * N;
			bo += size_t(x.ranks[k]) * N;
		}
		if (f32) {
			y32 = c.scratch<float>(S_ADF_FIRST + 11, size_t(N));
			res32 = c.scratch<float>(S_ADF_FIRST + 12, size_t(N));
			k_to_f32<<<unsigned(std::min<long long>((N + 255) / 256, 4096)), 256, 0, c.stream>>>(y32, y, N);
			XTT_CUDA(cudaGetLastError());
			c.count_launch();
			float* Fa = c.scratch<float>(S_ADF_FIRST + 8, fo);
			float* Ba = c.scratch<float>(S_ADF_FIRST + 9, bo);
			F32.assign(d, nullptr);
			B32.assign(d, nullptr);
			fo = bo = 0;
			for (int k = 0; k < d; ++k) {
				F32[k] = Fa + fo;
				B32[k] = Ba + bo;
				fo += size_t(x.ranks[k + 1]) * N;
				bo += size_t(x.ranks[k]) * N;
			}
		} else {
			double* Fa = c.scratch<double>(S_ADF_FIRST + 8, fo);
			double* Ba = c.scratch<double>(S_ADF_FIRST + 9, bo);
			F.assign(d, nullptr);
			B.assign(d, nullptr);
			fo = bo = 0;
			for (int k = 0; k < d; ++k) {
				F[k] = Fa + fo;
				B[k] = Ba + bo;
				fo += size_t(x.ranks[k + 1]) * N;
				bo += size_t(x.ranks[k]) * N;
			}
		}
		// res_grad: warps of 64 samples, kAdfResWarps per block; slice norms: 1024 samples per block
		chunk = 64;
		res_blocks = std::max<long long>(1, (N + chunk * kAdfResWarps - 1) / (chunk * kAdfResWarps));
		norm_chunk = 1024;
		norm_blocks = std::max<long long>(1, (N + norm_chunk - 1) / norm_chunk);
		gpart = c.scratch<double>(S_ADF_FIRST + 3, size_t(res_blocks) * maxr * maxn * maxr);
		npart = c.scratch<double>(S_ADF_FIRST + 4, size_t(norm_blocks) * maxn);
		rrpart = c.scratch<double>(S_ADF_FIRST + 5, size_t(res_blocks));
		G = c.scratch<double>(S_ADF_FIRST + 6, size_t(maxr) * maxn * maxr);
		nrm = c.scratch<double>(S_ADF_FIRST + 7, size_t(maxn) + 8);
		rr = nrm + maxn;
	}
	template <class S>
	AdfLevelT<S> level(int k, const double* X, const std::vector<S*>& Fs, const std::vector<S*>& Bs) const {
		AdfLevelT<S> L;
		L.pos = pos + size_t(k) * N;
		L.F = k > 0 ? Fs[k - 1] : nullptr;
		L.B = k + 1 < d ? Bs[k + 1] : nullptr;
		L.X = X;
		L.r0 = int(x.ranks[k]);
		L.n = int(x.dims[k]);
		L.r1 = int(x.ranks[k + 1]);
		L.N = N;
		return L;
	}
	AdfLevel level(int k, const double* X) const { return level<double>(k, X, F, B); }
	template <class S>
	size_t res_smem(int k) const {
		AdfResSmem<S> l{int(x.ranks[k] * x.ranks[k + 1]), int(x.dims[k]), int(x.ranks[k]), int(x.ranks[k + 1])};
		return size_t(l.total()) * sizeof(S);
	}
	// res (mode 0) or given res (mode 1), G into Gout, and sum res^2 into rr[0]
	void res_grad(int k, int mode, const double* X, double* Gout, double gscale) {
		const int len = int(x.ranks[k] * x.dims[k] * x.ranks[k + 1]);
		if (fast) {
			const int mx = 100 * 1024;
			func_attr_once(k_adf_res_grad<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
			func_attr_once(k_adf_res_grad<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
			ProfScope ps(c, "adf_res_grad");
			if (f32)
				k_adf_res_grad<float><<<unsigned(res_blocks), kAdfResThreads, res_smem<float>(k), c.stream>>>(
				    level<float>(k, X, F32, B32), y32, res32, mode, gpart, rrpart, chunk);
			else
				k_adf_res_grad<double><<<unsigned(res_blocks), kAdfResThreads, res_smem<double>(k), c.stream>>>(
				    level(k, X), y, res, mode, gpart, rrpart, chunk);
			c.count_launch();
			sum_parts(c, gpart, res_blocks, len, Gout, gscale);
			sum_parts(c, rrpart, res_blocks, 1, rr, 1.0);
		} else {
			const AdfLevel L = level(k, X);
			if (mode == 0) k_adf_res_generic<<<std::max<long long>(1, std::min<long long>((N + 255) / 256, 4096)), 256, 0, c.stream>>>(L, y, res);
			k_adf_grad_generic<<<std::max(1, (len + 127) / 128), 128, 0, c.stream>>>(L, res, Gout);
			if (gscale != 1.0) scale(c, Gout, gscale, size_t(len));
			dot_async(c, res, res, size_t(N), 20);
			XTT_CUDA(cudaMemcpyAsync(rr, c.d_dbl + 20, sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
			c.count_launch(2);
		}
		XTT_CUDA(cudaGetLastError());
	}
	void slicenorm(int k) {
		if (fast) {
			ProfScope ps(c, "adf_slicenorm");
			if (f32)
				k_adf_slicenorm<float><<<unsigned(norm_blocks), kAdfNormThreads, 0, c.stream>>>(
				    level<float>(k, x.core[k], F32, B32), G, npart, norm_chunk);
			else
				k_adf_slicenorm<double><<<unsigned(norm_blocks), kAdfNormThreads, 0, c.stream>>>(level(k, x.core[k]), G,
				                                                                                  npart, norm_chunk);
			c.count_launch();
			sum_parts(c, npart, norm_blocks, int(x.dims[k]), nrm, 1.0);
		} else {
			k_adf_slicenorm_generic<<<1, 32, 0, c.stream>>>(level(k, x.core[k]), G, nrm);
			c.count_launch();
		}
		XTT_CUDA(cudaGetLastError());
	}
	void forward(int k) {
		const int r0 = int(x.ranks[k]), n = int(x.dims[k]), r1 = int(x.ranks[k + 1]);
		const unsigned bl = unsigned(std::max<long long>(1, std::min<long long>((N + 255) / 256, (long long)c.num_sms * 8)));
		ProfScope ps(c, "adf_stack");
		if (f32)
			k_adf_forward<float><<<bl, 256, size_t(r0) * n * r1 * sizeof(float), c.stream>>>(
			    pos + size_t(k) * N, k > 0 ? F32[k - 1] : nullptr, x.core[k], F32[k], r0, n, r1, N);
		else
			k_adf_forward<double><<<bl, 256, size_t(r0) * n * r1 * sizeof(double), c.stream>>>(
			    pos + size_t(k) * N, k > 0 ? F[k - 1] : nullptr, x.core[k], F[k], r0, n, r1, N);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	}
	void backward(int k) {
		const int r0 = int(x.ranks[k]), n = int(x.dims[k]), r1 = int(x.ranks[k + 1]);
		const unsigned bl = unsigned(std::max<long long>(1, std::min<long long>((N + 255) / 256, (long long)c.num_sms * 8)));
		ProfScope ps(c, "adf_stack");
		if (f32)
			k_adf_backward<float><<<bl, 256, size_t(r0) * n * r1 * sizeof(float), c.stream>>>(
			    pos + size_t(k) * N, k + 1 < d ? B32[k + 1] : nullptr, x.core[k], B32[k], r0, n, r1, N);
		else
			k_adf_backward<double><<<bl, 256, size_t(r0) * n * r1 * sizeof(double), c.stream>>>(
			    pos + size_t(k) * N, k + 1 < d ? B[k + 1] : nullptr, x.core[k], B[k], r0, n, r1, N);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	}
	double read_rr() {
		XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 30, rr, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		return c.h_dbl[30];
	}
};

}  // namespace

// update_x at core k followed by move_core(k + 1, keepRank) in ONE launch when the core
// fits the narrow-core factorisation (ranks <= 8, at most 128 rows): the step, the QR of the
// updated core and the absorption of R into core k + 1. False if it does not fit.
static bool update_and_move_right(Tensor& x, int k, const double* G, const double* nrm) {
	if (!(x.canonicalized && x.core_position == k)) return false;
	TransferArgs t;
	t.from = x.core[k];
	t.to = x.core[k + 1];
	t.r0 = int(x.ranks[k]); t.nf = int(x.dims[k]); t.r1 = int(x.ranks[k + 1]);
	t.rt = t.r1; t.nt = int(x.dims[k + 1]); t.r2 = int(x.ranks[k + 2]);
	t.right = 1;
	t.G = G;
	t.nrm = nrm;
	if (!transfer_narrow_fits(t)) return false;
	Context& c = *x.ctx;
	{
		ProfScope ps(c, "qr");
		launch_transfer_narrow(t, c.stream);
	}
	c.count_launch();
	x.core_position = k + 1;
	return true;
}

AdfResult adf(Tensor& x, const int64_t* positions, const double* values, long long N, int64_t max_iter,
              double target, double min_dec, int precision, const std::vector<int64_t>* max_ranks,
              const std::function<void(Tensor&)>& add_random_rank_one) {
	// ADFVariant::InternalSolver::solve (adf.cpp:566-604) with solve_with_current_ranks
	// (adf.cpp:489-542). Without max_ranks x keeps its ranks; with them (the operator()
	// overload taking maxRanks, adf.h:263-266) every run that stops early at lower ranks is
	// followed by a rank increase (adf.cpp:590-602) and another run.
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op, "ADF needs a TT tensor");
	XTT_REQUIRE(N > 0, "need at very least one measurement");
	XTT_REQUIRE(!max_ranks || int(max_ranks->size()) == x.d - 1, "maxRanks needs one entry per inner bond");
	double ny2 = 0;
	for (long long s = 0; s < N; ++s) ny2 += values[s] * values[s];
	const double norm_y = std::sqrt(ny2);
	move_core(x, 0, false);  // canonicalize_left (adf.cpp:582)
	AdfResult out;
	// members of the reference's solver: they carry over between runs at different ranks
	double residual_norm = DBL_MAX, last_residual_norm = DBL_MAX;
	int64_t it = 0;
	bool f32 = false;
	const int d = x.d;
	auto inner_ranks = [&] { return std::vector<int64_t>(x.ranks.begin() + 1, x.ranks.end() - 1); };
	auto solve_with_current_ranks = [&] {
		// the stacks are sized for the current ranks (resize_stack_tensors, adf.cpp:194-204)
		AdfData D(c, x, positions, values, N, precision != XTT_PRECISION_FP64);
		f32 = D.f32;
		double dec1 = 0, dec2 = 0, dec3 = 0;
		// From the second iteration at these ranks on, both halves of an iteration repeat
		// the same launches with the same arguments (core d-1 -> 0, backward stacks,
		// residual; then the sweep): each is recorded once as a graph and replayed. Not
		// while per-class profiling times the launches one by one.
		ReplayGraph start_graph, sweep_graph;
		const bool graphs = !c.profiling;
		auto start = [&] {
			// move_core(0): from a canonical position p the moves p -> 0 one step at a time,
			// each backward stack B_k on the aux stream as soon as core k is right-orthogonal
			// (at once for k > p), beside the next move
			if (!x.canonicalized) {
				move_core(x, 0, true);
				for (int k = d - 1; k > 0; --k) D.backward(k);
			} else {
				const int p = int(x.core_position);
				for (int k = d - 1; k > 0; --k) {
					if (k <= p) move_core(x, k - 1, true);
					c.fork();
					OnAux on(c);
					D.backward(k);
				}
				c.join();
			}
			D.res_grad(0, 0, x.core[0], D.G, 1.0);
		};
		auto sweep = [&] {
			for (int k = 0; k < d; ++k) {
				if (k > 0) D.res_grad(k, 0, x.core[k], D.G, 1.0);
				D.slicenorm(k);
				if (k + 1 < d && update_and_move_right(x, k, D.G, D.nrm)) {
					D.forward(k);
					continue;
				}
				adf_update(c, x.core[k], D.G, D.nrm, int(x.ranks[k]), int(x.dims[k]), int(x.ranks[k + 1]));
				if (k + 1 < d) {
					move_core(x, k + 1, true);
					D.forward(k);
				}
			}
		};
		int64_t local = 0;  // iterations at these ranks so far
		for (; max_iter == 0 || it < max_iter; ++it, ++local) {
			if (graphs && local >= 1 && d > 1) {
				start_graph.run(c, start);
				x.canonicalized = true;
				x.core_position = 0;
			} else {
				start();
			}
			last_residual_norm = residual_norm;
			residual_norm = std::sqrt(D.read_rr()) / norm_y;
			out.trace.push_back(residual_norm);
			out.trace_iteration.push_back(it);
			out.trace_ranks.push_back(inner_ranks());
			const double dec4 = dec3;
			dec3 = dec2;
			dec2 = dec1;
			dec1 = residual_norm / last_residual_norm;
			if (residual_norm < target || dec1 * dec2 * dec3 * dec4 > std::pow(min_dec, 4)) break;
			if (graphs && local >= 1 && d > 1) {
				sweep_graph.run(c, sweep);
				x.canonicalized = true;
				x.core_position = d - 1;
			} else {
				sweep();
			}
		}
	};
	solve_with_current_ranks();
	if (max_ranks) {
		XTT_REQUIRE(bool(add_random_rank_one), "the rank increase needs a source of random rank-one tensors");
		const std::vector<int64_t> mr = reduce_to_maximal_ranks(*max_ranks, x.dims);
		while (residual_norm > target && inner_ranks() != mr && (max_iter == 0 || it < max_iter)) {
			// x += 1e-6 ||x|| r / ||r|| for a random rank-one TT r, then round(maxRanks)
			move_core(x, 0, true);
			add_random_rank_one(x);
			round_tt(x, mr, kXerusEpsilon, nullptr);
			solve_with_current_ranks();
		}
	}
	out.residual = residual_norm;
	out.checked_residual = residual_norm;
	out.iterations = it;
	if (f32) {
		// FP64 check of the FP32 form: ||P(x) - y|| / ||y|| from FP64 entries of the FP64 cores
		std::vector<double> e(N);
		entries(x, positions, N, e.data());
		double s2 = 0;
		for (long long i = 0; i < N; ++i) s2 += (e[i] - values[i]) * (e[i] - values[i]);
		out.checked_residual = std::sqrt(s2) / norm_y;
	}
	return out;
}

// ------------------------------------------------------------ IHT

__global__ void k_iht_add(double* y, const double* x, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		y[i] += x[i];
}

static void run_gemm_chain(Context& c, const GemmChain& ch) {
	for (int i = 0; i < ch.ns; ++i) gemm(c, ch.g[i]);
}

IhtResult iht(Tensor& x, const int64_t* positions, const double* values, long long N, int64_t max_iter) {
	// IHT (src/xerus/algorithms/iht.cpp:29-155) with an iteration cap. largeX = x + sum_s w_s
	// e_{pos_s} (w_s = beta alpha (y_s - cur_s)) is never formed: its rank-(r + N) block
	// structure splits every contraction of the ALS sweep into a dense part (the
	// environments of newX against x: the operator-free ALS stacks and local projection)
	// and a per-sample part (newX's backward / forward products at the samples, the ADF
	// stacks, weighted by w_s: ADF's projected-gradient kernel with w in place of the
	// residual). Each trial: newX = x moved to core 0, right stacks, then left to right
	// core k = dense + per-sample projection, move on (keepRank), push the left stacks.
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op, "IHT needs a TT tensor");
	XTT_REQUIRE(N > 0, "need at very least one measurement");
	XTT_REQUIRE(max_iter >= 0, "max_iter must be >= 0");
	const int d = x.d;
	Tensor nx(&c, false, d, x.dims.data(), x.ranks.data());
	nx.copy_from(x);
	AdfData D(c, nx, positions, values, N, false);
	// dense environments (x rank first, newX rank second, as the operator-free ALS stacks)
	std::vector<size_t> off(d + 2, 0);
	size_t maxcore = 1, maxr2 = 1;
	for (int k = 0; k <= d; ++k) {
		off[k + 1] = off[k] + size_t(x.ranks[k]) * x.ranks[k];
		maxr2 = std::max(maxr2, size_t(x.ranks[k]) * x.ranks[k]);
	}
	for (int k = 0; k < d; ++k) maxcore = std::max(maxcore, x.core_size(k));
	double* Rb = c.scratch<double>(S_ADF_FIRST + 20, off[d + 1]);
	double* Lb = c.scratch<double>(S_ADF_FIRST + 21, 2 * maxr2);
	double* tmp = c.scratch<double>(S_ADF_FIRST + 22, maxcore);
	double* G = c.scratch<double>(S_ADF_FIRST + 23, maxcore);
	std::vector<double> cur(N), w(N), e(N);
	auto resid = [&](const Tensor& t) {
		entries(t, positions, N, e.data());
		double s2 = 0;
		for (long long i = 0; i < N; ++i) s2 += (values[i] - e[i]) * (values[i] - e[i]);
		return std::sqrt(s2);
	};
	IhtResult out;
	double alpha = 1.0, residual = 1.0;
	for (int64_t it = 0; it < max_iter; ++it) {
		entries(x, positions, N, cur.data());
		double best = residual * 2, new_alpha = alpha;
		for (double beta = 1 / 1.1; beta < 1.1 * 1.5; beta *= 1.1) {
			for (long long i = 0; i < N; ++i) w[i] = beta * alpha * (values[i] - cur[i]);
			XTT_CUDA(cudaMemcpyAsync(D.res, w.data(), N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
			nx.copy_from(x);
			move_core(nx, 0, true);
			fill(c, Rb + off[d], 1.0, 1);
			for (int k = d - 1; k > 0; --k) {
				run_gemm_chain(c, plan_push_right_rhs(Rb + off[k + 1], x.core[k], nx.core[k], Rb + off[k], tmp,
				                                      x.ranks[k], nx.ranks[k], x.dims[k], x.ranks[k + 1],
				                                      nx.ranks[k + 1]));
				D.backward(k);
			}
			double* lcur = Lb;
			double* lnext = Lb + maxr2;
			fill(c, lcur, 1.0, 1);
			for (int k = 0; k < d; ++k) {
				const long long len = (long long)nx.core_size(k);
				run_gemm_chain(c, plan_local_rhs1(lcur, x.core[k], Rb + off[k + 1], nx.core[k], tmp, nx.ranks[k],
				                                  nx.ranks[k + 1], x.ranks[k], x.ranks[k + 1], x.dims[k]));
				D.res_grad(k, 1, nx.core[k], G, 1.0);
				k_iht_add<<<unsigned(std::min<long long>((len + 255) / 256, 1024)), 256, 0, c.stream>>>(nx.core[k], G,
				                                                                                       len);
				XTT_CUDA(cudaGetLastError());
				c.count_launch();
				if (k + 1 < d) {
					move_core(nx, k + 1, true);
					run_gemm_chain(c, plan_push_left_rhs(lcur, x.core[k], nx.core[k], lnext, tmp, x.ranks[k],
					                                     nx.ranks[k], x.dims[k], x.ranks[k + 1], nx.ranks[k + 1]));
					std::swap(lcur, lnext);
					D.forward(k);
				}
			}
			const double r = resid(nx);
			if (r <= best) {
				x.copy_from(nx);
				best = r;
				new_alpha = alpha * beta;
			}
		}
		residual = best;
		alpha = new_alpha;
		out.trace.push_back(best);
	}
	c.sync();
	out.residual = residual;
	return out;
}

// ------------------------------------------------------------ rank-one measurements
//
// ADFVariant::InternalSolver<RankOneMeasurementSet> (adf.cpp:233-288, 333-357, 405-408,
// 481-487): a sample is <x, u_1 (x) ... (x) u_d> with a vector u_k per mode, so a stack
// update contracts the core with the sample's mixed component sum_i u_k[i] X_k[:, i, :];
// the projected gradient takes every entry of u_k; the slice norms collapse into one
// total (position_or_zero is 0) and update_x takes one step for the whole core. The
// vectors are stored mode-major (entry i of sample s at i*N + s), like the stacks.

constexpr int kR1Threads = 128;
constexpr int kR1Warps = kR1Threads / 32;
constexpr int kR1MaxN = 16;

struct R1Level {
	const double* U;  // this mode's vectors: n x N
	const double* F;  // F_{k-1}: r0 x N (nullptr: the constant 1)
	const double* B;  // B_{k+1}: r1 x N (nullptr: the constant 1)
	const double* X;  // core (r0, n, r1)
	int r0, n, r1;
	long long N;
};

// <f, M(u) b> for one sample with the core (or gradient) in shared memory
__device__ __forceinline__ double r1_value(const double* Xs, const R1Level& L, long long s, const double* f,
                                           const double* b) {
	double v = 0.0;
	for (int a = 0; a < L.r0; ++a) {
		double t = 0.0;
		for (int i = 0; i < L.n; ++i) {
			const double* xr = Xs + (a * L.n + i) * L.r1;
			double w = 0.0;
			for (int c = 0; c < L.r1; ++c) w = fma(xr[c], b[c], w);
			t = fma(L.U[(long long)i * L.N + s], w, t);
		}
		v = fma(f[a], t, v);
	}
	return v;
}

// B_k[a][s] = sum_i u[i] sum_c X[a,i,c] B_{k+1}[c][s]  (update_backward_stack, adf.cpp:234-249)
__global__ void k_r1_backward(R1Level L, double* Bo) {
	extern __shared__ double xs_r1[];
	for (int e = threadIdx.x; e < L.r0 * L.n * L.r1; e += blockDim.x) xs_r1[e] = L.X[e];
	__syncthreads();
	for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < L.N; s += (long long)gridDim.x * blockDim.x) {
		double b[kAdfMaxR];
		for (int c = 0; c < L.r1; ++c) b[c] = L.B ? L.B[c * L.N + s] : 1.0;
		for (int a = 0; a < L.r0; ++a) {
			double t = 0.0;
			for (int i = 0; i < L.n; ++i) {
				const double* xr = xs_r1 + (a * L.n + i) * L.r1;
				double w = 0.0;
				for (int c = 0; c < L.r1; ++c) w = fma(xr[c], b[c], w);
				t = fma(L.U[(long long)i * L.N + s], w, t);
			}
			Bo[a * L.N + s] = t;
		}
	}
}

// F_k[c][s] = sum_a F_{k-1}[a][s] sum_i u[i] X[a,i,c]  (update_forward_stack, adf.cpp:271-288)
__global__ void k_r1_forward(R1Level L, double* Fo) {
	extern __shared__ double xs_r1[];
	for (int e = threadIdx.x; e < L.r0 * L.n * L.r1; e += blockDim.x) xs_r1[e] = L.X[e];
	__syncthreads();
	for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < L.N; s += (long long)gridDim.x * blockDim.x) {
		double f[kAdfMaxR], u[kR1MaxN];
		for (int a = 0; a < L.r0; ++a) f[a] = L.F ? L.F[a * L.N + s] : 1.0;
		for (int i = 0; i < L.n; ++i) u[i] = L.U[(long long)i * L.N + s];
		for (int c = 0; c < L.r1; ++c) {
			double t = 0.0;
			for (int a = 0; a < L.r0; ++a) {
				double w = 0.0;
				for (int i = 0; i < L.n; ++i) w = fma(u[i], xs_r1[(a * L.n + i) * L.r1 + c], w);
				t = fma(f[a], w, t);
			}
			Fo[c * L.N + s] = t;
		}
	}
}

// res_s and per-block partials of G (r0, n, r1) and sum res^2 (calculate_residual,
// calculate_projected_gradient with perform_dyadic_product, adf.cpp:290-357). Lanes own the
// (a, c) pairs and, for them, every slice i in registers; samples are staged 32 at a time
// (res F premultiplied, B, u) and added in order; warps summed in order (deterministic).
__global__ void __launch_bounds__(kR1Threads) k_r1_res_grad(R1Level L, const double* y, double* res, double* gpart,
                                                            double* rrpart, long long chunk) {
	extern __shared__ double sm_r1[];
	const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	const int r0 = L.r0, n = L.n, r1 = L.r1, P = r0 * r1;
	double* Xs = sm_r1;                                   // r0 n r1
	double* RF = Xs + r0 * n * r1 + wib * (r0 + r1 + n) * 33;  // per warp: r0 + r1 + n rows of 33
	double* BB = RF + r0 * 33;
	double* UU = BB + r1 * 33;
	double* Gw = Xs + r0 * n * r1 + kR1Warps * (r0 + r1 + n) * 33;  // per warp n P, for the block sum
	__shared__ double rrw[kR1Warps];
	for (int e = threadIdx.x; e < r0 * n * r1; e += blockDim.x) Xs[e] = L.X[e];
	__syncthreads();
	int pa[kAdfPairsPerLane], pc[kAdfPairsPerLane];
	double acc[kAdfPairsPerLane][kR1MaxN];
#pragma unroll
	for (int t = 0; t < kAdfPairsPerLane; ++t) {
		const int p = lane + 32 * t;
		pa[t] = p < P ? p / r1 : 0;
		pc[t] = p < P ? p - pa[t] * r1 : 0;
#pragma unroll
		for (int i = 0; i < kR1MaxN; ++i) acc[t][i] = 0.0;
	}
	double rr = 0.0;
	const long long s0 = ((long long)blockIdx.x * kR1Warps + wib) * chunk, s1 = min(L.N, s0 + chunk);
	for (long long base = s0; base < s1; base += 32) {
		const long long s = base + lane;
		if (s < s1) {
			double f[kAdfMaxR], b[kAdfMaxR];
			for (int a = 0; a < r0; ++a) f[a] = L.F ? L.F[a * L.N + s] : 1.0;
			for (int c = 0; c < r1; ++c) b[c] = L.B ? L.B[c * L.N + s] : 1.0;
			const double rs = y[s] - r1_value(Xs, L, s, f, b);
			res[s] = rs;
			rr = fma(rs, rs, rr);
			for (int a = 0; a < r0; ++a) RF[a * 33 + lane] = rs * f[a];
			for (int c = 0; c < r1; ++c) BB[c * 33 + lane] = b[c];
			for (int i = 0; i < n; ++i) UU[i * 33 + lane] = L.U[(long long)i * L.N + s];
		}
		__syncwarp();
		const int cnt = int((s1 - base) < 32 ? (s1 - base) : 32);
		for (int j = 0; j < cnt; ++j) {
#pragma unroll
			for (int t = 0; t < kAdfPairsPerLane; ++t) {
				if (lane + 32 * t >= P) continue;
				const double q = RF[pa[t] * 33 + j] * BB[pc[t] * 33 + j];
#pragma unroll
				for (int i = 0; i < kR1MaxN; ++i)
					if (i < n) acc[t][i] = fma(q, UU[i * 33 + j], acc[t][i]);
			}
		}
		__syncwarp();
	}
	// the warp's accumulators into shared memory, then the block sum in warp order
	double* gw = Gw + wib * n * P;
#pragma unroll
	for (int t = 0; t < kAdfPairsPerLane; ++t) {
		const int p = lane + 32 * t;
		if (p >= P) continue;
#pragma unroll
		for (int i = 0; i < kR1MaxN; ++i)
			if (i < n) gw[i * P + p] = acc[t][i];
	}
	rr = warp_sum(rr);
	if (lane == 0) rrw[wib] = rr;
	__syncthreads();
	double* gp = gpart + (long long)blockIdx.x * r0 * n * r1;
	for (int e = threadIdx.x; e < n * P; e += blockDim.x) {
		double t = 0;
		for (int q = 0; q < kR1Warps; ++q) t += Gw[q * n * P + e];
		const int i = e / P, p = e - i * P, a = p / r1, c = p - a * r1;
		gp[(a * n + i) * r1 + c] = t;
	}
	if (threadIdx.x == 0) {
		double t = 0;
		for (int q = 0; q < kR1Warps; ++q) t += rrw[q];
		rrpart[blockIdx.x] = t;
	}
}

// per-block partials of sum_s <F[s], M_G(u_s) B[s]>^2 (calculate_slicewise_norm_A_projGrad
// with every sample in slot 0, adf.cpp:413-465)
__global__ void __launch_bounds__(kR1Threads) k_r1_norm(R1Level L, const double* G, double* npart, long long chunk) {
	__shared__ double Gs[kAdfMaxR * kR1MaxN * kAdfMaxR];
	__shared__ double red[32];
	for (int e = threadIdx.x; e < L.r0 * L.n * L.r1; e += blockDim.x) Gs[e] = G[e];
	__syncthreads();
	double acc = 0.0;
	const long long s0 = (long long)blockIdx.x * chunk, s1 = min(L.N, s0 + chunk);
	for (long long s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
		double f[kAdfMaxR], b[kAdfMaxR];
		for (int a = 0; a < L.r0; ++a) f[a] = L.F ? L.F[a * L.N + s] : 1.0;
		for (int c = 0; c < L.r1; ++c) b[c] = L.B ? L.B[c * L.N + s] : 1.0;
		const double v = r1_value(Gs, L, s, f, b);
		acc = fma(v, v, acc);
	}
	acc = block_sum(acc, red);
	if (threadIdx.x == 0) npart[blockIdx.x] = acc;
}

// X += (||G||^2 / nrm) G  (update_x for rank-one sets, adf.cpp:481-487); one block
__global__ void k_r1_update(double* X, const double* G, const double* nrm, int len) {
	__shared__ double sc[32];
	double s = 0.0;
	for (int e = threadIdx.x; e < len; e += blockDim.x) s = fma(G[e], G[e], s);
	const double step = block_sum(s, sc) / nrm[0];
	for (int e = threadIdx.x; e < len; e += blockDim.x) X[e] = fma(step, G[e], X[e]);
}

AdfResult adf_rank_one(Tensor& x, const double* vectors, const double* values, long long N, int64_t max_iter,
                       double target, double min_dec) {
	// ADFVariant::InternalSolver<RankOneMeasurementSet>::solve (adf.cpp:489-604) with x at its ranks
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op, "ADF needs a TT tensor");
	XTT_REQUIRE(N > 0, "need at very least one measurement");
	const int d = x.d;
	int64_t maxr = 1, maxn = 1, sum_n = 0;
	for (int k = 0; k <= d; ++k) maxr = std::max(maxr, x.ranks[k]);
	for (int k = 0; k < d; ++k) {
		maxn = std::max(maxn, x.dims[k]);
		sum_n += x.dims[k];
	}
	XTT_REQUIRE(maxr <= kAdfMaxR && maxn <= kR1MaxN && maxr * maxr <= 32 * kAdfPairsPerLane,
	            "rank-one ADF on the device needs ranks <= 8 and mode sizes <= 16");
	double ny2 = 0;
	for (long long s = 0; s < N; ++s) ny2 += values[s] * values[s];
	const double norm_y = std::sqrt(ny2);
	move_core(x, 0, false);  // canonicalize_left (adf.cpp:582)
	// device data: vectors mode-major, values, residuals, stacks, partials
	std::vector<double> hu(size_t(sum_n) * N);
	std::vector<size_t> uoff(d, 0);
	for (int k = 1; k < d; ++k) uoff[k] = uoff[k - 1] + size_t(x.dims[k - 1]) * N;
	for (long long s = 0; s < N; ++s) {
		size_t col = 0;
		for (int k = 0; k < d; ++k)
			for (int64_t i = 0; i < x.dims[k]; ++i, ++col) hu[uoff[k] + size_t(i) * N + s] = vectors[size_t(s) * sum_n + col];
	}
	double* U = c.scratch<double>(S_ADF_FIRST + 13, hu.size());
	double* y = c.scratch<double>(S_ADF_FIRST + 1, N);
	double* res = c.scratch<double>(S_ADF_FIRST + 2, N);
	XTT_CUDA(cudaMemcpyAsync(U, hu.data(), hu.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
	XTT_CUDA(cudaMemcpyAsync(y, values, N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
	size_t fo = 0, bo = 0;
	for (int k = 0; k < d; ++k) {
		fo += size_t(x.ranks[k + 1]) * N;
		bo += size_t(x.ranks[k]) * N;
	}
	double* Fa = c.scratch<double>(S_ADF_FIRST + 8, fo);
	double* Ba = c.scratch<double>(S_ADF_FIRST + 9, bo);
	std::vector<double*> F(d), B(d);
	fo = bo = 0;
	for (int k = 0; k < d; ++k) {
		F[k] = Fa + fo;
		B[k] = Ba + bo;
		fo += size_t(x.ranks[k + 1]) * N;
		bo += size_t(x.ranks[k]) * N;
	}
	const long long chunk = 64, res_blocks = std::max<long long>(1, (N + chunk * kR1Warps - 1) / (chunk * kR1Warps));
	const long long norm_chunk = 1024, norm_blocks = std::max<long long>(1, (N + norm_chunk - 1) / norm_chunk);
	double* gpart = c.scratch<double>(S_ADF_FIRST + 3, size_t(res_blocks) * maxr * maxn * maxr);
	double* npart = c.scratch<double>(S_ADF_FIRST + 4, size_t(norm_blocks));
	double* rrpart = c.scratch<double>(S_ADF_FIRST + 5, size_t(res_blocks));
	double* G = c.scratch<double>(S_ADF_FIRST + 6, size_t(maxr) * maxn * maxr);
	double* nrm = c.scratch<double>(S_ADF_FIRST + 7, 2);
	double* rr = nrm + 1;
	auto level = [&](int k, const double* X) {
		R1Level L;
		L.U = U + uoff[k];
		L.F = k > 0 ? F[k - 1] : nullptr;
		L.B = k + 1 < d ? B[k + 1] : nullptr;
		L.X = X;
		L.r0 = int(x.ranks[k]);
		L.n = int(x.dims[k]);
		L.r1 = int(x.ranks[k + 1]);
		L.N = N;
		return L;
	};
	const unsigned sbl = unsigned(std::max<long long>(1, std::min<long long>((N + 255) / 256, (long long)c.num_sms * 8)));
	auto backward = [&](int k) {
		const R1Level L = level(k, x.core[k]);
		ProfScope ps(c, "adf_stack");
		k_r1_backward<<<sbl, 256, size_t(L.r0) * L.n * L.r1 * sizeof(double), c.stream>>>(L, B[k]);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	};
	auto forward = [&](int k) {
		const R1Level L = level(k, x.core[k]);
		ProfScope ps(c, "adf_stack");
		k_r1_forward<<<sbl, 256, size_t(L.r0) * L.n * L.r1 * sizeof(double), c.stream>>>(L, F[k]);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	};
	func_attr_once(k_r1_res_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
	auto res_grad = [&](int k) {
		const R1Level L = level(k, x.core[k]);
		const int P = L.r0 * L.r1, len = L.r0 * L.n * L.r1;
		const size_t smem = (size_t(len) + size_t(kR1Warps) * (L.r0 + L.r1 + L.n) * 33 + size_t(kR1Warps) * L.n * P) *
		                    sizeof(double);
		ProfScope ps(c, "adf_res_grad");
		k_r1_res_grad<<<unsigned(res_blocks), kR1Threads, smem, c.stream>>>(L, y, res, gpart, rrpart, chunk);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		sum_parts(c, gpart, res_blocks, len, G, 1.0);
		sum_parts(c, rrpart, res_blocks, 1, rr, 1.0);
	};
	AdfResult out;
	double residual_norm = DBL_MAX, last_residual_norm = DBL_MAX;
	double dec1 = 0, dec2 = 0, dec3 = 0;
	for (int64_t it = 0; max_iter == 0 || it < max_iter; ++it) {
		move_core(x, 0, true);
		for (int k = d - 1; k > 0; --k) backward(k);
		res_grad(0);
		XTT_CUDA(cudaMemcpyAsync(c.h_dbl + 30, rr, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		last_residual_norm = residual_norm;
		residual_norm = std::sqrt(c.h_dbl[30]) / norm_y;
		out.trace.push_back(residual_norm);
		const double dec4 = dec3;
		dec3 = dec2;
		dec2 = dec1;
		dec1 = residual_norm / last_residual_norm;
		if (residual_norm < target || dec1 * dec2 * dec3 * dec4 > std::pow(min_dec, 4)) break;
		for (int k = 0; k < d; ++k) {
			if (k > 0) res_grad(k);
			{
				const R1Level L = level(k, x.core[k]);
				ProfScope ps(c, "adf_slicenorm");
				k_r1_norm<<<unsigned(norm_blocks), kR1Threads, 0, c.stream>>>(L, G, npart, norm_chunk);
				XTT_CUDA(cudaGetLastError());
				c.count_launch();
				sum_parts(c, npart, norm_blocks, 1, nrm, 1.0);
			}
			k_r1_update<<<1, 128, 0, c.stream>>>(x.core[k], G, nrm, int(x.core_size(k)));
			XTT_CUDA(cudaGetLastError());
			c.count_launch();
			if (k + 1 < d) {
				move_core(x, k + 1, true);
				forward(k);
			}
		}
	}
	out.residual = residual_norm;
	out.checked_residual = residual_norm;
	return out;
}

double adf_gradient(const Tensor& xc, const int64_t* positions, const double* values, long long N,
                    std::vector<double>& grad) {
	// loss 0.5 ||P(x) - y||^2 and d loss / d X_k = -sum_s res_s F_{k-1}[s] (x) e_{i_s} (x) B_{k+1}[s]
	Tensor& x = const_cast<Tensor&>(xc);
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op && N > 0, "ADF gradient needs a TT tensor and samples");
	AdfData D(c, x, positions, values, N);
	const int d = x.d;
	for (int k = 0; k + 1 < d; ++k) D.forward(k);
	for (int k = d - 1; k > 0; --k) D.backward(k);
	grad.assign(x.total_size(), 0.0);
	double* Gk = c.scratch<double>(S_ADF_FIRST + 10, x.total_size());
	size_t off = 0;
	// residual from the last level (mode 0 at k = d-1), then gradients with the fixed residual
	std::vector<size_t> offs(d);
	for (int k = 0; k < d; ++k) {
		offs[k] = off;
		off += x.core_size(k);
	}
	D.res_grad(d - 1, 0, x.core[d - 1], Gk + offs[d - 1], -1.0);
	for (int k = 0; k + 1 < d; ++k) D.res_grad(k, 1, x.core[k], Gk + offs[k], -1.0);
	const double loss = 0.5 * D.read_rr();
	XTT_CUDA(cudaMemcpyAsync(grad.data(), Gk, sizeof(double) * grad.size(), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	return loss;
}

}  // namespace xtt
