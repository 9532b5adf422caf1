// TT operations of the xerus sweep path on device-resident tensors:
// move_core / transfer_core, round / round_edge, the dot-product zipper,
// frob_norm, sampled entries, operator application and the FP64 residual.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <tuple>

#include <cooperative_groups.h>

#include "engine.cuh"

namespace xtt {

// ------------------------------------------------------------ kernel attributes

void func_attr_once(const void* kernel, cudaFuncAttribute attr, int value) {
	static std::mutex mu;
	static std::set<std::tuple<int, const void*, int, int>> done;
	int dev = 0;
	XTT_CUDA(cudaGetDevice(&dev));
	const auto key = std::make_tuple(dev, kernel, int(attr), value);
	std::lock_guard<std::mutex> lock(mu);
	if (done.count(key)) return;
	XTT_CUDA(cudaFuncSetAttribute(kernel, attr, value));
	done.insert(key);
}

// ------------------------------------------------------------ context

Context::Context(int dev) : device(dev) {
	XTT_CUDA(cudaSetDevice(dev));
	XTT_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
	stream = own;
	XTT_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
	XTT_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
	XTT_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
	XTT_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
	XTT_CUDA(cudaMalloc(&d_status, sizeof(int)));
	XTT_CUDA(cudaMalloc(&d_barrier, 2 * sizeof(unsigned)));
	XTT_CUDA(cudaMalloc(&d_ints, 64 * sizeof(int)));
	XTT_CUDA(cudaMalloc(&d_dbl, 64 * sizeof(double)));
	XTT_CUDA(cudaMallocHost(&h_ints, 64 * sizeof(int)));
	XTT_CUDA(cudaMallocHost(&h_dbl, 64 * sizeof(double)));
	XTT_CUDA(cudaMemset(d_status, 0, sizeof(int)));
	XTT_CUDA(cudaMemset(d_barrier, 0, 2 * sizeof(unsigned)));
	slots.resize(S_MAX);
}

Context::~Context() {
	cudaSetDevice(device);
	cudaStreamSynchronize(stream);
	cudaStreamSynchronize(aux);
	for (auto& e : graph_cache) delete e.second;
	for (auto& s : slots)
		if (s.p) cudaFree(s.p);
	cudaFree(d_status);
	cudaFree(d_barrier);
	cudaFree(d_ints);
	cudaFree(d_dbl);
	cudaFreeHost(h_ints);
	cudaFreeHost(h_dbl);
	if (batch_exec) cudaGraphExecDestroy(batch_exec);
	if (batch_host) cudaFreeHost(batch_host);
	cudaEventDestroy(ev_fork);
	cudaEventDestroy(ev_join);
	cudaStreamDestroy(aux);
	cudaStreamDestroy(own);
}

void Context::fork() {
	XTT_CUDA(cudaEventRecord(ev_fork, stream));
	XTT_CUDA(cudaStreamWaitEvent(aux, ev_fork, 0));
}

void Context::join() {
	XTT_CUDA(cudaEventRecord(ev_join, aux));
	XTT_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
}

void* Context::scratch_bytes(int id, size_t bytes) {
	XTT_REQUIRE(id >= 0 && id < S_MAX, "scratch id");
	Slot& s = slots[id];
	if (s.bytes < bytes) {
		const size_t nb = std::max(bytes, s.bytes * 3 / 2) + 256;
		if (s.p) {
			XTT_CUDA(cudaStreamSynchronize(own));  // either stream may still use the old buffer
			XTT_CUDA(cudaStreamSynchronize(aux));
			if (stream != own) XTT_CUDA(cudaStreamSynchronize(stream));
			XTT_CUDA(cudaFree(s.p));
			s.p = nullptr;
		}
		cudaError_t e = cudaMalloc(&s.p, nb);
		if (e != cudaSuccess) throw Error(XTT_ERR_NO_MEMORY, "device allocation of scratch failed");
		s.bytes = nb;
	}
	return s.p;
}

void Context::check_status() {
	int st = 0;
	XTT_CUDA(cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost));
	if (st != DEV_OK) {
		XTT_CUDA(cudaMemset(d_status, 0, sizeof(int)));
		XTT_CUDA(cudaMemset(d_barrier, 0, 2 * sizeof(unsigned)));
		switch (st) {
			case DEV_TIMEOUT: throw Error(XTT_ERR_TIMEOUT, "a device-side wait timed out");
			case DEV_NOT_CONVERGED: throw Error(XTT_ERR_NOT_CONVERGED, "iteration cap reached on the device");
			case DEV_BREAKDOWN: throw Error(XTT_ERR_NUMERIC, "numerical breakdown (non-SPD operator or NaN)");
			default: throw Error(XTT_ERR_CAPACITY, "device kernel rejected a size");
		}
	}
}

void Context::sync() {
	XTT_CUDA(cudaStreamSynchronize(stream));
	check_status();
}

ProfScope::ProfScope(Context& cc, const char* n, double by, double fl) : c(cc), name(n), bytes(by), flops(fl) {
	if (!c.profiling) return;
	XTT_CUDA(cudaEventCreate(&a));
	XTT_CUDA(cudaEventCreate(&b));
	XTT_CUDA(cudaEventRecord(a, c.stream));
}

ProfScope::~ProfScope() {
	if (!a) return;
	cudaEventRecord(b, c.stream);
	c.pending.push_back(Context::Timed{name, a, b, bytes, flops});
}

void Context::resolve_profile() {
	for (auto& t : pending) {
		float ms = 0;
		XTT_CUDA(cudaEventSynchronize(t.stop));
		XTT_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
		cudaEventDestroy(t.start);
		cudaEventDestroy(t.stop);
		auto it = std::find_if(profile.begin(), profile.end(), [&](const auto& e) { return e.first == t.name; });
		if (it == profile.end()) {
			profile.emplace_back(t.name, ProfileEntry{});
			it = profile.end() - 1;
		}
		it->second.launches += 1;
		it->second.ms += ms;
		it->second.bytes += t.bytes;
		it->second.flops += t.flops;
	}
	pending.clear();
}

int Context::read_int(int idx) {
	XTT_CUDA(cudaMemcpyAsync(h_ints + idx, d_ints + idx, sizeof(int), cudaMemcpyDeviceToHost, stream));
	sync();
	return h_ints[idx];
}

void Context::read_ints(int lo, int hi) {
	XTT_CUDA(cudaMemcpyAsync(h_ints + lo, d_ints + lo, sizeof(int) * size_t(hi - lo), cudaMemcpyDeviceToHost, stream));
	sync();
}

// ------------------------------------------------------------ tensors

Tensor::Tensor(Context* c, bool is_op, int order, const int64_t* dims_, const int64_t* ranks_)
    : ctx(c), op(is_op), d(order), dims(dims_, dims_ + order), ranks(ranks_, ranks_ + order + 1) {
	XTT_REQUIRE(order >= 1, "order must be positive");
	XTT_REQUIRE(ranks[0] == 1 && ranks[order] == 1, "boundary ranks must be 1");
	for (int k = 0; k < order; ++k) XTT_REQUIRE(dims[k] > 0, "dimension 0 is not valid");
	for (int k = 0; k <= order; ++k) XTT_REQUIRE(ranks[k] > 0, "rank 0 is not valid");
	core.assign(d, nullptr);
	cap.assign(d, 0);
	for (int k = 0; k < d; ++k) {
		const size_t sz = core_size(k);
		if (cudaMalloc(&core[k], std::max<size_t>(sz, 1) * sizeof(double)) != cudaSuccess)
			throw Error(XTT_ERR_NO_MEMORY, "device allocation of a TT core failed");
		cap[k] = std::max<size_t>(sz, 1);
		XTT_CUDA(cudaMemsetAsync(core[k], 0, sz * sizeof(double), ctx->stream));
	}
}

Tensor::~Tensor() {
	if (ctx) cudaStreamSynchronize(ctx->stream);
	for (double* p : core)
		if (p) cudaFree(p);
}

size_t Tensor::total_size() const {
	size_t s = 0;
	for (int k = 0; k < d; ++k) s += core_size(k);
	return s;
}

void Tensor::reshape_core(int k, int64_t r0, int64_t r1) {
	const size_t sz = size_t(r0) * size_t(n(k)) * size_t(r1);
	if (sz > cap[k]) {
		XTT_CUDA(cudaStreamSynchronize(ctx->stream));
		XTT_CUDA(cudaFree(core[k]));
		core[k] = nullptr;
		const size_t nc = std::max(sz, cap[k] * 3 / 2);
		if (cudaMalloc(&core[k], nc * sizeof(double)) != cudaSuccess)
			throw Error(XTT_ERR_NO_MEMORY, "device allocation of a TT core failed");
		cap[k] = nc;
	}
	ranks[k] = r0;
	ranks[k + 1] = r1;
}

void Tensor::copy_from(const Tensor& o) {
	XTT_REQUIRE(o.d == d && o.dims == dims && o.op == op, "copy between different shapes");
	for (int k = 0; k < d; ++k) {
		const size_t sz = o.core_size(k);
		if (sz > cap[k]) {
			XTT_CUDA(cudaStreamSynchronize(ctx->stream));
			XTT_CUDA(cudaFree(core[k]));
			XTT_CUDA(cudaMalloc(&core[k], sz * sizeof(double)));
			cap[k] = sz;
		}
	}
	ranks = o.ranks;
	for (int k = 0; k < d; ++k) copy_d2d(*ctx, core[k], o.core[k], core_size(k));
	canonicalized = o.canonicalized;
	core_position = o.core_position;
}

// ------------------------------------------------------------ kernels

template <class T>
__global__ void __launch_bounds__(kGemmThreads) k_gemm(Gemm<T> g) {
	__shared__ GemmSmem<T> sm;
	gemm_tile(g, blockIdx.x, sm);
}

template <class T>
void check_gemm(const Gemm<T>& g) {
	XTT_REQUIRE(g.lenA >= 0 && g.lenB >= 0 && g.lenC >= 0, "internal: GEMM launched without operand lengths");
	XTT_REQUIRE(g.strides_nonnegative(), "internal: negative GEMM stride");
	XTT_REQUIRE(g.K <= 0 || (g.A && g.B), "internal: GEMM operand missing");
	XTT_REQUIRE(g.max_off_A() < g.lenA || g.K <= 0, "internal: GEMM operand A out of bounds");
	XTT_REQUIRE(g.max_off_B() < g.lenB || g.K <= 0, "internal: GEMM operand B out of bounds");
	XTT_REQUIRE(g.C && g.max_off_C() < g.lenC, "internal: GEMM output out of bounds");
	XTT_REQUIRE(!g.D || g.max_off_C() < g.lenC, "internal: GEMM epilogue operand out of bounds");
}
template void check_gemm<double>(const Gemm<double>&);
template void check_gemm<float>(const Gemm<float>&);

// Split-K tile GEMM: the S CTAs of one cluster (S = cluster size) compute the
// same TS x TS output tile over disjoint K ranges; their partial sums meet in
// the rank-0 CTA through distributed shared memory, added in rank order
// (deterministic), and rank 0 runs the epilogue. S = 1 is a plain tile GEMM.
template <class T, int TS>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_sk(Gemm<T> g, int S, int kchunk) {
	constexpr int R = TS / 16;
	__shared__ TileSmem<T, TS> sm;
	__shared__ T part[R * R][kGemmThreads];
	const long long tile = blockIdx.x / S;
	const int ks = blockIdx.x % S;
	const int kb = ks * kchunk, ke = min(g.K, kb + kchunk);
	T acc[R][R];
	gemm_tile_acc<T, TS>(g, tile, kb, ke, sm, acc);
	if (S == 1) {
		gemm_tile_store<T, TS>(g, tile, acc);
		return;
	}
	namespace cgn = cooperative_groups;
	cgn::cluster_group cl = cgn::this_cluster();
#pragma unroll
	for (int i = 0; i < R; ++i)
#pragma unroll
		for (int j = 0; j < R; ++j) part[i * R + j][threadIdx.x] = acc[i][j];
	cl.sync();
	if (cl.block_rank() == 0) {
#pragma unroll
		for (int i = 0; i < R; ++i)
#pragma unroll
			for (int j = 0; j < R; ++j) {
				T v[8];
#pragma unroll
				for (int p = 0; p < 8; ++p) {
					const T t = cl.map_shared_rank(&part[i * R + j][threadIdx.x], p < S ? p : 0)[0];
					v[p] = p < S ? t : T(0);
				}
				T s = T(0);
#pragma unroll
				for (int p = 0; p < 8; ++p) s += v[p];
				acc[i][j] = s;
			}
		gemm_tile_store<T, TS>(g, tile, acc);
	}
	cl.sync();  // the partials stay readable until rank 0 has summed them
}

// Launch shape: 32 x 32 tiles when they already cover the SMs, else 16 x 16
// tiles and up to 8-way split K so that FP64 work spreads over the GPU (GB300
// retires about two FP64 FMAs per SM and clock, so one tile on one SM is slow).
template <class T>
static void launch_gemm_sk(Context& c, const Gemm<T>& g) {
	const long long t32 = g.tiles();
	XTT_REQUIRE(t32 < (1ll << 26), "GEMM too large");
	const long long target = 2ll * c.num_sms;
	if (t32 >= target || g.K <= 16) {
		k_gemm_sk<T, 32><<<unsigned(t32), kGemmThreads, 0, c.stream>>>(g, 1, std::max(g.K, 1));
		XTT_CUDA(cudaGetLastError());
		return;
	}
	const long long t16 = (long long)g.batch * ((g.M + 15) / 16) * ((g.N + 15) / 16);
	int S = int(std::min<long long>(8, std::max<long long>(1, (target + t16 - 1) / t16)));
	S = std::min(S, std::max(1, g.K / 16));  // at least 16 K per CTA
	const int kchunk = (g.K + S - 1) / S;
	S = (g.K + kchunk - 1) / kchunk;
	if (S == 1) {
		k_gemm_sk<T, 16><<<unsigned(t16), kGemmThreads, 0, c.stream>>>(g, 1, g.K);
		XTT_CUDA(cudaGetLastError());
		return;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(unsigned(t16 * S));
	cfg.blockDim = dim3(kGemmThreads);
	cfg.stream = c.stream;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = S;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	XTT_CUDA(cudaLaunchKernelEx(&cfg, k_gemm_sk<T, 16>, g, S, kchunk));
}

void gemm(Context& c, const Gemm<double>& g) {
	if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return;
	if (c.tc_active && !g.D && g.K > 0) {  // precision form: the contraction on the tensor cores
		gemm_tc(c, g, c.tc_active);
		return;
	}
	check_gemm(g);
	const double mn = double(g.batch) * g.M * g.N, mk = double(g.M) * g.K, kn = double(g.K) * g.N;
	const bool df = c.df_gemm && !g.D && 2.0 * mn * g.K >= kDfGemmMinFlops;
	ProfScope ps(c, df ? "gemm_df" : "gemm", 8.0 * (double(g.batch) * (mk + kn) + mn), 2.0 * mn * g.K);
	if (df) {
		gemm_df(c, g);
		return;
	}
	launch_gemm_sk(c, g);
	c.count_launch();
}

void gemm_f(Context& c, const Gemm<float>& g) {
	if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return;
	check_gemm(g);
	k_gemm<float><<<unsigned(g.tiles()), kGemmThreads, 0, c.stream>>>(g);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

__global__ void k_fill(double* x, double v, size_t n) {
	for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) x[i] = v;
}
__global__ void k_scale(double* x, double f, size_t n) {
	for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) x[i] *= f;
}

static unsigned grid_for(size_t n, int threads = 256) {
	return unsigned(std::max<size_t>(1, std::min<size_t>((n + threads - 1) / threads, 4096)));
}

void copy_d2d(Context& c, double* dst, const double* src, size_t count) {
	if (count == 0 || dst == src) return;
	XTT_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
}

void fill(Context& c, double* dst, double v, size_t count) {
	if (!count) return;
	k_fill<<<grid_for(count), 256, 0, c.stream>>>(dst, v, count);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

void scale(Context& c, double* x, double f, size_t count) {
	if (!count) return;
	k_scale<<<grid_for(count), 256, 0, c.stream>>>(x, f, count);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

constexpr int kRedBlocks = 64;

__global__ void k_dot_partial(const double* a, const double* b, size_t n, double* partial) {
	__shared__ double sc[32];
	double s = 0;
	for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
		s += a[i] * b[i];
	s = block_sum(s, sc);
	if (threadIdx.x == 0) partial[blockIdx.x] = s;
}
__global__ void k_sum_partials(const double* partial, int np, double* out) {
	__shared__ double sc[32];
	double s = 0;
	for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
	s = block_sum(s, sc);
	if (threadIdx.x == 0) *out = s;
}

void dot_async(Context& c, const double* a, const double* b, size_t count, int slot) {
	double* part = c.scratch<double>(S_RED, kRedBlocks);
	k_dot_partial<<<kRedBlocks, 256, 0, c.stream>>>(a, b, count, part);
	k_sum_partials<<<1, 64, 0, c.stream>>>(part, kRedBlocks, c.d_dbl + slot);
	XTT_CUDA(cudaGetLastError());
	c.count_launch(2);
}

void sumsq_async(Context& c, const double* x, size_t count, int slot) { dot_async(c, x, x, count, slot); }

static double read_dbl(Context& c, int slot) {
	XTT_CUDA(cudaMemcpyAsync(c.h_dbl + slot, c.d_dbl + slot, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	return c.h_dbl[slot];
}

// out(c, a, b) = in(a, b, c) for in of shape (A, B, C)
__global__ void k_cab(double* out, const double* in, int A, int B, int C) {
	const size_t n = size_t(A) * B * C;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < n; e += size_t(gridDim.x) * blockDim.x) {
		const int c = int(e / (size_t(A) * B));
		const size_t r = e % (size_t(A) * B);
		const int a = int(r / B), b = int(r % B);
		out[e] = in[(size_t(a) * B + b) * C + c];
	}
}

// out (M x s) = in^T (in: s x M) scaled by S per column
__global__ void k_transpose_scale(double* out, const double* in, const double* S, int s, int M) {
	const size_t n = size_t(s) * M;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < n; e += size_t(gridDim.x) * blockDim.x) {
		const int j = int(e / s), c = int(e % s);
		out[e] = in[size_t(c) * M + j] * S[c];
	}
}

// rows of X (s x M) scaled by S
__global__ void k_scale_rows(double* X, const double* S, int s, int M) {
	const size_t n = size_t(s) * M;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < n; e += size_t(gridDim.x) * blockDim.x)
		X[e] *= S[e / M];
}

__global__ void k_scale_cols(double* X, const double* S, int m, int k) {
	const size_t n = size_t(m) * k;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < n; e += size_t(gridDim.x) * blockDim.x)
		X[e] *= S[e % k];
}

void scale_rows(Context& c, double* X, const double* S, int rows, int cols) {
	if (size_t(rows) * cols == 0) return;
	k_scale_rows<<<grid_for(size_t(rows) * cols), 256, 0, c.stream>>>(X, S, rows, cols);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

void scale_cols(Context& c, double* X, const double* S, int rows, int cols) {
	if (size_t(rows) * cols == 0) return;
	k_scale_cols<<<grid_for(size_t(rows) * cols), 256, 0, c.stream>>>(X, S, rows, cols);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
}

// ------------------------------------------------------------ move_core

std::vector<int64_t> reduce_to_maximal_ranks(std::vector<int64_t> r, const std::vector<int64_t>& n) {
	// src/xerus/ttNetwork.cpp:369-402 with n = the product of the component's external dimensions
	const size_t d = n.size();
	int64_t cur = 1;
	for (size_t i = 0; i + 1 < d; ++i) {
		cur *= n[i];
		if (cur < r[i]) r[i] = cur;
		else cur = r[i];
	}
	cur = 1;
	for (size_t i = 1; i < d; ++i) {
		cur *= n[d - i];
		if (cur < r[d - i - 1]) r[d - i - 1] = cur;
		else cur = r[d - i - 1];
	}
	return r;
}

bool exceeds_maximal_ranks(const Tensor& x) {
	std::vector<int64_t> inner(x.ranks.begin() + 1, x.ranks.end() - 1), nn(x.d);
	for (int k = 0; k < x.d; ++k) nn[k] = x.n(k);
	return reduce_to_maximal_ranks(inner, nn) != inner;
}

// ------------------------------------------------------------ Cholesky QR of well-conditioned cores
// The rank-revealing factorisations of round (its left-orthogonalisation and the two per
// bond) by Cholesky QR with Newton-Schulz re-orthogonalisation, all FP64 products but one
// FP32 Cholesky of a Gram matrix: for the tall A_w (m_w x n_w; A or A^T),
//   G = A_w^T A_w;  R_32 = chol(G) in FP32, Q_1 = A_w R_32^{-1};
//   three steps Q <- Q (3 I - Q^T Q) / 2 (each squares the orthogonality defect);
//   C = Q^T A_w, so A_w = Q C with Q orthonormal to rounding.
// Householder QR on GB300 is a chain of ~n_w dependent column steps whose FP64 latencies
// (a reduction, a square root and a division each) and cluster barriers no parallelism
// hides; here the chain is the FP32 Cholesky only. The factorisation is accepted when
// every Cholesky pivot keeps 1e-6 of its column's squared norm (kappa(A) below ~1e3,
// far from the reference's rank rule |R_kk| < 16 eps R_00, which therefore keeps all
// n_w columns: rank_out = n_w) and the last step's defect max|Q^T Q - I| is below 1e-7
// (so Q is orthonormal to ~1e-14); otherwise a flag is set and the caller runs the
// pivoted Householder QR. Q and C differ from Householder's by an orthogonal n_w x n_w
// factor (Q C is the same): round uses them only through Q C-invariant products.
constexpr int kGqSlots = 6;  // scratch ids per concurrent factorisation
constexpr size_t kGraphCacheMax = 64;  // captured launch sequences kept per context
constexpr int kGqMaxCols = 128;
constexpr int kGqNsSteps = 3;

// FP32 Cholesky G = R^T R (G scaled to unit largest diagonal) with R^{-1} built alongside:
// the symmetric elimination E G E^T = D (E unit lower triangular, its rows updated with
// the same multipliers as G's) gives R = D^{1/2} E^{-T}, so R^{-1} = E^T D^{-1/2}; written
// (FP64, scaled back) to Rinv (n x n row-major, zero below the diagonal). One CTA of
// kGqRows x 32 threads (rows x columns), n <= NMAX; one barrier per pivot, every thread
// reading the pivot itself, and each thread's updates staged as all loads, then all
// stores (the compiler cannot reorder shared-memory stores and later loads).
constexpr int kGqRows = 16;
template <int NMAX>
__global__ void __launch_bounds__(kGqRows * 32) k_gq_chol32(const double* __restrict__ G, int n,
                                                            double* __restrict__ Rinv, int* flag) {
	constexpr int U = NMAX / 32, RPT = NMAX / kGqRows;
	extern __shared__ float gq_s[];
	const int ld = n + 1, tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
	float* S = gq_s;            // n x ld: G, eliminated in its upper triangle
	float* E = gq_s + n * ld;   // n x ld: the elimination, unit lower triangular
	__shared__ float s_rs[kGqMaxCols], s_d0[kGqMaxCols];
	__shared__ double s_scale;
	__shared__ int s_bad;
	if (tid < 32) {  // the largest diagonal entry, read by one warp in parallel
		double mx = 0;
		for (int i = tid; i < n; i += 32) mx = fmax(mx, G[(long long)i * n + i]);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
		if (tid == 0) {
			s_scale = mx > 0 ? 1.0 / mx : 0.0;
			s_bad = !(mx > 0);
		}
	}
	__syncthreads();
	const double sc = s_scale;
	for (int i = ty; i < n; i += kGqRows)  // rows by warp, columns by lane
		for (int j = tx; j < n; j += 32) {
			const float v = float(G[(long long)i * n + j] * sc);
			S[i * ld + j] = v;
			E[i * ld + j] = i == j ? 1.f : 0.f;
			if (i == j) s_d0[i] = v;
		}
	__syncthreads();
	for (int k = 0; k < n; ++k) {
		float d = S[k * ld + k];
		if (!(d > 1e-6f * s_d0[k])) {
			if (tid == 0) s_bad = 1;
			d = 1.f;
		}
		const float inv = __fdividef(1.f, d);
		if (tid == 0) s_rs[k] = rsqrtf(d);
		float sk[U], ek[U], l[RPT], sv[RPT][U], ev[RPT][U];
#pragma unroll
		for (int u = 0; u < U; ++u) {
			const int j = tx + 32 * u;
			sk[u] = j < n ? S[k * ld + j] : 0.f;
			ek[u] = j <= k ? E[k * ld + j] : 0.f;
		}
#pragma unroll
		for (int rr = 0; rr < RPT; ++rr) {
			const int i = k + 1 + ty + kGqRows * rr;
			l[rr] = i < n ? S[k * ld + i] * inv : 0.f;
#pragma unroll
			for (int u = 0; u < U; ++u) {
				const int j = tx + 32 * u;
				sv[rr][u] = i < n && j >= i && j < n ? S[i * ld + j] : 0.f;
				ev[rr][u] = i < n && j <= k ? E[i * ld + j] : 0.f;
			}
		}
#pragma unroll
		for (int rr = 0; rr < RPT; ++rr) {
			const int i = k + 1 + ty + kGqRows * rr;
#pragma unroll
			for (int u = 0; u < U; ++u) {
				const int j = tx + 32 * u;
				if (i < n && j >= i && j < n) S[i * ld + j] = fmaf(-l[rr], sk[u], sv[rr][u]);
				if (i < n && j <= k) E[i * ld + j] = fmaf(-l[rr], ek[u], ev[rr][u]);
			}
		}
		__syncthreads();
	}
	const double back = sqrt(sc);
	for (int a = ty; a < n; a += kGqRows)
		for (int b = tx; b < n; b += 32) Rinv[(long long)a * n + b] = b >= a ? double(E[b * ld + a] * s_rs[b]) * back : 0.0;
	if (tid == 0 && s_bad) atomicExch(flag, 1);
}

// H = (3 I - G) / 2 for the Newton-Schulz step; on the last step the defect gate and
// the rank. One thread per entry.
__global__ void k_gq_ns(const double* __restrict__ G, double* __restrict__ H, int n, int last, int* flag, int* rank_out) {
	int bad = 0;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
		const int i = e / n, j = e % n;
		const double dev = G[e] - (i == j ? 1.0 : 0.0);
		if (!(fabs(dev) < 1e-7)) bad = 1;
		H[e] = (i == j ? 1.0 : 0.0) - 0.5 * dev;
	}
	if (last) {
		if (bad) atomicExch(flag, 1);
		if (blockIdx.x == 0 && threadIdx.x == 0 && rank_out) *rank_out = n;
	}
}

static Gemm<double> gq_gemm(int M, int N, int K, const double* A, long long sAm, long long sAk, long long lenA,
                            const double* B, long long sBk, long long sBn, long long lenB, double* C, long long sCm,
                            long long sCn, long long lenC) {
	Gemm<double> g;
	g.M = M; g.N = N; g.K = K;
	g.A = A; g.sAm = sAm; g.sAk = sAk;
	g.B = B; g.sBk = sBk; g.sBn = sBn;
	g.C = C; g.sCm = sCm; g.sCn = sCn;
	g.lens(lenA, lenB, lenC);
	return g;
}

static bool gram_qr_fits(const QrArgs& a) {
	const int mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n;
	return a.pivot && a.want_q && nw >= 16 && nw <= kGqMaxCols && mw >= nw;
}

// Enqueues the Cholesky QR of `a` (gram_qr_fits) on the context's stream with the scratch
// of `slot` (0 or 1); `flag` (a device int, cleared here) is set where the caller must
// run the Householder QR instead. Writes a.Q, a.C and *a.rank_out in a.'s layouts.
static void gram_qr(Context& c, const QrArgs& a, int slot, int* flag) {
	Fp64ContractionScope fp64(c);
	const bool tr = a.transpose != 0;
	const int mw = tr ? a.n : a.m, nw = tr ? a.m : a.n;
	const long long sr = tr ? 1 : a.lda, sc = tr ? a.lda : 1;  // A_w[i][j] = A[i sr + j sc]
	const long long lenA = (long long)(a.m - 1) * a.lda + a.n, nn = (long long)nw * nw, mn = (long long)mw * nw;
	const int id = S_GQ_FIRST + slot * kGqSlots;
	double* G = c.scratch<double>(id + 0, nn);
	double* Ri = c.scratch<double>(id + 1, nn);
	double* H = c.scratch<double>(id + 2, nn);
	double* Qa0 = c.scratch<double>(id + 3, mn);
	double* Qb0 = c.scratch<double>(id + 4, mn);
	if (nw > 64)
		func_attr_once(k_gq_chol32<kGqMaxCols>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		               int(2 * kGqMaxCols * (kGqMaxCols + 1) * sizeof(float)));
	// the 13 launches in stream order, reading the factor from Ain
	auto launches = [&](const double* Ain) {
		double *Qa = Qa0, *Qb = Qb0;
		XTT_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), c.stream));
		gemm(c, gq_gemm(nw, nw, mw, Ain, sc, sr, lenA, Ain, sr, sc, lenA, G, nw, 1, nn));  // A_w^T A_w
		const size_t smem = 2 * size_t(nw) * (nw + 1) * sizeof(float);
		if (nw <= 64) k_gq_chol32<64><<<1, kGqRows * 32, smem, c.stream>>>(G, nw, Ri, flag);
		else k_gq_chol32<kGqMaxCols><<<1, kGqRows * 32, smem, c.stream>>>(G, nw, Ri, flag);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		gemm(c, gq_gemm(mw, nw, nw, Ain, sr, sc, lenA, Ri, nw, 1, nn, Qa, nw, 1, mn));  // Q_1 = A_w R^{-1}
		// the output layouts: tr == 0: Q (m x n_w) ld n_w, C (n_w x n) ld n; tr == 1: Q (n_w x n)
		// ld n (= Q_w^T), C (m x n_w) ld n_w (= C_w^T)
		const long long qm = tr ? 1 : nw, qn = tr ? mw : 1;
		for (int it = 0; it < kGqNsSteps; ++it) {
			const bool last = it + 1 == kGqNsSteps;
			gemm(c, gq_gemm(nw, nw, mw, Qa, 1, nw, mn, Qa, nw, 1, mn, G, nw, 1, nn));  // Q^T Q
			k_gq_ns<<<(unsigned(nn) + 255) / 256, 256, 0, c.stream>>>(G, H, nw, last, flag, a.rank_out);
			XTT_CUDA(cudaGetLastError());
			c.count_launch();
			if (last) gemm(c, gq_gemm(mw, nw, nw, Qa, nw, 1, mn, H, nw, 1, nn, a.Q, qm, qn, mn));
			else gemm(c, gq_gemm(mw, nw, nw, Qa, nw, 1, mn, H, nw, 1, nn, Qb, nw, 1, mn));
			std::swap(Qa, Qb);
		}
		// C_w = Q_w^T A_w, Q_w read back from a.Q
		gemm(c, gq_gemm(nw, nw, mw, a.Q, tr ? mw : 1, tr ? 1 : nw, mn, Ain, sr, sc, lenA, a.C, tr ? 1 : nw,
		                tr ? nw : 1, nn));
	};
	if (c.profiling) {  // per-launch timing: no graph
		launches(a.A);
		return;
	}
	// replayed as one CUDA graph per shape and buffer set: the factor is first copied into a
	// staging buffer the graph reads (the cores it factors live in different buffers)
	double* As = c.scratch<double>(id + 5, size_t(lenA));
	copy_d2d(c, As, a.A, size_t(lenA));
	const std::vector<long long> key = {1, a.m, a.n, a.lda, a.transpose, slot, (long long)(uintptr_t)As,
	                                    (long long)(uintptr_t)G, (long long)(uintptr_t)Ri, (long long)(uintptr_t)H,
	                                    (long long)(uintptr_t)Qa0, (long long)(uintptr_t)Qb0,
	                                    (long long)(uintptr_t)a.Q, (long long)(uintptr_t)a.C,
	                                    (long long)(uintptr_t)a.rank_out, (long long)(uintptr_t)flag};
	ReplayGraph* g = nullptr;
	for (auto& e : c.graph_cache)
		if (e.first == key) g = e.second;
	if (!g) {
		if (c.graph_cache.size() >= kGraphCacheMax) {  // bounded: the oldest entry goes, idle on both streams
			XTT_CUDA(cudaStreamSynchronize(c.own));
			XTT_CUDA(cudaStreamSynchronize(c.aux));
			XTT_CUDA(cudaStreamSynchronize(c.stream));
			delete c.graph_cache.front().second;
			c.graph_cache.erase(c.graph_cache.begin());
		}
		g = new ReplayGraph();
		c.graph_cache.emplace_back(key, g);
	}
	g->run(c, [&] { launches(As); });
}

// ------------------------------------------------------------ blocked Householder QR
// For factorisations with more than 64 columns (the keepRank moves of rank-128 sweeps), the
// cluster QR spreads each column step over 16 SMs only, and its trailing updates are FP64
// work those SMs retire at ~2 FMAs per clock. Blocked instead (dgeqrf's scheme): panels of
// kQbBlock columns are factored by the cluster kernel, which writes their reflectors V_p
// and tau; the trailing columns are updated as three FP64 GEMMs over the whole GPU,
// A_2 -= V_p T_p^T (V_p^T A_2), with T_p dlarft's forward factor (T_ii = tau_i,
// T(0:i, i) = -tau_i T(0:i, 0:i) V_p(:, 0:i)^T v_i); and Q = B_0 B_1 .. [I; 0] with
// B_p = I - V_p T_p V_p^T is formed backward the same way, Q(j0:, j0:) -= V_p (T_p (V_p^T
// Q(j0:, j0:))) (columns left of j0 are unit vectors with zeros below row j0, which B_p
// leaves unchanged). The reflectors and R are those of the unblocked factorisation up to
// rounding (the same dlarfg vectors, in the same order).
constexpr int kQbBlock = 32;
static_assert(S_GQ_FIRST + 2 * kGqSlots <= S_RES_MEET && S_RES_MEET < S_QB,
              "scratch ids of the Gram QR, the residual and the blocked QR overlap");

// T_p of one panel from its Gram G = V_p^T V_p (jb x jb) and tau: thread r owns row r.
__global__ void k_wy_t(const double* __restrict__ G, const double* __restrict__ tau, double* __restrict__ T, int jb) {
	__shared__ double sG[kQbBlock][kQbBlock + 1];
	__shared__ double sT[kQbBlock][kQbBlock + 1];
	const int r = threadIdx.x;
	for (int e = r; e < jb * jb; e += blockDim.x) sG[e / jb][e % jb] = G[e];
	__syncwarp();
	if (r < jb) {
		for (int i = 0; i < jb; ++i) {
			double v = 0.0;
			if (r == i) {
				v = tau[i];
			} else if (r < i) {
				double acc = 0.0;
				for (int t = r; t < i; ++t) acc = fma(sT[r][t], sG[t][i], acc);
				v = -tau[i] * acc;
			}
			sT[r][i] = v;
		}
		for (int i = 0; i < jb; ++i) T[r * jb + i] = sT[r][i];
	}
}

// dst[i][c] (row / column strides) = src[i * ss + c * sc] for i < m, c < n.
__global__ void k_copy2d(double* dst, long long dr, long long dc, const double* src, long long sr, long long sc, int m,
                         int n) {
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)m * n;
	     e += (long long)gridDim.x * blockDim.x) {
		const int i = int(e / n), c = int(e % n);
		dst[i * dr + c * dc] = src[i * sr + c * sc];
	}
}

__global__ void k_zero2d(double* dst, long long dr, long long dc, int m, int n) {
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)m * n;
	     e += (long long)gridDim.x * blockDim.x)
		dst[(e / n) * dr + (e % n) * dc] = 0.0;
}

// Q_w = [I_kq; 0] (mw x kq) at Q with row / column strides.
__global__ void k_eye_rect(double* Q, int mw, int kq, long long sr, long long sc) {
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)mw * kq;
	     e += (long long)gridDim.x * blockDim.x) {
		const int i = int(e / kq), c = int(e % kq);
		Q[i * sr + c * sc] = i == c ? 1.0 : 0.0;
	}
}

// Unpivoted QR with Q (tall, k_q > 64) blocked as above; false (nothing done) where the
// cluster kernel does not take a panel.
static bool qr_blocked(Context& c, const QrArgs& a) {
	const bool tr = a.transpose != 0;
	const int mw = tr ? a.n : a.m, nw = tr ? a.m : a.n, kq = std::min(mw, nw);
	if (a.pivot || !a.want_q || kq <= 64 || mw < nw || mw - (kq - 1) / kQbBlock * kQbBlock < 48) return false;
	const int np = (kq + kQbBlock - 1) / kQbBlock;
	if (kq - (np - 1) * kQbBlock < 8) return false;  // every panel needs 8 columns for the cluster kernel
	const size_t nb2 = size_t(kQbBlock) * kQbBlock, nwk = size_t(kQbBlock) * nw, nA = size_t(mw) * nw;
	// working copy of A_w, the panels' reflectors (mw x kQbBlock each, rows from j0), tau,
	// T per panel, the panel's R, and the GEMM temporaries
	double* Wk = c.scratch<double>(S_QB, nA + size_t(np) * mw * kQbBlock + kq + size_t(np) * nb2 + 2 * nb2 + 2 * nwk);
	double* Vall = Wk + nA;
	double* tau = Vall + size_t(np) * mw * kQbBlock;
	double* Tall = tau + kq;
	double *G = Tall + size_t(np) * nb2, *Rp = G + nb2, *W1 = Rp + nb2, *W2 = W1 + nwk;
	Fp64ContractionScope fp64(c);
	const long long asr = tr ? 1 : a.lda, asc = tr ? a.lda : 1;  // A_w[i][j] = A[i asr + j asc]
	k_copy2d<<<grid_for(nA), 256, 0, c.stream>>>(Wk, nw, 1, a.A, asr, asc, mw, nw);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	// R (kq x nw) into a.C: tr == 0, C (kq x n) ld n; tr == 1, C (m x kq) ld kq = R^T
	const long long csr = tr ? 1 : nw, csc = tr ? kq : 1;
	auto mk = [](int M, int N, int K, const double* A, long long sAm, long long sAk, long long lenA, const double* B,
	             long long sBk, long long sBn, long long lenB, double* C, long long sCm, long long sCn, long long lenC,
	             double alpha, double beta) {
		Gemm<double> g;
		g.M = M; g.N = N; g.K = K;
		g.A = A; g.sAm = sAm; g.sAk = sAk;
		g.B = B; g.sBk = sBk; g.sBn = sBn;
		g.C = C; g.sCm = sCm; g.sCn = sCn;
		g.alpha = alpha; g.beta = beta;
		g.lens(lenA, lenB, lenC);
		return g;
	};
	const long long lw = (long long)nA;
	for (int p = 0; p < np; ++p) {
		const int j0 = p * kQbBlock, jb = std::min(kQbBlock, kq - j0), mp = mw - j0, n2 = nw - j0 - jb;
		double* Vp = Vall + size_t(p) * mw * kQbBlock;  // mp x jb, ld jb
		double* Tp = Tall + size_t(p) * nb2;
		QrArgs ap;
		ap.A = Wk + (long long)j0 * nw + j0; ap.lda = nw; ap.m = mp; ap.n = jb; ap.transpose = 0; ap.pivot = 0;
		ap.want_q = 1; ap.C = Rp; ap.Q = nullptr; ap.rank_out = nullptr; ap.V_out = Vp; ap.tau_out = tau + j0;
		ap.work = nullptr;
		if (!launch_qr_reflectors(ap, c.stream)) {
			XTT_REQUIRE(p == 0, "internal: blocked QR panel does not fit the cluster kernel");
			return false;  // nothing done yet
		}
		c.count_launch();
		// R_pp (jb x jb) and zeros left of it in rows j0.., into C
		k_copy2d<<<grid_for(size_t(jb) * jb), 256, 0, c.stream>>>(a.C + j0 * csr + j0 * csc, csr, csc, Rp, jb, 1, jb, jb);
		if (j0 > 0) k_zero2d<<<grid_for(size_t(jb) * j0), 256, 0, c.stream>>>(a.C + j0 * csr, csr, csc, jb, j0);
		XTT_CUDA(cudaGetLastError());
		c.count_launch(j0 > 0 ? 2 : 1);
		const long long lv = (long long)mp * jb;
		gemm(c, mk(jb, jb, mp, Vp, 1, jb, lv, Vp, jb, 1, lv, G, jb, 1, (long long)nb2, 1.0, 0.0));  // V_p^T V_p
		k_wy_t<<<1, 32, 0, c.stream>>>(G, tau + j0, Tp, jb);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		if (n2 > 0) {
			double* A2 = Wk + (long long)j0 * nw + j0 + jb;  // mp x n2, ld nw
			const long long la2 = lw - ((long long)j0 * nw + j0 + jb);
			gemm(c, mk(jb, n2, mp, Vp, 1, jb, lv, A2, nw, 1, la2, W1, n2, 1, (long long)nwk, 1.0, 0.0));  // V^T A2
			gemm(c, mk(jb, n2, jb, Tp, 1, jb, (long long)nb2, W1, n2, 1, (long long)nwk, W2, n2, 1, (long long)nwk, 1.0,
			           0.0));  // T^T W1
			gemm(c, mk(mp, n2, jb, Vp, jb, 1, lv, W2, n2, 1, (long long)nwk, A2, nw, 1, la2, -1.0, 1.0));  // A2 -= V W2
			// R_12: the panel rows of the updated trailing columns
			k_copy2d<<<grid_for(size_t(jb) * n2), 256, 0, c.stream>>>(a.C + j0 * csr + (j0 + jb) * csc, csr, csc, A2, nw,
			                                                          1, jb, n2);
			XTT_CUDA(cudaGetLastError());
			c.count_launch();
		}
	}
	// Q_w[i][col] at a.Q[i qsr + col qsc]: tr == 0, Q (m x k) ld k; tr == 1, Q^T (k x n) ld n
	const long long qsr = tr ? 1 : kq, qsc = tr ? mw : 1, lq = (long long)mw * kq;
	k_eye_rect<<<grid_for(size_t(mw) * kq), 256, 0, c.stream>>>(a.Q, mw, kq, qsr, qsc);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	for (int p = np - 1; p >= 0; --p) {
		const int j0 = p * kQbBlock, jb = std::min(kQbBlock, kq - j0), mr = mw - j0, nc = kq - j0;
		const double* Vp = Vall + size_t(p) * mw * kQbBlock;
		const double* Tp = Tall + size_t(p) * nb2;
		const long long lv = (long long)mr * jb;
		double* Qb = a.Q + j0 * qsr + j0 * qsc;
		const long long lqb = lq - (j0 * qsr + j0 * qsc);
		gemm(c, mk(jb, nc, mr, Vp, 1, jb, lv, Qb, qsr, qsc, lqb, W1, nc, 1, (long long)nwk, 1.0, 0.0));  // V^T Q
		gemm(c, mk(jb, nc, jb, Tp, jb, 1, (long long)nb2, W1, nc, 1, (long long)nwk, W2, nc, 1, (long long)nwk, 1.0,
		           0.0));  // T W1
		gemm(c, mk(mr, nc, jb, Vp, jb, 1, lv, W2, nc, 1, (long long)nwk, Qb, qsr, qsc, lqb, -1.0, 1.0));  // Q -= V W2
	}
	return true;
}

// The rank-revealing QR of transfer_core / round: Cholesky QR where the context asks for
// it and the shape fits, the pivoted Householder QR otherwise or when its gate fails.
// Returns the rank when the host knows it already (the Cholesky QR keeps all columns),
// else -1: the rank is then in *a.rank_out (not synchronised).
static int rank_revealing_qr(Context& c, QrArgs& a) {
	if (!a.pivot) {
		ProfScope ps(c, "qr", qr_work_bytes(a), qr_work_flops(a));
		if (qr_blocked(c, a)) return std::min(a.m, a.n);
	}
	if (c.gram_qr && gram_qr_fits(a)) {
		ProfScope ps(c, "qr_gram", qr_work_bytes(a), qr_work_flops(a));
		int* flag = c.d_ints + 12;
		gram_qr(c, a, 0, flag);
		if (c.read_int(12) == 0) return a.transpose ? a.m : a.n;
	}
	ProfScope ps(c, "qr", qr_work_bytes(a), qr_work_flops(a));
	launch_qr(a, c.stream);
	c.count_launch();
	return -1;
}

void transfer_core(Tensor& x, int from, int to, bool rr) {
	Context& c = *x.ctx;
	const int64_t r0 = x.ranks[from], nf = x.n(from), r1 = x.ranks[from + 1];
	if (!rr) {
		// small cores: factorisation and absorption in one launch, ranks unchanged
		TransferArgs t;
		t.from = x.core[from];
		t.to = x.core[to];
		t.r0 = int(r0); t.nf = int(nf); t.r1 = int(r1);
		t.right = to == from + 1;
		t.rt = int(x.ranks[to]); t.nt = int(x.n(to)); t.r2 = int(x.ranks[to + 1]);
		if (transfer_narrow_fits(t) || transfer_small_fits(t)) {
			QrArgs q;  // for the declared work only
			q.m = t.right ? int(r0 * nf) : int(r0); q.n = t.right ? int(r1) : int(nf * r1); q.transpose = t.right ? 0 : 1;
			ProfScope ps(c, "qr", qr_work_bytes(q), qr_work_flops(q));
			// the narrow-core kernel where it fits (measured 28 vs 39 us for 48 x 6), else the
			// block one: on GB300 one warp issues its FP64 instructions one at a time (~64 cycles
			// each, no overlap within a warp); both spread independent columns over four warps
			if (transfer_narrow_fits(t)) launch_transfer_narrow(t, c.stream);
			else launch_transfer_small(t, c.stream);
			c.count_launch();
			return;
		}
	}
	QrArgs a;
	if (to == from + 1) {
		const int m = int(r0 * nf), n = int(r1), kq = std::min(m, n);
		double* Q = c.scratch<double>(S_QR_Q, size_t(m) * kq);
		double* C = c.scratch<double>(S_QR_C, size_t(kq) * n);
		const size_t wk = qr_work_doubles(m, n);
		a.A = x.core[from]; a.lda = n; a.m = m; a.n = n; a.transpose = 0; a.pivot = rr ? 1 : 0;
		a.work = wk ? c.scratch<double>(S_QR_WORK, wk) : nullptr;
		a.Q = Q; a.C = C; a.rank_out = c.d_ints;
		const int known = rank_revealing_qr(c, a);
		const int rank = known >= 0 ? known : rr ? c.read_int(0) : kq;
		const int64_t nt = x.n(to), r2 = x.ranks[to + 1];
		// new right neighbour: C (rank x r1) * core_to (r1 x nt*r2)
		double* T = c.scratch<double>(S_GEMM_A, size_t(rank) * nt * r2);
		Gemm<double> g;
		g.M = rank; g.N = int(nt * r2); g.K = int(r1);
		g.A = C; g.sAm = r1; g.sAk = 1;
		g.B = x.core[to]; g.sBk = nt * r2; g.sBn = 1;
		g.C = T; g.sCm = nt * r2; g.sCn = 1;
		g.lens((long long)kq * n, (long long)x.core_size(to), (long long)rank * nt * r2);
		gemm(c, g);
		x.reshape_core(from, r0, rank);
		copy_d2d(c, x.core[from], Q, size_t(m) * rank);
		x.reshape_core(to, rank, r2);
		copy_d2d(c, x.core[to], T, size_t(rank) * nt * r2);
	} else {
		XTT_REQUIRE(to + 1 == from, "transfer_core between non-neighbours");
		const int m = int(r0), n = int(nf * r1), kq = std::min(m, n);
		double* Q = c.scratch<double>(S_QR_Q, size_t(kq) * n);
		double* C = c.scratch<double>(S_QR_C, size_t(m) * kq);
		const size_t wk = qr_work_doubles(n, m);
		a.A = x.core[from]; a.lda = n; a.m = m; a.n = n; a.transpose = 1; a.pivot = rr ? 1 : 0;
		a.work = wk ? c.scratch<double>(S_QR_WORK, wk) : nullptr;
		a.Q = Q; a.C = C; a.rank_out = c.d_ints;
		const int known = rank_revealing_qr(c, a);
		const int rank = known >= 0 ? known : rr ? c.read_int(0) : kq;
		const int64_t rt = x.ranks[to], nt = x.n(to);
		// new left neighbour: core_to (rt*nt x r0) * C (r0 x rank)
		double* T = c.scratch<double>(S_GEMM_A, size_t(rt) * nt * rank);
		Gemm<double> g;
		g.M = int(rt * nt); g.N = rank; g.K = int(r0);
		g.A = x.core[to]; g.sAm = r0; g.sAk = 1;
		g.B = C; g.sBk = rank; g.sBn = 1;
		g.C = T; g.sCm = rank; g.sCn = 1;
		g.lens((long long)x.core_size(to), (long long)m * kq, (long long)rt * nt * rank);
		gemm(c, g);
		x.reshape_core(from, rank, r1);
		copy_d2d(c, x.core[from], Q, size_t(rank) * n);
		x.reshape_core(to, rt, rank);
		copy_d2d(c, x.core[to], T, size_t(rt) * nt * rank);
	}
}

void move_core(Tensor& x, int64_t pos, bool keep_rank) {
	// TTNetwork::move_core, src/xerus/ttNetwork.cpp:581-628
	XTT_REQUIRE(pos >= 0 && pos < x.d, "illegal core position");
	const int d = x.d;
	if (x.canonicalized) {
		for (int64_t n = x.core_position; n < pos; ++n) transfer_core(x, int(n), int(n + 1), !keep_rank);
		for (int64_t n = x.core_position; n > pos; --n) transfer_core(x, int(n), int(n - 1), !keep_rank);
	} else {
		for (int64_t n = 0; n < pos; ++n) transfer_core(x, int(n), int(n + 1), !keep_rank);
		for (int64_t n = d - 1; n > pos; --n) transfer_core(x, int(n), int(n - 1), !keep_rank);
	}
	while (exceeds_maximal_ranks(x)) {
		for (int64_t n = pos; n > 0; --n) transfer_core(x, int(n), int(n - 1), !keep_rank);
		for (int n = 0; n + 1 < d; ++n) transfer_core(x, n, n + 1, !keep_rank);
		for (int64_t n = d - 1; n > pos; --n) transfer_core(x, int(n), int(n - 1), !keep_rank);
	}
	x.canonicalized = true;
	x.core_position = pos;
}

// ------------------------------------------------------------ round

__global__ void k_f2d(double* out, const float* in, size_t n) {
	for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
		out[i] = double(in[i]);
}

// ------------------------------------------------------------ SVD refinement by products
// Square X = U Sigma V^T from approximate factors (the FP32 Jacobi's V, U from X V) by the
// Newton-type refinement of Ogita and Aishima ("Iterative refinement for singular value
// decomposition based on matrix multiplication", J. Comput. Appl. Math. 369, 2020): with
// U = U^(I + F), V = V^(I + G), the conditions U^T U = I, V^T V = I and U^T X V = Sigma,
// to first order in F and G, give for R = I - U^T U, S = I - V^T V, T = U^T X V:
//   sigma_i = T_ii / (1 - (R_ii + S_ii) / 2),  F_ii = R_ii / 2,  G_ii = S_ii / 2,
//   F_ij = (a s_j + b s_i) / (s_j^2 - s_i^2),  G_ij = (a s_i + b s_j) / (s_j^2 - s_i^2)
//   with a = T_ij + s_j R_ij, b = T_ji + s_j S_ij (i != j).
// Each step is four FP64 products (U^T U and V^T V as one batched launch) and an
// elementwise kernel, with no rotation sweeps (each of whose steps ends in a barrier).
// The error squares per step: the FP32 start (~1e-4 in the vectors, FP32 rounding over
// the relative gaps) reaches FP64 rounding in three. Near-equal or near-zero singular
// values, where first-order corrections are not small, and a last step whose corrections
// are still above 1e-9 set a flag: the caller then runs the FP64 Jacobi sweeps instead.
constexpr int kOaSteps = 3;

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

// Columns of Y = X V normalised into U (both q x q row-major); a zero column sets the flag.
__global__ void k_oa_normalize(const double* Y, double* U, int q, int* flag) {
	const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
	for (int c = blockIdx.x * warps + (threadIdx.x >> 5); c < q; c += gridDim.x * warps) {
		double s = 0;
		for (int i = lane; i < q; i += 32) s = fma(Y[(long long)i * q + c], Y[(long long)i * q + c], s);
		s = sqrt(warp_sum(s));
		if (!(s > 0.0)) {
			if (lane == 0) atomicExch(flag, 1);
			continue;
		}
		const double inv = 1.0 / s;
		for (int i = lane; i < q; i += 32) U[(long long)i * q + c] = Y[(long long)i * q + c] * inv;
	}
}

// PQ = [U^T U | V^T V], T = U^T X V (q x q each). One row i per block (grid-stride):
// sigma_i into sig, rows i of I + F and I + G into FG = [I + F | I + G]. The flag is set
// for a relative gap below 1e-5, a singular value below 1e-13 of the largest, or (last
// step) a correction above 1e-9.
__global__ void k_oa_correct(const double* PQ, const double* T, double* FG, double* sig, int q, int last, int* flag) {
	extern __shared__ double s_sig[];
	__shared__ double s_max[32];
	const long long qq = (long long)q * q;
	const double* P = PQ;
	const double* Qm = PQ + qq;
	for (int j = threadIdx.x; j < q; j += blockDim.x) {
		const double r = 1.0 - P[(long long)j * q + j], t = 1.0 - Qm[(long long)j * q + j];
		s_sig[j] = T[(long long)j * q + j] / (1.0 - 0.5 * (r + t));
	}
	__syncthreads();
	double mx = 0;
	for (int j = threadIdx.x; j < q; j += blockDim.x) mx = fmax(mx, fabs(s_sig[j]));
	mx = warp_max(mx);
	if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
	__syncthreads();
	double smax = 0;
	for (int w = 0; w < int(blockDim.x >> 5); ++w) smax = fmax(smax, s_max[w]);
	int bad = 0;
	for (int i = blockIdx.x; i < q; i += gridDim.x) {
		const double si = s_sig[i];
		if (threadIdx.x == 0) {
			sig[i] = si;
			if (!(si > 1e-13 * smax)) bad = 1;
		}
		for (int j = threadIdx.x; j < q; j += blockDim.x) {
			const long long ij = (long long)i * q + j, ji = (long long)j * q + i;
			double f, g;
			if (i == j) {
				f = 0.5 * (1.0 - P[ij]);
				g = 0.5 * (1.0 - Qm[ij]);
			} else {
				const double sj = s_sig[j], dif = sj - si;
				if (!(fabs(dif) > 1e-5 * fmax(fabs(si), fabs(sj)))) {
					bad = 1;
					f = g = 0.0;
				} else {
					const double a = T[ij] - sj * P[ij], b = T[ji] - sj * Qm[ij], inv = 1.0 / (dif * (sj + si));
					f = (a * sj + b * si) * inv;
					g = (a * si + b * sj) * inv;
				}
			}
			if (last && (fabs(f) > 1e-9 || fabs(g) > 1e-9)) bad = 1;
			FG[ij] = f + (i == j ? 1.0 : 0.0);
			FG[qq + ij] = g + (i == j ? 1.0 : 0.0);
		}
	}
	if (bad) atomicExch(flag, 1);
}

// Sort descending, the reference's truncation (rank cap, first j >= 1 with S_j <= eps S_0),
// the sign gauge (largest |entry| of each kept left vector positive, first on ties), and
// U (m x rank), S, V^T (rank x n); nothing when the flag is set.
__global__ void k_oa_finish(const double* UV, const double* sig_g, int q, SvdArgs a, const int* flag) {
	if (*flag) return;
	extern __shared__ double s_fin[];  // sigma (q doubles), then the order (q ints)
	double* sig = s_fin;
	int* s_order = reinterpret_cast<int*>(s_fin + q);
	__shared__ int s_rank;
	__shared__ double s_sign[1024];
	const double* Uh = UV;
	const double* Vh = UV + (long long)q * q;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	for (int c = tid; c < q; c += blockDim.x) sig[c] = sig_g[c];
	__syncthreads();
	for (int c = tid; c < q; c += blockDim.x) {
		int pos = 0;
		for (int o = 0; o < q; ++o) pos += (sig[o] > sig[c]) || (sig[o] == sig[c] && o < c);
		s_order[pos] = c;
	}
	__syncthreads();
	if (tid == 0) {
		int rank = q;
		if (a.max_rank > 0 && a.max_rank < rank) rank = a.max_rank;
		const double s0 = sig[s_order[0]];
		for (int j = 1; j < rank; ++j)
			if (sig[s_order[j]] <= a.eps * s0) { rank = j; break; }
		s_rank = rank;
		if (a.rank_out) *a.rank_out = rank;
	}
	__syncthreads();
	const int rank = s_rank;
	for (int k = warp; k < rank; k += nwarps) {
		const int c = s_order[k];
		double best = -1.0, val = 0.0;
		int bi = 1 << 30;
		for (int i = lane; i < q; i += 32) {
			const double u = Uh[(long long)i * q + c];
			if (fabs(u) > best) { best = fabs(u); val = u; bi = i; }
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			const double ob = __shfl_xor_sync(0xffffffffu, best, o);
			const double ov = __shfl_xor_sync(0xffffffffu, val, o);
			const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
			if (ob > best || (ob == best && oi < bi)) { best = ob; val = ov; bi = oi; }
		}
		if (lane == 0) s_sign[k] = val < 0.0 ? -1.0 : 1.0;
	}
	__syncthreads();
	for (int k = tid; k < rank; k += blockDim.x) a.S[k] = sig[s_order[k]];
	for (int i = warp; i < q; i += nwarps)  // rows by warp, columns by lane
		for (int k = lane; k < rank; k += 32) a.U[(long long)i * rank + k] = s_sign[k] * Uh[(long long)i * q + s_order[k]];
	for (int k = warp; k < rank; k += nwarps)
		for (int j = lane; j < q; j += 32) a.Vt[(long long)k * q + j] = s_sign[k] * Vh[(long long)j * q + s_order[k]];
}

// C = A B for q x q row-major operands (A transposed when ta), `batch` pairs at stride q^2.
static Gemm<double> sq_gemm(int q, const double* A, bool ta, long long lda, const double* B, double* C, int batch = 1) {
	const long long qq = (long long)q * q;
	Gemm<double> g;
	g.M = q; g.N = q; g.K = q; g.batch = batch;
	g.A = A; g.sAm = ta ? 1 : lda; g.sAk = ta ? lda : 1; g.sAb = qq;
	g.B = B; g.sBk = q; g.sBn = 1; g.sBb = qq;
	g.C = C; g.sCm = q; g.sCn = 1; g.sCb = qq;
	g.lens((batch - 1) * qq + (long long)(q - 1) * lda + q, batch * qq, batch * qq);
	return g;
}

// X (q x q, leading dimension a.ldx) from W (the FP32 Jacobi's right factor, FP64):
// kOaSteps refinement steps, then the outputs of `a`. `ok` false (nothing written) if
// the flag was set; `rank` the kept rank when it was read with the flag (-1 otherwise).
struct RefineResult {
	bool ok;
	int rank;
};
static RefineResult svd_refine_square(Context& c, const SvdArgs& a, const double* W, int q) {
	XTT_REQUIRE(q <= 1024, "internal: refinement sized for q <= 1024");
	const size_t qq = size_t(q) * q;
	double* UV = c.scratch<double>(S_SVD_RF_U, 2 * qq);    // [U | V]
	double* UV2 = c.scratch<double>(S_SVD_RF_V, 2 * qq);   // the next [U | V]
	double* M = c.scratch<double>(S_SVD_RF_M, 6 * qq + q);  // [P | Q], Z, T, [I + F | I + G], sigma
	double *PQ = M, *Z = M + 2 * qq, *T = M + 3 * qq, *FG = M + 4 * qq, *sig = M + 6 * qq;
	int* flag = c.d_ints + 6;
	XTT_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), c.stream));
	copy_d2d(c, UV + qq, W, qq);
	gemm(c, sq_gemm(q, a.X, false, a.ldx, UV + qq, Z));  // Y = X V
	k_oa_normalize<<<std::max(1, q / 8), 256, 0, c.stream>>>(Z, UV, q, flag);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	for (int it = 0; it < kOaSteps; ++it) {
		gemm(c, sq_gemm(q, UV, true, q, UV, PQ, 2));       // [U^T U | V^T V]
		gemm(c, sq_gemm(q, a.X, false, a.ldx, UV + qq, Z));  // X V
		gemm(c, sq_gemm(q, UV, true, q, Z, T));              // U^T X V
		k_oa_correct<<<std::min(q, 64), 128, size_t(q) * sizeof(double), c.stream>>>(PQ, T, FG, sig, q,
		                                                                               it == kOaSteps - 1, flag);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
		gemm(c, sq_gemm(q, UV, false, q, FG, UV2, 2));  // [U (I + F) | V (I + G)]
		std::swap(UV, UV2);
	}
	k_oa_finish<<<1, 256, size_t(q) * (sizeof(double) + sizeof(int)), c.stream>>>(UV, sig, q, a, flag);
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	// one host read for the flag and, where it is a context int, the rank
	const long long ri = a.rank_out ? (long long)(a.rank_out - c.d_ints) : -1;
	if (ri >= 0 && ri < 64) {
		c.read_ints(int(std::min<long long>(ri, 6)), int(std::max<long long>(ri, 6)) + 1);
		return {c.h_ints[6] == 0, c.h_ints[6] == 0 ? c.h_ints[ri] : -1};
	}
	return {c.read_int(6) == 0, -1};
}

// One-sided Jacobi of a.X (through launch_svd). Mixed precision where it fits (svd_path
// AUTO, columns orthogonalised, 32..: one CTA holds the matrix in FP32): FP32 sweeps to
// FP32 orthogonality in one CTA give a rotation W32. Square X: the product refinement
// above takes it to FP64 accuracy. Otherwise (or when the refinement flags its input):
// two Newton-Schulz steps in FP64, W <- 1.5 W - 0.5 W (W^T W), make it orthogonal to
// rounding (each squares the 1e-7 defect); the FP64 cluster Jacobi then starts from X W
// with V = W and needs only the few sweeps of its quadratic phase. Same singular values,
// truncation and gauge.
// `mixed` false: plain FP64 Jacobi (after the QR preconditioning, whose R^T already
// converges in 6-10 sweeps, the FP32 stage measured slower than it saves).
static int jacobi(Context& c, SvdArgs& a, bool mixed) {
	const bool tall = a.m > a.n || (a.m == a.n && !a.orth_rows);
	const int p = tall ? a.m : a.n, q = tall ? a.n : a.m;
	if (mixed && c.svd_path == XTT_SVD_PATH_AUTO && tall && !a.V0 && q >= 32 && svd_f32_fits(p, q)) {
		Fp64ContractionScope fp64(c);
		const size_t qq = size_t(q) * q;
		float* w32 = c.scratch<float>(S_SVD_MX_W32, qq);
		{
			ProfScope ps(c, "svd_f32");
			launch_svd_f32(a.X, a.ldx, p, q, w32, c.stream);
		}
		double* W = c.scratch<double>(S_SVD_MX_W, qq);
		double* W2 = c.scratch<double>(S_SVD_MX_W2, qq);
		double* G = c.scratch<double>(S_SVD_MX_G, qq);
		k_f2d<<<unsigned(std::min<size_t>(1024, (qq + 255) / 256)), 256, 0, c.stream>>>(W, w32, qq);
		c.count_launch(2);
		XTT_CUDA(cudaGetLastError());
		// square: refine the FP32 factors by products instead of Jacobi sweeps
		if (p == q && q <= 1024) {
			ProfScope ps(c, "svd_refine");
			const RefineResult rr = svd_refine_square(c, a, W, q);
			if (rr.ok) return rr.rank;
		}
		ProfScope ps(c, "svd_sweeps");
		for (int it = 0; it < 2; ++it) {
			Gemm<double> g1;  // G = W^T W
			g1.M = q; g1.N = q; g1.K = q;
			g1.A = W; g1.sAm = 1; g1.sAk = q;
			g1.B = W; g1.sBk = q; g1.sBn = 1;
			g1.C = G; g1.sCm = q; g1.sCn = 1;
			g1.lens((long long)qq, (long long)qq, (long long)qq);
			gemm(c, g1);
			copy_d2d(c, W2, W, qq);
			Gemm<double> g2;  // W2 = 1.5 W - 0.5 W G
			g2.M = q; g2.N = q; g2.K = q;
			g2.A = W; g2.sAm = q; g2.sAk = 1;
			g2.B = G; g2.sBk = q; g2.sBn = 1;
			g2.C = W2; g2.sCm = q; g2.sCn = 1;
			g2.alpha = -0.5; g2.beta = 1.5;
			g2.lens((long long)qq, (long long)qq, (long long)qq);
			gemm(c, g2);
			std::swap(W, W2);
		}
		double* B0 = c.scratch<double>(S_SVD_MX_B0, size_t(p) * q);
		Gemm<double> g3;  // B0 = X W
		g3.M = p; g3.N = q; g3.K = q;
		g3.A = a.X; g3.sAm = a.ldx; g3.sAk = 1;
		g3.B = W; g3.sBk = q; g3.sBn = 1;
		g3.C = B0; g3.sCm = q; g3.sCn = 1;
		g3.lens((long long)(p - 1) * a.ldx + q, (long long)qq, (long long)p * q);
		gemm(c, g3);
		SvdArgs b = a;
		b.X = B0;
		b.ldx = q;
		b.m = p;
		b.n = q;
		b.orth_rows = 0;
		b.V0 = W;
		const size_t wk = svd_work_doubles(p, q);
		b.work = wk ? c.scratch<double>(S_SVD_WORK, wk) : nullptr;
		launch_svd(b, c.stream);
		c.count_launch();
		return -1;
	}
	const size_t wk = svd_work_doubles(a.m, a.n);
	a.work = wk ? c.scratch<double>(S_SVD_WORK, wk) : nullptr;
	launch_svd(a, c.stream);
	c.count_launch();
	return -1;
}

int run_svd(Context& c, SvdArgs& a, bool graded) {
	ProfScope ps(c, "svd");
	if (graded && c.svd_path == XTT_SVD_PATH_AUTO && svd_pc_fits(a.m, a.n)) {
		size_t nq, nc, nqr, nsv;
		svd_pc_workspace(a.m, a.n, nq, nc, nqr, nsv);
		SvdPcWork w;
		w.q = c.scratch<double>(S_SVD_PC_Q, nq);
		w.c = c.scratch<double>(S_SVD_PC_C, nc);
		(a.m >= a.n ? w.u : w.vt) = c.scratch<double>(S_SVD_PC_UV, nc);
		if (a.m >= a.n) {
			w.ct = c.scratch<double>(S_SVD_PC_CT, nc);
			w.ut = c.scratch<double>(S_SVD_PC_UT, nc);
		}
		w.qr_work = nqr ? c.scratch<double>(S_SVD_PC_QRW, nqr) : nullptr;
		w.svd_work = nsv ? c.scratch<double>(S_SVD_WORK, nsv) : nullptr;
		launch_svd_pc_qr(a, w, c.d_ints + 4, c.stream);
		const int kept = c.read_int(4);  // rows of the pivoted R the Jacobi phase needs
		SvdArgs sa = svd_pc_jacobi(a, w, kept, c.stream);
		jacobi(c, sa, false);
		svd_pc_finish(a, w, kept, c.stream);
		c.count_launch(3);
		return -1;
	}
	return jacobi(c, a, true);
}

static int svd_into(Context& c, const double* X, int m, int n, int max_rank, double eps, double*& U, double*& S,
                    double*& Vt) {
	const int q = std::min(m, n);
	U = c.scratch<double>(S_SVD_U, size_t(m) * q);
	S = c.scratch<double>(S_SVD_S, size_t(q));
	Vt = c.scratch<double>(S_SVD_VT, size_t(q) * n);
	SvdArgs a;
	a.X = X; a.ldx = n; a.m = m; a.n = n; a.max_rank = max_rank; a.eps = eps;
	a.U = U; a.S = S; a.Vt = Vt; a.rank_out = c.d_ints + 1; a.status = c.d_status;
	const int known = run_svd(c, a);
	return known >= 0 ? known : c.read_int(1);
}

__global__ void k_eye(double* I, int n) {
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x)
		I[e] = e / n == e % n ? 1.0 : 0.0;
}

// to_orth: core `to` has orthonormal columns (round's left-orthogonalised cores). Its QC is
// then T = T I (Q_T = T, C_B = I, full rank: the reference's pivoted QR of such a matrix has
// |R_kk| = 1 and keeps every column), and only F is factored.
static void round_edge(Tensor& x, int from, int to, int64_t max_rank, double eps, std::vector<double>* spectra,
                       bool to_orth) {
	// TensorNetwork::round_edge (src/xerus/tensorNetwork.cpp:678-818) for from = core k+1, to = core k.
	Context& c = *x.ctx;
	const int64_t r = x.ranks[from], nF = x.n(from), rF = x.ranks[from + 1];
	const int64_t rT = x.ranks[to], nT = x.n(to);
	const double sizeF = double(r * nF * rF), sizeT = double(rT * nT * r);
	const int mr = max_rank >= (int64_t(1) << 31) - 1 ? 0 : int(max_rank);
	double *U, *S, *Vt;
	int s;
	if (5.0 * sizeF * sizeT >= 6.0 * std::pow(double(r), 4)) {
		// F = C_A Q_F (CQ), T = Q_T C_B (QC), X = C_A^T C_B^T
		QrArgs a;
		const int mF = int(r), nFc = int(nF * rF);
		double* CA = c.scratch<double>(S_ROUND_CA, size_t(mF) * std::min(mF, nFc));
		double* QF = c.scratch<double>(S_ROUND_QA, size_t(std::min(mF, nFc)) * nFc);
		size_t wk = qr_work_doubles(nFc, mF);
		a.A = x.core[from]; a.lda = nFc; a.m = mF; a.n = nFc; a.transpose = 1; a.pivot = 1;
		a.work = wk ? c.scratch<double>(S_QR_WORK, wk) : nullptr;
		a.Q = QF; a.C = CA; a.rank_out = c.d_ints + 2;
		// the two factorisations are independent: T's on the aux stream, F's on the main one
		c.fork();
		const int mT = int(rT * nT), nTc = int(r);
		const bool skip_b = to_orth && mT >= nTc;
		double* QT = skip_b ? x.core[to] : c.scratch<double>(S_ROUND_QB, size_t(mT) * std::min(mT, nTc));
		double* CB = c.scratch<double>(S_ROUND_CB, size_t(std::min(mT, nTc)) * nTc);
		wk = qr_work_doubles(mT, nTc);
		QrArgs b;
		b.A = x.core[to]; b.lda = nTc; b.m = mT; b.n = nTc; b.transpose = 0; b.pivot = 1;
		b.work = wk ? c.scratch<double>(S_ROUND_X, wk) : nullptr;  // not S_QR_WORK: runs beside a
		b.Q = QT; b.C = CB; b.rank_out = c.d_ints + 3;
		const bool gb = !skip_b && c.gram_qr && gram_qr_fits(b), ga = c.gram_qr && gram_qr_fits(a);
		if (skip_b) {
			k_eye<<<unsigned((nTc * nTc + 255) / 256), 256, 0, c.stream>>>(CB, nTc);
			XTT_CUDA(cudaGetLastError());
			c.count_launch();
		}
		if (!skip_b) {
			OnAux aux(c);
			if (gb) {
				ProfScope ps(c, "qr_gram", qr_work_bytes(b), qr_work_flops(b));
				gram_qr(c, b, 1, c.d_ints + 13);
			} else {
				ProfScope ps(c, "qr", qr_work_bytes(b), qr_work_flops(b));
				launch_qr(b, c.stream);
				c.count_launch();
			}
		}
		if (ga) {
			ProfScope ps(c, "qr_gram", qr_work_bytes(a), qr_work_flops(a));
			gram_qr(c, a, 0, c.d_ints + 12);
		} else {
			ProfScope ps(c, "qr", qr_work_bytes(a), qr_work_flops(a));
			launch_qr(a, c.stream);
			c.count_launch();
		}
		c.join();
		// one read for the ranks and the Cholesky QRs' gates; a gate that failed: the pivoted
		// Householder QR instead, and its rank
		c.read_ints(2, 14);
		bool again = false;
		if (ga && c.h_ints[12]) {
			ProfScope ps(c, "qr", qr_work_bytes(a), qr_work_flops(a));
			launch_qr(a, c.stream);
			c.count_launch();
			again = true;
		}
		if (gb && c.h_ints[13]) {
			ProfScope ps(c, "qr", qr_work_bytes(b), qr_work_flops(b));
			launch_qr(b, c.stream);
			c.count_launch();
			again = true;
		}
		if (again) c.read_ints(2, 4);
		const int ka = c.h_ints[2], kb = skip_b ? nTc : c.h_ints[3];
		double* X = c.scratch<double>(S_GEMM_B, size_t(ka) * kb);
		Gemm<double> g;
		g.M = ka; g.N = kb; g.K = int(r);
		g.A = CA; g.sAm = 1; g.sAk = ka;
		g.B = CB; g.sBk = 1; g.sBn = r;
		g.C = X; g.sCm = kb; g.sCn = 1;
		g.lens((long long)mF * std::min(mF, nFc), (long long)std::min(mT, nTc) * nTc, (long long)ka * kb);
		gemm(c, g);
		s = svd_into(c, X, ka, kb, mr, eps, U, S, Vt);
		// coreB = S Vt ; F' = U^T Q_F ; T' = Q_T coreB^T
		scale_rows(c, Vt, S, s, kb);
		double* Fn = c.scratch<double>(S_RES_CORE0, size_t(s) * nFc);
		Gemm<double> gf;
		gf.M = s; gf.N = nFc; gf.K = ka;
		gf.A = U; gf.sAm = 1; gf.sAk = s;
		gf.B = QF; gf.sBk = nFc; gf.sBn = 1;
		gf.C = Fn; gf.sCm = nFc; gf.sCn = 1;
		gf.lens((long long)ka * std::min(ka, kb), (long long)std::min(mF, nFc) * nFc, (long long)s * nFc);
		gemm(c, gf);
		double* Tn = c.scratch<double>(S_RES_CORE1, size_t(mT) * s);
		Gemm<double> gt;
		gt.M = mT; gt.N = s; gt.K = kb;
		gt.A = QT; gt.sAm = kb; gt.sAk = 1;
		gt.B = Vt; gt.sBk = 1; gt.sBn = kb;
		gt.C = Tn; gt.sCm = s; gt.sCn = 1;
		gt.lens((long long)mT * std::min(mT, nTc), (long long)std::min(ka, kb) * kb, (long long)mT * s);
		gemm(c, gt);
		x.reshape_core(from, s, rF);
		copy_d2d(c, x.core[from], Fn, size_t(s) * nFc);
		x.reshape_core(to, rT, s);
		copy_d2d(c, x.core[to], Tn, size_t(mT) * s);
	} else {
		// X = F^T T^T : (nF rF) x (rT nT)
		const int mX = int(nF * rF), nX = int(rT * nT);
		double* X = c.scratch<double>(S_GEMM_B, size_t(mX) * nX);
		Gemm<double> g;
		g.M = mX; g.N = nX; g.K = int(r);
		g.A = x.core[from]; g.sAm = 1; g.sAk = nF * rF;
		g.B = x.core[to]; g.sBk = 1; g.sBn = r;
		g.C = X; g.sCm = nX; g.sCn = 1;
		g.lens((long long)x.core_size(from), (long long)x.core_size(to), (long long)mX * nX);
		gemm(c, g);
		s = svd_into(c, X, mX, nX, mr, eps, U, S, Vt);
		x.reshape_core(from, s, rF);
		k_cab<<<grid_for(size_t(mX) * s), 256, 0, c.stream>>>(x.core[from], U, int(nF), int(rF), s);
		x.reshape_core(to, rT, s);
		k_transpose_scale<<<grid_for(size_t(nX) * s), 256, 0, c.stream>>>(x.core[to], Vt, S, s, nX);
		c.count_launch(2);
	}
	XTT_CUDA(cudaGetLastError());
	if (spectra) {
		std::vector<double> h(s);
		XTT_CUDA(cudaMemcpyAsync(h.data(), S, sizeof(double) * s, cudaMemcpyDeviceToHost, c.stream));
		c.sync();
		spectra->insert(spectra->end(), h.begin(), h.end());
	}
}

void round_tt(Tensor& x, const std::vector<int64_t>& max_ranks, double eps, std::vector<double>* spectra) {
	// TTNetwork::round(maxRanks, eps), src/xerus/ttNetwork.cpp:643-665
	XTT_REQUIRE(eps < 1.0 && eps >= 0.0, "_eps must be in [0, 1)");
	XTT_REQUIRE(int(max_ranks.size()) + 1 == x.d, "there must be exactly order-1 maxRanks");
	for (auto m : max_ranks) XTT_REQUIRE(m > 0, "rounding to rank 0 is not possible");
	const bool init_canon = x.canonicalized;
	const int64_t init_pos = x.core_position;
	const int d = x.d;
	GramQrScope gram(*x.ctx);
	move_core(x, d - 1, false);
	// after move_core(d - 1) every core left of the one being truncated has orthonormal columns
	for (int i = 0; i + 1 < d; ++i) round_edge(x, d - 1 - i, d - 2 - i, max_ranks[d - 2 - i], eps, spectra, true);
	x.canonicalized = true;
	x.core_position = 0;
	if (init_canon) move_core(x, init_pos, false);
}

// ------------------------------------------------------------ contractions

// Zipper M_k = sum over cores 0..k-1 of x (x) y; returns <x, y>.
double dot(const Tensor& x, const Tensor& y) {
	XTT_REQUIRE(x.d == y.d && x.dims == y.dims && x.op == y.op, "dot of tensors with different dimensions");
	Context& c = *x.ctx;
	int64_t maxr = 1;
	for (int k = 0; k <= x.d; ++k) maxr = std::max({maxr, x.ranks[k], y.ranks[k]});
	int64_t maxn = 1;
	for (int k = 0; k < x.d; ++k) maxn = std::max(maxn, x.n(k));
	double* M = c.scratch<double>(S_ZIP_M, size_t(maxr) * maxr);
	double* M2 = c.scratch<double>(S_ZIP_M2, size_t(maxr) * maxr);
	double* T = c.scratch<double>(S_ZIP_T, size_t(maxr) * maxn * maxr);
	fill(c, M, 1.0, 1);
	for (int k = 0; k < x.d; ++k) {
		const int64_t rx = x.ranks[k], rx1 = x.ranks[k + 1], ry = y.ranks[k], ry1 = y.ranks[k + 1], n = x.n(k);
		Gemm<double> g;  // T[b][(i, a')] = sum_a M[a][b] x[a][(i, a')]
		g.M = int(ry); g.N = int(n * rx1); g.K = int(rx);
		g.A = M; g.sAm = 1; g.sAk = ry;
		g.B = x.core[k]; g.sBk = n * rx1; g.sBn = 1;
		g.C = T; g.sCm = n * rx1; g.sCn = 1;
		g.lens(maxr * maxr, (long long)x.core_size(k), maxr * maxn * maxr);
		gemm(c, g);
		Gemm<double> h;  // M'[a'][b'] = sum_{(b,i)} T[(b,i)][a'] y[(b,i)][b']
		h.M = int(rx1); h.N = int(ry1); h.K = int(ry * n);
		h.A = T; h.sAm = 1; h.sAk = rx1;
		h.B = y.core[k]; h.sBk = ry1; h.sBn = 1;
		h.C = M2; h.sCm = ry1; h.sCn = 1;
		h.lens(maxr * maxn * maxr, (long long)y.core_size(k), maxr * maxr);
		gemm(c, h);
		std::swap(M, M2);
	}
	XTT_CUDA(cudaMemcpyAsync(c.h_dbl, M, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	return c.h_dbl[0];
}

double frob_norm(const Tensor& x) {
	// TTNetwork::frob_norm, src/xerus/ttNetwork.cpp:781-789
	if (x.canonicalized) {
		Context& c = *x.ctx;
		const int k = int(x.core_position);
		sumsq_async(c, x.core[k], x.core_size(k), 0);
		return std::sqrt(read_dbl(c, 0));
	}
	return std::sqrt(dot(x, x));
}

double orthogonal_norm(Tensor& x) {
	for (int k = 0; k + 1 < x.d; ++k) transfer_core(x, k, k + 1, false);
	x.canonicalized = true;
	x.core_position = x.d - 1;
	Context& c = *x.ctx;
	sumsq_async(c, x.core[x.d - 1], x.core_size(x.d - 1), 0);
	return std::sqrt(read_dbl(c, 0));
}

// y[(K,a), i, (L,b)] = sum_j A[K,i,j,L] x[a,j,b]
__global__ void k_op_apply(double* y, const double* A, const double* x, int K, int L, int n, int ra, int rb) {
	const size_t total = size_t(K) * ra * n * L * rb;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
		size_t t = e;
		const int b = int(t % rb); t /= rb;
		const int l = int(t % L); t /= L;
		const int i = int(t % n); t /= n;
		const int a = int(t % ra); t /= ra;
		const int k = int(t);
		double s = 0;
		for (int j = 0; j < n; ++j)
			s += A[((size_t(k) * n + i) * n + j) * L + l] * x[(size_t(a) * n + j) * rb + b];
		y[e] = s;
	}
}

void op_apply_tt(const Tensor& A, const Tensor& x, Tensor& y) {
	XTT_REQUIRE(A.op && !x.op && A.d == x.d && A.dims == x.dims, "operator and tensor dimensions differ");
	Context& c = *x.ctx;
	for (int k = 0; k < x.d; ++k) {
		const int K = int(A.ranks[k]), L = int(A.ranks[k + 1]), ra = int(x.ranks[k]), rb = int(x.ranks[k + 1]);
		const int n = int(x.dims[k]);
		y.reshape_core(k, int64_t(K) * ra, int64_t(L) * rb);
		k_op_apply<<<grid_for(y.core_size(k)), 256, 0, c.stream>>>(y.core[k], A.core[k], x.core[k], K, L, n, ra, rb);
		c.count_launch();
	}
	XTT_CUDA(cudaGetLastError());
	y.canonicalized = false;
}

// One core of the operator product A B (TTStack<true> contracted, src/xerus/ttStack.cpp:47-173):
// C((k l), i, j, (k' l')) = sum_m A(k, i, m, k') B(l, m, j, l').
__global__ void k_op_op(double* C, const double* A, const double* B, int K, int L, int Kb, int Lb, int n) {
	const size_t total = size_t(K) * Kb * n * n * L * Lb;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
		size_t t = e;
		const int l2 = int(t % Lb); t /= Lb;
		const int k2 = int(t % L); t /= L;
		const int j = int(t % n); t /= n;
		const int i = int(t % n); t /= n;
		const int l = int(t % Kb);
		const int k = int(t / Kb);
		double s = 0;
		for (int m = 0; m < n; ++m)
			s = fma(A[((size_t(k) * n + i) * n + m) * L + k2], B[((size_t(l) * n + m) * n + j) * Lb + l2], s);
		C[e] = s;
	}
}

void tt_apply(const Tensor& A, const Tensor& x, Tensor& y) {
	// A(i/2, j/2) * x(j&0) cast to a TT (TTStack, src/xerus/ttStack.cpp:47-173; specialised
	// contraction, src/xerus/ttNetwork.cpp:886-967): core ranks R_k r_k, and the result is
	// canonicalised (rank-revealing move_core) at A's core position when A is canonical.
	XTT_REQUIRE(A.op && A.d == x.d && A.dims == x.dims && y.d == x.d && y.op == x.op && y.dims == x.dims,
	            "operator and tensor dimensions differ");
	Context& c = *x.ctx;
	if (!x.op) {
		op_apply_tt(A, x, y);
	} else {
		for (int k = 0; k < x.d; ++k) {
			const int K = int(A.ranks[k]), L = int(A.ranks[k + 1]), Kb = int(x.ranks[k]), Lb = int(x.ranks[k + 1]);
			const int n = int(x.dims[k]);
			y.reshape_core(k, int64_t(K) * Kb, int64_t(L) * Lb);
			k_op_op<<<grid_for(y.core_size(k)), 256, 0, c.stream>>>(y.core[k], A.core[k], x.core[k], K, L, Kb, Lb, n);
			c.count_launch();
		}
		XTT_CUDA(cudaGetLastError());
	}
	y.canonicalized = false;
	if (A.canonicalized) move_core(y, A.core_position, false);
}

// Block core of p + f q (TT sum, src/xerus/ttNetwork.cpp:796-847): out (P0+Q0 or 1, n, P1+Q1 or 1)
// with p in the leading block and q in the trailing one, q scaled by f in the first core.
__global__ void k_block_core(double* out, const double* p, const double* q, int P0, int P1, int Q0, int Q1, int n,
                             int first, int last, double f) {
	const int O0 = first ? 1 : P0 + Q0, O1 = last ? 1 : P1 + Q1;
	const size_t total = size_t(O0) * n * O1;
	for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
		const int o1 = int(e % O1);
		const int i = int((e / O1) % n);
		const int o0 = int(e / (size_t(O1) * n));
		double v = 0;
		// p block at (0.., 0..)
		if (o0 < P0 && o1 < P1) v += p[(size_t(o0) * n + i) * P1 + o1];
		const int q0 = first ? o0 : o0 - P0, q1 = last ? o1 : o1 - P1;
		if (q0 >= 0 && q0 < Q0 && q1 >= 0 && q1 < Q1) v += (first ? f : 1.0) * q[(size_t(q0) * n + i) * Q1 + q1];
		out[e] = v;
	}
}

void tt_add(Tensor& x, const Tensor& y, double f) {
	// x += f y (TTNetwork::operator+= / -=, src/xerus/ttNetwork.cpp:796-856): block cores of
	// ranks r + s; a canonical x is canonicalised again at its core position (rank-revealing
	// move_core), which can lower the ranks.
	XTT_REQUIRE(x.op == y.op && x.d == y.d && x.dims == y.dims, "The dimensions in TT sum must coincide");
	Context& c = *x.ctx;
	const int d = x.d;
	const bool canon = x.canonicalized;
	const int64_t pos = x.core_position;
	const std::vector<int64_t> xr = x.ranks;  // reshape_core below rewrites x.ranks as it goes
	for (int k = 0; k < d; ++k) {
		const int n = int(x.n(k));
		const int P0 = int(xr[k]), P1 = int(xr[k + 1]), Q0 = int(y.ranks[k]), Q1 = int(y.ranks[k + 1]);
		const int first = k == 0, last = k == d - 1;
		const int O0 = first ? 1 : P0 + Q0, O1 = last ? 1 : P1 + Q1;
		const size_t ny = size_t(O0) * n * O1;
		double* T = c.scratch<double>(S_GEMM_A, ny);
		k_block_core<<<grid_for(ny), 256, 0, c.stream>>>(T, x.core[k], y.core[k], P0, P1, Q0, Q1, n, first, last, f);
		c.count_launch();
		XTT_CUDA(cudaGetLastError());
		x.reshape_core(k, O0, O1);
		copy_d2d(c, x.core[k], T, ny);
	}
	x.canonicalized = false;
	if (canon && d > 1) move_core(x, pos, false);
	else if (canon) x.canonicalized = true;  // one component: component(0) += (ttNetwork.cpp:809-812)
}

double residual(const Tensor& A, const Tensor& x, const Tensor& b) { return residual(&A, x, b); }

// The residual's two-core meeting (below) where its GEMMs stay under this many flops.
constexpr double kResMeetMaxFlops = 2e8;

double residual(const Tensor* Ap, const Tensor& x, const Tensor& b) {
	// ||A x - b|| / ||b|| (src/xerus/algorithms/als.cpp:258-261; A null: ||x - b|| / ||b||,
	// als.cpp:301) without cancellation. The block
	// cores Y_k of y = A x - b (TT sum, src/xerus/ttNetwork.cpp:796-856) are formed one at a time
	// and orthogonalised from both ends at once: cores 0..mid-1 left to right on the context's
	// stream (Householder QR, only the triangular factor R is carried), cores d-1..mid+2 right to
	// left on the aux stream (LQ, only the factor L is carried). The two halves meet over the two
	// cores mid, mid+1 (mid = (d-2)/2, so the two chains are equally long and the widest
	// factorisation, the one a single meeting core would leave to one side, is not needed):
	// ||y|| = ||R Y_mid Y_mid+1 L||, three GEMMs; where that product would cost more than
	// kResMeetMaxFlops (large ranks), they meet over core d/2 alone: ||y|| = ||R Y_mid L||.
	// Neither the residual TT nor any orthogonal factor is stored.
	XTT_REQUIRE(x.dims == b.dims && !x.op && !b.op && (!Ap || (Ap->dims == x.dims && Ap->op)),
	            "x and b dimensions differ");
	Context& c = *x.ctx;
	const int d = x.d;
	const double nb = frob_norm(b);
	auto opr = [&](int k) -> int64_t { return Ap ? Ap->ranks[k] : 1; };
	size_t cap_core = 1, cap_r = 1;
	for (int k = 0; k < d; ++k) {
		const size_t p0 = size_t(opr(k) * x.ranks[k] + b.ranks[k]), p1 = size_t(opr(k + 1) * x.ranks[k + 1] + b.ranks[k + 1]);
		cap_core = std::max(cap_core, p0 * size_t(x.dims[k]) * p1);
		cap_r = std::max({cap_r, p0 * p1, p0 * p0, p1 * p1});
	}
	struct Bufs {
		double *ax, *Y, *Z, *R;
	};
	auto bufs = [&](int i0, int i1, int i2) {
		Bufs f;
		f.ax = c.scratch<double>(i0, cap_core);
		f.Y = c.scratch<double>(i1, cap_core);
		f.Z = c.scratch<double>(i2, 2 * cap_core + cap_r);
		f.R = f.Z + 2 * cap_core;
		return f;
	};
	const Bufs lb = bufs(S_RES_CORE0, S_RES_CORE1, S_RES_R), rb_ = bufs(S_RES_CORE0B, S_RES_CORE1B, S_RES_RB);
	struct Dims {
		int n, O0, O1;
	};
	// block core k of A x - b into f.Y on the current stream
	auto block = [&](int k, const Bufs& f) {
		const int K = int(opr(k)), L = int(opr(k + 1)), ra = int(x.ranks[k]), rb = int(x.ranks[k + 1]);
		const int n = int(x.dims[k]);
		const int P0 = K * ra, P1 = L * rb, Q0 = int(b.ranks[k]), Q1 = int(b.ranks[k + 1]);
		const int first = k == 0, last = k == d - 1;
		const int O0 = first ? 1 : P0 + Q0, O1 = last ? 1 : P1 + Q1;
		const size_t nax = size_t(P0) * n * P1, ny = size_t(O0) * n * O1;
		if (Ap) {
			k_op_apply<<<grid_for(nax), 256, 0, c.stream>>>(f.ax, Ap->core[k], x.core[k], K, L, n, ra, rb);
			c.count_launch();
		} else {
			copy_d2d(c, f.ax, x.core[k], nax);
		}
		k_block_core<<<grid_for(ny), 256, 0, c.stream>>>(f.Y, f.ax, b.core[k], P0, P1, Q0, Q1, n, first, last, -1.0);
		c.count_launch();
		XTT_CUDA(cudaGetLastError());
		return Dims{n, O0, O1};
	};
	auto qr_r_only = [&](double* Zp, int m, int ncol, int transpose, double* out) {
		QrArgs a;
		const int mw = transpose ? ncol : m, nw = transpose ? m : ncol;
		const size_t wk = qr_work_doubles(mw, nw);
		a.A = Zp; a.lda = ncol; a.m = m; a.n = ncol; a.transpose = transpose; a.pivot = 0; a.want_q = 0;
		a.work = wk ? c.scratch<double>(c.stream == c.aux ? S_QR_WORKB : S_QR_WORK, wk) : nullptr;
		a.Q = nullptr; a.C = out; a.rank_out = nullptr;
		ProfScope ps(c, "qr", qr_work_bytes(a), qr_work_flops(a));
		launch_qr(a, c.stream);
		c.count_launch();
	};
	// the meeting: two cores when their product is cheap (the left carry's rows at mid follow
	// rr <- min(rr n_k, O_k+1) along the chain)
	auto bond = [&](int k) -> int64_t { return k == 0 || k == d ? 1 : opr(k) * x.ranks[k] + b.ranks[k]; };
	bool two = false;
	if (d >= 2) {
		const int m2 = (d - 2) / 2;
		int64_t rows = 1;
		for (int k = 0; k < m2; ++k) rows = std::min<int64_t>(rows * x.dims[k], bond(k + 1));
		const double flops = 2.0 * double(rows * x.dims[m2]) * double(bond(m2 + 1)) *
		                     double(x.dims[m2 + 1] * bond(m2 + 2));
		two = flops <= kResMeetMaxFlops;
	}
	const int mid = two ? (d - 2) / 2 : d / 2;
	const int right_end = two ? mid + 1 : mid;  // the right chain stops above this core
	// right half on the aux stream: carry L (O1_k x rl), starting from [1]
	int64_t rl = 1;
	double* Lc = rb_.R;
	c.fork();
	{
		OnAux on(c);
		fill(c, Lc, 1.0, 1);
		for (int k = d - 1; k > right_end; --k) {
			const Dims dm = block(k, rb_);
			Gemm<double> g;  // Z = Y_k ((O0 n) x O1) * L (O1 x rl)
			g.M = dm.O0 * dm.n; g.N = int(rl); g.K = dm.O1;
			g.A = rb_.Y; g.sAm = dm.O1; g.sAk = 1;
			g.B = Lc; g.sBk = rl; g.sBn = 1;
			g.C = rb_.Z; g.sCm = rl; g.sCn = 1;
			g.lens((long long)cap_core, (long long)cap_r, (long long)2 * cap_core);
			gemm(c, g);
			// L <- left factor of Z viewed as O0 x (n rl)  (LQ, L only)
			const int ncol = int(dm.n * rl), kq = std::min(dm.O0, ncol);
			XTT_REQUIRE(size_t(dm.O0) * kq <= cap_r, "internal: residual carry too small");
			qr_r_only(rb_.Z, dm.O0, ncol, 1, Lc);
			rl = kq;
		}
	}
	// left half on the context's stream, concurrently with the right half: carry R (rr x O0_k),
	// starting from [1]
	int64_t rr = 1;
	fill(c, lb.R, 1.0, 1);
	for (int k = 0; k < mid; ++k) {
		const Dims dm = block(k, lb);
		Gemm<double> g;  // Z = R (rr x O0) * Y (O0 x n O1)
		g.M = int(rr); g.N = dm.n * dm.O1; g.K = dm.O0;
		g.A = lb.R; g.sAm = dm.O0; g.sAk = 1;
		g.B = lb.Y; g.sBk = dm.n * dm.O1; g.sBn = 1;
		g.C = lb.Z; g.sCm = dm.n * dm.O1; g.sCn = 1;
		g.lens((long long)cap_r, (long long)cap_core, (long long)2 * cap_core);
		gemm(c, g);
		const int m = int(rr * dm.n), kq = std::min(m, dm.O1);
		XTT_REQUIRE(size_t(kq) * dm.O1 <= cap_r, "internal: residual carry too small");
		qr_r_only(lb.Z, m, dm.O1, 0, lb.R);
		rr = kq;
	}
	c.join();  // the meeting reads the right half's carry L
	const Dims dm = block(mid, lb);
	Gemm<double> g1;  // Z = R (rr x O0) * Y_mid (O0 x n O1)
	g1.M = int(rr); g1.N = dm.n * dm.O1; g1.K = dm.O0;
	g1.A = lb.R; g1.sAm = dm.O0; g1.sAk = 1;
	g1.B = lb.Y; g1.sBk = dm.n * dm.O1; g1.sBn = 1;
	g1.C = lb.Z; g1.sCm = dm.n * dm.O1; g1.sCn = 1;
	g1.lens((long long)cap_r, (long long)cap_core, (long long)2 * cap_core);
	gemm(c, g1);
	if (!two) {
		// one core: W = Z L, ||y|| = ||W||
		Gemm<double> g2;  // W = Z ((rr n) x O1) * L (O1 x rl)
		g2.M = int(rr * dm.n); g2.N = int(rl); g2.K = dm.O1;
		g2.A = lb.Z; g2.sAm = dm.O1; g2.sAk = 1;
		g2.B = Lc; g2.sBk = rl; g2.sBn = 1;
		g2.C = lb.ax; g2.sCm = rl; g2.sCn = 1;
		g2.lens((long long)2 * cap_core, (long long)cap_r, (long long)cap_core);
		XTT_REQUIRE(size_t(rr) * dm.n * rl <= cap_core, "internal: residual meeting block too small");
		gemm(c, g2);
		sumsq_async(c, lb.ax, size_t(rr) * dm.n * rl, 0);
		return std::sqrt(read_dbl(c, 0)) / nb;
	}
	// two cores: W = ((R Y_mid) Y_mid+1) L, ||y|| = ||W|| (the right chain's buffers are free:
	// the join above ordered its work before this)
	const Dims dn = block(mid + 1, rb_);
	XTT_REQUIRE(dn.O0 == dm.O1, "internal: residual meeting ranks differ");
	const size_t rows2 = size_t(rr) * dm.n * dn.n;  // (a, i_mid, i_mid+1)
	double* Z2 = c.scratch<double>(S_RES_MEET, rows2 * size_t(dn.O1 + rl));
	double* W = Z2 + rows2 * dn.O1;
	Gemm<double> g2;  // Z2 = Z ((rr n) x O1) * Y_mid+1 (O1 x n' O2)
	g2.M = int(rr * dm.n); g2.N = dn.n * dn.O1; g2.K = dm.O1;
	g2.A = lb.Z; g2.sAm = dm.O1; g2.sAk = 1;
	g2.B = rb_.Y; g2.sBk = dn.n * dn.O1; g2.sBn = 1;
	g2.C = Z2; g2.sCm = dn.n * dn.O1; g2.sCn = 1;
	g2.lens((long long)2 * cap_core, (long long)cap_core, (long long)(rows2 * dn.O1));
	gemm(c, g2);
	Gemm<double> g3;  // W = Z2 ((rr n n') x O2) * L (O2 x rl)
	g3.M = int(rows2); g3.N = int(rl); g3.K = dn.O1;
	g3.A = Z2; g3.sAm = dn.O1; g3.sAk = 1;
	g3.B = Lc; g3.sBk = rl; g3.sBn = 1;
	g3.C = W; g3.sCm = rl; g3.sCn = 1;
	g3.lens((long long)(rows2 * dn.O1), (long long)cap_r, (long long)(rows2 * rl));
	gemm(c, g3);
	sumsq_async(c, W, rows2 * size_t(rl), 0);
	return std::sqrt(read_dbl(c, 0)) / nb;
}

// One block per sample: v <- v * x_k[:, i_k, :]
__global__ void k_entries(const double* const* cores, const int64_t* ranks, const int64_t* dims, int d,
                          const int64_t* pos, int64_t count, double* out, int maxr) {
	extern __shared__ double buf[];
	double* v = buf;
	double* w = buf + maxr;
	for (int64_t s = blockIdx.x; s < count; s += gridDim.x) {
		if (threadIdx.x == 0) v[0] = 1.0;
		__syncthreads();
		for (int k = 0; k < d; ++k) {
			const int r0 = int(ranks[k]), r1 = int(ranks[k + 1]), n = int(dims[k]);
			const int64_t i = pos[s * d + k];
			const double* c = cores[k];
			for (int b = threadIdx.x; b < r1; b += blockDim.x) {
				double acc = 0;
				for (int a = 0; a < r0; ++a) acc += v[a] * c[(size_t(a) * n + i) * r1 + b];
				w[b] = acc;
			}
			__syncthreads();
			for (int b = threadIdx.x; b < r1; b += blockDim.x) v[b] = w[b];
			__syncthreads();
		}
		if (threadIdx.x == 0) out[s] = v[0];
		__syncthreads();
	}
}

// One block per sample: v <- v * sum_i u_k[i] x_k[:, i, :] (RankOneMeasurementSet::measure,
// src/xerus/measurments.cpp:397-...); u holds each sample's concatenated vectors (row stride su).
__global__ void k_entries_r1(const double* const* cores, const int64_t* ranks, const int64_t* dims, int d,
                             const double* u, long long su, int64_t count, double* out, int maxr) {
	extern __shared__ double buf[];
	double* v = buf;
	double* w = buf + maxr;
	for (int64_t s = blockIdx.x; s < count; s += gridDim.x) {
		if (threadIdx.x == 0) v[0] = 1.0;
		__syncthreads();
		const double* us = u + s * su;
		for (int k = 0; k < d; ++k) {
			const int r0 = int(ranks[k]), r1 = int(ranks[k + 1]), n = int(dims[k]);
			const double* c = cores[k];
			for (int b = threadIdx.x; b < r1; b += blockDim.x) {
				double acc = 0;
				for (int a = 0; a < r0; ++a) {
					double t = 0;
					for (int i = 0; i < n; ++i) t = fma(us[i], c[(size_t(a) * n + i) * r1 + b], t);
					acc = fma(v[a], t, acc);
				}
				w[b] = acc;
			}
			__syncthreads();
			for (int b = threadIdx.x; b < r1; b += blockDim.x) v[b] = w[b];
			__syncthreads();
			us += n;
		}
		if (threadIdx.x == 0) out[s] = v[0];
		__syncthreads();
	}
}

void entries_rank_one(const Tensor& x, const double* vectors, int64_t count, double* out) {
	XTT_REQUIRE(!x.op, "measurements of a TT operator are not supported");
	Context& c = *x.ctx;
	if (count == 0) return;
	int64_t maxr = 1, su = 0;
	for (auto r : x.ranks) maxr = std::max(maxr, r);
	for (auto n : x.dims) su += n;
	const size_t meta = size_t(x.d) * 2 + 1;
	int64_t* dmeta = c.scratch<int64_t>(S_ENT_META, meta);
	std::vector<int64_t> hm(meta);
	for (int k = 0; k < x.d; ++k) hm[k] = x.dims[k];
	for (int k = 0; k <= x.d; ++k) hm[x.d + k] = x.ranks[k];
	double** dcores = c.scratch<double*>(S_ENT_CORES, x.d);
	std::vector<double*> hc(x.core.begin(), x.core.end());
	double* du = c.scratch<double>(S_ADF_FIRST + 14, size_t(count) * su);
	double* dout = c.scratch<double>(S_ENT_OUT, count);
	XTT_CUDA(cudaMemcpyAsync(dmeta, hm.data(), hm.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c.stream));
	XTT_CUDA(cudaMemcpyAsync(dcores, hc.data(), hc.size() * sizeof(double*), cudaMemcpyHostToDevice, c.stream));
	XTT_CUDA(cudaMemcpyAsync(du, vectors, sizeof(double) * count * su, cudaMemcpyHostToDevice, c.stream));
	const unsigned blocks = unsigned(std::min<int64_t>(count, 8192));
	k_entries_r1<<<blocks, 128, 2 * maxr * sizeof(double), c.stream>>>(dcores, dmeta + x.d, dmeta, x.d, du, su, count,
	                                                                    dout, int(maxr));
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	XTT_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * count, cudaMemcpyDeviceToHost, c.stream));
	c.sync();
}

void entries(const Tensor& x, const int64_t* positions, int64_t count, double* out) {
	XTT_REQUIRE(!x.op, "entries of a TT operator are not supported");
	Context& c = *x.ctx;
	if (count == 0) return;
	for (int64_t s = 0; s < count; ++s)
		for (int k = 0; k < x.d; ++k)
			XTT_REQUIRE(positions[s * x.d + k] >= 0 && positions[s * x.d + k] < x.dims[k], "position out of range");
	int64_t maxr = 1;
	for (auto r : x.ranks) maxr = std::max(maxr, r);
	const size_t meta = size_t(x.d) * 3 + 1;
	int64_t* dmeta = c.scratch<int64_t>(S_ENT_META, meta + size_t(count) * x.d);
	std::vector<int64_t> hm(meta + size_t(count) * x.d);
	for (int k = 0; k < x.d; ++k) { hm[k] = x.dims[k]; }
	for (int k = 0; k <= x.d; ++k) hm[x.d + k] = x.ranks[k];
	std::memcpy(hm.data() + meta, positions, sizeof(int64_t) * count * x.d);
	double** dcores = c.scratch<double*>(S_ENT_CORES, x.d);
	std::vector<double*> hc(x.core.begin(), x.core.end());
	double* dout = c.scratch<double>(S_ENT_OUT, count);
	XTT_CUDA(cudaMemcpyAsync(dmeta, hm.data(), hm.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c.stream));
	XTT_CUDA(cudaMemcpyAsync(dcores, hc.data(), hc.size() * sizeof(double*), cudaMemcpyHostToDevice, c.stream));
	const unsigned blocks = unsigned(std::min<int64_t>(count, 8192));
	k_entries<<<blocks, 128, 2 * maxr * sizeof(double), c.stream>>>(dcores, dmeta + x.d, dmeta, x.d, dmeta + meta,
	                                                                 count, dout, int(maxr));
	XTT_CUDA(cudaGetLastError());
	c.count_launch();
	XTT_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * count, cudaMemcpyDeviceToHost, c.stream));
	c.sync();
}

}  // namespace xtt
