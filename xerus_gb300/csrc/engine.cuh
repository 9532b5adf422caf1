// Host-side engine of the TT sweep library: contexts (one CUDA stream, a
// device status word, scratch buffers), device-resident TT tensors and the
// operations of the xerus sweep path built from the kernels.
//
// Shapes are authoritative on the host. Kernels get explicit shapes; the only
// host<->device synchronisations inside an operation are the reads of a rank
// that a rank-revealing factorisation decided on the device (QC/CQ in
// move_core(keepRank=false), SVD truncation in round and DMRG).
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <functional>
#include <vector>

#include "common.cuh"
#include "gemm.cuh"
#include "linalg.cuh"

namespace xtt {

struct Context {
	int device = 0;
	cudaStream_t own = nullptr;
	cudaStream_t stream = nullptr;
	cudaStream_t aux = nullptr;              // second stream for work that runs beside `stream`
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	int num_sms = 0;
	int* d_status = nullptr;       // DeviceStatus word
	unsigned* d_barrier = nullptr; // grid barrier count/phase
	int* d_ints = nullptr;         // small device results (ranks), 64 ints
	int* h_ints = nullptr;         // pinned mirror
	double* d_dbl = nullptr;       // small device results (norms, dots), 64 doubles
	double* h_dbl = nullptr;       // pinned mirror
	long long launches = 0;
	int cg_path = XTT_CG_PATH_AUTO;  // xtt_cg_path: which local CG kernel family runs
	int svd_path = XTT_SVD_PATH_AUTO;  // xtt_svd_path: QR-preconditioned or plain Jacobi SVD
	// precision form of round / move_core / dot (xtt_context_set_contraction_precision):
	// 0 FP64 GEMMs; 3 split TF32, 1 TF32 on the tensor cores. Applied only while
	// `tc_active` is set, which those three entry points do for their duration.
	int contraction_terms = 0;
	int tc_active = 0;
	// while set (DfGemmScope), FP64 GEMMs of at least kDfGemmMinFlops run in double-float
	// tiles (FP32 pairs, ~1e-15 of sum |a b|): the environment pushes of the mixed sweeps
	int df_gemm = 0;
	bool gram_qr = false;  // rank-revealing QRs by Cholesky QR where well-conditioned (GramQrScope)
	// CUDA graphs of fixed launch sequences, by the shapes and buffers they were captured with
	std::vector<std::pair<std::vector<long long>, struct ReplayGraph*>> graph_cache;
	// batched ALS: the CUDA graph of the last batch launch (replayed while its
	// signature holds), its pinned descriptor staging, and autotuned launch shapes
	unsigned long long batch_key = 0;
	cudaGraphExec_t batch_exec = nullptr;
	void* batch_host = nullptr;
	size_t batch_host_bytes = 0;
	struct BatchTuned {
		unsigned long long sig;
		int threads, per_sm, tile;
	};
	std::vector<BatchTuned> batch_tuned;  // the batch autotuner's choices per batch signature
	int tensors = 0;        // live tensors created on this context
	bool closing = false;   // destroy requested; freed when the last tensor goes
	struct Slot {
		void* p = nullptr;
		size_t bytes = 0;
	};
	std::vector<Slot> slots;

	explicit Context(int dev);
	~Context();
	// Scratch buffer `id` with at least `count` elements of T (contents undefined).
	template <class T>
	T* scratch(int id, size_t count) {
		return static_cast<T*>(scratch_bytes(id, count * sizeof(T)));
	}
	void* scratch_bytes(int id, size_t bytes);
	void sync();                      // stream sync + device status check
	// aux waits for everything issued so far on stream / stream waits for aux
	void fork();
	void join();
	void check_status();              // reads d_status (after a sync) and throws on failure
	int read_int(int idx);            // sync + d_ints[idx]
	void read_ints(int lo, int hi);   // sync + d_ints[lo, hi) into h_ints
	void count_launch(int n = 1) { launches += n; }

	// Optional per-kernel-class timing: CUDA events recorded on the context's
	// stream around each launch of a class, resolved when read.
	bool profiling = false;
	struct Timed {
		std::string name;
		cudaEvent_t start, stop;
		double bytes, flops;
	};
	std::vector<Timed> pending;
	struct ProfileEntry {
		long long launches = 0;
		double ms = 0;
		double bytes = 0, flops = 0;  // algorithmic work the launch sites declared
	};
	std::vector<std::pair<std::string, ProfileEntry>> profile;
	void resolve_profile();
};

// RAII scope recording a launch class's start and stop events when profiling.
// `bytes` / `flops`: the algorithmic work of the scope (minimal operand traffic,
// arithmetic), accumulated per class for roofline figures.
struct ProfScope {
	Context& c;
	const char* name;
	double bytes, flops;
	cudaEvent_t a = nullptr, b = nullptr;
	ProfScope(Context& cc, const char* n, double bytes = 0, double flops = 0);
	~ProfScope();
};

// Records the launches `body` issues on the context's stream once as a CUDA graph and
// replays the graph on every later run: for launch sequences that repeat with the same
// arguments (an ADF sweep at fixed ranks), where issuing ~100 small launches one by one
// from the host costs more than the kernels. The body must not synchronise or
// allocate; host-side state it would change must be set by the caller after a replay.
struct ReplayGraph {
	cudaGraphExec_t exec = nullptr;
	int64_t launches = 0;
	ReplayGraph() = default;
	ReplayGraph(const ReplayGraph&) = delete;
	ReplayGraph& operator=(const ReplayGraph&) = delete;
	~ReplayGraph() {
		if (exec) cudaGraphExecDestroy(exec);
	}
	template <class F>
	void run(Context& c, F&& body) {
		if (!exec) {
			const int64_t l0 = c.launches;
			cudaGraph_t g = nullptr;
			XTT_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
			try {
				body();
			} catch (...) {
				cudaGraph_t t = nullptr;
				cudaStreamEndCapture(c.stream, &t);
				if (t) cudaGraphDestroy(t);
				cudaGetLastError();
				throw;
			}
			XTT_CUDA(cudaStreamEndCapture(c.stream, &g));
			const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
			cudaGraphDestroy(g);
			XTT_CUDA(e);
			launches = c.launches - l0;  // the body counted its launches once
		} else {
			c.count_launch(int(launches));
		}
		XTT_CUDA(cudaGraphLaunch(exec, c.stream));
	}
};

// Applies the context's contraction precision for its scope (round, move_core, dot).
struct ContractionPrecisionScope {
	Context& c;
	int saved;
	explicit ContractionPrecisionScope(Context& cc) : c(cc), saved(cc.tc_active) { c.tc_active = c.contraction_terms; }
	~ContractionPrecisionScope() { c.tc_active = saved; }
};

// Keeps the engine's contractions FP64 for its scope (factorisation internals).
struct Fp64ContractionScope {
	Context& c;
	int saved;
	explicit Fp64ContractionScope(Context& cc) : c(cc), saved(cc.tc_active) { c.tc_active = 0; }
	~Fp64ContractionScope() { c.tc_active = saved; }
};

// Rank-revealing QRs of its scope by Cholesky QR where well-conditioned (round and the
// public move_core; the library's internal canonicalisations keep Householder QR).
struct GramQrScope {
	Context& c;
	bool saved;
	explicit GramQrScope(Context& cc) : c(cc), saved(cc.gram_qr) { c.gram_qr = true; }
	~GramQrScope() { c.gram_qr = saved; }
};

// Issues the launches of its scope on the context's aux stream.
struct OnAux {
	Context& c;
	cudaStream_t saved;
	explicit OnAux(Context& cc) : c(cc), saved(cc.stream) { c.stream = c.aux; }
	~OnAux() { c.stream = saved; }
};

// Scratch slot ids (one per purpose, so nested operations never share a buffer).
enum ScratchId : int {
	S_QR_Q = 0, S_QR_C, S_QR_WORK, S_GEMM_A, S_GEMM_B, S_SVD_U, S_SVD_S, S_SVD_VT, S_SVD_WORK,
	S_ROUND_X, S_ROUND_QA, S_ROUND_QB, S_ROUND_CA, S_ROUND_CB, S_ZIP_M, S_ZIP_T, S_ZIP_M2,
	S_RES_CORE0, S_RES_CORE1, S_RES_R, S_RED, S_ENT_META, S_ENT_CORES, S_ENT_OUT,
	S_RES_CORE0B, S_RES_CORE1B, S_RES_RB, S_QR_WORKB, S_BATCH_META, S_BATCH_WORK, S_BATCH_BACKUP,
	S_SVD_PC_Q, S_SVD_PC_C, S_SVD_PC_UV, S_SVD_PC_QRW, S_GEMM_TC_WORK, S_SVD_PC_CT, S_SVD_PC_UT,
	S_SVD_MX_W32, S_SVD_MX_W, S_SVD_MX_W2, S_SVD_MX_G, S_SVD_MX_B0, S_TMA_A, S_TMA_B, S_SVD_RF_U, S_SVD_RF_V,
	S_SVD_RF_M, S_GQ_FIRST,  // 2 x kGqSlots ids from here: the Gram QR's buffers for two concurrent factorisations
	S_RES_MEET = 60,         // the residual's two-core meeting products
	S_QB = 61,               // the blocked Q formation's reflectors and products
	S_ALS_FIRST = 64,
	S_ADF_FIRST = 128,
	S_MAX = 192
};

struct Tensor {
	Context* ctx = nullptr;
	bool op = false;
	int d = 0;
	std::vector<int64_t> dims;
	std::vector<int64_t> ranks;     // d+1, ranks[0] = ranks[d] = 1
	std::vector<double*> core;      // device pointers
	std::vector<size_t> cap;        // capacity (doubles) of each core buffer
	bool canonicalized = false;
	int64_t core_position = 0;

	Tensor(Context* c, bool is_op, int order, const int64_t* dims_, const int64_t* ranks_);
	~Tensor();
	Tensor(const Tensor&) = delete;
	Tensor& operator=(const Tensor&) = delete;

	int64_t n(int k) const { return op ? dims[k] * dims[k] : dims[k]; }
	size_t core_size(int k) const { return size_t(ranks[k]) * size_t(n(k)) * size_t(ranks[k + 1]); }
	size_t total_size() const;
	// Resize core k for new ranks (content undefined when the buffer grows).
	void reshape_core(int k, int64_t r0, int64_t r1);
	void copy_from(const Tensor& o);  // same order/dims; takes ranks, cores and canonical state
};

// Host-side validation of a GEMM descriptor against its operand lengths (throws).
template <class T>
void check_gemm(const Gemm<T>& g);
// The same GEMM on the tensor cores (tcgen05, TF32 products, FP32 accumulation;
// terms = 3: split TF32 with FP32-level products, terms = 1: plain TF32).
template <class T>
void gemm_tc(Context& c, const Gemm<T>& g, int terms);
// The TMA-fed form of gemm_tc (operands split into K-major pieces, streamed by
// cp.async.bulk.tensor): false if the driver cannot describe them as tensor maps.
template <class T>
bool gemm_tc_tma(Context& c, const Gemm<T>& g, int terms);

// Stream-ordered helpers.
void gemm(Context& c, const Gemm<double>& g);
// C = alpha A B + beta C in double-float tiles (FP64 operands as FP32 pairs on the CUDA
// cores, error-free products, TwoSum sums; K split across CTAs when the tiles leave SMs idle)
void gemm_df(Context& c, const Gemm<double>& g);
constexpr double kDfGemmMinFlops = 4e6;
struct DfGemmScope {
	Context& c;
	int saved;
	DfGemmScope(Context& cc, bool on) : c(cc), saved(cc.df_gemm) { c.df_gemm = on ? 1 : saved; }
	~DfGemmScope() { c.df_gemm = saved; }
};
void gemm_f(Context& c, const Gemm<float>& g);
void copy_d2d(Context& c, double* dst, const double* src, size_t count);
void fill(Context& c, double* dst, double v, size_t count);
void scale(Context& c, double* x, double f, size_t count);
// Truncated SVD a.X = a.U diag(a.S) a.Vt on the context's stream (kernel class "svd").
// `graded`: the caller expects a decaying spectrum (a DMRG two-site solution); then,
// where it fits and svd_path allows, QR-preconditioned Jacobi runs (a third of the
// plain sweeps there; on unstructured matrices, e.g. rounding a random TT, it saves
// no sweeps and its QR costs more than it saves). The workspace (a.work) is taken
// from the context's scratch here.
// Returns the kept rank when the host already read it, else -1 (then it is in *a.rank_out).
int run_svd(Context& c, SvdArgs& a, bool graded = false);
void scale_rows(Context& c, double* X, const double* S, int rows, int cols);  // X (rows x cols) *= S[row]
void scale_cols(Context& c, double* X, const double* S, int rows, int cols);  // X (rows x cols) *= S[col]
// Sum of squares of x into ctx.d_dbl[slot] (deterministic two-level reduction).
void sumsq_async(Context& c, const double* x, size_t count, int slot);
// sum_i a[i] * b[i] into ctx.d_dbl[slot] (deterministic two-level reduction).
void dot_async(Context& c, const double* a, const double* b, size_t count, int slot);

// TT operations (xerus semantics).
void transfer_core(Tensor& x, int from, int to, bool allow_rank_reduction);
void move_core(Tensor& x, int64_t pos, bool keep_rank);
void round_tt(Tensor& x, const std::vector<int64_t>& max_ranks, double eps, std::vector<double>* spectra);
double dot(const Tensor& x, const Tensor& y);
double frob_norm(const Tensor& x);
double orthogonal_norm(Tensor& x);  // destroys x's gauge (QR sweep), returns ||x||
double residual(const Tensor& A, const Tensor& x, const Tensor& b);
// ||x - b|| / ||b|| (A null: the identity)
double residual(const Tensor* A, const Tensor& x, const Tensor& b);
void entries(const Tensor& x, const int64_t* positions, int64_t count, double* out);
bool exceeds_maximal_ranks(const Tensor& x);
std::vector<int64_t> reduce_to_maximal_ranks(std::vector<int64_t> ranks, const std::vector<int64_t>& dims);

// xerus's binary data file of a TTTensor / TTOperator (fileio.cu).
struct TtFile {
	bool op = false;
	std::vector<int64_t> dims, ranks;  // ranks d+1
	std::vector<double> cores;         // row-major cores, concatenated
	bool canonicalized = false;
	int64_t core_position = 0;
};
std::vector<uint8_t> tt_file_encode(bool op, const std::vector<int64_t>& dims, const std::vector<int64_t>& ranks,
                                    const double* cores, bool canonicalized, int64_t core_position);
TtFile tt_file_decode(const uint8_t* data, size_t size);
std::vector<uint8_t> read_file(const std::string& path);
void write_file(const std::string& path, const std::vector<uint8_t>& bytes);

// y <- A x as a TT (cores R_k r_k), allocating y's cores.
void op_apply_tt(const Tensor& A, const Tensor& x, Tensor& y);
// y = A x (x a TT tensor or operator); canonicalised at A's core position when A is canonical.
void tt_apply(const Tensor& A, const Tensor& x, Tensor& y);
// x += f y; a canonical x is canonicalised again (rank-revealing) at its core position.
void tt_add(Tensor& x, const Tensor& y, double f);

// ADF for single-point samples (positions: N x d, row-major).
struct AdfResult {
	double residual = 0;          // the iteration's own residual (FP32 in the FP32 form)
	double checked_residual = 0;  // FP64 residual of the returned x
	int64_t iterations = 0;       // the solver's iteration counter at the end
	std::vector<double> trace;    // PerformanceData: residual, iteration count and inner ranks per point
	std::vector<int64_t> trace_iteration;
	std::vector<std::vector<int64_t>> trace_ranks;
};
// xerus's EPSILON (include/xerus/basic.h:50), the default cutoff of TTNetwork::round
constexpr double kXerusEpsilon = 8 * 2.220446049250313e-16;
// precision: XTT_PRECISION_FP64, or XTT_PRECISION_MIXED for FP32 stacks and
// per-sample arithmetic with FP64 cores, QR and final check. max_ranks (d-1 inner
// ranks) switches on the rank increase; add_random_rank_one then adds
// 1e-6 ||x|| r / ||r|| for a fresh random rank-one TT r to x (canonical at core 0).
AdfResult adf(Tensor& x, const int64_t* positions, const double* values, long long N, int64_t max_iter, double target,
              double min_dec, int precision = XTT_PRECISION_FP64, const std::vector<int64_t>* max_ranks = nullptr,
              const std::function<void(Tensor&)>& add_random_rank_one = {});
// IHT for single-point samples (positions: N x d, row-major) with an iteration cap.
struct IhtResult {
	double residual = 0;          // ||y - P(x)|| of the returned x (absolute, as the reference)
	std::vector<double> trace;    // the best residual of every iteration
};
IhtResult iht(Tensor& x, const int64_t* positions, const double* values, long long N, int64_t max_iter);
// Riemannian CG on the fixed-rank TT manifold (GeometricCGVariant with the submanifold
// retraction and projective vector transport); A null: minimise ||x - b||.
struct RiemannReport {
	double residual = 0;         // ||b - A x|| of the result (absolute, as the reference returns)
	int64_t steps = 0;
	std::vector<double> trace;   // residual before the first step and after every step
};
RiemannReport geometric_cg(const Tensor* A, Tensor& x, const Tensor& b, int64_t num_steps, double eps, bool assume_spd,
                           int retraction = XTT_RETRACTION_SUBMANIFOLD);
// SteepestDescentVariant with SubmanifoldRetractionII (absolute stopping tests, as the reference)
RiemannReport steepest_descent(const Tensor* A, Tensor& x, const Tensor& b, int64_t num_steps, double eps,
                               bool assume_spd, int retraction = XTT_RETRACTION_SUBMANIFOLD);
// ADF on rank-one measurements (RankOneMeasurementSet): vectors holds, per sample, the
// concatenated vectors u_1 .. u_d (N x sum n_k, row-major). FP64.
AdfResult adf_rank_one(Tensor& x, const double* vectors, const double* values, long long N, int64_t max_iter,
                       double target, double min_dec);
// RankOneMeasurementSet::measure(TensorNetwork): <x, u_1 (x) ... (x) u_d> per sample.
void entries_rank_one(const Tensor& x, const double* vectors, int64_t count, double* out);
double adf_gradient(const Tensor& x, const int64_t* positions, const double* values, long long N,
                    std::vector<double>& grad);

}  // namespace xtt
