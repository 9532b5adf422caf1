/*
 * xtt.h - C ABI of the GB300-native Tensor-Train sweep engine (libxtt.so).
 *
 * The library keeps TT tensors and TT operators resident on one CUDA device and
 * runs the xerus sweep path on it: TTNetwork::move_core / round / frob_norm, the
 * TT dot product, ALSVariant::solve (ALS_SPD, DMRG_SPD, ASD_SPD) and ADFVariant
 * for single-point measurement sets. Every entry point takes plain pointers and
 * sizes, returns an xtt_status, and leaves a message for xtt_last_error() when it
 * fails. A context owns one CUDA stream; calls on one context are serialised by
 * the caller (one host thread per context), different contexts are independent.
 *
 * Layout: a TT tensor of order d has cores (r_{k-1}, n_k, r_k), a TT operator
 * cores (R_{k-1}, n_k, n_k, R_k), all row-major FP64 (last index fastest) with
 * boundary ranks r_0 = r_d = 1, exactly as xerus stores its component tensors
 * (include/xerus/ttNetwork.h:145-150, include/xerus/tensor.h:536). Host buffers
 * hold the cores concatenated in order.
 *
 * Each declaration names the reference interface it replaces (paths relative to
 * the xerus 3.0.1 source tree).
 */
#ifndef XTT_H
#define XTT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum xtt_status {
	XTT_OK = 0,
	XTT_ERR_ARGUMENT = 1,        /* bad shape, index or option: xerus REQUIRE failure (misc/check.h:60-65) */
	XTT_ERR_CUDA = 2,            /* a CUDA runtime call failed */
	XTT_ERR_NOT_CONVERGED = 3,   /* a local solver or the SVD hit its iteration cap */
	XTT_ERR_NUMERIC = 4,         /* NaN/Inf or a breakdown (non-SPD local operator) */
	XTT_ERR_TIMEOUT = 5,         /* a bounded device-side wait gave up */
	XTT_ERR_CAPACITY = 6,        /* a size exceeds a fixed limit of the library */
	XTT_ERR_NO_MEMORY = 7
} xtt_status;

typedef enum xtt_precision {
	XTT_PRECISION_FP64 = 0,      /* plain form: FP64 everywhere */
	XTT_PRECISION_MIXED = 1      /* local solves in FP32 with FP64 iterative refinement (residual
	                                updates and the sweeps' large environment pushes in
	                                double-float, ~1e-15 relative) */
} xtt_precision;

typedef struct xtt_context xtt_context;
typedef struct xtt_tensor xtt_tensor;

/* Message of the last failing call on this host thread ("" if none). */
const char* xtt_last_error(void);
const char* xtt_version(void);

/* --------------------------------------------------------------- context */
int xtt_context_create(int device, xtt_context** out);
int xtt_context_destroy(xtt_context* ctx);
/* Use an existing cudaStream_t (passed as void*); NULL restores the context's own stream. */
int xtt_context_set_stream(xtt_context* ctx, void* stream);
int xtt_context_synchronize(xtt_context* ctx);
/* Number of kernels this context has launched so far (a counter, for measurements). */
int xtt_context_kernel_launches(xtt_context* ctx, int64_t* count);
/* Per-kernel-class timing with CUDA events on the context's stream (the analogue
 * of xerus's XERUS_PA_START/END accumulators, include/xerus/misc/performanceAnalysis.h:30-39).
 * enable = 1 starts (and clears) it, 0 stops it. Classes: "cg_fp64", "cg_mixed",
 * "cg_tc", "gemm", "gemm_df" (double-float GEMMs of the mixed sweeps), "gemm_tc", "qr",
 * "qr_gram", "svd", "adf_res_grad", "adf_slicenorm", "adf_stack". */
int xtt_context_profile(xtt_context* ctx, int enable);
/* Launch count and total milliseconds of one class since profiling started (0 if none). */
int xtt_context_profile_get(xtt_context* ctx, const char* name, int64_t* launches, double* milliseconds);
/* Algorithmic work the launches of one class declared since profiling started:
 * minimal operand bytes and arithmetic (0 for classes whose work depends on
 * device-side iteration counts, e.g. the CG solves). */
int xtt_context_profile_work(xtt_context* ctx, const char* name, double* bytes, double* flops);

/* Which kernel family runs the local conjugate-gradient solves of xtt_als (no
 * reference counterpart; the reference factors the local system densely,
 * src/xerus/algorithms/als.cpp:43-71). AUTO: one thread-block cluster with all
 * operands in shared memory when the local system fits (up to 16 CTAs), else
 * the grid-wide cooperative kernel; for mixed-precision solves at a site whose
 * rank is 64 or more or whose local system has 16384 unknowns or more, the
 * tensor-core form (FP64 refinement of FP32 CG whose operator stages run as
 * split-TF32 tcgen05 GEMMs). GRID: always the grid-wide
 * kernel. TENSOR: the tensor-core form for every mixed-precision solve. Results
 * agree to the CG tolerance; the choice only changes speed. */
typedef enum xtt_cg_path { XTT_CG_PATH_AUTO = 0, XTT_CG_PATH_GRID = 1, XTT_CG_PATH_TENSOR = 2 } xtt_cg_path;
int xtt_context_set_cg_path(xtt_context* ctx, int path);

/* Which SVD runs the truncations (the reference calls LAPACK's dgesdd,
 * src/xerus/blasLapackWrapper.cpp:288-340). AUTO: for the DMRG split of xtt_als a
 * column-pivoted QR, then one-sided Jacobi on R^T (a third of the sweeps on the
 * split's decaying spectra); for xtt_round (and splits the QR path does not take)
 * FP32 Jacobi sweeps in one CTA, orthogonalised in FP64, then the FP64 Jacobi from
 * that start (a few sweeps); where the smaller side is 32..512. JACOBI: always plain
 * FP64 one-sided Jacobi. All keep the same singular values, truncation rule and sign
 * gauge; results agree to rounding. */
typedef enum xtt_svd_path { XTT_SVD_PATH_AUTO = 0, XTT_SVD_PATH_JACOBI = 1 } xtt_svd_path;
int xtt_context_set_svd_path(xtt_context* ctx, int path);

/* Precision form of xtt_round, xtt_move_core and xtt_dot (TTNetwork::round,
 * move_core and the TT dot product, include/xerus/ttNetwork.h:330-420): 0 keeps
 * every contraction FP64 (the reference's arithmetic); 3 runs the contractions
 * (R absorption, bond products, singular-vector absorption, the dot-product
 * zipper) as split-TF32 tensor-core GEMMs with FP32 accumulation (two TF32 pieces
 * per operand, three products), 6 as split-BF16 GEMMs (three BF16 pieces per
 * operand, the six products of weight >= 2^-16), 1 as plain TF32. The operands
 * are split once per GEMM into K-major pieces that TMA (cp.async.bulk.tensor)
 * streams into the MMAs' shared-memory stages. The QR and SVD factorisations stay
 * FP64 in every form. Other entry points (the solvers) always contract in FP64. */
int xtt_context_set_contraction_precision(xtt_context* ctx, int terms);

/* C (m x n) = A (m x k) B (k x n) on the tensor cores (tcgen05 MMAs, FP32
 * accumulation in tensor memory), FP64 row-major device matrices with leading
 * dimensions lda, ldb, ldc; terms = 3 splits each operand into two TF32 pieces
 * (FP32-level products), 6 into three BF16 pieces (FP32-level products on the
 * 16-bit MMA path), 1 is plain TF32; terms = 2 runs the CUDA-core double-float
 * tiles of the mixed local solves' residual updates and environment pushes instead
 * (each FP64 operand as an FP32 pair, error-free FMA products, TwoSum accumulation:
 * ~1e-15 of sum |a b|; K split across CTAs when the tiles leave SMs idle). The building block of the precision forms
 * (no reference counterpart: the reference multiplies in FP64 through BLAS,
 * src/xerus/blasLapackWrapper.cpp:96-147); exposed to check it against an FP64
 * product. Asynchronous on the context's stream. */
int xtt_gemm_tc(xtt_context* ctx, int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                int64_t ldb, double* C, int64_t ldc, int32_t terms);

/* ---------------------------------------------------------------- tensors */
/* TTNetwork(dims) + set_component: a device TT with the given ranks (order+1
 * entries, r_0 = r_d = 1), all cores zero, not canonical.
 * Replaces TTTensor/TTOperator construction (include/xerus/ttNetwork.h:44-100). */
int xtt_tensor_create(xtt_context* ctx, int is_operator, int64_t order, const int64_t* dims,
                      const int64_t* ranks, xtt_tensor** out);
int xtt_tensor_destroy(xtt_tensor* t);
/* Deep copy (TTNetwork copy constructor). */
int xtt_tensor_copy(const xtt_tensor* src, xtt_tensor** out);
int xtt_tensor_order(const xtt_tensor* t, int64_t* order);
int xtt_tensor_dims(const xtt_tensor* t, int64_t* dims);
/* Current ranks, order+1 entries (TTNetwork::ranks, include/xerus/ttNetwork.h:394, plus the boundary 1s). */
int xtt_tensor_ranks(const xtt_tensor* t, int64_t* ranks);
/* Number of doubles of all cores at the current ranks. */
int xtt_tensor_size(const xtt_tensor* t, int64_t* count);
/* Host <-> device copies of all cores (count must equal xtt_tensor_size). */
int xtt_tensor_set_cores(xtt_tensor* t, const double* host, int64_t count);
int xtt_tensor_get_cores(const xtt_tensor* t, double* host, int64_t count);
/* Replace the whole tensor with new ranks and cores (TTNetwork::set_component for every core). */
int xtt_tensor_assign(xtt_tensor* t, const int64_t* ranks, const double* host, int64_t count);
/* TTNetwork::canonicalized / corePosition (include/xerus/ttNetwork.h:66-72) and assume_core_position (:421). */
int xtt_tensor_get_canonical(const xtt_tensor* t, int* canonicalized, int64_t* core_position);
int xtt_tensor_set_canonical(xtt_tensor* t, int canonicalized, int64_t core_position);
/* x *= f on the core (TTNetwork::operator*=, src/xerus/ttNetwork.cpp:859-868). */
int xtt_tensor_scale(xtt_tensor* t, double f);

/* ------------------------------------------------------------- random state */
/* Reseeds the library's random engine (std::mt19937_64, the analogue of
 * xerus::misc::randomEngine, src/xerus/misc/random.cpp:29) and resets its normal
 * distribution (drops a cached polar variate). Thread-local, like the reference. */
int xtt_random_seed(uint64_t seed);
/* TTNetwork::random(dims, ranks, normal(mean, stddev)) (include/xerus/ttNetwork.h:128-155):
 * ranks has order-1 inner entries, reduced to the maximal ranks; entries drawn
 * core by core in row-major order on the host from the library engine, then
 * move_core(0) with rank-revealing QR on the device. */
int xtt_tensor_random(xtt_context* ctx, int64_t order, const int64_t* dims, const int64_t* inner_ranks,
                      double mean, double stddev, xtt_tensor** out);
/* SinglePointMeasurementSet::random(num, dims) positions
 * (src/xerus/measurments.cpp:42-47, 222-248): out holds num*order indices, sorted. */
int xtt_random_positions(int64_t num, int64_t order, const int64_t* dims, int64_t* out);
/* Draws `count` values from N(mean, stddev) with the library engine (what a caller
 * of std::normal_distribution on misc::randomEngine gets). */
int xtt_random_normal(double mean, double stddev, int64_t count, double* out);

/* ----------------------------------------------------------- core movement */
/* TTNetwork::move_core(position, keepRank) (include/xerus/ttNetwork.h:413,
 * src/xerus/ttNetwork.cpp:581-628): keep_rank != 0 uses plain QR/LQ, else
 * rank-revealing pivoted QR with the cutoff |R_kk| < 16 eps R_00. */
int xtt_move_core(xtt_tensor* x, int64_t position, int keep_rank);
/* TTNetwork::round(maxRanks, eps) (include/xerus/ttNetwork.h:352-373,
 * src/xerus/ttNetwork.cpp:643-665). max_ranks has order-1 entries (use
 * INT64_MAX for "no cap"). If spectra is not NULL it receives the kept singular
 * values of each bond in sweep order (right to left), at most spectra_capacity. */
int xtt_round(xtt_tensor* x, const int64_t* max_ranks, double eps, double* spectra, int64_t spectra_capacity,
              int64_t* spectra_count);

/* ---------------------------------------------------------- contractions */
/* Full contraction value_t(x(i&0) * y(i&0)) of two TT tensors of equal dims
 * (src/xerus/indexedTensorReadOnly.cpp:58-61 via tensorNetwork.cpp:1253-1333). */
int xtt_dot(const xtt_tensor* x, const xtt_tensor* y, double* out);
/* TTNetwork::frob_norm (src/xerus/ttNetwork.cpp:781-789): the core norm when
 * canonical, else sqrt(<x,x>). */
int xtt_frob_norm(const xtt_tensor* x, double* out);
/* ||A x - b|| / ||b|| in FP64, through an orthogonalising sweep of the TT A x - b
 * (no cancellation). Replaces ALSVariant's residual_f (src/xerus/algorithms/als.cpp:258-261). */
int xtt_residual(const xtt_tensor* A, const xtt_tensor* x, const xtt_tensor* b, double* out);
/* A(i/2, j/2) * x(j&0) cast to a TT: the TTStack product (src/xerus/ttStack.cpp:47-173,
 * src/xerus/ttNetwork.cpp:886-967) with core ranks R_k r_k; x a TT tensor (out a TT
 * tensor) or a TT operator (out a TT operator, A x as operators). out is created on
 * x's context; it is canonicalised (rank-revealing move_core) at A's core position
 * when A is canonical, as the reference's stack cast does. */
int xtt_apply(const xtt_tensor* A, const xtt_tensor* x, xtt_tensor** out);
/* x += alpha y: TTNetwork::operator+= (alpha = 1) and operator-= (alpha = -1)
 * (src/xerus/ttNetwork.cpp:796-856); block cores of ranks r + s, then, when x was
 * canonical, a rank-revealing move_core back to its core position. */
int xtt_add(xtt_tensor* x, const xtt_tensor* y, double alpha);
/* Entries of x at `count` multi-indices (count*order int64, row-major):
 * SinglePointMeasurementSet::measure(TensorNetwork) (src/xerus/measurments.cpp:125-153). */
int xtt_entries(const xtt_tensor* x, const int64_t* positions, int64_t count, double* out);

/* The TT dot product of xtt_dot on caller-owned device memory, for callers
 * that cannot allocate device memory (for example when a framework's caching
 * allocator already owns the device memory, or on paths where cudaMalloc /
 * cudaFree and cudaFree's implicit synchronisation are not acceptable). It
 * allocates nothing: its intermediates live in a fixed 2.25 MiB __device__
 * array inside libxtt.so, one per device, kept until the library is unloaded.
 * No counterpart in the reference.
 * x_cores / y_cores: the cores concatenated (as xtt_tensor_get_cores lays them
 * out) in device memory of the current device; x_ranks / y_ranks: order+1 host
 * entries; result: one double of device memory, written asynchronously on
 * `stream` (a cudaStream_t, NULL = legacy default stream). Limits: every rank
 * <= 128 and every mode size <= 16, else XTT_ERR_CAPACITY before any launch.
 * The first call on a device looks up the array's device address; make it
 * before any stream capture on that device. The address is kept for the life of
 * the process: resetting the device (cudaDeviceReset) after that first call is
 * not supported. All calls share the array:
 * calls whose kernels may overlap on the GPU race and must be serialised. */
int xtt_dot_noalloc(int64_t order, const int64_t* dims, const int64_t* x_ranks, const double* x_cores,
                    const int64_t* y_ranks, const double* y_cores, double* result, void* stream);

/* ----------------------------------------------------------------- files */
/* xerus's binary data files for TTTensor / TTOperator: misc::save_to_file /
 * load_from_file (include/xerus/misc/fileIO.h:103-162) with the TTNetwork,
 * TensorNetwork and Tensor stream writers (src/xerus/ttNetwork.cpp:1454-1488,
 * src/xerus/tensorNetwork.cpp:1429-1500, src/xerus/tensor.cpp:1781-1830). Files
 * written here are byte-identical to the reference's for the same tensor; files
 * from the reference load here (dense or sparse components; binary format only). */
int xtt_tensor_save(const xtt_tensor* t, const char* path);
int xtt_tensor_load(xtt_context* ctx, const char* path, xtt_tensor** out);
/* The same format from / into host memory. encode: size receives the byte
 * count; buffer may be NULL to query it. decode: dims (order) and ranks
 * (order + 1) are written if both are non-NULL, cores if non-NULL. */
int xtt_file_encode(int is_operator, int64_t order, const int64_t* dims, const int64_t* ranks, const double* cores,
                    int canonicalized, int64_t core_position, uint8_t* buffer, int64_t capacity, int64_t* size);
int xtt_file_decode(const uint8_t* buffer, int64_t size, int* is_operator, int64_t* order, int64_t* dims,
                    int64_t* ranks, int64_t dims_capacity, double* cores, int64_t cores_capacity, int64_t* cores_count,
                    int* canonicalized, int64_t* core_position);

/* ------------------------------------------------------------------- ALS */
typedef struct xtt_als_options {
	int32_t sites;                   /* ALSVariant::sites: 1 = ALS, 2 = DMRG (als.h:112) */
	int32_t local_solver;            /* 0 = exact local solve (lapack_solver, als.cpp:43), 1 = one steepest-descent step (ASD_solver, als.cpp:73) */
	int32_t preserve_core_position;  /* ALSVariant::preserveCorePosition (als.h:117) */
	int32_t precision;               /* xtt_precision */
	int64_t num_half_sweeps;         /* 0 = until convergence (als.h:113) */
	double convergence_epsilon;      /* |dE| threshold (als.h:114), default 1e-6 */
	double local_tolerance;          /* relative residual of the local CG solve, default 1e-13 */
	int64_t local_max_iterations;    /* CG iteration cap per local solve, 0 = 10*N */
	double residual_target;          /* > 0: also stop after the first half-sweep whose FP64 residual <= target */
	int32_t record_residuals;        /* 1: FP64 residual after every micro-step into the trace (costly) */
	int32_t max_rank;                /* DMRG only: > 0 lets the 2-site split grow ranks up to this cap */
	double svd_epsilon;              /* DMRG only, with max_rank > 0: relative singular value cutoff */
	int32_t exact_environment;       /* DMRG only: 0 reproduces the reference's decreasing half-sweep, which
	                                    contracts core k (not k+1) into the right environment
	                                    (src/xerus/algorithms/als.cpp:371); 1 contracts core k+1, and the
	                                    last split of each half-sweep leaves S on the side the next one
	                                    starts from, so every environment is orthonormal and the local
	                                    systems keep the operator's condition number */
	int32_t assume_spd;              /* ALSVariant::assumeSPD (als.h:115), default 1. 0: least squares
	                                    ||A x - b|| through the projections of A^T A and A^T b (ALS, DMRG,
	                                    ASD; als.cpp:184-215); the energy is then the residual */
	int32_t use_residual;            /* ALSVariant::useResidualForEndCriterion (als.h:116) */
	int32_t reserved;
} xtt_als_options;

typedef struct xtt_als_report {
	double energy;                   /* the value ALSVariant::operator() returns */
	double residual;                 /* FP64 ||A x - b|| / ||b|| of the result */
	int64_t half_sweeps;
	int64_t micro_steps;
	int64_t local_iterations;        /* total CG iterations (FP32 + FP64) */
	int64_t refinements;             /* FP64 refinement passes (mixed precision) */
	int64_t trace_count;             /* entries written to each trace */
} xtt_als_report;

int xtt_als_default_options(xtt_als_options* opt);
/* ALSVariant::solve(A, x, b, numHalfSweeps, convergenceEpsilon, perfData)
 * (src/xerus/algorithms/als.cpp:483-553, include/xerus/algorithms/als.h:152-207),
 * for a symmetric positive definite operator (assume_spd = 1) or any operator
 * (assume_spd = 0). A = NULL is the operator-free form x ~ b (the overloads
 * without an operator, als.h:181-206; sites = 1 only). x is updated in place.
 * The traces (optional, trace_capacity entries each) receive, per recorded
 * point, the residual (if record_residuals: ||A x - b|| / ||b||, or ||x - b||
 * without an operator, as the reference's PerformanceData) and the flags of
 * PerformanceData (0, 1 = half sweep, 3 = full sweep; als.h:109-110); energies
 * gets the energy at the end of every half-sweep. report->residual is always
 * relative (||x - b|| / ||b|| without an operator). */
int xtt_als(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, const xtt_als_options* opt,
            xtt_als_report* report, double* residual_trace, int64_t* flag_trace, double* energy_trace,
            int64_t trace_capacity);

/* Batched ALS_SPD over `count` independent instances (no reference counterpart
 * as one call: each instance is what ALSVariant::solve does for one problem,
 * src/xerus/algorithms/als.cpp:483-553, with sites = 1 and the exact local
 * solver). Instances may differ in order (<= 16), mode sizes and ranks (x ranks
 * <= 64, maximal-reduced); all tensors live on ctx. One persistent launch: each
 * CTA sweeps one instance at a time, instances taken longest-first. The launch
 * (descriptor upload, counter reset, kernel, result download) is captured as a
 * CUDA graph and replayed by later calls with the same batch signature. With
 * autotune = 1 the first call of a signature times the launch shapes
 * (threads x CTAs per SM), then the register tile shapes of the GEMMs and of the
 * local operator at the fastest launch shape, on the batch itself, restoring x
 * between trials, and caches the fastest. num_half_sweeps (or, when 0, the energy criterion) is
 * capped at 1024 half-sweeps per instance. x[i] is updated in place (and left canonical at its
 * start position if preserve_core_position, else where the sweep ended);
 * energies[i] receives what ALSVariant::operator() returns for instance i. */
typedef struct xtt_batch_report {
	double milliseconds;   /* device time of the batched launch */
	int32_t threads;       /* launch shape used */
	int32_t ctas_per_sm;
	int32_t ctas;
	int32_t tile;          /* register tiles: 0 one output per thread; 1 GEMM 2 x 2 and local
	                          operator 2 rows per thread; 2 GEMM 4 x 2 and 4 rows */
} xtt_batch_report;
int xtt_als_batch(xtt_context* ctx, int64_t count, const xtt_tensor* const* A, xtt_tensor* const* x,
                  const xtt_tensor* const* b, const xtt_als_options* opt, int autotune, double* energies,
                  int64_t* local_iterations, xtt_batch_report* report);

/* Gradient of the ALS energy J(x) = <x, A x> - 2 <x, b> with respect to every
 * core of x (no gauge condition), for symmetric A: dJ/dX_k = 2 (L_k A_k R_k x_k -
 * Lb_k b_k Rb_k) with environments built from all other cores. grad receives the
 * cores concatenated like xtt_tensor_get_cores. At a canonical x with core k it
 * equals -2 times the ASD_solver step direction (src/xerus/algorithms/als.cpp:81). */
int xtt_als_energy_gradient(const xtt_tensor* A, const xtt_tensor* x, const xtt_tensor* b, double* energy,
                            double* grad, int64_t count);

/* ------------------------------------------------------------------- ADF */
typedef struct xtt_adf_options {
	int64_t max_iterations;          /* ADFVariant::maxIterations (adf.h:233), 0 = unlimited */
	double target_residual;          /* ADFVariant::targetResidualNorm (adf.h:234) */
	double min_decrease;             /* ADFVariant::minimalResidualNormDecrease (adf.h:235) */
	int32_t precision;               /* XTT_PRECISION_FP64; XTT_PRECISION_MIXED: FP32 stacks and per-sample
	                                    arithmetic, FP64 cores and QR, FP64-checked final residual (no
	                                    reference counterpart) */
	int32_t reserved;
} xtt_adf_options;

/* ADFVariant(maxIter, target, minDecrease)(x, SinglePointMeasurementSet{positions, values})
 * (include/xerus/algorithms/adf.h:248-252, src/xerus/algorithms/adf.cpp:489-604), x at its
 * maximal ranks. positions: num*order int64 (row-major), need not be sorted. residual_trace
 * receives the relative residual at the start of every iteration (PerformanceData). */
int xtt_adf(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num,
            const xtt_adf_options* opt, double* final_residual, double* residual_trace,
            int64_t trace_capacity, int64_t* trace_count);

/* ADFVariant(maxIter, target, minDecrease)(x, SinglePointMeasurementSet, maxRanks)
 * (include/xerus/algorithms/adf.h:263-266, src/xerus/algorithms/adf.cpp:566-604): x may
 * start below max_ranks (order-1 inner ranks, reduced to the maximal ranks). Whenever a
 * run at the current ranks stops early (stagnation) with the residual above the target
 * and ranks below max_ranks, a random rank-one TT from the library's random state
 * (xtt_random_seed), scaled to 1e-6 ||x||, is added and x is rounded to max_ranks
 * (adf.cpp:590-602); the iteration count carries on. The traces receive, per recorded
 * point (PerformanceData), the relative residual, the iteration count and the order-1
 * inner ranks (rank_trace: trace_capacity x (order-1)); each may be NULL. */
int xtt_adf_max_ranks(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num,
                      const int64_t* max_ranks, const xtt_adf_options* opt, double* final_residual,
                      double* residual_trace, int64_t* iteration_trace, int64_t* rank_trace, int64_t trace_capacity,
                      int64_t* trace_count);

/* GeometricCGVariant(numSteps, convergenceEpsilon, assumeSPD, SubmanifoldRetractionI,
 * ProjectiveVectorTransport)(A, x, b, numSteps, perfData) (src/xerus/algorithms/cg.cpp:34-120,
 * retractions.cpp, steepestDescent.cpp:37-80): Riemannian CG on the TT manifold of x's
 * ranks; A = NULL minimises ||x - b||. x must be canonical at core 0 (as the reference
 * requires) and is updated in place. residual receives ||b - A x|| (absolute, what the
 * reference returns); residual_trace the residual before the first and after every step. */
int xtt_geometric_cg(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                     double convergence_epsilon, int assume_spd, double* residual, double* residual_trace,
                     int64_t trace_capacity, int64_t* trace_count);
/* SteepestDescentVariant(numSteps, convergenceEpsilon, assumeSPD, SubmanifoldRetractionII)
 * (src/xerus/algorithms/steepestDescent.cpp:83-175): same arguments and results as
 * xtt_geometric_cg (the stopping tests are absolute, as in the reference). */
int xtt_steepest_descent(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                         double convergence_epsilon, int assume_spd, double* residual, double* residual_trace,
                         int64_t trace_capacity, int64_t* trace_count);

/* IHT(x, SinglePointMeasurementSet, perfData) (include/xerus/algorithms/iht.h:32,
 * src/xerus/algorithms/iht.cpp:29-155) for at most max_iterations iterations (the
 * reference has no stopping test and runs 10^6). Per iteration the steps beta alpha
 * (beta = 1/1.1, 1, 1.1, .., < 1.65) of y - P(x) are each taken by one ALS sweep of x
 * towards x + the step (the rank-(r + N) tensor is never formed); a trial no worse than
 * the best so far is kept, as in the reference. x keeps its ranks. residual receives
 * ||y - P(x)|| (absolute), residual_trace the best residual of every iteration. */
int xtt_iht(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num, int64_t max_iterations,
            double* residual, double* residual_trace, int64_t trace_capacity, int64_t* trace_count);

/* The retractions of src/xerus/algorithms/retractions.cpp for the Riemannian solvers:
 * SUBMANIFOLD: SubmanifoldRetractionI / II (:222-236), componentwise addition of the
 * tangent components, then move_core(0, keepRank) - what xtt_geometric_cg and
 * xtt_steepest_descent use. HOSVD: HOSVDRetractionI / II (:43-55), the step added as a
 * TT of larger rank (the tangent vector's added_to_base, or x + step), then
 * round(oldRanks). ALS: ALSRetractionI / II (:57-69), ALSVariant(1, 2, lapack_solver,
 * false) without an operator fits x (its ranks kept) to that TT. */
typedef enum xtt_retraction {
	XTT_RETRACTION_SUBMANIFOLD = 0,
	XTT_RETRACTION_HOSVD = 1,
	XTT_RETRACTION_ALS = 2
} xtt_retraction;
/* xtt_geometric_cg / xtt_steepest_descent with the retraction chosen
 * (GeometricCGVariant(..., retraction, ProjectiveVectorTransport), include/xerus/algorithms/cg.h:55-62;
 * SteepestDescentVariant(..., retraction), include/xerus/algorithms/steepestDescent.h:60-63). */
int xtt_geometric_cg_retraction(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                                double convergence_epsilon, int assume_spd, int retraction, double* residual,
                                double* residual_trace, int64_t trace_capacity, int64_t* trace_count);
int xtt_steepest_descent_retraction(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                                    double convergence_epsilon, int assume_spd, int retraction, double* residual,
                                    double* residual_trace, int64_t trace_capacity, int64_t* trace_count);

/* RankOneMeasurementSet (include/xerus/measurments.h:94-140): a sample is
 * <x, u_1 (x) ... (x) u_d> for vectors u_k of length n_k; `vectors` holds each
 * sample's vectors concatenated (num x sum n_k doubles, row-major).
 * xtt_random_rank_one: RankOneMeasurementSet::random(num, dims)
 * (src/xerus/measurments.cpp:522-544): Gaussian vectors from the library's random
 * state (Tensor::random per mode), sorted as the reference sorts them.
 * xtt_entries_rank_one: RankOneMeasurementSet::measure(TensorNetwork).
 * xtt_adf_rank_one: ADFVariant(maxIter, target, minDecrease)(x, RankOneMeasurementSet)
 * (src/xerus/algorithms/adf.cpp:233-288, 333-357, 405-408, 481-487), FP64 only, ranks
 * <= 8 and mode sizes <= 16 on the device. */
int xtt_random_rank_one(int64_t num, int64_t order, const int64_t* dims, double* vectors);
int xtt_entries_rank_one(const xtt_tensor* x, const double* vectors, int64_t count, double* out);
int xtt_adf_rank_one(xtt_tensor* x, const double* vectors, const double* values, int64_t num,
                     const xtt_adf_options* opt, double* final_residual, double* residual_trace,
                     int64_t trace_capacity, int64_t* trace_count);
/* Loss 0.5 ||P_Omega(x) - y||^2 and its gradient with respect to every core of x
 * (adjoint of the sampled-entry map; at the core position it is minus
 * ADF's projected gradient, src/xerus/algorithms/adf.cpp:359-396). */
int xtt_adf_gradient(const xtt_tensor* x, const int64_t* positions, const double* values, int64_t num,
                     double* loss, double* grad, int64_t count);

#ifdef __cplusplus
}
#endif
#endif /* XTT_H */
