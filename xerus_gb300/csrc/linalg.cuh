// Dense FP64 factorisations of TT cores on the device: Householder QR (plain
// or with column pivoting and the reference's rank rule) and a one-sided Jacobi
// SVD with the reference's truncation rule. One CTA per factorisation; the
// matrix is staged in shared memory when it fits, else in a global workspace.
#pragma once

#include "common.cuh"

namespace xtt {

struct QrArgs {
	const double* A = nullptr;  // input, row-major with leading dimension lda
	long long lda = 0;
	int m = 0, n = 0;           // A is m x n
	int transpose = 0;          // factor A^T instead of A (for LQ / CQ)
	int pivot = 0;              // column pivoting + rank rule (QC / CQ)
	double* work = nullptr;     // global workspace (mw*nw doubles) when shared memory is too small
	// Outputs, written after the rank is known:
	//  transpose == 0: A = Q C, Q (m x rank) row-major ld rank, C (rank x n) row-major ld n
	//  transpose == 1: A = C Q, C (m x rank) row-major ld rank, Q (rank x n) row-major ld n
	double* Q = nullptr;
	double* C = nullptr;
	int* rank_out = nullptr;    // device int
	int want_q = 1;             // 0: only C (the triangular factor) is written, Q is not formed
	int rank_rule = 1;          // 0 with pivot: keep all min(m, n) rows of R (pivoting only)
	double rank_tol = 16 * 2.220446049250313e-16;  // the rank rule: first k with |R_kk| < rank_tol R_00
	// reflector output instead of Q (launch_qr_reflectors): V (m_w x k_q row-major, unit lower
	// trapezoidal: the dlarfg vectors of the factored m_w x n_w matrix) and tau (k_q)
	double* V_out = nullptr;
	double* tau_out = nullptr;
};

struct SvdArgs {
	const double* X = nullptr;  // m x n row-major, leading dimension ldx
	long long ldx = 0;
	int m = 0, n = 0;
	int max_rank = 0;           // 0 = no cap
	double eps = 0.0;           // drop from the first j >= 1 with S[j] <= eps * S[0]
	double* work = nullptr;     // global workspace when shared memory is too small
	double* U = nullptr;        // m x rank, ld rank
	double* S = nullptr;        // rank
	double* Vt = nullptr;       // rank x n, ld n
	int* rank_out = nullptr;
	int* status = nullptr;
	int max_sweeps = 60;
	int orth_rows = 0;          // square X only: orthogonalise the rows (Jacobi on X^T) instead of the columns
	const double* V0 = nullptr; // columns orthogonalised (tall): the starting right factor (n x n row-major)
	                            // instead of the identity; X is then X_orig V0 and V = V0 J
};

// Algorithmic work of one factorisation: operand bytes read and written once
// (A, the triangular factor, Q if formed) and Householder flops (2 m n^2 - 2/3 n^3
// for the factor, the same again to form Q).
inline double qr_work_bytes(const QrArgs& a) {
	const double mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n, kq = mw < nw ? mw : nw;
	return 8.0 * (mw * nw + kq * nw + (a.want_q ? mw * kq : 0.0));
}
inline double qr_work_flops(const QrArgs& a) {
	const double mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n, kq = mw < nw ? mw : nw;
	const double f = 2.0 * mw * nw * kq - 2.0 / 3.0 * kq * kq * kq;
	return a.want_q ? 2.0 * f : f;
}

// Launchers (stream-ordered, asynchronous).
void launch_qr(const QrArgs& a, cudaStream_t s);
// The one-barrier cluster QR writing C and the reflectors (a.V_out, a.tau_out) instead of Q,
// for callers that form Q by blocked WY products; false (nothing launched) where that kernel
// does not take the shape.
bool launch_qr_reflectors(const QrArgs& a, cudaStream_t s);

// transfer_core with keepRank of a small core in one launch (QR / LQ of core `from`, Q in
// place, the triangular factor absorbed into core `to`), for the shapes transfer_small_fits accepts.
struct TransferArgs {
	double* from = nullptr;
	double* to = nullptr;
	int r0 = 0, nf = 0, r1 = 0;  // core from (r0, nf, r1)
	int rt = 0, nt = 0, r2 = 0;  // core to: (r1, nt, r2) moving right, (rt, nt, r0) moving left
	int right = 1;
	// optional, moving right by one warp only: first the ADF step core_from[:, i, :] +=
	// (||G_i||^2 / nrm[i]) G_i on each slice i (G shaped like core_from)
	const double* G = nullptr;
	const double* nrm = nullptr;
};
bool transfer_small_fits(const TransferArgs& t);
void launch_transfer_small(const TransferArgs& t, cudaStream_t s);
// One CTA of four warps: cores with at most 8 columns (of the factored matrix) and 128 rows.
bool transfer_narrow_fits(const TransferArgs& t);
void launch_transfer_narrow(const TransferArgs& t, cudaStream_t s);
size_t qr_work_doubles(int m, int n);        // global workspace needed (0 if shared memory suffices)
void launch_svd(const SvdArgs& a, cudaStream_t s);
size_t svd_work_doubles(int m, int n);

// Truncated SVD of X (m x n) preconditioned by a column-pivoted QR (Drmac and Veselic,
// "New fast and accurate Jacobi SVD algorithm", SIAM J. Matrix Anal. Appl. 29 (2008)):
// X P = Q R, then one-sided Jacobi on R^T, whose columns (the rows of a pivoted R) are
// graded and nearly orthogonal, so it converges in a few sweeps where Jacobi on X takes
// tens. Same outputs, rank rule and sign gauge (largest |entry| of each left vector
// positive) as launch_svd. Workspace sizes: svd_pc_workspace; shapes: svd_pc_fits.
struct SvdPcWork {
	double* q = nullptr;   // m x k or k x n (k = min(m, n))
	double* c = nullptr;   // k x k
	double* u = nullptr;   // k x k
	double* vt = nullptr;  // k x k
	double* ct = nullptr;  // k x k (m >= n: the transposed factor)
	double* ut = nullptr;  // k x k (m >= n: the Jacobi left factor)
	double* qr_work = nullptr;
	double* svd_work = nullptr;
};
bool svd_pc_fits(int m, int n);
void svd_pc_workspace(int m, int n, size_t& q, size_t& c, size_t& qr_work, size_t& svd_work);
// Phase 1: the pivoted QR; writes to the device int `kept` how many rows of R the
// Jacobi phase needs (rows below a tolerance tied to a.eps are dropped, see
// svd_pc_row_tol). Phase 2 (the caller has read `kept` to the host): svd_pc_jacobi
// returns the arguments of the Jacobi SVD (always of a tall matrix: R^T or P R^T),
// the caller runs it, and svd_pc_finish forms the factors of X.
double svd_pc_row_tol(const SvdArgs& a);
void launch_svd_pc_qr(const SvdArgs& a, const SvdPcWork& w, int* kept, cudaStream_t s);
SvdArgs svd_pc_jacobi(const SvdArgs& a, const SvdPcWork& w, int kept, cudaStream_t s);
void svd_pc_finish(const SvdArgs& a, const SvdPcWork& w, int kept, cudaStream_t s);

// FP32 stage of the mixed-precision Jacobi: one-sided Jacobi in FP32 on the columns of
// the p x q matrix X (row-major, ld ldx; scaled by a power of two into FP32 range) in
// one CTA, to FP32 orthogonality; writes the accumulated rotations W (q x q
// row-major, FP32). svd_f32_fits: the shape fits one CTA's shared memory.
bool svd_f32_fits(int p, int q);
void launch_svd_f32(const double* X, long long ldx, int p, int q, float* W, cudaStream_t s);

}  // namespace xtt
