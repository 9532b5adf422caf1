// FP64 Householder QR (optionally column-pivoted, rank-revealing) and one-sided
// Jacobi SVD, one CTA per factorisation.
//
// QR follows LAPACK's conventions so that rank decisions and signs agree with
// the reference's dgeqp3/dgeqrf path (src/xerus/blasLapackWrapper.cpp:243-438):
// reflector H = I - tau v v^T with v_j = 1, beta = -sign(alpha) ||(alpha, x)||,
// pivot = first column of largest remaining norm, rank = first k with
// |R[k,k]| < 16 eps R[0,0] (R[0,0] signed, as in the reference), Q formed in
// place by backward accumulation (dorg2r's scheme).
//
// The SVD orthogonalises the columns of the taller orientation by plane
// rotations (Hestenes' one-sided Jacobi, cyclic round-robin ordering so a warp
// owns one disjoint column pair per step), then sorts the singular values in
// descending order and applies the truncation rule of calculate_svd
// (src/xerus/tensor.cpp:1463-1474).
#include <cfloat>

#include <cooperative_groups.h>

#include "blk_qr.cuh"
#include "linalg.cuh"

namespace xtt {

constexpr int kQrThreads = 512;
constexpr int kSvdThreads = 512;
constexpr size_t kDynSmemMax = 200 * 1024;

__host__ __device__ static size_t qr_aux_doubles(int mw, int nw) { return size_t(mw < nw ? mw : nw) + size_t(nw) + size_t(nw + 1) / 2 + 2; }

size_t qr_work_doubles(int m, int n) {
	const size_t need = (qr_aux_doubles(m, n) + size_t(m) * n) * sizeof(double);
	return need <= kDynSmemMax ? 0 : size_t(m) * n;
}

__global__ void __launch_bounds__(kQrThreads) k_qr(QrArgs a, int use_smem) {
	extern __shared__ double dyn[];
	__shared__ double red[16][33];
	__shared__ double wsh[32];
	__shared__ double sred[32];
	__shared__ double s_scal, s_beta;
	__shared__ int s_idx[32];
	__shared__ int s_rank;
	const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
	const int mw = a.transpose ? a.n : a.m;
	const int nw = a.transpose ? a.m : a.n;
	const int kq = min(mw, nw);
	double* tau = dyn;
	double* cn2 = dyn + kq;
	int* perm = reinterpret_cast<int*>(dyn + kq + nw);
	double* W = use_smem ? dyn + qr_aux_doubles(mw, nw) : a.work;
	auto w = [&](int i, int j) -> double& { return W[(long long)i * nw + j]; };

	for (long long e = tid; e < (long long)mw * nw; e += blockDim.x) {
		const int i = int(e / nw), j = int(e % nw);
		W[e] = a.transpose ? a.A[(long long)j * a.lda + i] : a.A[(long long)i * a.lda + j];
	}
	for (int j = tid; j < nw; j += blockDim.x) perm[j] = j;
	__syncthreads();
	if (a.pivot) {
		for (int cb = 0; cb < nw; cb += 32) {
			const int c = cb + tx;
			double part = 0;
			if (c < nw)
				for (int i = ty; i < mw; i += 16) part += w(i, c) * w(i, c);
			red[ty][tx] = part;
			__syncthreads();
			if (ty == 0 && c < nw) {
				double s = 0;
				for (int t = 0; t < 16; ++t) s += red[t][tx];
				cn2[c] = s;
			}
			__syncthreads();
		}
	}

	for (int j = 0; j < kq; ++j) {
		if (a.pivot) {
			// first column of maximal remaining norm (idamax semantics)
			double best = -1.0;
			int bi = nw;
			for (int c = j + tid; c < nw; c += blockDim.x)
				if (cn2[c] > best) { best = cn2[c]; bi = c; }
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				const double ob = __shfl_xor_sync(0xffffffffu, best, o);
				const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
				if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
			}
			if (tx == 0) { sred[ty] = best; s_idx[ty] = bi; }
			__syncthreads();
			if (tid == 0) {
				double b = -1.0;
				int ix = nw;
				for (int t = 0; t < (int)(blockDim.x >> 5); ++t)
					if (sred[t] > b || (sred[t] == b && s_idx[t] < ix)) { b = sred[t]; ix = s_idx[t]; }
				s_idx[0] = ix;
			}
			__syncthreads();
			const int p = s_idx[0];
			if (p != j && p < nw) {
				for (int i = tid; i < mw; i += blockDim.x) {
					const double t = w(i, j);
					w(i, j) = w(i, p);
					w(i, p) = t;
				}
				if (tid == 0) {
					const double t = cn2[j]; cn2[j] = cn2[p]; cn2[p] = t;
					const int q = perm[j]; perm[j] = perm[p]; perm[p] = q;
				}
			}
			__syncthreads();
		}
		// Householder reflector of column j (dlarfg)
		double part = 0;
		for (int i = j + 1 + tid; i < mw; i += blockDim.x) part += w(i, j) * w(i, j);
		const double xnorm2 = block_sum(part, sred);
		if (tid == 0) {
			const double alpha = w(j, j);
			if (xnorm2 == 0.0) {
				tau[j] = 0.0;
				s_scal = 1.0;
				s_beta = alpha;
			} else {
				const double beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
				tau[j] = (beta - alpha) / beta;
				s_scal = 1.0 / (alpha - beta);
				s_beta = beta;
			}
		}
		__syncthreads();
		const double scal = s_scal;
		for (int i = j + 1 + tid; i < mw; i += blockDim.x) w(i, j) *= scal;
		if (tid == 0) w(j, j) = s_beta;
		__syncthreads();
		const double tj = tau[j];
		if (tj != 0.0 || a.pivot) {
			for (int cb = j + 1; cb < nw; cb += 32) {
				const int c = cb + tx;
				double pt = 0;
				if (c < nw && tj != 0.0) {
					if (ty == 0) pt = w(j, c);
					for (int i = j + 1 + ty; i < mw; i += 16) pt += w(i, j) * w(i, c);
				}
				red[ty][tx] = pt;
				__syncthreads();
				if (ty == 0) {
					double s = 0;
					for (int t = 0; t < 16; ++t) s += red[t][tx];
					wsh[tx] = tj * s;
				}
				__syncthreads();
				double nrm = 0;
				if (c < nw) {
					const double wc = wsh[tx];
					if (ty == 0) w(j, c) -= wc;
					for (int i = j + 1 + ty; i < mw; i += 16) {
						const double v = w(i, c) - wc * w(i, j);
						w(i, c) = v;
						nrm += v * v;
					}
				}
				if (a.pivot) {
					red[ty][tx] = nrm;
					__syncthreads();
					if (ty == 0 && c < nw) {
						double s = 0;
						for (int t = 0; t < 16; ++t) s += red[t][tx];
						cn2[c] = s;
					}
				}
				__syncthreads();
			}
		}
	}
	__syncthreads();
	if (tid == 0) {
		int rank = kq;
		if (a.pivot && a.rank_rule) {
			const double r00 = w(0, 0);
			for (int k = 1; k < kq; ++k)
				if (fabs(w(k, k)) < a.rank_tol * r00) { rank = k; break; }
		}
		s_rank = rank;
		if (a.rank_out) *a.rank_out = rank;
	}
	__syncthreads();
	const int rank = s_rank;
	// C (upper triangle of the first `rank` rows, columns un-permuted)
	for (long long e = tid; e < (long long)rank * nw; e += blockDim.x) {
		const int r = int(e / nw), j = int(e % nw);
		const double v = (r <= j) ? w(r, j) : 0.0;
		if (!a.transpose) a.C[(long long)r * nw + perm[j]] = v;
		else a.C[(long long)perm[j] * rank + r] = v;
	}
	__syncthreads();
	if (!a.want_q) return;
	// Q = H_0 ... H_{rank-1} [I; 0], in place in the first `rank` columns
	for (int j = rank - 1; j >= 0; --j) {
		const double tj = tau[j];
		if (j < rank - 1 && tj != 0.0) {
			for (int cb = j + 1; cb < rank; cb += 32) {
				const int c = cb + tx;
				double pt = 0;
				if (c < rank)
					for (int i = j + 1 + ty; i < mw; i += 16) pt += w(i, j) * w(i, c);
				red[ty][tx] = pt;  // row j of column c is zero here
				__syncthreads();
				if (ty == 0) {
					double s = 0;
					for (int t = 0; t < 16; ++t) s += red[t][tx];
					wsh[tx] = tj * s;
				}
				__syncthreads();
				if (c < rank) {
					const double wc = wsh[tx];
					if (ty == 0) w(j, c) = -wc;
					for (int i = j + 1 + ty; i < mw; i += 16) w(i, c) -= wc * w(i, j);
				}
				__syncthreads();
			}
		}
		for (int i = tid; i < mw; i += blockDim.x) {
			if (i > j) w(i, j) *= -tj;
			else if (i == j) w(i, j) = 1.0 - tj;
			else w(i, j) = 0.0;
		}
		__syncthreads();
	}
	for (long long e = tid; e < (long long)mw * rank; e += blockDim.x) {
		const int i = int(e / rank), c = int(e % rank);
		const double v = w(i, c);
		if (!a.transpose) a.Q[(long long)i * rank + c] = v;
		else a.Q[(long long)c * mw + i] = v;
	}
}

// ----------------------------------------------------------- cluster QR
//
// The same factorisation with the rows of the working matrix split across the
// CTAs of one thread-block cluster (up to 16 SMs), each holding its row block
// in shared memory. Per column j: every CTA contributes partial sums over its
// rows (column norm below the diagonal, then w = v^T A[:, j+1:]) to a buffer
// in its own shared memory, one hardware cluster barrier later every CTA sums
// all CTAs' partials through distributed shared memory in rank order, so all
// CTAs hold bit-identical reflectors and update only their own rows. Partial
// buffers alternate with the column's parity, which is what lets two barriers
// per column (three with pivoting) suffice. GB300's FP64 rate per SM (~8
// GFLOP/s) is what this buys back: the trailing updates run on 16 SMs.

constexpr int kQcThreads = 256;

struct QcLayout {
	int mb, nw, kq;
	__host__ __device__ size_t wl() const { return 0; }
	__host__ __device__ size_t vec() const { return size_t(mb) * nw; }
	__host__ __device__ size_t nrm() const { return vec() + 2 * size_t(nw); }
	__host__ __device__ size_t cn2() const { return nrm() + 2 * size_t(nw); }
	__host__ __device__ size_t tau() const { return cn2() + nw; }
	__host__ __device__ size_t scl() const { return tau() + kq; }
	__host__ __device__ size_t dg() const { return scl() + 8; }
	__host__ __device__ size_t perm() const { return dg() + mb; }
	__host__ __device__ size_t total() const { return perm() + size_t(nw + 1) / 2 + 1; }
};

// Sum over the cluster's CTAs, in rank order, of local[idx] in each CTA's shared
// memory. All remote loads are issued before the first add (one round trip
// instead of P); ranks >= P read rank 0 and contribute an exact zero.
__device__ __forceinline__ double cluster_sum_at(cooperative_groups::cluster_group& cl, double* local, int idx,
                                                 int P) {
	double v[16];
#pragma unroll
	for (int p = 0; p < 16; ++p) {
		const double t = cl.map_shared_rank(local, p < P ? p : 0)[idx];
		v[p] = p < P ? t : 0.0;
	}
	double s = 0;
#pragma unroll
	for (int p = 0; p < 16; ++p) s += v[p];
	return s;
}

__global__ void __launch_bounds__(kQcThreads) k_qr_cluster(QrArgs a, QcLayout lay) {
	namespace cg = cooperative_groups;
	cg::cluster_group cl = cg::this_cluster();
	const int P = int(cl.num_blocks()), me = int(cl.block_rank());
	const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, NY = kQcThreads / 32;
	const int mw = a.transpose ? a.n : a.m, nw = lay.nw, kq = lay.kq, mb = lay.mb;
	const int r0 = me * mb, r1 = min(mw, r0 + mb), nl = max(0, r1 - r0);
	extern __shared__ double sm[];
	double* Wl = sm + lay.wl();
	double* vec = sm + lay.vec();
	double* nrm = sm + lay.nrm();
	double* cn2 = sm + lay.cn2();
	double* tau = sm + lay.tau();
	double* scl = sm + lay.scl();
	double* dg = sm + lay.dg();
	int* perm = reinterpret_cast<int*>(sm + lay.perm());
	__shared__ double red[kQcThreads / 32][33];
	__shared__ double s_w[32];
	__shared__ double s_coef[3];
	__shared__ int s_idx[kQcThreads / 32];
	__shared__ double s_best[kQcThreads / 32];
	auto w = [&](int il, int j) -> double& { return Wl[(long long)il * nw + j]; };

	for (long long e = tid; e < (long long)nl * nw; e += blockDim.x) {
		const int il = int(e / nw), j = int(e % nw), gi = r0 + il;
		w(il, j) = a.transpose ? a.A[(long long)j * a.lda + gi] : a.A[(long long)gi * a.lda + j];
	}
	for (int j = tid; j < nw; j += blockDim.x) perm[j] = j;
	__syncthreads();
	// column c partial sums over local rows il >= lo of f(il, c) into dst[c] (c in [c0, nw))
	auto colsum = [&](int c0, int lo, double* dst, auto f) {
		for (int cb = c0; cb < nw; cb += 32) {
			const int c = cb + tx;
			double pt = 0;
			if (c < nw)
				for (int il = lo + ty; il < nl; il += NY) pt += f(il, c);
			red[ty][tx] = pt;
			__syncthreads();
			if (ty == 0 && c < nw) {
				double s = 0;
				for (int t = 0; t < NY; ++t) s += red[t][tx];
				dst[c] = s;
			}
			__syncthreads();
		}
	};
	auto lo_of = [&](int g) { return min(max(g - r0, 0), nl); };  // first local row with global index >= g
	if (a.pivot) {
		colsum(0, 0, nrm, [&](int il, int c) { return w(il, c) * w(il, c); });
		cl.sync();
		for (int c = tid; c < nw; c += blockDim.x) cn2[c] = cluster_sum_at(cl, nrm, c, P);
		__syncthreads();
	}
	for (int j = 0; j < kq; ++j) {
		const int par = j & 1;
		double* vecp = vec + par * nw;
		double* nrmp = nrm + (1 - par) * nw;  // the initial norms used buffer 0
		double* sclp = scl + par * 4;
		if (a.pivot) {
			double best = -1.0;
			int bi = nw;
			for (int c = j + tid; c < nw; c += blockDim.x)
				if (cn2[c] > best) { best = cn2[c]; bi = c; }
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				const double ob = __shfl_xor_sync(0xffffffffu, best, o);
				const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
				if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
			}
			if (tx == 0) { s_best[ty] = best; s_idx[ty] = bi; }
			__syncthreads();
			if (tid == 0) {
				double b = -1.0;
				int ix = nw;
				for (int t = 0; t < NY; ++t)
					if (s_best[t] > b || (s_best[t] == b && s_idx[t] < ix)) { b = s_best[t]; ix = s_idx[t]; }
				s_idx[0] = ix;
			}
			__syncthreads();
			const int p = s_idx[0];
			if (p != j && p < nw) {
				for (int il = tid; il < nl; il += blockDim.x) {
					const double t = w(il, j);
					w(il, j) = w(il, p);
					w(il, p) = t;
				}
				if (tid == 0) {
					const double t = cn2[j]; cn2[j] = cn2[p]; cn2[p] = t;
					const int q = perm[j]; perm[j] = perm[p]; perm[p] = q;
				}
			}
			__syncthreads();
		}
		// reflector of column j: partial norm below the diagonal and alpha from the owner of row j
		{
			double part = 0;
			for (int il = lo_of(j + 1) + tid; il < nl; il += blockDim.x) part += w(il, j) * w(il, j);
			__shared__ double sc[32];
			part = block_sum(part, sc);
			if (tid == 0) {
				sclp[0] = part;
				sclp[1] = (j >= r0 && j < r1) ? w(j - r0, j) : 0.0;
			}
		}
		cl.sync();
		if (tid < 2) s_coef[tid] = cluster_sum_at(cl, sclp, tid, P);
		__syncthreads();
		if (tid == 0) {
			const double xn2 = s_coef[0], alpha = s_coef[1];
			double t = 0, scal = 1.0, beta = alpha;
			if (xn2 != 0.0) {
				beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
				t = (beta - alpha) / beta;
				scal = 1.0 / (alpha - beta);
			}
			tau[j] = t;
			s_coef[0] = t;
			s_coef[1] = scal;
			s_coef[2] = beta;
		}
		__syncthreads();
		const double tj = s_coef[0], scal = s_coef[1];
		for (int il = lo_of(j + 1) + tid; il < nl; il += blockDim.x) w(il, j) *= scal;
		if (tid == 0 && j >= r0 && j < r1) w(j - r0, j) = s_coef[2];
		__syncthreads();
		// w = v^T A[:, j+1:] over local rows >= j (v_j = 1)
		const int lo = lo_of(j);
		colsum(j + 1, lo, vecp, [&](int il, int c) { return (r0 + il == j ? 1.0 : w(il, j)) * w(il, c); });
		cl.sync();
		for (int cb = j + 1; cb < nw; cb += 32) {
			const int c = cb + tx;
			if (ty == 0) s_w[tx] = c < nw ? tj * cluster_sum_at(cl, vecp, c, P) : 0.0;
			__syncthreads();
			double nr = 0;
			if (c < nw) {
				const double wc = s_w[tx];
				for (int il = lo + ty; il < nl; il += NY) {
					const double v = (r0 + il == j) ? 1.0 : w(il, j);
					const double u = w(il, c) - wc * v;
					w(il, c) = u;
					if (r0 + il > j) nr += u * u;
				}
			}
			if (a.pivot) {
				red[ty][tx] = nr;
				__syncthreads();
				if (ty == 0 && c < nw) {
					double s = 0;
					for (int t = 0; t < NY; ++t) s += red[t][tx];
					nrmp[c] = s;
				}
			}
			__syncthreads();
		}
		if (a.pivot) {
			cl.sync();
			for (int c = j + 1 + tid; c < nw; c += blockDim.x) cn2[c] = cluster_sum_at(cl, nrmp, c, P);
			__syncthreads();
		}
	}
	// rank rule: every CTA reads the diagonal through DSMEM and decides identically
	for (int il = tid; il < nl; il += blockDim.x) dg[il] = (r0 + il < kq) ? w(il, r0 + il) : 0.0;
	cl.sync();
	__shared__ int s_rank;
	// the whole diagonal, gathered in parallel into this CTA's (now unused) column-norm buffer
	double* diag = nrm;
	if (a.pivot)
		for (int k = tid; k < kq; k += blockDim.x) diag[k] = cl.map_shared_rank(dg, k / mb)[k - (k / mb) * mb];
	__syncthreads();
	if (tid == 0) {
		int rank = kq;
		if (a.pivot && a.rank_rule) {
			const double r00 = diag[0];
			for (int k = 1; k < kq; ++k)
				if (fabs(diag[k]) < a.rank_tol * r00) { rank = k; break; }
		}
		s_rank = rank;
		if (me == 0 && a.rank_out) *a.rank_out = rank;
	}
	__syncthreads();
	const int rank = s_rank;
	for (long long e = tid; e < (long long)nl * nw; e += blockDim.x) {
		const int il = int(e / nw), jj = int(e % nw), r = r0 + il;
		if (r >= rank) continue;
		const double v = (r <= jj) ? w(il, jj) : 0.0;
		if (!a.transpose) a.C[(long long)r * nw + perm[jj]] = v;
		else a.C[(long long)perm[jj] * rank + r] = v;
	}
	if (!a.want_q) {
		cl.sync();  // keep every CTA's shared memory alive until all remote reads are done
		return;
	}
	__syncthreads();
	for (int j = rank - 1; j >= 0; --j) {
		const int par = j & 1;
		double* vecp = vec + par * nw;
		const double tj = tau[j];
		const int lo = lo_of(j + 1);
		if (j < rank - 1) {
			// w_c = sum_{rows > j} v_i Q[i][c] for c in (j, rank); row j of those columns is zero
			for (int cb = j + 1; cb < rank; cb += 32) {
				const int c = cb + tx;
				double pt = 0;
				if (c < rank)
					for (int il = lo + ty; il < nl; il += NY) pt += w(il, j) * w(il, c);
				red[ty][tx] = pt;
				__syncthreads();
				if (ty == 0 && c < rank) {
					double s = 0;
					for (int t = 0; t < NY; ++t) s += red[t][tx];
					vecp[c] = s;
				}
				__syncthreads();
			}
			cl.sync();
			for (int cb = j + 1; cb < rank; cb += 32) {
				const int c = cb + tx;
				if (ty == 0) s_w[tx] = c < rank ? tj * cluster_sum_at(cl, vecp, c, P) : 0.0;
				__syncthreads();
				if (c < rank) {
					const double wc = s_w[tx];
					if (ty == 0 && j >= r0 && j < r1) w(j - r0, c) = -wc;
					for (int il = lo + ty; il < nl; il += NY) w(il, c) -= wc * w(il, j);
				}
				__syncthreads();
			}
		}
		for (int il = tid; il < nl; il += blockDim.x) {
			const int gi = r0 + il;
			if (gi > j) w(il, j) *= -tj;
			else if (gi == j) w(il, j) = 1.0 - tj;
			else w(il, j) = 0.0;
		}
		__syncthreads();
	}
	for (long long e = tid; e < (long long)nl * rank; e += blockDim.x) {
		const int il = int(e / rank), c = int(e % rank), gi = r0 + il;
		const double v = w(il, c);
		if (!a.transpose) a.Q[(long long)gi * rank + c] = v;
		else a.Q[(long long)c * mw + gi] = v;
	}
	cl.sync();  // no CTA leaves while others may still read its shared memory
}

// ----------------------------------------------------------- cluster QR, no pivoting
//
// The unpivoted factorisation (the residual's R-only sweeps and move_core with
// keepRank) with the same row-block distribution, arranged around GB300's FP64
// pipe, which takes ~64 cycles per warp instruction: no FP64 reduction runs as
// a long dependent chain. Per column j, two cluster barriers: (1) the partial
// norms of column j below the diagonal (computed during the previous column's
// update) and the diagonal entry meet in a 16-lane shuffle tree; (2) the
// partials w_c = v^T A[:, c] of each CTA's rows meet in per-column 8+8 trees.
// Inside a CTA each thread owns one column of one row group; row groups are
// combined in fixed order. Every CTA computes bit-identical reflectors.

// Sum of f(il) for il in [ia, ib) with four interleaved accumulators (short
// dependent FP64 chains), combined in a fixed order.
template <class F>
__device__ __forceinline__ double chain4(int ia, int ib, F f) {
	double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
	int il = ia;
	for (; il + 3 < ib; il += 4) {
		a0 += f(il);
		a1 += f(il + 1);
		a2 += f(il + 2);
		a3 += f(il + 3);
	}
	for (; il < ib; ++il) a0 += f(il);
	return (a0 + a1) + (a2 + a3);
}

constexpr int kQ2Threads = 256;

struct Qc2Layout {
	int mb, nw, kq, ldw;
	__host__ __device__ size_t vecw() const { return size_t(mb) * ldw; }
	__host__ __device__ size_t slot() const { return vecw() + 2 * size_t(nw); }
	__host__ __device__ size_t tau() const { return slot() + 4; }
	__host__ __device__ size_t sw() const { return tau() + kq; }
	__host__ __device__ size_t part() const { return sw() + nw; }
	__host__ __device__ size_t partn() const { return part() + 8 * 256; }
	__host__ __device__ size_t coef() const { return partn() + 8; }
	// column pivoting: exchanged (norm below the diagonal, diagonal entry) pairs per column,
	// their cluster totals, and the permutation (ints)
	__host__ __device__ size_t pslot() const { return coef() + 4; }
	__host__ __device__ size_t tb() const { return pslot() + 4 * size_t(nw); }
	__host__ __device__ size_t td() const { return tb() + nw; }
	__host__ __device__ size_t perm() const { return td() + nw; }
	__host__ __device__ size_t total() const { return perm() + size_t(nw + 1) / 2 + 1; }
};

// Column-chunk geometry of the thread-per-(column, row group) mapping.
struct ColMap {
	int Cc, ncw, G;
	__device__ ColMap(int C, int cb) {
		Cc = min(256, C - cb);
		ncw = (Cc + 31) >> 5;
		G = ncw > 0 ? max(1, 8 / ncw) : 1;
	}
};

__global__ void __launch_bounds__(kQ2Threads) k_qr_cl2(QrArgs a, Qc2Layout lay) {
	namespace cg = cooperative_groups;
	cg::cluster_group cl = cg::this_cluster();
	const int P = int(cl.num_blocks()), me = int(cl.block_rank());
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int mw = a.transpose ? a.n : a.m, nw = lay.nw, kq = lay.kq, mb = lay.mb, ldw = lay.ldw;
	const int r0 = me * mb, r1 = min(mw, r0 + mb), nl = max(0, r1 - r0);
	extern __shared__ double sm[];
	double* W = sm;
	double* vecw = sm + lay.vecw();
	double* slot = sm + lay.slot();
	double* tau = sm + lay.tau();
	double* sw = sm + lay.sw();
	double* part = sm + lay.part();
	double* partn = sm + lay.partn();
	double* coef = sm + lay.coef();
	double* pslot = sm + lay.pslot();
	double* tb = sm + lay.tb();
	double* td = sm + lay.td();
	int* perm = reinterpret_cast<int*>(sm + lay.perm());
	__shared__ double s_best[kQ2Threads / 32];
	__shared__ int s_bidx[kQ2Threads / 32];
	auto w = [&](int il, int c) -> double& { return W[(long long)il * ldw + c]; };
	auto lo_of = [&](int g) { return min(max(g - r0, 0), nl); };

	for (long long e = tid; e < (long long)nl * nw; e += kQ2Threads) {
		const int il = int(e / nw), c = int(e % nw), gi = r0 + il;
		w(il, c) = a.transpose ? a.A[(long long)c * a.lda + gi] : a.A[(long long)gi * a.lda + c];
	}
	for (int c = tid; c < nw; c += kQ2Threads) perm[c] = c;
	__syncthreads();
	if (a.pivot) {
		// column 0's exchange: per column the norm below row 0 and the row-0 entry
		for (int c = tid; c < nw; c += kQ2Threads) {
			double sb = 0;
			for (int il = lo_of(1); il < nl; ++il) sb = fma(w(il, c), w(il, c), sb);
			pslot[2 * c] = sb;
			pslot[2 * c + 1] = (0 >= r0 && 0 < r1) ? w(0 - r0, c) : 0.0;
		}
	} else if (warp == 0) {
		double s = 0;
		for (int il = lo_of(1) + lane; il < nl; il += 32) s = fma(w(il, 0), w(il, 0), s);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (lane == 0) coef[3] = s;
	}
	__syncthreads();
	for (int j = 0; j < kq; ++j) {
		const int par = j & 1;
		double* vp = vecw + par * nw;
		double* sl = slot + par * 2;
		if (a.pivot) {
			double* ps = pslot + par * 2 * nw;
			cl.sync();
			for (int c = j + tid; c < nw; c += kQ2Threads) {
				tb[c] = cluster_sum_at(cl, ps, 2 * c, P);
				td[c] = cluster_sum_at(cl, ps, 2 * c + 1, P);
			}
			__syncthreads();
			// pivot: the first column of largest remaining norm (idamax order), identical in every CTA
			double best = -1.0;
			int bi = nw;
			for (int c = j + tid; c < nw; c += kQ2Threads) {
				const double v = tb[c] + td[c] * td[c];
				if (v > best) { best = v; bi = c; }
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				const double ob = __shfl_xor_sync(0xffffffffu, best, o);
				const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
				if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
			}
			if (lane == 0) { s_best[warp] = best; s_bidx[warp] = bi; }
			__syncthreads();
			int pv = nw;
			{
				double b = -1.0;
				for (int t = 0; t < kQ2Threads / 32; ++t)
					if (s_best[t] > b || (s_best[t] == b && s_bidx[t] < pv)) { b = s_best[t]; pv = s_bidx[t]; }
			}
			if (pv != j && pv < nw) {
				for (int il = tid; il < nl; il += kQ2Threads) {
					const double t = w(il, j);
					w(il, j) = w(il, pv);
					w(il, pv) = t;
				}
				__syncthreads();
				if (tid == 0) {
					double t = tb[j]; tb[j] = tb[pv]; tb[pv] = t;
					t = td[j]; td[j] = td[pv]; td[pv] = t;
					const int q = perm[j]; perm[j] = perm[pv]; perm[pv] = q;
				}
			}
			__syncthreads();
			if (tid == 0) {
				const double xn2 = tb[j], alpha = td[j];
				double tt, scal, beta;
				reflector_scalars(alpha, xn2, beta, tt, scal);
				tau[j] = tt;
				coef[0] = scal;
				coef[1] = beta;
				coef[2] = tt;
			}
		} else {
		if (tid == 0) {
			sl[0] = coef[3];
			sl[1] = (j >= r0 && j < r1) ? w(j - r0, j) : 0.0;
		}
		cl.sync();
		if (warp == 0) {
			const int src = lane & 15, which = lane >> 4;
			const double t = cl.map_shared_rank(sl, src < P ? src : 0)[which];
			double v = src < P ? t : 0.0;
#pragma unroll
			for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
			const double alpha = __shfl_sync(0xffffffffu, v, 16);
			if (lane == 0) {
				const double xn2 = v;
				double tt, scal, beta;
				reflector_scalars(alpha, xn2, beta, tt, scal);
				tau[j] = tt;
				coef[0] = scal;
				coef[1] = beta;
				coef[2] = tt;
			}
		}
		}
		__syncthreads();
		const double scal = coef[0], tj = coef[2];
		for (int il = lo_of(j + 1) + tid; il < nl; il += kQ2Threads) w(il, j) *= scal;
		if (tid == 0 && j >= r0 && j < r1) w(j - r0, j) = coef[1];
		__syncthreads();
		const int c0 = j + 1, C = nw - c0, lo = lo_of(j), nrows = nl - lo;
		// partial w_c over this CTA's rows >= j
		for (int cb = 0; cb < C; cb += 256) {
			const ColMap cm(C, cb);
			const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
			if (g < cm.G && ci < cm.Cc) {
				const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
				double acc = 0;
				acc = chain4(ia, ib, [&](int il) { return ((r0 + il == j) ? 1.0 : w(il, j)) * w(il, c); });
				part[g * 256 + ci] = acc;
			}
			__syncthreads();
			if (tid < cm.Cc) {
				double s = 0;
				for (int gg = 0; gg < cm.G; ++gg) s += part[gg * 256 + tid];
				vp[c0 + cb + tid] = s;
			}
			__syncthreads();
		}
		cl.sync();
		// totals over the cluster: two threads per column, 8 ranks each, then one shuffle
		for (int cb = 0; cb < C; cb += 128) {
			const int Cc = min(128, C - cb), ci = tid >> 1, h = tid & 1;
			double s = 0;
			if (ci < Cc) {
				const int c = c0 + cb + ci;
				double v[8];
#pragma unroll
				for (int q = 0; q < 8; ++q) {
					const int p = 8 * h + q;
					const double t = cl.map_shared_rank(vp, p < P ? p : 0)[c];
					v[q] = p < P ? t : 0.0;
				}
				s = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
			}
			s += __shfl_xor_sync(0xffffffffu, s, 1);
			if (ci < Cc && h == 0) sw[c0 + cb + ci] = tj * s;
		}
		__syncthreads();
		// update, and the partial norms below row j+1 for the next column step (pivoting: of every
		// remaining column, with the row-(j+1) entries; else of column j+1 only)
		int G0 = 1;
		double* psn = pslot + ((j + 1) & 1) * 2 * nw;
		for (int cb = 0; cb < C; cb += 256) {
			const ColMap cm(C, cb);
			if (cb == 0) G0 = cm.G;
			const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
			if (g < cm.G && ci < cm.Cc) {
				const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
				const double wc = sw[c];
				for (int il = ia; il < ib; ++il) w(il, c) = fma(-wc, (r0 + il == j) ? 1.0 : w(il, j), w(il, c));
				const int is = max(ia, j + 2 - r0);  // rows below j+1
				const double ns = chain4(is < ia ? ia : is, ib, [&](int il) { return w(il, c) * w(il, c); });
				if (a.pivot) part[g * 256 + ci] = ns;
				else if (c == j + 1) partn[g] = ns;
			}
			if (a.pivot) {
				__syncthreads();
				if (tid < cm.Cc) {
					const int c = c0 + cb + tid;
					double sb = 0;
					for (int gg = 0; gg < cm.G; ++gg) sb += part[gg * 256 + tid];
					psn[2 * c] = sb;
					psn[2 * c + 1] = (j + 1 >= r0 && j + 1 < r1) ? w(j + 1 - r0, c) : 0.0;
				}
				__syncthreads();
			}
		}
		__syncthreads();
		if (tid == 0) {
			double s = 0;
			if (C > 0)
				for (int gg = 0; gg < G0; ++gg) s += partn[gg];
			coef[3] = s;
		}
		__syncthreads();
	}
	int rank = kq;
	if (a.pivot && a.rank_rule) {
		// the reference's rank rule on R's diagonal, gathered from its owners (|R_kk| < 16 eps R_00)
		cl.sync();
		for (int k = tid; k < kq; k += kQ2Threads) {
			const int owner = k / mb;
			tb[k] = cl.map_shared_rank(W, owner)[(long long)(k - owner * mb) * ldw + k];
		}
		__syncthreads();
		if (tid == 0) {
			int rk = kq;
			for (int k = 1; k < kq; ++k)
				if (fabs(tb[k]) < a.rank_tol * tb[0]) { rk = k; break; }
			coef[3] = double(rk);
		}
		__syncthreads();
		rank = int(coef[3]);
		cl.sync();  // the diagonal reads are done before anything rewrites W
	}
	if (me == 0 && tid == 0 && a.rank_out) *a.rank_out = rank;
	for (long long e = tid; e < (long long)nl * nw; e += kQ2Threads) {
		const int il = int(e / nw), c = int(e % nw), r = r0 + il;
		if (r >= rank) continue;
		const double v = (r <= c) ? w(il, c) : 0.0;
		if (!a.transpose) a.C[(long long)r * nw + perm[c]] = v;
		else a.C[(long long)perm[c] * rank + r] = v;
	}
	if (!a.want_q) {
		cl.sync();  // every CTA's shared memory stays alive until all remote reads are done
		return;
	}
	__syncthreads();
	// Q in place, backward accumulation of the reflectors (dorg2r)
	for (int j = rank - 1; j >= 0; --j) {
		const int par = j & 1;
		double* vp = vecw + par * nw;
		const double tj = tau[j];
		const int c0 = j + 1, C = rank - c0, lo = lo_of(j + 1), nrows = nl - lo;
		if (C > 0) {
			for (int cb = 0; cb < C; cb += 256) {
				const ColMap cm(C, cb);
				const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
				if (g < cm.G && ci < cm.Cc) {
					const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
					double acc = 0;
					acc = chain4(ia, ib, [&](int il) { return w(il, j) * w(il, c); });
					part[g * 256 + ci] = acc;
				}
				__syncthreads();
				if (tid < cm.Cc) {
					double s = 0;
					for (int gg = 0; gg < cm.G; ++gg) s += part[gg * 256 + tid];
					vp[c0 + cb + tid] = s;
				}
				__syncthreads();
			}
			cl.sync();
			for (int cb = 0; cb < C; cb += 128) {
				const int Cc = min(128, C - cb), ci = tid >> 1, h = tid & 1;
				double s = 0;
				if (ci < Cc) {
					const int c = c0 + cb + ci;
					double v[8];
#pragma unroll
					for (int q = 0; q < 8; ++q) {
						const int p = 8 * h + q;
						const double t = cl.map_shared_rank(vp, p < P ? p : 0)[c];
						v[q] = p < P ? t : 0.0;
					}
					s = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
				}
				s += __shfl_xor_sync(0xffffffffu, s, 1);
				if (ci < Cc && h == 0) sw[c0 + cb + ci] = tj * s;
			}
			__syncthreads();
			for (int cb = 0; cb < C; cb += 256) {
				const ColMap cm(C, cb);
				const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
				if (g < cm.G && ci < cm.Cc) {
					const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
					const double wc = sw[c];
					for (int il = ia; il < ib; ++il) w(il, c) = fma(-wc, w(il, j), w(il, c));
					if (g == 0 && j >= r0 && j < r1) w(j - r0, c) = -wc;
				}
			}
			__syncthreads();
		}
		for (int il = tid; il < nl; il += kQ2Threads) {
			const int gi = r0 + il;
			if (gi > j) w(il, j) *= -tj;
			else if (gi == j) w(il, j) = 1.0 - tj;
			else w(il, j) = 0.0;
		}
		__syncthreads();
	}
	for (long long e = tid; e < (long long)nl * rank; e += kQ2Threads) {
		const int il = int(e / rank), c = int(e % rank), gi = r0 + il;
		const double v = w(il, c);
		if (!a.transpose) a.Q[(long long)gi * rank + c] = v;
		else a.Q[(long long)c * mw + gi] = v;
	}
	cl.sync();
}

// Unpivoted Householder QR / LQ across a cluster with ONE cluster barrier per
// column. Rows are split over the CTAs as in k_qr_cl2. Each step needs, summed
// over the cluster, the column's squared norm below the diagonal (sigma), its
// diagonal entry (alpha), and for every trailing column c the dot product with
// the column below the diagonal (D_c) and c's diagonal-row entry (E_c). With
// v = [1; x * scal], the reflector's product with column c is
// v^T a_c = E_c + scal D_c, so all of them come from one exchange instead of a
// norm exchange followed by a dot-product exchange. Each CTA writes its
// partials for step j+1 into its own shared memory (two parities) while
// finishing step j; after the barrier every CTA reads the P partials of the
// fields it needs from the other CTAs and sums them in rank order, so all CTAs
// form bit-identical reflectors. Q (if wanted) is accumulated backwards
// (dorg2r order) with the same exchange, one barrier per reflector.
constexpr int kQ1Threads = 256;

struct Qc1Layout {
	int P, mb, nw, kq, ldw, S;  // S: fields per parity (sigma, alpha, D_c, E_c)
	__host__ __device__ size_t red() const { return size_t(mb) * ldw; }
	__host__ __device__ size_t tot() const { return red() + 2 * size_t(S); }
	__host__ __device__ size_t tau() const { return tot() + size_t(S); }
	__host__ __device__ size_t part() const { return tau() + kq; }
	// column pivoting: squared partial column norms (vn1^2, vn2^2 of dlaqp2), this CTA's partial squared
	// norms for exact (re)computation, R's diagonal, the permutation and recompute flags (ints)
	__host__ __device__ size_t vn1() const { return part() + 8 * 256; }
	__host__ __device__ size_t vn2() const { return vn1() + nw; }
	__host__ __device__ size_t rec() const { return vn2() + nw; }
	__host__ __device__ size_t beta() const { return rec() + nw; }
	__host__ __device__ size_t ints() const { return beta() + kq; }
	// Q by the compact WY form (wy = 1): the Gram totals of the reflectors (strict upper
	// part), V's top kq x kq block, and V T for this CTA's rows
	int wy;
	__host__ __device__ size_t gram() const { return ints() + size_t(nw) + 2; }
	__host__ __device__ size_t vt() const { return gram() + (wy ? size_t(kq) * (kq - 1) / 2 : 0); }
	__host__ __device__ size_t wr() const { return vt() + (wy ? size_t(kq) * kq : 0); }
	__host__ __device__ size_t total() const { return wr() + (wy ? size_t(mb) * kq : 0); }
};

__global__ void __launch_bounds__(kQ1Threads, 1) k_qr_cl1(QrArgs a, Qc1Layout lay) {
	namespace cg = cooperative_groups;
	cg::cluster_group cl = cg::this_cluster();
	const int P = lay.P, me = int(cl.block_rank());
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int mw = a.transpose ? a.n : a.m, nw = lay.nw, kq = lay.kq, mb = lay.mb, ldw = lay.ldw, S = lay.S;
	const int r0 = me * mb, r1 = min(mw, r0 + mb), nl = max(0, r1 - r0);
	extern __shared__ double sm[];
	double* W = sm;
	double* red = sm + lay.red();
	double* tot = sm + lay.tot();
	double* tau = sm + lay.tau();
	double* part = sm + lay.part();
	double* vn1 = sm + lay.vn1();
	double* vn2 = sm + lay.vn2();
	double* rec = sm + lay.rec();
	double* betas = sm + lay.beta();
	int* perm = reinterpret_cast<int*>(sm + lay.ints());
	int* flag = perm + nw;  // nw recompute flags, then the "any" flag
	__shared__ long long s_best[kQ1Threads / 32];
	__shared__ int s_bidx[kQ1Threads / 32];
	__shared__ double s_coef[3];
	auto w = [&](int il, int c) -> double& { return W[(long long)il * ldw + c]; };
	auto lo_of = [&](int g) { return min(max(g - r0, 0), nl); };

	for (long long e = tid; e < (long long)nl * nw; e += kQ1Threads) {
		const int il = int(e / nw), c = int(e % nw), gi = r0 + il;
		w(il, c) = a.transpose ? a.A[(long long)c * a.lda + gi] : a.A[(long long)gi * a.lda + c];
	}
	__syncthreads();

	// pivoting (dlaqp2 order): exact squared norms of columns [c0, nw) over rows >= row0,
	// summed over the cluster into `out` (one barrier), only where sel(c)
	auto exact_norms = [&](int c0, int row0, auto sel, auto out) {
		const int lo = lo_of(row0);
		for (int c = c0 + tid; c < nw; c += kQ1Threads) {
			double a0 = 0, a1 = 0;
			int il = lo;
			for (; il + 1 < nl; il += 2) {
				a0 = fma(w(il, c), w(il, c), a0);
				a1 = fma(w(il + 1, c), w(il + 1, c), a1);
			}
			if (il < nl) a0 = fma(w(il, c), w(il, c), a0);
			rec[c] = a0 + a1;
		}
		__syncthreads();
		cl.sync();
		for (int c = c0 + tid; c < nw; c += kQ1Threads) {
			if (!sel(c)) continue;
			double t = 0;
			for (int q = 0; q < P; ++q) t += cl.map_shared_rank(rec, q)[c];
			out(c, t);
		}
		__syncthreads();
	};
	// the first column of largest vn1 in [c0, nw) (idamax order; vn1 holds squares, same order),
	// swapped into column c0. vn1 >= 0, so its IEEE bit patterns order like its values: the
	// search compares 64-bit integers (FP64 comparisons occupy GB300's slow FP64 pipe).
	auto pivot_into = [&](int c0) {
		long long best = -1;
		int bi = nw;
		for (int c = c0 + tid; c < nw; c += kQ1Threads) {
			const long long v = __double_as_longlong(vn1[c]);
			if (v > best) { best = v; bi = c; }
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
			const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
			if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
		}
		if (lane == 0) { s_best[warp] = best; s_bidx[warp] = bi; }
		__syncthreads();
		int pv = nw;
		{
			long long b = -1;
			for (int t = 0; t < kQ1Threads / 32; ++t)
				if (s_best[t] > b || (s_best[t] == b && s_bidx[t] < pv)) { b = s_best[t]; pv = s_bidx[t]; }
		}
		if (pv != c0 && pv < nw) {
			for (int il = tid; il < nl; il += kQ1Threads) {
				const double t = w(il, c0);
				w(il, c0) = w(il, pv);
				w(il, pv) = t;
			}
			if (tid == 0) {
				double t = vn1[c0]; vn1[c0] = vn1[pv]; vn1[pv] = t;
				t = vn2[c0]; vn2[c0] = vn2[pv]; vn2[pv] = t;
				const int q = perm[c0]; perm[c0] = perm[pv]; perm[pv] = q;
			}
		}
		__syncthreads();
	};
	if (a.pivot) {
		for (int c = tid; c < nw; c += kQ1Threads) perm[c] = c;
		exact_norms(0, 0, [](int) { return true; }, [&](int c, double t) { vn1[c] = vn2[c] = t; });
		pivot_into(0);
	}

	// this CTA's partials of step jn (rows > jn) into its own slot of parity jn & 1:
	// field 0 sigma, 1 alpha, 2 + c D_c, 2 + nw + c E_c
	auto publish = [&](int jn) {
		double* slot = red + (jn & 1) * size_t(S);
		const int lo = lo_of(jn + 1), nrows = nl - lo, C = nw - jn;  // columns jn (sigma) .. nw-1
		const bool owner = jn >= r0 && jn < r1;
		for (int cb = 0; cb < C; cb += 256) {
			const ColMap cm(C, cb);
			const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
			if (g < cm.G && ci < cm.Cc) {
				const int c = jn + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
				part[g * 256 + ci] = chain4(ia, ib, [&](int il) { return w(il, jn) * w(il, c); });
			}
			__syncthreads();
			if (tid < cm.Cc) {
				const int c = jn + cb + tid;
				double sd = 0;
				for (int gg = 0; gg < cm.G; ++gg) sd += part[gg * 256 + tid];
				slot[c == jn ? 0 : 2 + c] = sd;
				slot[c == jn ? 1 : 2 + nw + c] = owner ? w(jn - r0, c) : 0.0;
			}
			__syncthreads();
		}
	};
	// cluster totals into tot[], rank order: fields 0, 1 (if head), then [2 + c0, 2 + c0 + C)
	// and, if head, [2 + nw + c0, 2 + nw + c0 + C)
	// (alpha and E_c are nonzero only in the CTA owning the diagonal row: read there, not summed)
	auto gather = [&](int par, bool head, int c0, int C) {
		const int nv = head ? 2 + 2 * C : C;
		const int owner = min((c0 - 1) / mb, P - 1);
		for (int v = tid; v < nv; v += kQ1Threads) {
			const int f = !head ? 2 + c0 + v : v < 2 ? v : v < 2 + C ? 2 + c0 + (v - 2) : 2 + nw + c0 + (v - 2 - C);
			if (head && (f == 1 || f >= 2 + nw)) {
				tot[f] = cl.map_shared_rank(red, owner)[par * S + f];
				continue;
			}
			double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
			int q = 0;
			for (; q + 3 < P; q += 4) {
				a0 += cl.map_shared_rank(red, q + 0)[par * S + f];
				a1 += cl.map_shared_rank(red, q + 1)[par * S + f];
				a2 += cl.map_shared_rank(red, q + 2)[par * S + f];
				a3 += cl.map_shared_rank(red, q + 3)[par * S + f];
			}
			for (; q < P; ++q) a0 += cl.map_shared_rank(red, q)[par * S + f];
			tot[f] = (a0 + a1) + (a2 + a3);
		}
	};

	publish(0);
	for (int j = 0; j < kq; ++j) {
		const int par = j & 1;
		cl.sync();
		// totals: sigma, alpha (fields 0, 1), D_c and E_c of the trailing columns
		const int c0 = j + 1, C = nw - c0;
		gather(par, true, c0, C);
		__syncthreads();
		// the reflector's scalars, once per CTA (a square root and a division: redundant
		// copies in every thread would queue on the FP64 pipe)
		if (tid == 0) {
			double b0, t0, s0;
			reflector_scalars(tot[1], tot[0], b0, t0, s0);
			s_coef[0] = b0;
			s_coef[1] = t0;
			s_coef[2] = s0;
			tau[j] = t0;
		}
		__syncthreads();
		const double beta = s_coef[0], tt = s_coef[1], scal = s_coef[2];
		// the reflector below the diagonal (v = x scal) and R_jj
		for (int il = lo_of(j + 1) + tid; il < nl; il += kQ1Threads) w(il, j) *= scal;
		if (tid == 0 && j >= r0 && j < r1) w(j - r0, j) = beta;
		__syncthreads();
		// trailing columns, rows >= j: a_c -= tau (E_c + scal D_c) v, v = [1; x scal]
		const int lo = lo_of(j), nrows = nl - lo;
		for (int cb = 0; cb < C; cb += 256) {
			const ColMap cm(C, cb);
			const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
			if (g < cm.G && ci < cm.Cc) {
				const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
				const double wc = tt * fma(scal, tot[2 + c], tot[2 + nw + c]);
				for (int il = ia; il < ib; ++il) w(il, c) = fma(-wc, (r0 + il == j) ? 1.0 : w(il, j), w(il, c));
			}
		}
		__syncthreads();
		if (tid == 0) betas[j] = beta;
		if (a.pivot && j + 1 < kq) {
			// downdate the partial norms with the new row j (R_jc = E_c - wc), recomputing
			// them exactly where the downdate lost accuracy (dlaqp2, tol3z = sqrt(eps)). The
			// norms are kept squared: dlaqp2's test temp (vn1/vn2)^2 <= tol3z with
			// temp = 1 - (R_jc/vn1)^2 is (vn1^2 - R_jc^2) / vn2^2 <= tol3z, and its update
			// vn1 sqrt(temp) is sqrt(vn1^2 - R_jc^2): no division or square root per column.
			if (tid == 0) flag[nw] = 0;
			__syncthreads();
			const double tol3z = sqrt(DBL_EPSILON / 2);
			for (int c = c0 + tid; c < nw; c += kQ1Threads) {
				flag[c] = 0;
				if (vn1[c] != 0.0) {
					const double e = tot[2 + nw + c];
					const double rjc = e - tt * fma(scal, tot[2 + c], e);
					const double nsq = fmax(0.0, fma(-rjc, rjc, vn1[c]));
					if (nsq <= tol3z * vn2[c]) {
						flag[c] = 1;
						flag[nw] = 1;
					} else {
						vn1[c] = nsq;
					}
				}
			}
			__syncthreads();
			if (flag[nw])
				exact_norms(c0, j + 1, [&](int c) { return flag[c] != 0; },
				            [&](int c, double t) { vn1[c] = vn2[c] = t; });
			pivot_into(c0);
		}
		// the next step's partials (columns > j)
		if (j + 1 < kq) publish(j + 1);
	}
	__syncthreads();
	int rank = kq;
	if (a.pivot && a.rank_rule)  // the reference's rank rule on R's diagonal: |R_kk| < 16 eps R_00 (signed R_00)
		for (int k = 1; k < kq; ++k)
			if (fabs(betas[k]) < a.rank_tol * betas[0]) { rank = k; break; }
	if (me == 0 && tid == 0 && a.rank_out) *a.rank_out = rank;
	for (long long e = tid; e < (long long)nl * nw; e += kQ1Threads) {
		const int il = int(e / nw), c = int(e % nw), r = r0 + il;
		if (r >= rank) continue;
		const double v = (r <= c) ? w(il, c) : 0.0;
		const int pc = a.pivot ? perm[c] : c;
		if (!a.transpose) a.C[(long long)r * nw + pc] = v;
		else a.C[(long long)pc * rank + r] = v;
	}
	cl.sync();  // every CTA has read the last partials before they are rewritten or freed
	if (!a.want_q) return;
	if (a.V_out) {
		// the reflectors for a blocked Q formation outside: rows of this CTA, unit diagonal
		for (long long e = tid; e < (long long)nl * kq; e += kQ1Threads) {
			const int il = int(e / kq), c = int(e % kq), gi = r0 + il;
			a.V_out[(long long)gi * kq + c] = gi == c ? 1.0 : (gi > c ? w(il, c) : 0.0);
		}
		if (me == 0)
			for (int c = tid; c < kq; c += kQ1Threads) a.tau_out[c] = tau[c];
		cl.sync();
		return;
	}
	if (lay.wy) {
		// Q = [I; 0] - V T V_top^T with the UT transform T^{-1} = diag(1/tau) + striu(V^T V)
		// (Joffrain, Low, Quintana-Orti, van de Geijn, Van Zee, "Accumulating Householder
		// transformations, revisited", 2006): one Gram reduction over the cluster and
		// CTA-local triangular work replace the reflector-by-reflector accumulation.
		const int n = rank, np = n * (n - 1) / 2;
		double* gt = sm + lay.gram();
		double* vt = sm + lay.vt();
		double* wr = sm + lay.wr();
		auto vv = [&](int il, int j) -> double {
			const int gi = r0 + il;
			return gi == j ? 1.0 : (gi > j ? w(il, j) : 0.0);
		};
		// this CTA's partial Gram of the reflectors, pair p = j (j - 1) / 2 + l for l < j
		for (int p = tid; p < np; p += kQ1Threads) {
			int j = int((1.0f + sqrtf(1.0f + 8.0f * float(p))) * 0.5f);
			while (j * (j - 1) / 2 > p) --j;
			while ((j + 1) * j / 2 <= p) ++j;
			const int l = p - j * (j - 1) / 2;
			double a0 = 0, a1 = 0;
			int il = lo_of(j);
			for (; il + 1 < nl; il += 2) {
				a0 = fma(vv(il, l), vv(il, j), a0);
				a1 = fma(vv(il + 1, l), vv(il + 1, j), a1);
			}
			if (il < nl) a0 = fma(vv(il, l), vv(il, j), a0);
			part[p] = a0 + a1;
		}
		__syncthreads();
		cl.sync();
		// totals of this CTA's share of the pairs (rank order), and V's top block from its owners
		const int bs = (np + P - 1) / P, p0 = me * bs, p1 = min(np, p0 + bs);
		for (int p = p0 + tid; p < p1; p += kQ1Threads) {
			double t0 = 0, t1 = 0;
			int q = 0;
			for (; q + 1 < P; q += 2) {
				t0 += cl.map_shared_rank(part, q)[p];
				t1 += cl.map_shared_rank(part, q + 1)[p];
			}
			if (q < P) t0 += cl.map_shared_rank(part, q)[p];
			gt[p] = t0 + t1;
		}
		for (int e = tid; e < n * n; e += kQ1Threads) {
			const int c = e / n, j = e - c * n;
			double v = c == j ? 1.0 : 0.0;
			if (c > j) {
				const int ow = c / mb;
				v = cl.map_shared_rank(W, ow)[(long long)(c - ow * mb) * ldw + j];
			}
			vt[e] = v;
		}
		__syncthreads();
		cl.sync();
		// the other CTAs' shares of the Gram totals
		for (int p = tid; p < np; p += kQ1Threads)
			if (p < p0 || p >= p1) gt[p] = cl.map_shared_rank(gt, min(p / bs, P - 1))[p];
		// wr = V_rows T: forward substitution on wr T^{-1} = V_rows, column by column
		for (int e = tid; e < nl * n; e += kQ1Threads) {
			const int il = e / n, j = e - il * n;
			wr[e] = j == 0 ? tau[0] * vv(il, 0) : vv(il, j);
		}
		__syncthreads();
		for (int j = 0; j + 1 < n; ++j) {
			const int m = n - j - 1;
			for (int e = tid; e < nl * m; e += kQ1Threads) {
				const int il = e / m, l = j + 1 + (e - il * m);
				const double t = fma(-wr[il * n + j], gt[l * (l - 1) / 2 + j], wr[il * n + l]);
				wr[il * n + l] = l == j + 1 ? tau[l] * t : t;
			}
			__syncthreads();
		}
		// Q_rows = E_rows - wr V_top^T (V_top unit lower triangular)
		for (int e = tid; e < nl * n; e += kQ1Threads) {
			const int il = e / n, c = e - il * n;
			double a0 = 0, a1 = 0;
			int j = 0;
			for (; j + 1 <= c; j += 2) {
				a0 = fma(wr[il * n + j], vt[c * n + j], a0);
				a1 = fma(wr[il * n + j + 1], vt[c * n + j + 1], a1);
			}
			if (j <= c) a0 = fma(wr[il * n + j], vt[c * n + j], a0);
			w(il, c) = (r0 + il == c ? 1.0 : 0.0) - (a0 + a1);
		}
		__syncthreads();
	} else {
	// Q in place, backward accumulation of the reflectors (dorg2r)
	for (int j = rank - 1; j >= 0; --j) {
		const double tj = tau[j];
		const int c0 = j + 1, C = rank - c0, lo = lo_of(j + 1), nrows = nl - lo, par = j & 1;
		if (C > 0) {
			double* slot = red + par * size_t(S);
			for (int cb = 0; cb < C; cb += 256) {
				const ColMap cm(C, cb);
				const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
				if (g < cm.G && ci < cm.Cc) {
					const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
					part[g * 256 + ci] = chain4(ia, ib, [&](int il) { return w(il, j) * w(il, c); });
				}
				__syncthreads();
				if (tid < cm.Cc) {
					double sd = 0;
					for (int gg = 0; gg < cm.G; ++gg) sd += part[gg * 256 + tid];
					slot[2 + c0 + cb + tid] = sd;
				}
				__syncthreads();
			}
			cl.sync();
			gather(par, false, c0, C);
			__syncthreads();
			for (int cb = 0; cb < C; cb += 256) {
				const ColMap cm(C, cb);
				const int g = warp / cm.ncw, ci = (warp % cm.ncw) * 32 + lane, chunk = (nrows + cm.G - 1) / cm.G;
				if (g < cm.G && ci < cm.Cc) {
					const int c = c0 + cb + ci, ia = lo + g * chunk, ib = min(nl, ia + chunk);
					const double wc = tj * tot[2 + c];
					for (int il = ia; il < ib; ++il) w(il, c) = fma(-wc, w(il, j), w(il, c));
					if (g == 0 && j >= r0 && j < r1) w(j - r0, c) = -wc;
				}
			}
			__syncthreads();
		}
		for (int il = tid; il < nl; il += kQ1Threads) {
			const int gi = r0 + il;
			if (gi > j) w(il, j) *= -tj;
			else if (gi == j) w(il, j) = 1.0 - tj;
			else w(il, j) = 0.0;
		}
		__syncthreads();
	}
	}
	for (long long e = tid; e < (long long)nl * rank; e += kQ1Threads) {
		const int il = int(e / rank), c = int(e % rank), gi = r0 + il;
		const double v = w(il, c);
		if (!a.transpose) a.Q[(long long)gi * rank + c] = v;
		else a.Q[(long long)c * mw + gi] = v;
	}
	cl.sync();  // every CTA's shared memory stays alive until the last remote reads are done
}

static int qr_cl1_size(int mw, int nw, bool want_q, Qc1Layout& lay) {
	if (mw < 48 || nw < 8) return 0;
	int P = std::min(16, (mw + 15) / 16);
	lay.mb = (mw + P - 1) / P;
	P = (mw + lay.mb - 1) / lay.mb;
	lay.P = P;
	lay.nw = nw;
	lay.kq = std::min(mw, nw);
	lay.ldw = nw | 1;
	lay.S = 2 + 2 * nw;
	lay.wy = want_q && lay.kq <= 64 ? 1 : 0;  // the partial Gram fits the 2048-entry `part` region
	if (lay.wy && lay.total() * sizeof(double) > kDynSmemMax) lay.wy = 0;
	if (lay.total() * sizeof(double) > kDynSmemMax) return 0;
	return P;
}

static int qr_cl2_size(int mw, int nw, Qc2Layout& lay) {
	if (mw < 48 || nw < 8) return 0;
	int P = std::min(16, (mw + 15) / 16);
	lay.mb = (mw + P - 1) / P;
	P = (mw + lay.mb - 1) / lay.mb;
	lay.nw = nw;
	lay.kq = std::min(mw, nw);
	lay.ldw = nw | 1;
	if (lay.total() * sizeof(double) > kDynSmemMax) return 0;
	return P;
}

// Small unpivoted factorisations (the rank-6 cores of ADF's move_core, short
// residual factors): one CTA of 128 threads running the block Householder QR,
// the working copy in dynamic shared memory.
constexpr int kQrSmallThreads = 128;
constexpr int kQrSmallMaxRows = 512;

__global__ void __launch_bounds__(kQrSmallThreads) k_qr_small(QrArgs a) {
	extern __shared__ double w_small[];
	__shared__ BlkQrSmem sh;
	const int mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n;
	blk_qr(a.A, a.lda, a.m, a.n, a.transpose, w_small, a.C, a.Q, a.want_q != 0, sh);
	if (threadIdx.x == 0 && a.rank_out) *a.rank_out = mw < nw ? mw : nw;
}

// transfer_core with keepRank for small cores in one launch: Householder QR of
// core `from` (LQ when moving left) in shared memory, Q written back in place,
// and the triangular factor absorbed into core `to` (R * core_to moving right,
// core_to * L moving left). The rank is unchanged (it never exceeds the other
// dimension of the factored matrix).
__global__ void __launch_bounds__(kQrSmallThreads) k_transfer_small(TransferArgs t) {
	extern __shared__ double sm_t[];
	__shared__ BlkQrSmem sh;
	const int tid = threadIdx.x;
	if (t.right) {
		const int mw = t.r0 * t.nf, nw = t.r1, n2 = t.nt * t.r2;
		double* W = sm_t;
		double* C = W + size_t(mw) * nw;
		double* T = C + size_t(nw) * nw;
		for (int e = tid; e < nw * n2; e += blockDim.x) T[e] = t.to[e];
		blk_qr(t.from, nw, mw, nw, 0, W, C, t.from, true, sh);
		for (int e = tid; e < nw * n2; e += blockDim.x) {
			const int i = e / n2, c = e - i * n2;
			double acc = 0;
			for (int k = i; k < nw; ++k) acc = fma(C[i * nw + k], T[k * n2 + c], acc);
			t.to[e] = acc;
		}
	} else {
		const int nw = t.r0, mw = t.nf * t.r1, m2 = t.rt * t.nt;
		double* W = sm_t;
		double* C = W + size_t(mw) * nw;
		double* T = C + size_t(nw) * nw;
		for (int e = tid; e < m2 * nw; e += blockDim.x) T[e] = t.to[e];
		blk_qr(t.from, mw, t.r0, mw, 1, W, C, t.from, true, sh);
		for (int e = tid; e < m2 * nw; e += blockDim.x) {
			const int i = e / nw, c = e - i * nw;
			double acc = 0;
			for (int k = c; k < nw; ++k) acc = fma(T[i * nw + k], C[k * nw + c], acc);
			t.to[e] = acc;
		}
	}
}

// transfer_core with keepRank for narrow cores (at most 8 columns, at most 128 rows) by
// one CTA of four warps, the matrix in shared memory: the same Householder QR as blk_qr
// (dlarfg conventions, reflectors below the diagonal, dorg2r's backward Q formation) and
// the same absorption of R into the neighbour. Its use is the ADF sweep, where it also
// applies the core's gradient step first (one launch instead of two). Measured on GB300:
// a warp issues its FP64 instructions one at a time (~64 cycles each, independent ones
// included), so the trailing columns' dot products and updates of a column step, which
// are independent, go to different warps (each SM sub-partition has its own FP64
// issue); the column's norm and reflector scalars stay one chain.
constexpr int kTwCols = 8, kTwRptMax = 4, kTwMaxSlices = 16, kTwWarps = 4;

template <int R>
__device__ __forceinline__ double tree_sum(const double* v) {
	if constexpr (R == 1) return v[0];
	else if constexpr (R == 2) return v[0] + v[1];
	else if constexpr (R == 3) return (v[0] + v[1]) + v[2];
	else return (v[0] + v[1]) + (v[2] + v[3]);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// RPT rows per lane (mw <= 32 RPT): in every warp lane l covers rows l, l + 32, .. of the
// columns that warp owns; column loops stay loops (compact code for instructions that
// run once or a few times).
template <int RPT>
__global__ void __launch_bounds__(32 * kTwWarps) k_transfer_narrow(TransferArgs t) {
	__shared__ double sA[32 * kTwRptMax][kTwCols + 1];
	__shared__ double sV[32 * kTwRptMax][kTwCols + 1];
	__shared__ double sR[kTwCols][kTwCols];
	__shared__ double sTau[kTwCols];
	__shared__ double sStep[kTwMaxSlices];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
	const int mw = t.right ? t.r0 * t.nf : t.nf * t.r1, nw = t.right ? t.r1 : t.r0;
#pragma unroll 1
	for (int e = tid; e < 32 * RPT * kTwCols; e += nt) {
		const int row = e / kTwCols, c = e % kTwCols;
		sA[row][c] = (row < mw && c < nw) ? (t.right ? t.from[row * nw + c] : t.from[c * mw + row]) : 0.0;
	}
	if (t.G) {
		// the ADF step on every slice i of core_from (rows (a, i), i = row mod n): thread i adds
		// slice i's squares and divides (the n divisions side by side), then all threads update
		const int n = t.nf;
		__syncthreads();
		if (tid < n) {
			double sum = 0.0;
#pragma unroll 1
			for (int row = tid; row < mw; row += n)
#pragma unroll 1
				for (int c = 0; c < nw; ++c) sum = fma(t.G[row * nw + c], t.G[row * nw + c], sum);
			sStep[tid] = sum / t.nrm[tid];
		}
		__syncthreads();
#pragma unroll 1
		for (int e = tid; e < mw * nw; e += nt) {
			const int row = e / nw, c = e % nw;
			sA[row][c] = fma(sStep[row % n], t.G[e], sA[row][c]);
		}
	}
	__syncthreads();
	// Householder QR, one barrier per column: every warp reads column j into registers,
	// forms ||x||^2 and the reflector scalars itself (the same instructions on the same
	// data in every warp: identical results, the FP64 chains of different warps overlap)
	// and the dot products x^T a_c of the columns it owns, then updates those columns,
	// a_c -= tau (a_jc + scal x^T a_c) [1; scal x]. Column j itself is written (scaled
	// below the diagonal, beta on it) by warp 0 after the barrier, while the next column's
	// work, which does not read it, runs. Rows >= mw are zero.
	double scal_prev = 1.0, beta_prev = 0.0;
#pragma unroll 1
	for (int j = 0; j < nw; ++j) {
		double x[RPT];
#pragma unroll
		for (int u = 0; u < RPT; ++u) {
			const int row = lane + 32 * u;
			x[u] = row > j ? sA[row][j] : 0.0;
		}
		double pu[RPT];
#pragma unroll
		for (int u = 0; u < RPT; ++u) pu[u] = x[u] * x[u];
		const double xn2 = warp_sum_d(tree_sum<RPT>(pu));
		double beta, tj, scal;
		reflector_scalars(sA[j][j], xn2, beta, tj, scal);
		if (warp == 0 && j > 0) {  // column j - 1, nobody reads it any more
#pragma unroll
			for (int u = 0; u < RPT; ++u) {
				const int row = lane + 32 * u;
				if (row > j - 1) sA[row][j - 1] *= scal_prev;
			}
			if (lane == 0) sA[j - 1][j - 1] = beta_prev;
		}
#pragma unroll 1
		for (int c = j + 1 + warp; c < nw; c += kTwWarps) {
			double pv[RPT];
#pragma unroll
			for (int u = 0; u < RPT; ++u) pv[u] = x[u] * sA[lane + 32 * u][c];
			const double ajc = sA[j][c];
			const double wc = tj * fma(scal, warp_sum_d(tree_sum<RPT>(pv)), ajc);
			const double ws = wc * scal;
#pragma unroll
			for (int u = 0; u < RPT; ++u) {
				const int row = lane + 32 * u;
				if (row > j) sA[row][c] = fma(-ws, x[u], sA[row][c]);
			}
			if (lane == 0) sA[j][c] = ajc - wc;
		}
		if (tid == 0) sTau[j] = tj;
		scal_prev = scal;
		beta_prev = beta;
		__syncthreads();
	}
	if (warp == 0 && nw > 0) {
		const int j = nw - 1;
#pragma unroll
		for (int u = 0; u < RPT; ++u) {
			const int row = lane + 32 * u;
			if (row > j) sA[row][j] *= scal_prev;
		}
		if (lane == 0) sA[j][j] = beta_prev;
	}
	__syncthreads();
	// R, and the reflectors copied aside (the Q formation reads them there while it
	// overwrites sA column by column)
	for (int e = tid; e < kTwCols * kTwCols; e += nt) {
		const int i = e / kTwCols, c = e % kTwCols;
		sR[i][c] = (i < nw && c < nw && c >= i) ? sA[i][c] : 0.0;
	}
#pragma unroll 1
	for (int e = tid; e < 32 * RPT * kTwCols; e += nt) sV[e / kTwCols][e % kTwCols] = sA[e / kTwCols][e % kTwCols];
	__syncthreads();
	// Q in place of the reflectors (dorg2r, backward), one barrier per step: every warp
	// takes v_j from the copy, updates the trailing columns it owns; warp 0 rewrites
	// column j, which no warp reads in this step
#pragma unroll 1
	for (int j = nw - 1; j >= 0; --j) {
		const double tj = sTau[j];
		double v[RPT];
#pragma unroll
		for (int u = 0; u < RPT; ++u) {
			const int row = lane + 32 * u;
			v[u] = row > j ? sV[row][j] : 0.0;
		}
#pragma unroll 1
		for (int c = j + 1 + warp; c < nw; c += kTwWarps) {
			double pv[RPT];
#pragma unroll
			for (int u = 0; u < RPT; ++u) pv[u] = v[u] * sA[lane + 32 * u][c];
			const double wc = tj * warp_sum_d(tree_sum<RPT>(pv));
#pragma unroll
			for (int u = 0; u < RPT; ++u) {
				const int row = lane + 32 * u;
				if (row > j) sA[row][c] = fma(-wc, v[u], sA[row][c]);
			}
			if (lane == 0) sA[j][c] = -wc;
		}
		if (warp == 0) {
#pragma unroll
			for (int u = 0; u < RPT; ++u) {
				const int row = lane + 32 * u;
				sA[row][j] = row > j ? -tj * v[u] : (row == j ? 1.0 - tj : 0.0);
			}
		}
		__syncthreads();
	}
	// the neighbour absorbs R (right: R * core_to; left: core_to * R^T), each thread reading
	// whole columns (right) or rows (left) of core_to before writing them
	if (t.right) {
		const int n2 = t.nt * t.r2;
#pragma unroll 1
		for (int col = tid; col < n2; col += nt) {
			double v[kTwCols];
#pragma unroll
			for (int k = 0; k < kTwCols; ++k) v[k] = k < nw ? t.to[k * n2 + col] : 0.0;
#pragma unroll
			for (int i = 0; i < kTwCols; ++i) {
				if (i >= nw) continue;
				double acc = 0.0;
#pragma unroll
				for (int k = i; k < kTwCols; ++k) acc = fma(sR[i][k], v[k], acc);
				t.to[i * n2 + col] = acc;
			}
		}
	} else {
		const int m2 = t.rt * t.nt;
#pragma unroll 1
		for (int row = tid; row < m2; row += nt) {
			double v[kTwCols];
#pragma unroll
			for (int k = 0; k < kTwCols; ++k) v[k] = k < nw ? t.to[row * nw + k] : 0.0;
#pragma unroll
			for (int c = 0; c < kTwCols; ++c) {
				if (c >= nw) continue;
				double acc = 0.0;
#pragma unroll
				for (int k = c; k < kTwCols; ++k) acc = fma(v[k], sR[c][k], acc);
				t.to[row * nw + c] = acc;
			}
		}
	}
	// Q: right, core_from (mw x nw); left, Q^T as core_from (nw x mw)
#pragma unroll 1
	for (int e = tid; e < mw * nw; e += nt) {
		const int row = e / nw, c = e % nw;
		if (t.right) t.from[row * nw + c] = sA[row][c];
		else t.from[c * mw + row] = sA[row][c];
	}
}

bool transfer_narrow_fits(const TransferArgs& t) {
	const int mw = t.right ? t.r0 * t.nf : t.nf * t.r1, nw = t.right ? t.r1 : t.r0;
	if (t.G && (!t.right || t.nf > kTwMaxSlices)) return false;
	return nw >= 1 && nw <= kTwCols && mw >= nw && mw <= 32 * kTwRptMax;
}

void launch_transfer_narrow(const TransferArgs& t, cudaStream_t s) {
	XTT_REQUIRE(transfer_narrow_fits(t), "internal: transfer_core shapes do not fit the narrow-core kernel");
	const int mw = t.right ? t.r0 * t.nf : t.nf * t.r1;
	if (mw <= 32) k_transfer_narrow<1><<<1, 32 * kTwWarps, 0, s>>>(t);
	else if (mw <= 64) k_transfer_narrow<2><<<1, 32 * kTwWarps, 0, s>>>(t);
	else if (mw <= 96) k_transfer_narrow<3><<<1, 32 * kTwWarps, 0, s>>>(t);
	else k_transfer_narrow<4><<<1, 32 * kTwWarps, 0, s>>>(t);
	XTT_CUDA(cudaGetLastError());
}

static size_t transfer_small_bytes(const TransferArgs& t) {
	const int mw = t.right ? t.r0 * t.nf : t.nf * t.r1, nw = t.right ? t.r1 : t.r0;
	const long long other = t.right ? (long long)t.nt * t.r2 : (long long)t.rt * t.nt;
	if (mw < nw || !(mw < 48 || nw < 8) || nw > kBlkQrMaxCols || mw > kQrSmallMaxRows) return 0;
	const size_t bytes = (size_t(mw) * nw + size_t(nw) * nw + size_t(nw) * other) * sizeof(double);
	return bytes > kDynSmemMax ? 0 : bytes;
}

bool transfer_small_fits(const TransferArgs& t) { return transfer_small_bytes(t) > 0; }

void launch_transfer_small(const TransferArgs& t, cudaStream_t s) {
	const size_t bytes = transfer_small_bytes(t);
	XTT_REQUIRE(bytes > 0, "internal: transfer_core shapes do not fit the one-launch kernel");
	func_attr_once(k_transfer_small, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
	k_transfer_small<<<1, kQrSmallThreads, bytes, s>>>(t);
	XTT_CUDA(cudaGetLastError());
}

// Cluster geometry for an mw x nw factorisation: 0 CTAs if the one-CTA kernel is used.
static int qr_cluster_size(int mw, int nw, QcLayout& lay) {
	if (mw < 48 || nw < 8) return 0;
	int P = std::min(16, (mw + 15) / 16);
	lay.mb = (mw + P - 1) / P;
	P = (mw + lay.mb - 1) / lay.mb;
	lay.nw = nw;
	lay.kq = std::min(mw, nw);
	if (lay.total() * sizeof(double) > kDynSmemMax) return 0;
	return P;
}

bool launch_qr_reflectors(const QrArgs& a, cudaStream_t s) {
	const int mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n;
	if (a.pivot || !a.want_q || !a.V_out || !a.tau_out) return false;
	Qc1Layout l1;
	const int P1 = qr_cl1_size(mw, nw, false, l1);  // no compact-WY buffers: Q is not formed here
	if (P1 <= 1) return false;
	func_attr_once(k_qr_cl1, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
	func_attr_once(k_qr_cl1, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(P1);
	cfg.blockDim = dim3(kQ1Threads);
	cfg.dynamicSmemBytes = l1.total() * sizeof(double);
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = P1;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	int clusters = 0;
	if (cudaOccupancyMaxActiveClusters(&clusters, k_qr_cl1, &cfg) != cudaSuccess || clusters <= 0) {
		cudaGetLastError();
		return false;
	}
	XTT_CUDA(cudaLaunchKernelEx(&cfg, k_qr_cl1, a, l1));
	return true;
}

void launch_qr(const QrArgs& a, cudaStream_t s) {
	const int mw = a.transpose ? a.n : a.m, nw = a.transpose ? a.m : a.n;
	if (!a.pivot && (mw < 48 || nw < 8) && nw <= kBlkQrMaxCols && mw <= kQrSmallMaxRows) {
		const size_t bytes = size_t(mw) * nw * sizeof(double);
		func_attr_once(k_qr_small, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
		if (bytes <= kDynSmemMax) {
			k_qr_small<<<1, kQrSmallThreads, bytes, s>>>(a);
			XTT_CUDA(cudaGetLastError());
			return;
		}
	}
	{
		Qc1Layout l1;
		const int P1 = qr_cl1_size(mw, nw, a.want_q != 0, l1);
		if (P1 > 1) {
			func_attr_once(k_qr_cl1, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
			func_attr_once(k_qr_cl1, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
			cudaLaunchConfig_t cfg = {};
			cfg.gridDim = dim3(P1);
			cfg.blockDim = dim3(kQ1Threads);
			cfg.dynamicSmemBytes = l1.total() * sizeof(double);
			cfg.stream = s;
			cudaLaunchAttribute at[1];
			at[0].id = cudaLaunchAttributeClusterDimension;
			at[0].val.clusterDim.x = P1;
			at[0].val.clusterDim.y = 1;
			at[0].val.clusterDim.z = 1;
			cfg.attrs = at;
			cfg.numAttrs = 1;
			int clusters = 0;
			if (cudaOccupancyMaxActiveClusters(&clusters, k_qr_cl1, &cfg) == cudaSuccess && clusters > 0) {
				XTT_CUDA(cudaLaunchKernelEx(&cfg, k_qr_cl1, a, l1));
				return;
			}
			cudaGetLastError();
		}
	}
	{
		Qc2Layout l2;
		const int P2 = qr_cl2_size(mw, nw, l2);
		if (P2 > 1) {
			func_attr_once(k_qr_cl2, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
			func_attr_once(k_qr_cl2, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
			cudaLaunchConfig_t cfg = {};
			cfg.gridDim = dim3(P2);
			cfg.blockDim = dim3(kQ2Threads);
			cfg.dynamicSmemBytes = l2.total() * sizeof(double);
			cfg.stream = s;
			cudaLaunchAttribute at[1];
			at[0].id = cudaLaunchAttributeClusterDimension;
			at[0].val.clusterDim.x = P2;
			at[0].val.clusterDim.y = 1;
			at[0].val.clusterDim.z = 1;
			cfg.attrs = at;
			cfg.numAttrs = 1;
			int clusters = 0;
			if (cudaOccupancyMaxActiveClusters(&clusters, k_qr_cl2, &cfg) == cudaSuccess && clusters > 0) {
				XTT_CUDA(cudaLaunchKernelEx(&cfg, k_qr_cl2, a, l2));
				return;
			}
			cudaGetLastError();
		}
	}
	QcLayout lay;
	const int P = qr_cluster_size(mw, nw, lay);
	if (P > 1) {
		func_attr_once(k_qr_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
		func_attr_once(k_qr_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(P);
		cfg.blockDim = dim3(kQcThreads);
		cfg.dynamicSmemBytes = lay.total() * sizeof(double);
		cfg.stream = s;
		cudaLaunchAttribute at[1];
		at[0].id = cudaLaunchAttributeClusterDimension;
		at[0].val.clusterDim.x = P;
		at[0].val.clusterDim.y = 1;
		at[0].val.clusterDim.z = 1;
		cfg.attrs = at;
		cfg.numAttrs = 1;
		int clusters = 0;
		if (cudaOccupancyMaxActiveClusters(&clusters, k_qr_cluster, &cfg) == cudaSuccess && clusters > 0) {
			XTT_CUDA(cudaLaunchKernelEx(&cfg, k_qr_cluster, a, lay));
			return;
		}
		cudaGetLastError();  // not schedulable as a cluster here: one CTA below
	}
	const size_t aux = qr_aux_doubles(mw, nw) * sizeof(double);
	const size_t full = aux + size_t(mw) * nw * sizeof(double);
	const int use_smem = full <= kDynSmemMax ? 1 : 0;
	XTT_REQUIRE(use_smem || a.work, "QR workspace missing");
	XTT_REQUIRE(aux <= kDynSmemMax, "QR: too many columns");
	func_attr_once(k_qr, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
	k_qr<<<1, kQrThreads, use_smem ? full : aux, s>>>(a, use_smem);
	XTT_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------- SVD

__host__ __device__ static size_t svd_aux_doubles(int q) { return 2 * size_t(q) + 2; }

size_t svd_work_doubles(int m, int n) {
	const int p = std::max(m, n), q = std::min(m, n);
	const size_t need = (svd_aux_doubles(q) + size_t(p) * q + size_t(q) * q) * sizeof(double);
	return need <= kDynSmemMax ? 0 : size_t(p) * q + size_t(q) * q;
}

// Jacobi rotation (c, s) annihilating the off-diagonal entry ga of the 2x2 Gram
// block [[al, ga], [ga, be]] (Rutishauser's t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
// zeta = (be - al) / (2 ga)), written with zeta's division folded into t:
// t = sign(zeta) |2 ga| / (|be - al| + sqrt((be - al)^2 + 4 ga^2)), c = rsqrt(1 + t^2),
// s = c t. Fewer dependent FP64 divisions (each ~400 cycles on GB300).
__device__ __forceinline__ void jacobi_rotation(double al, double be, double ga, double& c, double& s, double& t) {
	const double dba = be - al, g2 = 2.0 * ga;
	const double sg = (dba >= 0.0 ? 1.0 : -1.0) * (ga >= 0.0 ? 1.0 : -1.0);
	t = sg * fabs(g2) / (fabs(dba) + sqrt(fma(dba, dba, g2 * g2)));
	c = rsqrt(fma(t, t, 1.0));
	s = c * t;
}
__device__ __forceinline__ void jacobi_rotation(double al, double be, double ga, double& c, double& s) {
	double t;
	jacobi_rotation(al, be, ga, c, s, t);
}

// The same rotation with fewer FP64 instructions (GB300's FP64 pipe retires about
// one warp instruction per 60 cycles and SM partition): t is the root of
// F(t) = ga t^2 + (be - al) t - ga with |t| <= 1; an FP32 estimate (inputs scaled by
// a power of two through their exponent bits) is refined by two Newton steps in
// FP64 whose divisions use the FP32 reciprocal of F'(t0) (each step squares the
// relative error, 1e-7 -> 1e-14 -> rounding); c = 1/sqrt(1 + t^2) likewise from the
// FP32 rsqrt with two FP64 Newton steps, s = c t.
__device__ __forceinline__ void jacobi_rotation_fast(double al, double be, double ga, double& c, double& s,
                                                     double& t) {
	const double dba = be - al;
	const long long ed = (__double_as_longlong(dba) >> 52) & 0x7ff, eg = (__double_as_longlong(ga) >> 52) & 0x7ff;
	const long long e = ed > eg ? ed : eg;
	const double sc = __longlong_as_double((2046 - e) << 52);  // 2^(1023 - e): the larger input to [1, 2)
	const float df = float(dba * sc), gf = float(ga * sc);
	const float hf = sqrtf(fmaf(df, df, 4.f * gf * gf));
	float tf = 2.f * fabsf(gf) / (fabsf(df) + hf);
	if ((df < 0.f) != (gf < 0.f)) tf = -tf;
	const float fp = fmaf(2.f * gf, tf, df);  // F'(t0) / sc
	const double r = double(1.f / fp) * sc;    // ~ 1 / F'(t0)
	double tt = double(tf);
	tt = fma(-fma(fma(ga, tt, dba), tt, -ga), r, tt);
	tt = fma(-fma(fma(ga, tt, dba), tt, -ga), r, tt);
	const double u = fma(tt, tt, 1.0), hu = 0.5 * u;
	double y = double(rsqrtf(float(u)));
	y = y * fma(-hu, y * y, 1.5);
	y = y * fma(-hu, y * y, 1.5);
	t = tt;
	c = y;
	s = y * tt;
}

// The cluster Jacobi stops after a sweep whose rotations all had |ga| / sqrt(al be)
// below kQuadStop: in the quadratic phase the next sweep's off-diagonals are of order
// kQuadStop^2 sqrt(q), below the rotation threshold eps sqrt(p), so the sweep that
// would only confirm convergence is skipped.
constexpr double kQuadStop2 = 1e-18;  // kQuadStop = 1e-9

__global__ void __launch_bounds__(kSvdThreads) k_svd(SvdArgs a, int use_smem) {
	extern __shared__ double dyn[];
	__shared__ int s_rot, s_rank;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	const bool tall = a.m > a.n || (a.m == a.n && !a.orth_rows);
	const int p = tall ? a.m : a.n, q = tall ? a.n : a.m;
	const int qe = q + (q & 1);
	double* sig = dyn;
	int* order = reinterpret_cast<int*>(dyn + q);
	double* B = use_smem ? dyn + svd_aux_doubles(q) : a.work;  // column-major p x q
	double* V = B + (long long)p * q;                            // column-major q x q
	for (long long e = tid; e < (long long)p * q; e += blockDim.x) {
		const int c = int(e / p), i = int(e % p);
		B[e] = tall ? a.X[(long long)i * a.ldx + c] : a.X[(long long)c * a.ldx + i];
	}
	for (long long e = tid; e < (long long)q * q; e += blockDim.x) {
		const int c = int(e / q), i = int(e % q);
		V[e] = (tall && a.V0) ? a.V0[(long long)i * q + c] : (c == i ? 1.0 : 0.0);
	}
	__shared__ double s_red[32];
	double nl = 0;
	for (long long e = tid; e < (long long)p * q; e += blockDim.x) nl = fma(B[e], B[e], nl);
	// pairs with a column below 0.1 eps ||A||_F need no rotation: such columns end as singular
	// values far under every truncation threshold (8 eps S_0 >= 8 eps ||A||_F / sqrt(q)), and
	// rotating rounding noise against them keeps the sweep from converging
	const double negl = block_sum(nl, s_red) * (0.01 * DBL_EPSILON * DBL_EPSILON);
	__syncthreads();
	const double tol = DBL_EPSILON * sqrt(double(p));
	int sweep = 0;
	bool converged = (q < 2);
	for (; sweep < a.max_sweeps && !converged; ++sweep) {
		if (tid == 0) s_rot = 0;
		__syncthreads();
		for (int step = 0; step < qe - 1; ++step) {
			for (int pr = warp; pr < qe / 2; pr += nwarps) {
				const int k1 = pr, k2 = qe - 1 - pr;
				const int i = (k1 == 0) ? 0 : ((k1 - 1 + step) % (qe - 1)) + 1;
				const int j = (k2 == 0) ? 0 : ((k2 - 1 + step) % (qe - 1)) + 1;
				if (i >= q || j >= q) continue;
				double* bi = B + (long long)i * p;
				double* bj = B + (long long)j * p;
				double al = 0, be = 0, ga = 0;
				for (int r = lane; r < p; r += 32) {
					const double x = bi[r], y = bj[r];
					al += x * x;
					be += y * y;
					ga += x * y;
				}
				al = warp_sum(al);
				be = warp_sum(be);
				ga = warp_sum(ga);
				if (ga != 0.0 && fmin(al, be) > negl && fabs(ga) > tol * sqrt(al * be)) {
					double c, s;
					jacobi_rotation(al, be, ga, c, s);
					for (int r = lane; r < p; r += 32) {
						const double x = bi[r], y = bj[r];
						bi[r] = c * x - s * y;
						bj[r] = s * x + c * y;
					}
					double* vi = V + (long long)i * q;
					double* vj = V + (long long)j * q;
					for (int r = lane; r < q; r += 32) {
						const double x = vi[r], y = vj[r];
						vi[r] = c * x - s * y;
						vj[r] = s * x + c * y;
					}
					if (lane == 0) s_rot = 1;
				}
			}
			__syncthreads();
		}
		converged = (s_rot == 0);
		__syncthreads();
	}
	if (!converged) record_status(a.status, DEV_NOT_CONVERGED);
	for (int c = warp; c < q; c += nwarps) {
		double s = 0;
		for (int r = lane; r < p; r += 32) s += B[(long long)c * p + r] * B[(long long)c * p + r];
		s = warp_sum(s);
		if (lane == 0) sig[c] = sqrt(s);
	}
	__syncthreads();
	for (int c = tid; c < q; c += blockDim.x) {
		int pos = 0;
		for (int o = 0; o < q; ++o) pos += (sig[o] > sig[c]) || (sig[o] == sig[c] && o < c);
		order[pos] = c;
	}
	__syncthreads();
	if (tid == 0) {
		int rank = q;
		if (a.max_rank > 0 && a.max_rank < rank) rank = a.max_rank;
		const double s0 = sig[order[0]];
		for (int j = 1; j < rank; ++j)
			if (sig[order[j]] <= a.eps * s0) { rank = j; break; }
		s_rank = rank;
		if (a.rank_out) *a.rank_out = rank;
	}
	__syncthreads();
	const int rank = s_rank;
	// Canonical sign gauge: the entry of largest magnitude (first on ties) of
	// each kept left singular vector is made positive, the right vector follows.
	__shared__ double s_sign[1024];
	for (int k = warp; k < rank && k < 1024; k += nwarps) {
		const int c = order[k];
		double best = -1.0, val = 0.0;
		int bi = 1 << 30;
		for (int i = lane; i < a.m; i += 32) {
			const double u = tall ? B[(long long)c * p + i] : V[(long long)c * q + i];
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
	for (int k = tid; k < rank; k += blockDim.x) a.S[k] = sig[order[k]];
	// tall: X = Bn Sigma V^T (Bn: normalised B columns); wide: X^T = Bn Sigma V^T
	for (long long e = tid; e < (long long)a.m * rank; e += blockDim.x) {
		const int i = int(e / rank), k = int(e % rank), c = order[k];
		double v;
		if (tall) v = sig[c] > 0 ? B[(long long)c * p + i] / sig[c] : 0.0;
		else v = V[(long long)c * q + i];
		a.U[(long long)i * rank + k] = s_sign[k] * v;
	}
	for (long long e = tid; e < (long long)rank * a.n; e += blockDim.x) {
		const int k = int(e / a.n), j = int(e % a.n), c = order[k];
		double v;
		if (tall) v = V[(long long)c * q + j];
		else v = sig[c] > 0 ? B[(long long)c * p + j] / sig[c] : 0.0;
		a.Vt[(long long)k * a.n + j] = s_sign[k] * v;
	}
}

// ----------------------------------------------------------- cluster SVD
//
// The one-sided Jacobi SVD above with the pairs of each round-robin step spread
// over the CTAs of one cluster (up to 16), so the FP64 work of a step runs on
// up to 16 SMs: each CTA holds the columns of its pairs (the B part, p entries,
// followed by the V part, q entries) in a double buffer in shared memory,
// rotates its pairs (one warp per pair), and after one cluster barrier pulls
// the columns its pairs need in the next step from wherever they were. The
// sweep's convergence flag, the singular values, the rank and the order are
// exchanged through distributed shared memory, so every CTA takes identical
// decisions; each CTA writes its own columns of U, S and V^T.

constexpr int kSvcThreads = 256;

struct SvcLayout {
	int p, q, qe, P, ppc, cpc;
	// a column slot: the B part [0, p), the V part [p, p + q), its squared norm at p + q
	__host__ __device__ size_t colw() const { return size_t(p) + q + 1; }
	__host__ __device__ size_t buf(int b) const { return size_t(b) * cpc * colw(); }
	__host__ __device__ size_t sig() const { return 2 * size_t(cpc) * colw(); }
	__host__ __device__ size_t flg() const { return sig() + qe; }
	__host__ __device__ size_t ord() const { return flg() + 16; }  // ints, stored from here
	__host__ __device__ size_t total() const { return ord() + size_t(qe) + 8; }
};

// column at tournament position k in step t, and the position of column c in step t
__device__ __forceinline__ int svc_col(int k, int t, int qe) { return k == 0 ? 0 : ((k - 1 + t) % (qe - 1)) + 1; }
__device__ __forceinline__ int svc_pos(int c, int t, int qe) {
	if (c == 0) return 0;
	int v = (c - 1 - t) % (qe - 1);
	if (v < 0) v += qe - 1;
	return v + 1;
}

__global__ void __launch_bounds__(kSvcThreads) k_svd_cluster(SvdArgs a, SvcLayout lay) {
	namespace cg = cooperative_groups;
	cg::cluster_group cl = cg::this_cluster();
	extern __shared__ double sm[];
	const int me = int(cl.block_rank()), tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	const int p = lay.p, q = lay.q, qe = lay.qe, P = lay.P, ppc = lay.ppc, cpc = lay.cpc;
	const size_t cw = lay.colw();
	const bool tall = a.m > a.n || (a.m == a.n && !a.orth_rows);
	double* sig = sm + lay.sig();
	double* flg = sm + lay.flg();
	int* order = reinterpret_cast<int*>(sm + lay.ord());
	__shared__ int s_rank, s_stop;
	// slot s of this CTA at step t: its tournament position
	auto slot_pos = [&](int s) {
		const int pr = me * ppc + (s >> 1);
		return (s & 1) ? qe - 1 - pr : pr;
	};
	// initial columns (step 0)
	{
		double* b0 = sm + lay.buf(0);
		for (long long e = tid; e < (long long)cpc * cw; e += blockDim.x) {
			const int s = int(e / cw), off = int(e % cw);
			const int pr = me * ppc + (s >> 1);
			double v = 0.0;
			if (pr < qe / 2) {
				const int c = svc_col(slot_pos(s), 0, qe);
				if (c < q && off < p + q) {
					if (off < p) v = tall ? a.X[(long long)off * a.ldx + c] : a.X[(long long)c * a.ldx + off];
					else if (tall && a.V0) v = a.V0[(long long)(off - p) * q + c];
					else v = (off - p == c) ? 1.0 : 0.0;
				}
			}
			b0[e] = v;
		}
	}
	__syncthreads();
	// ||A||_F^2 over the cluster (see k_svd: pairs with a negligible column are not rotated)
	__shared__ double s_red[32];
	{
		double nl = 0;
		const double* b0 = sm + lay.buf(0);
		for (long long e = tid; e < (long long)cpc * cw; e += blockDim.x)
			if (int(e % cw) < p) nl = fma(b0[e], b0[e], nl);
		nl = block_sum(nl, s_red);
		cl.sync();  // every CTA runs before the first remote store
		if (tid < P) cl.map_shared_rank(sig, tid)[me] = nl;
		cl.sync();
	}
	double na2 = 0;
	for (int c = 0; c < P; ++c) na2 += sig[c];
	const double negl = na2 * (0.01 * DBL_EPSILON * DBL_EPSILON);
	const double tol2 = DBL_EPSILON * DBL_EPSILON * double(p);  // rotate when |ga| > eps sqrt(p) sqrt(al be)
	int cur = 0, t = 0, sweep = 0;
	bool converged = (q < 2);
	bool rot = false, big = false;
	long long steps_left = (long long)a.max_sweeps * (qe - 1);
	// where the column in this CTA's slot `sl` at step t sits at step tn (push target)
	auto dest_of = [&](int sl, int tn, int nb) {
		const int c = svc_col(slot_pos(sl), t, qe);
		const int k = svc_pos(c, tn, qe);
		const int opr = k < qe / 2 ? k : qe - 1 - k;
		const int oc = opr / ppc, os = 2 * (opr % ppc) + (k < qe / 2 ? 0 : 1);
		return cl.map_shared_rank(sm + lay.buf(nb), oc) + (size_t)os * cw;
	};
	while (!converged && steps_left > 0) {
		double* bc = sm + lay.buf(cur);
		const int tn = (t + 1) % (qe - 1);
		// each warp rotates its pair and stores the two columns straight into the slots they
		// occupy at the next step (remote stores into the other buffer; no separate exchange)
		for (int lp = warp; lp < ppc; lp += nwarps) {
			const int pr = me * ppc + lp;
			if (pr >= qe / 2) continue;
			const int i = svc_col(pr, t, qe), j = svc_col(qe - 1 - pr, t, qe);
			const double* bi = bc + (size_t)(2 * lp) * cw;
			const double* bj = bc + (size_t)(2 * lp + 1) * cw;
			double* di = dest_of(2 * lp, tn, cur ^ 1);
			double* dj = dest_of(2 * lp + 1, tn, cur ^ 1);
			bool rotate = false;
			double c = 1.0, sn = 0.0, tr = 0.0, al = 0.0, be = 0.0, ga = 0.0;
			// squared column norms: computed at the first step of a sweep (for every column,
			// also one paired with the padding column of an odd count), then carried with
			// the columns and updated by each rotation (al - t ga, be + t ga), so a step
			// needs one dot product instead of three (FP64 pipe)
			if (t == 0) {
				for (int r = lane; r < p; r += 32) {
					const double x = bi[r], y = bj[r];
					al = fma(x, x, al);
					be = fma(y, y, be);
					ga = fma(x, y, ga);
				}
				al = warp_sum(al);
				be = warp_sum(be);
			} else {
				if (i < q && j < q)
					for (int r = lane; r < p; r += 32) ga = fma(bi[r], bj[r], ga);
				al = bi[p + q];
				be = bj[p + q];
			}
			if (i < q && j < q) {
				ga = warp_sum(ga);
				rotate = ga != 0.0 && fmin(al, be) > negl && ga * ga > tol2 * al * be;
				if (rotate) jacobi_rotation_fast(al, be, ga, c, sn, tr);
			}
			if (rotate) {
				for (int r = lane; r < p + q; r += 32) {
					const double x = bi[r], y = bj[r];
					di[r] = c * x - sn * y;
					dj[r] = sn * x + c * y;
				}
				if (lane == 0) {
					di[p + q] = fma(-tr, ga, al);
					dj[p + q] = fma(tr, ga, be);
				}
				rot = true;
				big = big || ga * ga >= kQuadStop2 * al * be;
			} else {
				for (int r = lane; r < p + q; r += 32) {
					di[r] = bi[r];
					dj[r] = bj[r];
				}
				if (lane == 0) {
					di[p + q] = al;
					dj[p + q] = be;
				}
			}
		}
		const bool last_step = (t == qe - 2);
		if (last_step) {
			// 0: no rotation in the sweep, 1: only rotations below kQuadStop, 2: a larger one
			__shared__ int s_rot;
			if (tid == 0) s_rot = 0;
			__syncthreads();
			if (rot) atomicMax(&s_rot, big ? 2 : 1);
			__syncthreads();
			if (tid < P) cl.map_shared_rank(flg, tid)[me] = double(s_rot);
		}
		cl.sync();  // every column of step tn is in place
		--steps_left;
		cur ^= 1;
		t = tn;
		if (last_step) {
			++sweep;
			if (tid == 0) {
				double worst = 0;
				for (int c2 = 0; c2 < P; ++c2) worst = fmax(worst, flg[c2]);
				// a sweep whose rotations were all below kQuadStop leaves off-diagonals of
				// order kQuadStop^2 (quadratic phase), under the rotation threshold: done
				s_stop = worst < 1.5 ? 1 : 0;
			}
			__syncthreads();
			converged = s_stop != 0;
			rot = false;
			big = false;
			if (converged) break;  // uniform: every CTA read the same flags
		}
	}
	if (!converged && me == 0 && tid == 0) record_status(a.status, DEV_NOT_CONVERGED);
	// singular values of this CTA's columns, pushed to every CTA
	double* bc = sm + lay.buf(cur);
	for (int s = warp; s < cpc; s += nwarps) {
		const int pr = me * ppc + (s >> 1);
		if (pr >= qe / 2) continue;
		const int c = svc_col(slot_pos(s), t, qe);
		if (c >= q) continue;
		double v = 0;
		for (int r = lane; r < p; r += 32) v = fma(bc[(size_t)s * cw + r], bc[(size_t)s * cw + r], v);
		v = warp_sum(v);
		if (lane < P) cl.map_shared_rank(sig, lane)[c] = sqrt(v);
	}
	cl.sync();
	for (int c = tid; c < q; c += blockDim.x) {
		int pos = 0;
		for (int o = 0; o < q; ++o) pos += (sig[o] > sig[c]) || (sig[o] == sig[c] && o < c);
		order[pos] = c;
	}
	__syncthreads();
	if (tid == 0) {
		int rank = q;
		if (a.max_rank > 0 && a.max_rank < rank) rank = a.max_rank;
		const double s0 = sig[order[0]];
		for (int j = 1; j < rank; ++j)
			if (sig[order[j]] <= a.eps * s0) { rank = j; break; }
		s_rank = rank;
		if (me == 0 && a.rank_out) *a.rank_out = rank;
	}
	__syncthreads();
	const int rank = s_rank;
	if (me == 0)
		for (int k = tid; k < rank; k += blockDim.x) a.S[k] = sig[order[k]];
	// this CTA's kept columns: sign gauge (largest |entry| of the left vector positive), U, V^T
	for (int s = warp; s < cpc; s += nwarps) {
		const int pr = me * ppc + (s >> 1);
		if (pr >= qe / 2) continue;
		const int c = svc_col(slot_pos(s), t, qe);
		if (c >= q) continue;
		int k = 0;
		for (int o = 0; o < q; ++o) k += (sig[o] > sig[c]) || (sig[o] == sig[c] && o < c);
		if (k >= rank) continue;
		const double* col = bc + (size_t)s * cw;  // B part [0, p), V part [p, p + q)
		const double sc = sig[c];
		double best = -1.0, val = 0.0;
		int bi = 1 << 30;
		for (int i = lane; i < a.m; i += 32) {
			const double u = tall ? col[i] : col[p + i];
			if (fabs(u) > best) { best = fabs(u); val = u; bi = i; }
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			const double ob = __shfl_xor_sync(0xffffffffu, best, o);
			const double ov = __shfl_xor_sync(0xffffffffu, val, o);
			const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
			if (ob > best || (ob == best && oi < bi)) { best = ob; val = ov; bi = oi; }
		}
		const double sg = val < 0.0 ? -1.0 : 1.0;
		for (int i = lane; i < a.m; i += 32) {
			const double u = tall ? (sc > 0 ? col[i] / sc : 0.0) : col[p + i];
			a.U[(long long)i * rank + k] = sg * u;
		}
		for (int j = lane; j < a.n; j += 32) {
			const double v = tall ? col[p + j] : (sc > 0 ? col[j] / sc : 0.0);
			a.Vt[(long long)k * a.n + j] = sg * v;
		}
	}
	cl.sync();  // no CTA leaves while another may still read its shared memory
}

static int svd_cluster_size(int m, int n, SvcLayout& lay) {
	lay.p = std::max(m, n);
	lay.q = std::min(m, n);
	if (lay.q < 16 || lay.q > 512) return 0;
	lay.qe = lay.q + (lay.q & 1);
	const int pairs = lay.qe / 2;
	int P = std::min(16, pairs);
	lay.ppc = (pairs + P - 1) / P;
	lay.P = (pairs + lay.ppc - 1) / lay.ppc;
	lay.cpc = 2 * lay.ppc;
	if (lay.cpc > 64 || lay.total() * sizeof(double) > kDynSmemMax) return 0;
	return lay.P;
}

void launch_svd(const SvdArgs& a, cudaStream_t s) {
	const int p = std::max(a.m, a.n), q = std::min(a.m, a.n);
	const size_t aux = svd_aux_doubles(q) * sizeof(double);
	const size_t full = aux + (size_t(p) * q + size_t(q) * q) * sizeof(double);
	const int use_smem = full <= kDynSmemMax ? 1 : 0;
	XTT_REQUIRE(use_smem || a.work, "SVD workspace missing");
	XTT_REQUIRE(std::min(a.m, a.n) <= 1024 || (a.max_rank > 0 && a.max_rank <= 1024), "SVD: more than 1024 kept singular values");
	SvcLayout lay;
	const int P = svd_cluster_size(a.m, a.n, lay);
	if (P > 1) {
		func_attr_once(k_svd_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
		func_attr_once(k_svd_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(P);
		cfg.blockDim = dim3(kSvcThreads);
		cfg.dynamicSmemBytes = lay.total() * sizeof(double);
		cfg.stream = s;
		cudaLaunchAttribute at[1];
		at[0].id = cudaLaunchAttributeClusterDimension;
		at[0].val.clusterDim.x = P;
		at[0].val.clusterDim.y = 1;
		at[0].val.clusterDim.z = 1;
		cfg.attrs = at;
		cfg.numAttrs = 1;
		int clusters = 0;
		if (cudaOccupancyMaxActiveClusters(&clusters, k_svd_cluster, &cfg) == cudaSuccess && clusters > 0) {
			XTT_CUDA(cudaLaunchKernelEx(&cfg, k_svd_cluster, a, lay));
			return;
		}
		cudaGetLastError();
	}
	func_attr_once(k_svd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
	k_svd<<<1, kSvdThreads, use_smem ? full : aux, s>>>(a, use_smem);
	XTT_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------ QR-preconditioned SVD

constexpr int kSvdPcThreads = 256;
constexpr int kSvdPcMaxDim = 4096;  // the left epilogue stages m + k <= 4608 doubles (36 KB)

// m >= n: X = Q C, C = U_c S Vt_c, so U = Q U_c (m x rank) and Vt = Vt_c (already in
// place). CTA j forms column j of U (one warp per row, lanes over Q's row), then fixes
// the sign gauge: the largest |entry| of the column (lowest index on ties) positive,
// with row j of Vt flipped alike.
__global__ void __launch_bounds__(kSvdPcThreads) k_svd_pc_left(const double* __restrict__ Q, int m, int k,
                                                              const double* __restrict__ Uc, const int* rank_ptr,
                                                              double* __restrict__ U, double* __restrict__ Vt, int n) {
	const int j = blockIdx.x, rank = *rank_ptr;
	if (j >= rank) return;
	extern __shared__ double sm[];
	double* uc = sm;      // k
	double* col = sm + k;  // m
	__shared__ double s_best[kSvdPcThreads / 32], s_val[kSvdPcThreads / 32];
	__shared__ int s_idx[kSvdPcThreads / 32];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	for (int l = tid; l < k; l += blockDim.x) uc[l] = Uc[(long long)l * rank + j];
	__syncthreads();
	for (int i = warp; i < m; i += nwarps) {
		const double* qr = Q + (long long)i * k;
		double acc = 0.0;
		for (int l = lane; l < k; l += 32) acc = fma(qr[l], uc[l], acc);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
		if (lane == 0) col[i] = acc;
	}
	__syncthreads();
	double best = -1.0, val = 0.0;
	int bi = 1 << 30;
	for (int i = tid; i < m; i += blockDim.x)
		if (fabs(col[i]) > best) { best = fabs(col[i]); val = col[i]; bi = i; }
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const double ob = __shfl_xor_sync(0xffffffffu, best, o);
		const double ov = __shfl_xor_sync(0xffffffffu, val, o);
		const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
		if (ob > best || (ob == best && oi < bi)) { best = ob; val = ov; bi = oi; }
	}
	if (lane == 0) { s_best[warp] = best; s_val[warp] = val; s_idx[warp] = bi; }
	__syncthreads();
	if (tid == 0) {
		for (int w = 1; w < nwarps; ++w)
			if (s_best[w] > s_best[0] || (s_best[w] == s_best[0] && s_idx[w] < s_idx[0])) {
				s_best[0] = s_best[w]; s_val[0] = s_val[w]; s_idx[0] = s_idx[w];
			}
	}
	__syncthreads();
	const double sg = s_val[0] < 0.0 ? -1.0 : 1.0;
	for (int i = tid; i < m; i += blockDim.x) U[(long long)i * rank + j] = sg * col[i];
	if (sg < 0.0)
		for (int c = tid; c < n; c += blockDim.x) Vt[(long long)j * n + c] = -Vt[(long long)j * n + c];
}

// m < n: X = C Q, C = U_c S Vt_c, so U = U_c (written in place, its gauge is already
// the one wanted) and Vt = Vt_c Q (rank x n). CTA j forms row j, threads over Q's row.
__global__ void __launch_bounds__(kSvdPcThreads) k_svd_pc_right(const double* __restrict__ Q, int k, int n,
                                                               const double* __restrict__ Vtc, const int* rank_ptr,
                                                               double* __restrict__ Vt) {
	const int j = blockIdx.x, rank = *rank_ptr;
	if (j >= rank) return;
	extern __shared__ double vr[];  // k
	for (int l = threadIdx.x; l < k; l += blockDim.x) vr[l] = Vtc[(long long)j * k + l];
	__syncthreads();
	for (int c = threadIdx.x; c < n; c += blockDim.x) {
		double acc = 0.0;
		for (int l = 0; l < k; ++l) acc = fma(vr[l], Q[(long long)l * n + c], acc);
		Vt[(long long)j * n + c] = acc;
	}
}

bool svd_pc_fits(int m, int n) {
	const int k = std::min(m, n);
	SvcLayout lay;
	return k >= 32 && std::max(m, n) <= kSvdPcMaxDim && svd_cluster_size(k, k, lay) > 1;
}

void svd_pc_workspace(int m, int n, size_t& q, size_t& c, size_t& qr_work, size_t& svd_work) {
	const int k = std::min(m, n);
	q = size_t(m) * n;
	c = size_t(k) * k;
	qr_work = m >= n ? qr_work_doubles(m, n) : qr_work_doubles(n, m);
	svd_work = svd_work_doubles(k, k);
}

double svd_pc_row_tol(const SvdArgs& a) {
	// Rows of the pivoted R with |R_kk| < tol |R_00| are dropped before the Jacobi sweeps.
	// The dropped block has Frobenius norm <= sqrt(k) tol |R_00| <= sqrt(k) tol S[0], so
	// with tol = 1e-3 eps / sqrt(k) it moves every singular value by at most 1e-3 of the
	// truncation threshold eps S[0]. Only for cutoffs well above rounding (eps >= 1e-12);
	// at the fixed-rank cutoff (8 machine epsilons) every row is kept.
	const int k = std::min(a.m, a.n);
	return a.eps >= 1e-12 ? 1e-3 * a.eps / std::sqrt(double(k)) : 0.0;
}

void launch_svd_pc_qr(const SvdArgs& a, const SvdPcWork& w, int* kept, cudaStream_t s) {
	const int m = a.m, n = a.n;
	XTT_REQUIRE(svd_pc_fits(m, n) && w.q && w.c && kept, "preconditioned SVD: shape or workspace not covered");
	// X P = Q R: tall X = Q C (C = R P^T), wide X = C Q with the factorisation of X^T (C = P R^T);
	// `kept` receives the number of rows of R kept
	const double tol = svd_pc_row_tol(a);
	QrArgs qa;
	qa.A = a.X; qa.lda = a.ldx; qa.m = m; qa.n = n; qa.transpose = m >= n ? 0 : 1; qa.pivot = 1;
	qa.rank_rule = tol > 0.0 ? 1 : 0;
	qa.rank_tol = tol;
	qa.work = w.qr_work; qa.Q = w.q; qa.C = w.c; qa.rank_out = kept; qa.want_q = 1;
	launch_qr(qa, s);
}

// B (cols x rows, row-major) = A^T for A rows x cols with leading dimension lda.
__global__ void k_transpose_d(const double* __restrict__ A, int rows, int cols, long long lda, double* __restrict__ B) {
	__shared__ double tile[32][33];
	const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
	for (int y = threadIdx.y; y < 32; y += blockDim.y) {
		const int r = r0 + y, c = c0 + threadIdx.x;
		if (r < rows && c < cols) tile[y][threadIdx.x] = A[(long long)r * lda + c];
	}
	__syncthreads();
	for (int y = threadIdx.y; y < 32; y += blockDim.y) {
		const int c = c0 + y, r = r0 + threadIdx.x;
		if (r < rows && c < cols) B[(long long)c * rows + r] = tile[threadIdx.x][y];
	}
}

// m >= n: X = Q C', C' (kk x n) = Ct^T, and the Jacobi SVD of the tall Ct = U_t S Vt_t
// gives C' = Vt_t^T S U_t^T: U = Q Vt_t^T (m x rank) and Vt = U_t^T (rank x n). CTA j
// forms column j of U (one warp per row), fixes the sign gauge on it (largest |entry|
// positive, lowest index on ties) and writes row j of Vt with the same sign.
__global__ void __launch_bounds__(kSvdPcThreads) k_svd_pc_left_t(const double* __restrict__ Q, int m, int kk,
                                                                const double* __restrict__ Vtt,
                                                                const double* __restrict__ Ut, const int* rank_ptr,
                                                                double* __restrict__ U, double* __restrict__ Vt, int n) {
	const int j = blockIdx.x, rank = *rank_ptr;
	if (j >= rank) return;
	extern __shared__ double sm[];
	double* uc = sm;        // kk
	double* col = sm + kk;  // m
	__shared__ double s_best[kSvdPcThreads / 32], s_val[kSvdPcThreads / 32];
	__shared__ int s_idx[kSvdPcThreads / 32];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	for (int l = tid; l < kk; l += blockDim.x) uc[l] = Vtt[(long long)j * kk + l];
	__syncthreads();
	for (int i = warp; i < m; i += nwarps) {
		const double* qr = Q + (long long)i * kk;
		double acc = 0.0;
		for (int l = lane; l < kk; l += 32) acc = fma(qr[l], uc[l], acc);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
		if (lane == 0) col[i] = acc;
	}
	__syncthreads();
	double best = -1.0, val = 0.0;
	int bi = 1 << 30;
	for (int i = tid; i < m; i += blockDim.x)
		if (fabs(col[i]) > best) { best = fabs(col[i]); val = col[i]; bi = i; }
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const double ob = __shfl_xor_sync(0xffffffffu, best, o);
		const double ov = __shfl_xor_sync(0xffffffffu, val, o);
		const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
		if (ob > best || (ob == best && oi < bi)) { best = ob; val = ov; bi = oi; }
	}
	if (lane == 0) { s_best[warp] = best; s_val[warp] = val; s_idx[warp] = bi; }
	__syncthreads();
	if (tid == 0) {
		for (int w = 1; w < nwarps; ++w)
			if (s_best[w] > s_best[0] || (s_best[w] == s_best[0] && s_idx[w] < s_idx[0])) {
				s_best[0] = s_best[w]; s_val[0] = s_val[w]; s_idx[0] = s_idx[w];
			}
	}
	__syncthreads();
	const double sg = s_val[0] < 0.0 ? -1.0 : 1.0;
	for (int i = tid; i < m; i += blockDim.x) U[(long long)i * rank + j] = sg * col[i];
	for (int c = tid; c < n; c += blockDim.x) Vt[(long long)j * n + c] = sg * Ut[(long long)c * rank + j];
}

SvdArgs svd_pc_jacobi(const SvdArgs& a, const SvdPcWork& w, int kk, cudaStream_t s) {
	const int m = a.m, n = a.n, k = std::min(m, n);
	XTT_REQUIRE(a.rank_out && kk >= 1 && kk <= k, "preconditioned SVD: rank output missing or kept rows out of range");
	const bool tall = m >= n;
	XTT_REQUIRE(tall ? (w.u && w.ct && w.ut) : w.vt != nullptr, "preconditioned SVD: workspace missing");
	// Jacobi on R^T, always on the columns of a tall matrix: m >= n, C' (kk x n) is
	// transposed into Ct (n x kk); m < n, C (m x kk) is used as it is
	SvdArgs sa = a;
	sa.work = w.svd_work;
	sa.orth_rows = 0;
	sa.V0 = nullptr;
	if (tall) {
		const dim3 grid((n + 31) / 32, (kk + 31) / 32), block(32, 8);
		k_transpose_d<<<grid, block, 0, s>>>(w.c, kk, n, n, w.ct);
		XTT_CUDA(cudaGetLastError());
		sa.X = w.ct;
		sa.m = n;
		sa.n = kk;
		sa.ldx = kk;
		sa.U = w.ut;  // n x rank
		sa.Vt = w.u;  // rank x kk
	} else {
		sa.X = w.c;
		sa.m = m;
		sa.n = kk;
		sa.ldx = kk;
		sa.U = a.U;   // U = U_c, its gauge already the one wanted
		sa.Vt = w.vt;
	}
	return sa;
}

void svd_pc_finish(const SvdArgs& a, const SvdPcWork& w, int kk, cudaStream_t s) {
	const int m = a.m, n = a.n;
	if (m >= n) {
		const size_t smem = size_t(kk + m) * sizeof(double);
		k_svd_pc_left_t<<<kk, kSvdPcThreads, smem, s>>>(w.q, m, kk, w.u, w.ut, a.rank_out, a.U, a.Vt, n);
	} else {
		// V^T = Vt_c Q: Vt_c is rank x kk, Q kk x n
		k_svd_pc_right<<<kk, kSvdPcThreads, size_t(kk) * sizeof(double), s>>>(w.q, kk, n, w.vt, a.rank_out, a.Vt);
	}
	XTT_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------ FP32 Jacobi stage

// Column pairs are handled by groups of LPP lanes. Where the shapes allow (64 x 64: 8 lanes
// x 8 entries; p, q <= 64: 4 x 16; <= 128: 8 x 16) each lane keeps its entries of the pair's
// columns in registers between the dot products and the rotation, and the V columns are
// fetched before the reductions: a step is one round of independent shared-memory
// accesses, with fewer warps issuing it (the stage is one CTA, bound by its issue rate).
// The columns are stored at a stride congruent to LPP mod 32 (a multiple of 4), so the
// groups of a warp, which hold consecutive columns, read disjoint banks; for the full
// shapes (p = q = LPP NR) each lane's entries are contiguous and move as float4.
struct Svf32Shape {
	int lpp, nr;
};
__host__ __device__ inline Svf32Shape svf32_shape(int p, int q) {
	if (p == 64 && q == 64) return {8, 8};  // full: 2 warps per SM sub-partition (measured best of 4/8/16 lanes)
	if (p <= 64 && q <= 64) return {4, 16};
	if (p <= 128 && q <= 128) return {8, 16};
	return {16, 0};  // entries in loops
}
// column stride: congruent to `mod` mod 32 (the full 64 x 64 shape: 16, so the two groups
// of a quarter-warp, on consecutive columns, take the two halves of the banks)
__host__ __device__ inline int svf32_ldmod(int p, int q) {
	return p == 64 && q == 64 ? 16 : svf32_shape(p, q).lpp;
}
__host__ __device__ inline int svf32_ld(int rows, int mod) { return rows + ((mod - rows % 32) % 32 + 32) % 32; }
__host__ inline int svf32_threads(int q, int lpp) {
	// at least 8 warps for the staging loops (the sweeps use the pairs' warps only)
	const int pairs = (q + (q & 1)) / 2, per_warp = 32 / lpp;
	return std::min(1024, 32 * std::max(8, (pairs + per_warp - 1) / per_warp));
}
static size_t svf32_smem(int p, int q) {
	const int mod = svf32_ldmod(p, q);
	return (size_t(svf32_ld(p, mod)) * q + size_t(svf32_ld(q, mod)) * q) * sizeof(float);
}

bool svd_f32_fits(int p, int q) { return q >= 2 && p >= q && svf32_smem(p, q) <= kDynSmemMax; }

template <int LPP, int NR, bool FULL>
__device__ void svd_f32_sweeps(float* B, int ldb, float* V, int ldv, int p, int q, float negl, float tol2, float big2,
                               int max_sweeps, int& s_rot) {
	constexpr int kGroups = 32 / LPP;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	const int qe = q + (q & 1), grp = lane / LPP, gl = lane % LPP;
	for (int sweep = 0; sweep < max_sweeps; ++sweep) {
		if (tid == 0) s_rot = 0;
		__syncthreads();
		for (int t = 0; t < qe - 1; ++t) {
			// every lane of a warp takes part in its shuffles
			for (int lp0 = kGroups * warp; lp0 < qe / 2; lp0 += kGroups * nwarps) {
				const int lp = lp0 + grp;
				int i = 0, j = 0;
				bool ok = lp < qe / 2;
				if (ok) {
					// svc_col without the division: (k - 1 + t) mod (qe - 1) for k, t < qe - 1
					const int m = qe - 1, a = lp - 1 + t, b = qe - 2 - lp + t;
					i = lp == 0 ? 0 : (a >= m ? a - m : a) + 1;
					j = (b >= m ? b - m : b) + 1;
					ok = i < q && j < q;
				}
				float* bi = B + i * ldb;
				float* bj = B + j * ldb;
				float* vi = V + i * ldv;
				float* vj = V + j * ldv;
				float al = 0.f, be = 0.f, ga = 0.f;
				float x[NR > 0 ? NR : 1], y[NR > 0 ? NR : 1], vx[NR > 0 ? NR : 1], vy[NR > 0 ? NR : 1];
				if constexpr (FULL) {
					// lane gl holds the float4 chunks gl, gl + LPP, ...: 16-byte accesses, a group's
					// lanes on consecutive chunks
					if (ok) {
#pragma unroll
						for (int u = 0; u < NR; u += 4) {
							const int r = 4 * (gl + LPP * (u / 4));
							const float4 a = *reinterpret_cast<const float4*>(bi + r);
							const float4 b = *reinterpret_cast<const float4*>(bj + r);
							const float4 c = *reinterpret_cast<const float4*>(vi + r);
							const float4 e = *reinterpret_cast<const float4*>(vj + r);
							x[u] = a.x; x[u + 1] = a.y; x[u + 2] = a.z; x[u + 3] = a.w;
							y[u] = b.x; y[u + 1] = b.y; y[u + 2] = b.z; y[u + 3] = b.w;
							vx[u] = c.x; vx[u + 1] = c.y; vx[u + 2] = c.z; vx[u + 3] = c.w;
							vy[u] = e.x; vy[u + 1] = e.y; vy[u + 2] = e.z; vy[u + 3] = e.w;
						}
					} else {
#pragma unroll
						for (int u = 0; u < NR; ++u) x[u] = y[u] = vx[u] = vy[u] = 0.f;
					}
#pragma unroll
					for (int u = 0; u < NR; ++u) {
						al = fmaf(x[u], x[u], al);
						be = fmaf(y[u], y[u], be);
						ga = fmaf(x[u], y[u], ga);
					}
				} else if constexpr (NR > 0) {
#pragma unroll
					for (int u = 0; u < NR; ++u) {
						const int r = gl + LPP * u;
						x[u] = ok && r < p ? bi[r] : 0.f;
						y[u] = ok && r < p ? bj[r] : 0.f;
						vx[u] = ok && r < q ? vi[r] : 0.f;
						vy[u] = ok && r < q ? vj[r] : 0.f;
					}
#pragma unroll
					for (int u = 0; u < NR; ++u) {
						al = fmaf(x[u], x[u], al);
						be = fmaf(y[u], y[u], be);
						ga = fmaf(x[u], y[u], ga);
					}
				} else if (ok) {
					for (int r = gl; r < p; r += LPP) {
						const float a = bi[r], b = bj[r];
						al = fmaf(a, a, al);
						be = fmaf(b, b, be);
						ga = fmaf(a, b, ga);
					}
				}
#pragma unroll
				for (int o = LPP / 2; o > 0; o >>= 1) {
					al += __shfl_xor_sync(0xffffffffu, al, o);
					be += __shfl_xor_sync(0xffffffffu, be, o);
					ga += __shfl_xor_sync(0xffffffffu, ga, o);
				}
				const float ab = al * be, g2s = ga * ga;
				if (ok && ga != 0.f && fminf(al, be) > negl && g2s > tol2 * ab) {
					const float dba = be - al, g2 = 2.f * ga;
					float tt = __fdividef(fabsf(g2), fabsf(dba) + sqrtf(fmaf(dba, dba, g2 * g2)));
					if ((dba < 0.f) != (ga < 0.f)) tt = -tt;
					const float cs = rsqrtf(fmaf(tt, tt, 1.f)), sn = cs * tt;
					if constexpr (FULL) {
#pragma unroll
						for (int u = 0; u < NR; u += 4) {
							const int r = 4 * (gl + LPP * (u / 4));
							float4 a, b, c, e;
							a.x = cs * x[u] - sn * y[u]; a.y = cs * x[u + 1] - sn * y[u + 1];
							a.z = cs * x[u + 2] - sn * y[u + 2]; a.w = cs * x[u + 3] - sn * y[u + 3];
							b.x = sn * x[u] + cs * y[u]; b.y = sn * x[u + 1] + cs * y[u + 1];
							b.z = sn * x[u + 2] + cs * y[u + 2]; b.w = sn * x[u + 3] + cs * y[u + 3];
							c.x = cs * vx[u] - sn * vy[u]; c.y = cs * vx[u + 1] - sn * vy[u + 1];
							c.z = cs * vx[u + 2] - sn * vy[u + 2]; c.w = cs * vx[u + 3] - sn * vy[u + 3];
							e.x = sn * vx[u] + cs * vy[u]; e.y = sn * vx[u + 1] + cs * vy[u + 1];
							e.z = sn * vx[u + 2] + cs * vy[u + 2]; e.w = sn * vx[u + 3] + cs * vy[u + 3];
							*reinterpret_cast<float4*>(bi + r) = a;
							*reinterpret_cast<float4*>(bj + r) = b;
							*reinterpret_cast<float4*>(vi + r) = c;
							*reinterpret_cast<float4*>(vj + r) = e;
						}
					} else if constexpr (NR > 0) {
#pragma unroll
						for (int u = 0; u < NR; ++u) {
							const int r = gl + LPP * u;
							if (r < p) {
								bi[r] = cs * x[u] - sn * y[u];
								bj[r] = sn * x[u] + cs * y[u];
							}
							if (r < q) {
								vi[r] = cs * vx[u] - sn * vy[u];
								vj[r] = sn * vx[u] + cs * vy[u];
							}
						}
					} else {
						for (int r = gl; r < p; r += LPP) {
							const float a = bi[r], b = bj[r];
							bi[r] = cs * a - sn * b;
							bj[r] = sn * a + cs * b;
						}
						for (int r = gl; r < q; r += LPP) {
							const float a = vi[r], b = vj[r];
							vi[r] = cs * a - sn * b;
							vj[r] = sn * a + cs * b;
						}
					}
					if (gl == 0 && g2s > big2 * ab) s_rot = 1;
				}
			}
			__syncthreads();
		}
		if (s_rot == 0) break;  // uniform: read after the last step's barrier
		__syncthreads();         // everyone has read s_rot before it is reset
	}
}

// One CTA: B (p x q, column-major, stride ldb) and V (q x q, column-major, stride ldv) in
// FP32 shared memory; round-robin one-sided Jacobi until a sweep's largest |cos| between
// paired columns is below 3e-3 (or max_sweeps); W = V written row-major. The input is
// scaled by the power of two that brings its largest entry to [0.5, 1), so squares and
// sums stay in FP32 range. Its purpose is a start for the FP64 stage (the product
// refinement, or Jacobi sweeps that started from X W converge in a few).
template <int LPP, int NR, bool FULL>
__global__ void __launch_bounds__(NR > 0 ? 512 : 1024) k_svd_f32(const double* __restrict__ X, long long ldx, int p,
                                                                 int q, float* __restrict__ W, int max_sweeps) {
	extern __shared__ float fsm[];
	const int ldb = svf32_ld(p, svf32_ldmod(p, q)), ldv = svf32_ld(q, svf32_ldmod(p, q));
	float* B = fsm;
	float* V = fsm + (size_t)ldb * q;
	__shared__ double d_red[32];
	__shared__ float f_red[32];
	__shared__ int s_rot;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
	// scale: the exponent of max |X| (non-negative doubles order like their bit patterns)
	long long mx = 0;
	for (int i = warp; i < p; i += nwarps)  // rows by warp, columns by lane: no index division
		for (int c = lane; c < q; c += 32) {
			const long long bits = __double_as_longlong(X[(long long)i * ldx + c]) & 0x7fffffffffffffffLL;
			mx = bits > mx ? bits : mx;
		}
	{
		double dm = __longlong_as_double(mx);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
		if (lane == 0) d_red[warp] = dm;
		__syncthreads();
		if (tid == 0) {
			double m2 = 0;
			for (int w = 0; w < nwarps; ++w) m2 = fmax(m2, d_red[w]);
			d_red[0] = m2;
		}
		__syncthreads();
	}
	const long long ex = (__double_as_longlong(d_red[0]) >> 52) & 0x7ff;
	const double scale = ex > 0 ? __longlong_as_double((2045 - ex) << 52) : 1.0;  // 2^(1022 - ex)
	float fl = 0.f;
	for (int i = warp; i < p; i += nwarps)
		for (int c = lane; c < q; c += 32) {
			const float v = float(X[(long long)i * ldx + c] * scale);
			B[c * ldb + i] = v;
			fl = fmaf(v, v, fl);
		}
	for (int c = warp; c < q; c += nwarps)
		for (int i = lane; i < q; i += 32) V[c * ldv + i] = c == i ? 1.f : 0.f;
	const float fro = block_sum(fl, f_red);  // its barriers also publish B and V
	const float negl = fro * 1e-12f;
	// a start for the FP64 stage, not an SVD: FP32-level orthogonality, at most 12
	// sweeps (near FP32 rounding the sweeps would go on rotating noise)
	const float tol = 4.f * sqrtf(float(p)) * FLT_EPSILON, tol2 = tol * tol;
	// a sweep whose largest |cos| between paired columns is below 3e-3 leaves them at
	// FP32 rounding (the sweeps converge quadratically); the next would rotate noise
	const float big2 = 9e-6f;
	svd_f32_sweeps<LPP, NR, FULL>(B, ldb, V, ldv, p, q, negl, tol2, big2, max_sweeps, s_rot);
	for (int i = warp; i < q; i += nwarps)
		for (int c = lane; c < q; c += 32) W[i * q + c] = V[c * ldv + i];
}

template <int LPP, int NR, bool FULL>
static void launch_svd_f32_as(const double* X, long long ldx, int p, int q, float* W, cudaStream_t s) {
	func_attr_once(k_svd_f32<LPP, NR, FULL>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDynSmemMax));
	k_svd_f32<LPP, NR, FULL><<<1, svf32_threads(q, LPP), svf32_smem(p, q), s>>>(X, ldx, p, q, W, 12);
}

void launch_svd_f32(const double* X, long long ldx, int p, int q, float* W, cudaStream_t s) {
	XTT_REQUIRE(svd_f32_fits(p, q), "internal: FP32 Jacobi stage does not fit one CTA");
	const Svf32Shape sh = svf32_shape(p, q);
	// FULL: p = q = LPP NR, every register entry is a matrix entry (no bounds tests)
	if (sh.lpp == 8 && sh.nr == 8) launch_svd_f32_as<8, 8, true>(X, ldx, p, q, W, s);
	else if (sh.lpp == 4) launch_svd_f32_as<4, 16, false>(X, ldx, p, q, W, s);
	else if (sh.lpp == 8 && p == 128 && q == 128) launch_svd_f32_as<8, 16, true>(X, ldx, p, q, W, s);
	else if (sh.lpp == 8) launch_svd_f32_as<8, 16, false>(X, ldx, p, q, W, s);
	else launch_svd_f32_as<16, 0, false>(X, ldx, p, q, W, s);
	XTT_CUDA(cudaGetLastError());
}

}  // namespace xtt
