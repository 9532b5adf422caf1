// Householder QR of a small matrix by one CTA (any block size up to 512
// threads), used by the batched sweep and for small unpivoted factorisations.
#pragma once

#include "common.cuh"

namespace xtt {

constexpr int kBlkQrMaxCols = 64;

// Householder scalars of dlarfg from alpha and ||x||^2 below the diagonal:
// beta = -sign(alpha) sqrt(alpha^2 + xn2), tau = (beta - alpha) / beta,
// scal = 1 / (alpha - beta). With q = alpha - beta, tau = -q^2 / (beta q) and
// scal = beta / (beta q): one division instead of two (a dependent FP64 division
// costs ~400 cycles on GB300). Agrees with the two-division form to a few ulp.
__device__ __forceinline__ void reflector_scalars(double alpha, double xn2, double& beta, double& tau, double& scal) {
	beta = alpha;
	tau = 0.0;
	scal = 1.0;
	if (xn2 != 0.0) {
		beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
		const double q = alpha - beta;
		const double inv = 1.0 / (beta * q);
		tau = -(q * q) * inv;
		scal = beta * inv;
	}
}

struct BlkQrSmem {
	double red[32];
	double coef[4];
	double tau[kBlkQrMaxCols];
	double sw[kBlkQrMaxCols];
	double part[16 * kBlkQrMaxCols];
};

// Householder QR (unpivoted, LAPACK dgeqrf/dorg2r conventions) of the m x n
// matrix A (transpose: of A^T) by one CTA, in the workspace W (mw x nw).
// Writes C (kq x nw; transposed: nw x kq) and, if want_q, Q (mw x kq;
// transposed: kq x mw). nw <= kBlkQrMaxCols.
__device__ inline void blk_qr(const double* A, long long lda, int m, int n, int transpose, double* W, double* C, double* Q,
                       bool want_q, BlkQrSmem& sh) {
	const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
	const int mw = transpose ? n : m, nw = transpose ? m : n, kq = min(mw, nw);
	auto w = [&](int i, int j) -> double& { return W[(long long)i * nw + j]; };
	for (long long e = tid; e < (long long)mw * nw; e += nt) {
		const int i = int(e / nw), j = int(e % nw);
		W[e] = transpose ? A[(long long)j * lda + i] : A[(long long)i * lda + j];
	}
	__syncthreads();
	for (int j = 0; j < kq; ++j) {
		double part = 0;
		for (int i = j + 1 + tid; i < mw; i += nt) part = fma(w(i, j), w(i, j), part);
		const double xn2 = block_sum(part, sh.red);
		if (tid == 0) {
			const double alpha = w(j, j);
			double t, scal, beta;
			reflector_scalars(alpha, xn2, beta, t, scal);
			sh.tau[j] = t;
			sh.coef[0] = scal;
			sh.coef[1] = beta;
		}
		__syncthreads();
		const double scal = sh.coef[0], tj = sh.tau[j];
		for (int i = j + 1 + tid; i < mw; i += nt) w(i, j) *= scal;
		if (tid == 0) w(j, j) = sh.coef[1];
		__syncthreads();
		const int c0 = j + 1, Cn = nw - c0;
		if (Cn > 0) {
			const int ncw = (Cn + 31) >> 5, G = max(1, nwarps / ncw);
			const int g = warp / ncw, ci = (warp % ncw) * 32 + lane, rows = mw - j, chunk = (rows + G - 1) / G;
			const int ia = j + g * chunk, ib = min(mw, ia + chunk);
			if (g < G && ci < Cn) {
				const int c = c0 + ci;
				double acc = 0;
				for (int i = ia; i < ib; ++i) acc = fma(i == j ? 1.0 : w(i, j), w(i, c), acc);
				sh.part[g * kBlkQrMaxCols + ci] = acc;
			}
			__syncthreads();
			if (tid < Cn) {
				double s = 0;
				for (int gg = 0; gg < G; ++gg) s += sh.part[gg * kBlkQrMaxCols + tid];
				sh.sw[c0 + tid] = tj * s;
			}
			__syncthreads();
			if (g < G && ci < Cn) {
				const int c = c0 + ci;
				const double wc = sh.sw[c];
				for (int i = ia; i < ib; ++i) w(i, c) = fma(-wc, i == j ? 1.0 : w(i, j), w(i, c));
			}
			__syncthreads();
		}
	}
	for (long long e = tid; e < (long long)kq * nw; e += nt) {
		const int r = int(e / nw), c = int(e % nw);
		const double v = (r <= c) ? w(r, c) : 0.0;
		if (!transpose) C[(long long)r * nw + c] = v;
		else C[(long long)c * kq + r] = v;
	}
	__syncthreads();
	if (!want_q) return;
	for (int j = kq - 1; j >= 0; --j) {
		const double tj = sh.tau[j];
		const int c0 = j + 1, Cn = kq - c0;
		if (Cn > 0) {
			const int ncw = (Cn + 31) >> 5, G = max(1, nwarps / ncw);
			const int g = warp / ncw, ci = (warp % ncw) * 32 + lane, rows = mw - j - 1, chunk = (rows + G - 1) / G;
			const int ia = j + 1 + g * chunk, ib = min(mw, ia + chunk);
			if (g < G && ci < Cn) {
				const int c = c0 + ci;
				double acc = 0;
				for (int i = ia; i < ib; ++i) acc = fma(w(i, j), w(i, c), acc);
				sh.part[g * kBlkQrMaxCols + ci] = acc;
			}
			__syncthreads();
			if (tid < Cn) {
				double s = 0;
				for (int gg = 0; gg < G; ++gg) s += sh.part[gg * kBlkQrMaxCols + tid];
				sh.sw[c0 + tid] = tj * s;
			}
			__syncthreads();
			if (g < G && ci < Cn) {
				const int c = c0 + ci;
				const double wc = sh.sw[c];
				for (int i = ia; i < ib; ++i) w(i, c) = fma(-wc, w(i, j), w(i, c));
				if (g == 0) w(j, c) = -wc;
			}
			__syncthreads();
		}
		for (int i = tid; i < mw; i += nt) w(i, j) = i > j ? -tj * w(i, j) : (i == j ? 1.0 - tj : 0.0);
		__syncthreads();
	}
	for (long long e = tid; e < (long long)mw * kq; e += nt) {
		const int i = int(e / kq), c = int(e % kq);
		const double v = w(i, c);
		if (!transpose) Q[(long long)i * kq + c] = v;
		else Q[(long long)c * mw + i] = v;
	}
	__syncthreads();
}

}  // namespace xtt
