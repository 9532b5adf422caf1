// Tensor-core tile engine for the FP32 GEMM stages of a persistent (cooperative)
// kernel: the same operand staging and tcgen05 TF32 MMAs as k_tc_gemm, driven by
// the 256 threads of a CTA that keeps its tensor-memory accumulator and its two
// mbarriers for the whole launch. Tiles of one stage are taken round-robin by the
// CTAs of the grid (no split K); the caller separates stages with a grid barrier.
// Split TF32 only (hi*hi + hi*lo + lo*hi per K step, FP32-level products).
#pragma once

#include "gemm.cuh"
#include "tc.cuh"

namespace xtt {
namespace tc {

constexpr int kPM = 128, kPN = 64;
constexpr int kPThreads = 256;
constexpr int kPTileA = kPM * kTileK * 4, kPTileB = kPN * kTileK * 4;
constexpr int kPStage = 2 * (kPTileA + kPTileB);
constexpr int kPMaxChunks = 16;  // K <= 512 per stage
// dynamic shared memory the engine uses (after 1024-byte alignment)
constexpr int kPSmem = 2 * kPStage + int(sizeof(long long)) * (2 * (kPM + kPN) + 2 * kPMaxChunks * kTileK);

struct TcEngine {
	unsigned char* smem;  // kPSmem bytes, 1024-aligned
	uint64_t* bar;        // two initialised mbarriers
	int* s_ok;            // shared flag: 0 once a wait gave up
	float* red;           // 32 floats of shared scratch
	uint32_t tmem;        // kPN tensor-memory columns
	uint32_t gc;          // chunks committed by this CTA so far
	int* status;

	// Tiles start, start + stride, ... of g; returns, in thread 0, sum over them of C .* D
	// (when g.D is set), else 0.
	__device__ float tiles(const Gemm<float>& g, long long start, long long stride) {
		const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
		constexpr int AE = kPM * kTileK / kPThreads, BE = kPN * kTileK / kPThreads;
		constexpr uint32_t idesc = idesc_tf32(kPM, kPN);
		long long* moffA = reinterpret_cast<long long*>(smem + 2 * kPStage);
		long long* noffB = moffA + kPM;
		long long* moffC = noffB + kPN;
		long long* noffC = moffC + kPM;
		long long* koffA = noffC + kPN;
		long long* koffB = koffA + kPMaxChunks * kTileK;
		const uint32_t base = smem_u32(smem);
		const long long tn = (g.N + kPN - 1) / kPN, tm = (g.M + kPM - 1) / kPM, nt = (long long)g.batch * tm * tn;
		const int nk = (g.K + kTileK - 1) / kTileK;
		const bool a_kfast = g.sAk == 1, b_kfast = g.sBk == 1;
		float dsum = 0.f;
		for (long long tile = start; tile < nt; tile += stride) {
			const long long b = tile / (tm * tn), rem = tile - b * tm * tn;
			const int m0 = int(rem / tn) * kPM, n0 = int(rem % tn) * kPN;
			const float* A = g.A + b * g.sAb;
			const float* B = g.B + b * g.sBb;
			// offsets: row and K parts tabulated (offA(m, k) = offA(m, 0) + offA(0, k))
			for (int i = tid; i < kPM; i += kPThreads) {
				moffA[i] = m0 + i < g.M ? g.offA(m0 + i, 0) : -1;
				moffC[i] = m0 + i < g.M ? g.offC(m0 + i, 0) : -1;
			}
			for (int i = tid; i < kPN; i += kPThreads) {
				noffB[i] = n0 + i < g.N ? g.offB(0, n0 + i) : -1;
				noffC[i] = n0 + i < g.N ? g.offC(0, n0 + i) : -1;
			}
			for (int i = tid; i < nk * kTileK; i += kPThreads) {
				koffA[i] = i < g.K ? g.offA(0, i) : -1;
				koffB[i] = i < g.K ? g.offB(i, 0) : -1;
			}
			__syncthreads();
			for (int kc = 0; kc < nk; ++kc) {
				const uint32_t mygc = gc + uint32_t(kc);
				const int st = int(mygc & 1u);
				const long long* kA = koffA + kc * kTileK;
				const long long* kB = koffB + kc * kTileK;
				float va[AE], vb[BE];
#pragma unroll
				for (int j = 0; j < AE; ++j) {
					const int e = tid + j * kPThreads;
					const int m = a_kfast ? (e >> 5) : (e & (kPM - 1));
					const int k = a_kfast ? (e & 31) : (e >> 7);
					const long long om = moffA[m], ok = kA[k];
					va[j] = (om >= 0 && ok >= 0) ? A[om + ok] : 0.f;
				}
#pragma unroll
				for (int j = 0; j < BE; ++j) {
					const int e = tid + j * kPThreads;
					const int n = b_kfast ? (e >> 5) : (e & (kPN - 1));
					const int k = b_kfast ? (e & 31) : (e >> 6);
					const long long on = noffB[n], ok = kB[k];
					vb[j] = (on >= 0 && ok >= 0) ? B[on + ok] : 0.f;
				}
				if (mygc >= 2u) {
					// the MMAs that read this stage (committed two chunks ago) are done
					if (tid == 0 && *s_ok && !mbar_wait(&bar[st], ((mygc - 2u) >> 1) & 1u)) *s_ok = 0;
					__syncthreads();
				}
				unsigned char* sa = smem + st * kPStage;
				unsigned char* sb = sa + 2 * kPTileA;
#pragma unroll
				for (int j = 0; j < AE; ++j) {
					const int e = tid + j * kPThreads;
					const int m = a_kfast ? (e >> 5) : (e & (kPM - 1));
					const int k = a_kfast ? (e & 31) : (e >> 7);
					const float hi = to_tf32(va[j]);
					const uint32_t off = tile_offset(m, k);
					*reinterpret_cast<float*>(sa + off) = hi;
					*reinterpret_cast<float*>(sa + kPTileA + off) = to_tf32(va[j] - hi);
				}
#pragma unroll
				for (int j = 0; j < BE; ++j) {
					const int e = tid + j * kPThreads;
					const int n = b_kfast ? (e >> 5) : (e & (kPN - 1));
					const int k = b_kfast ? (e & 31) : (e >> 6);
					const float hi = to_tf32(vb[j]);
					const uint32_t off = tile_offset(n, k);
					*reinterpret_cast<float*>(sb + off) = hi;
					*reinterpret_cast<float*>(sb + kPTileB + off) = to_tf32(vb[j] - hi);
				}
				fence_async_smem();
				fence_before_sync();
				__syncthreads();
				if (tid == 0 && *s_ok) {
					fence_after_sync();
					const uint32_t a_hi = base + st * kPStage, b_hi = a_hi + 2 * kPTileA;
#pragma unroll
					for (int s = 0; s < kTileK / 8; ++s) {
						const uint32_t ko = uint32_t(s) * 2 * kCoreBytes;
						mma_tf32(tmem, smem_desc(a_hi + ko), smem_desc(b_hi + ko), idesc, !(kc == 0 && s == 0));
						mma_tf32(tmem, smem_desc(a_hi + ko), smem_desc(b_hi + kPTileB + ko), idesc, true);
						mma_tf32(tmem, smem_desc(a_hi + kPTileA + ko), smem_desc(b_hi + ko), idesc, true);
					}
					mma_commit(&bar[st]);
				}
			}
			gc += uint32_t(nk);
			if (tid == 0 && *s_ok && nk > 0 && !mbar_wait(&bar[(gc - 1u) & 1u], ((gc - 1u) >> 1) & 1u)) *s_ok = 0;
			__syncthreads();
			fence_after_sync();
			if (*s_ok) {
				// warp w: TMEM lanes (tile rows) 32 (w % 4) .., columns 32 (w / 4) ..
				const int q = warp & 3, h = warp >> 2;
				const int ml = q * 32 + lane, m = m0 + ml;
				const long long om = moffC[ml];
				float* C = g.C + b * g.sCb;
				const float* D = g.D ? g.D + b * g.sCb : nullptr;
#pragma unroll
				for (int c = 0; c < 32; c += 16) {
					float v[16];
					tmem_ld16(tmem + (uint32_t(q * 32) << 16) + uint32_t(h * 32 + c), v);
					if (m < g.M) {
#pragma unroll
						for (int i = 0; i < 16; ++i) {
							const int nl = h * 32 + c + i;
							if (n0 + nl < g.N) {
								const long long o = om + noffC[nl];
								const float r = g.beta == 0.f ? g.alpha * v[i] : fmaf(g.alpha, v[i], g.beta * C[o]);
								C[o] = r;
								if (D) dsum = fmaf(r, D[o], dsum);
							}
						}
					}
				}
			} else if (tid == 0) {
				record_status(status, DEV_TIMEOUT);
			}
			fence_before_sync();
			__syncthreads();  // accumulator read and tables consumed before the next tile
		}
		return g.D ? block_sum(dsum, red) : 0.f;
	}
};

}  // namespace tc
}  // namespace xtt
