// Tensor-core tile engine for the FP32 GEMM stages of a persistent (cooperative)
// kernel: the same operand staging and tcgen05 TF32 MMAs as k_tc_gemm, driven by
// the 256 threads of a CTA that keeps its tensor-memory accumulator and its two
// mbarriers for the whole launch. Work items of one stage (output tiles, split
// along K when the tiles alone leave CTAs idle) are taken round-robin by the CTAs
// of the grid. A split tile is finished by whichever CTA stores its last partial
// (a per-tile arrival counter): that CTA sums the tile's partials in split order,
// so the result does not depend on which CTA came last, and no grid barrier or
// separate pass is spent on the reduction.
// The caller separates stages with a grid barrier. Split TF32 only (hi*hi +
// hi*lo + lo*hi per K step, FP32-level products).
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
constexpr int kPMaxSplit = 8;    // parts of a stage split along K
// dynamic shared memory the engine uses (after 1024-byte alignment)
constexpr int kPSmem = 2 * kPStage + int(sizeof(long long)) * (2 * (kPM + kPN) + 2 * kPMaxChunks * kTileK);

// Split of a stage along K: S parts of cpk chunks (identical on the host, which sizes
// the partials workspace, and on the device).
__host__ __device__ inline void split_k(const Gemm<float>& g, int grid, int& S, int& cpk) {
	const long long tiles = (long long)g.batch * ((g.M + kPM - 1) / kPM) * ((g.N + kPN - 1) / kPN);
	const int nk = (g.K + kTileK - 1) / kTileK;
	S = 1;
	if (tiles < grid && nk > 1) {
		const long long want = (grid + tiles - 1) / tiles;
		S = int(want < kPMaxSplit ? want : kPMaxSplit);
		if (S > nk) S = nk;
	}
	cpk = (nk + S - 1) / S;
	S = cpk > 0 ? (nk + cpk - 1) / cpk : 1;
}
__host__ __device__ inline long long split_k_partials(const Gemm<float>& g, int grid) {
	int S, cpk;
	split_k(g, grid, S, cpk);
	const long long tiles = (long long)g.batch * ((g.M + kPM - 1) / kPM) * ((g.N + kPN - 1) / kPN);
	return S > 1 ? (long long)S * tiles * kPM * kPN : 0;
}

// Tiles of a stage that is split along K (the arrival counters it needs), 0 if unsplit.
__host__ __device__ inline int split_k_tiles(const Gemm<float>& g, int grid) {
	int S, cpk;
	split_k(g, grid, S, cpk);
	return S > 1 ? g.batch * ((g.M + kPM - 1) / kPM) * ((g.N + kPN - 1) / kPN) : 0;
}

// The engine's 32-bit index arithmetic: fewer than 2^31 outputs per stage.
__host__ __device__ inline bool stage_fits(const Gemm<float>& g) {
	return (long long)g.batch * g.M * g.N < (1ll << 31);
}

struct TcEngine {
	unsigned char* smem;  // kPSmem bytes, 1024-aligned
	uint64_t* bar;        // two initialised mbarriers
	int* s_ok;            // shared flag: 0 once a wait gave up
	int* s_last;          // shared: the last chunk index committed (-1: none)
	float* red;           // 32 floats of shared scratch
	uint32_t tmem;        // kPN tensor-memory columns
	uint32_t gc;          // chunks committed by this CTA so far
	int* status;
	float* part;          // split-K partials (split_k_partials floats for the largest stage)
	int* arrivals;        // per-tile arrival counters of split stages (zero between uses)
	int* s_fix;           // shared flag: this CTA finishes the current split tile

	// Element j of this thread's share of a staged operand tile (R rows x 32 K):
	// each warp instruction covers 4 rows x 8 consecutive K when K is the contiguous
	// index (32-byte sectors, 2-way bank conflicts in the core-matrix layout), else
	// 8 consecutive rows x 4 K (conflict-free); e = tid + j * kPThreads.
	template <int R>
	__device__ static void stage_rk(int e, bool kfast, int& r, int& k) {
		if (kfast) {
			r = ((e >> 7) << 2) | ((e >> 3) & 3);
			k = (((e >> 5) & 3) << 3) | (e & 7);
		} else {
			r = (((e >> 5) & (R / 8 - 1)) << 3) | (e & 7);
			k = ((e / (4 * R)) << 2) | ((e >> 3) & 3);
		}
	}

	// One stage over the grid; returns the sum over this CTA's outputs of C .* D
	// (when g.D is set), else 0. Ends with every C element written by its CTA (the
	// caller's grid barrier publishes them). Index arithmetic is 32-bit: the host
	// admits stages of fewer than 2^31 outputs (tc::stage_fits).
	template <class Grp>
	__device__ float tiles(const Gemm<float>& g, Grp& grp) {
		const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
		constexpr int AE = kPM * kTileK / kPThreads, BE = kPN * kTileK / kPThreads;
		constexpr int kTS = kPN + 4;  // row stride of the epilogue's transposed tile (conflict-free)
		constexpr uint32_t idesc = idesc_tf32(kPM, kPN);
		long long* moffA = reinterpret_cast<long long*>(smem + 2 * kPStage);
		long long* noffB = moffA + kPM;
		long long* moffC = noffB + kPN;
		long long* noffC = moffC + kPM;
		long long* koffA = noffC + kPN;
		long long* koffB = koffA + kPMaxChunks * kTileK;
		const uint32_t base = smem_u32(smem);
		const int tn = (g.N + kPN - 1) / kPN, tm = (g.M + kPM - 1) / kPM, nt = g.batch * tm * tn;
		const int nk_all = (g.K + kTileK - 1) / kTileK;
		const bool a_kfast = g.sAk == 1, b_kfast = g.sBk == 1;
		// the C tile goes out through shared memory when C's rows are contiguous (or
		// for split partials): coalesced stores instead of one row per lane
		const bool c_rows = g.sCn == 1 && g.Ni == 0;
		int S, cpk;
		split_k(g, grp.size(), S, cpk);
		float dsum = 0.f;
		for (int item = grp.rank(); item < nt * S; item += grp.size()) {
			const int tile = item % nt;
			const int ks = item / nt;
			const int kb = ks * cpk, nk = min(nk_all, kb + cpk) - kb;
			const int b = tile / (tm * tn), rem = tile - b * tm * tn;
			const int m0 = (rem / tn) * kPM, n0 = (rem % tn) * kPN;
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
				const int gk = kb * kTileK + i;
				koffA[i] = gk < g.K ? g.offA(0, gk) : -1;
				koffB[i] = gk < g.K ? g.offB(gk, 0) : -1;
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
					int m, k;
					stage_rk<kPM>(tid + j * kPThreads, a_kfast, m, k);
					const long long om = moffA[m], ok = kA[k];
					va[j] = (om >= 0 && ok >= 0) ? A[om + ok] : 0.f;
				}
#pragma unroll
				for (int j = 0; j < BE; ++j) {
					int n, k;
					stage_rk<kPN>(tid + j * kPThreads, b_kfast, n, k);
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
					int m, k;
					stage_rk<kPM>(tid + j * kPThreads, a_kfast, m, k);
					const float hi = to_tf32(va[j]);
					const uint32_t off = tile_offset(m, k);
					*reinterpret_cast<float*>(sa + off) = hi;
					*reinterpret_cast<float*>(sa + kPTileA + off) = to_tf32(va[j] - hi);
				}
#pragma unroll
				for (int j = 0; j < BE; ++j) {
					int n, k;
					stage_rk<kPN>(tid + j * kPThreads, b_kfast, n, k);
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
					*s_last = int(mygc);
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
				float* C = g.C + b * g.sCb;
				const float* D = g.D ? g.D + b * g.sCb : nullptr;
				float* P = S > 1 ? part + ((size_t)ks * nt + tile) * (kPM * kPN) : nullptr;
				if (P || c_rows) {
					// every MMA of this item has completed: the operand stages are free
					float* sT = reinterpret_cast<float*>(smem);
#pragma unroll
					for (int c = 0; c < 32; c += 16) {
						float v[16];
						tmem_ld16(tmem + (uint32_t(q * 32) << 16) + uint32_t(h * 32 + c), v);
#pragma unroll
						for (int i = 0; i < 16; i += 4)
							*reinterpret_cast<float4*>(sT + ml * kTS + h * 32 + c + i) =
							    make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
					}
					__syncthreads();
					if (P) {
						for (int idx = tid; idx < kPM * kPN; idx += kPThreads) P[idx] = sT[(idx / kPN) * kTS + idx % kPN];
						__syncthreads();  // every partial store of this CTA issued
						if (tid == 0) {
							__threadfence();
							const int last = atomicAdd(&arrivals[tile], 1) == S - 1;
							if (last) {
								arrivals[tile] = 0;  // every part has arrived: reset for the next use
								__threadfence();
							}
							*s_fix = last;
						}
						__syncthreads();
					}
					if (!P) {
						for (int idx = tid; idx < kPM * kPN; idx += kPThreads) {
							const int row = idx / kPN, col = idx % kPN;
							if (m0 + row >= g.M || n0 + col >= g.N) continue;
							const long long o = moffC[row] + noffC[col];
							const float v = sT[row * kTS + col];
							const float r = g.beta == 0.f ? g.alpha * v : fmaf(g.alpha, v, g.beta * C[o]);
							C[o] = r;
							if (D) dsum = fmaf(r, D[o], dsum);
						}
					} else if (*s_fix) {
						// the partials in split order: this CTA's own from shared memory, the others
						// through L2 (L1 is not coherent across CTAs); per part, the loads of all
						// this thread's 4-element groups are issued before their sums
						constexpr int G4 = kPM * kPN / 4 / kPThreads;
						const float4* P0 = reinterpret_cast<const float4*>(part + (size_t)tile * (kPM * kPN));
						const size_t ps4 = (size_t)nt * (kPM * kPN / 4);
						float4 acc[G4];
#pragma unroll
						for (int u = 0; u < G4; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
						for (int k = 0; k < S; ++k) {
							float4 v[G4];
#pragma unroll
							for (int u = 0; u < G4; ++u) {
								const int q4 = u * kPThreads + tid;
								v[u] = k == ks ? *reinterpret_cast<const float4*>(sT + ((4 * q4) / kPN) * kTS + (4 * q4) % kPN)
								               : __ldcg(P0 + k * ps4 + q4);
							}
#pragma unroll
							for (int u = 0; u < G4; ++u) {
								acc[u].x += v[u].x;
								acc[u].y += v[u].y;
								acc[u].z += v[u].z;
								acc[u].w += v[u].w;
							}
						}
#pragma unroll
						for (int u = 0; u < G4; ++u) {
							const int q4 = u * kPThreads + tid, row = (4 * q4) / kPN, col = (4 * q4) % kPN;
							if (m0 + row >= g.M) continue;
							const float a4[4] = {acc[u].x, acc[u].y, acc[u].z, acc[u].w};
#pragma unroll
							for (int e = 0; e < 4; ++e) {
								if (n0 + col + e >= g.N) continue;
								const long long o = moffC[row] + noffC[col + e];
								const float r = g.beta == 0.f ? g.alpha * a4[e] : fmaf(g.alpha, a4[e], g.beta * C[o]);
								C[o] = r;
								if (D) dsum = fmaf(r, D[o], dsum);
							}
						}
					}
				} else {
					const long long om = moffC[ml];
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
				}
			} else if (tid == 0) {
				record_status(status, DEV_TIMEOUT);
			}
			fence_before_sync();
			__syncthreads();  // accumulator read, tables and the transposed tile consumed before the next tile
		}
		return g.D ? block_sum(dsum, red) : 0.f;
	}
};

}  // namespace tc
}  // namespace xtt
