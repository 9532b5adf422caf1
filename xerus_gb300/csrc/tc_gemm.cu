// Tensor-core (tcgen05, TF32 with FP32 accumulation) tile GEMM for the
// contractions of the precision forms: the strided batched Gemm<T> descriptor of
// the sweep engine, C = alpha A B + beta C, operands FP64 or FP32 in global
// memory. A 128 x 64 output tile per CTA accumulates in 64 tensor-memory columns;
// 32-deep K chunks are staged (converted on the fly) into a double-buffered
// shared-memory ring while the previous chunk's MMAs run, one thread issues the
// MMAs and commits each chunk to the stage's mbarrier.
//
// terms = 3 is split TF32: each operand is a = hi + lo with hi = tf32(a) and
// lo = tf32(a - hi), and A B ~ hi_A hi_B + hi_A lo_B + lo_A hi_B (the lo lo term
// is below FP32 rounding) — FP32-level products at three MMAs per step.
// terms = 1 is plain TF32 (11-bit mantissa products).
#include "engine.cuh"
#include "tc.cuh"

namespace xtt {

namespace {

constexpr int kTcThreads = 128;  // 4 warps: warp w owns TMEM lanes (= tile rows) 32w .. 32w + 31
constexpr int kTcM = 128, kTcN = 64;
constexpr int kTileABytes = kTcM * tc::kTileK * 4;  // 16 KB
constexpr int kTileBBytes = kTcN * tc::kTileK * 4;  // 8 KB

// TF32 parts of one operand element: hi = tf32(v), lo = tf32(v - hi). FP32
// operands split in FP32 (v - hi is exact there); FP64 operands take the
// remainder in FP64 so that lo carries the bits below FP32 as well. On GB300 the
// FP64 path costs FP64-pipe instructions per element, the FP32 path none.
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo) {
	hi = tc::to_tf32(v);
	lo = tc::to_tf32(v - hi);
}
__device__ __forceinline__ void split_tf32(double v, float& hi, float& lo) {
	hi = tc::to_tf32(float(v));
	lo = tc::to_tf32(float(v - double(hi)));
}

template <int NT>
__host__ __device__ constexpr int stage_bytes() {
	return (NT == 3 ? 2 : 1) * (kTileABytes + kTileBBytes);
}

template <class T, int NT>
__global__ void __launch_bounds__(kTcThreads) k_tc_gemm(Gemm<T> g, int* status, int cpk, float* part) {
	extern __shared__ __align__(1024) unsigned char tsm[];
	__shared__ __align__(8) uint64_t bar[2];
	__shared__ uint32_t s_tmem;
	__shared__ int s_ok, s_last;  // s_last: the last chunk committed (-1: none)
	constexpr int SB = stage_bytes<NT>();
	constexpr int AE = kTcM * tc::kTileK / kTcThreads, BE = kTcN * tc::kTileK / kTcThreads;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const long long tn = (g.N + kTcN - 1) / kTcN, tm = (g.M + kTcM - 1) / kTcM;
	const long long b = blockIdx.x / (tm * tn), rem = blockIdx.x - b * tm * tn;
	const int m0 = int(rem / tn) * kTcM, n0 = int(rem % tn) * kTcN;
	const T* A = g.A + b * g.sAb;
	const T* B = g.B + b * g.sBb;
	if (warp == 0) tc::tmem_alloc(&s_tmem, kTcN);
	if (tid == 0) {
		tc::mbar_init(&bar[0], 1);
		tc::mbar_init(&bar[1], 1);
		tc::mbar_fence_init();
		s_ok = 1;
		s_last = -1;
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = s_tmem;
	const uint32_t base = tc::smem_u32(tsm);
	const bool a_kfast = g.sAk == 1, b_kfast = g.sBk == 1;
	// this CTA's K chunks (split K over blockIdx.y)
	const int nk_all = (g.K + tc::kTileK - 1) / tc::kTileK;
	const int kc0 = blockIdx.y * cpk, nk = max(0, min(nk_all, kc0 + cpk) - kc0);
	// element offsets split into a row part and a K part (offA(m, k) = offA(m, 0) + offA(0, k)),
	// tabulated once so that the staging loops do no index division; -1 marks padding
	long long* moffA = reinterpret_cast<long long*>(tsm + 2 * SB);
	long long* noffB = moffA + kTcM;
	long long* moffC = noffB + kTcN;
	long long* noffC = moffC + kTcM;
	long long* koffA = noffC + kTcN;
	long long* koffB = koffA + (size_t)cpk * tc::kTileK;
	for (int i = tid; i < kTcM; i += kTcThreads) {
		moffA[i] = m0 + i < g.M ? g.offA(m0 + i, 0) : -1;
		moffC[i] = m0 + i < g.M ? g.offC(m0 + i, 0) : -1;
	}
	for (int i = tid; i < kTcN; i += kTcThreads) {
		noffB[i] = n0 + i < g.N ? g.offB(0, n0 + i) : -1;
		noffC[i] = n0 + i < g.N ? g.offC(0, n0 + i) : -1;
	}
	for (int i = tid; i < nk * tc::kTileK; i += kTcThreads) {
		const int gk = kc0 * tc::kTileK + i;
		koffA[i] = gk < g.K ? g.offA(0, gk) : -1;
		koffB[i] = gk < g.K ? g.offB(gk, 0) : -1;
	}
	__syncthreads();
	constexpr uint32_t idesc = tc::idesc_tf32(kTcM, kTcN);
	for (int kc = 0; kc < nk; ++kc) {
		const int st = kc & 1;
		const long long* kA = koffA + kc * tc::kTileK;
		const long long* kB = koffB + kc * tc::kTileK;
		// all of this thread's operand loads in flight at once
		T va[AE], vb[BE];
#pragma unroll
		for (int j = 0; j < AE; ++j) {
			const int e = tid + j * kTcThreads;
			const int m = a_kfast ? (e >> 5) : (e & (kTcM - 1));
			const int k = a_kfast ? (e & 31) : (e >> 7);
			const long long om = moffA[m], ok = kA[k];
			va[j] = (om >= 0 && ok >= 0) ? A[om + ok] : T(0);
		}
#pragma unroll
		for (int j = 0; j < BE; ++j) {
			const int e = tid + j * kTcThreads;
			const int n = b_kfast ? (e >> 5) : (e & (kTcN - 1));
			const int k = b_kfast ? (e & 31) : (e >> 6);
			const long long on = noffB[n], ok = kB[k];
			vb[j] = (on >= 0 && ok >= 0) ? B[on + ok] : T(0);
		}
		if (kc >= 2) {
			if (tid == 0 && s_ok && !tc::mbar_wait(&bar[st], uint32_t(((kc - 2) >> 1) & 1))) s_ok = 0;
			__syncthreads();  // the MMAs that read this stage are done
		}
		unsigned char* sa = tsm + st * SB;
		unsigned char* sb = sa + (NT == 3 ? 2 : 1) * kTileABytes;
#pragma unroll
		for (int j = 0; j < AE; ++j) {
			const int e = tid + j * kTcThreads;
			const int m = a_kfast ? (e >> 5) : (e & (kTcM - 1));
			const int k = a_kfast ? (e & 31) : (e >> 7);
			float hi, lo;
			split_tf32(va[j], hi, lo);
			const uint32_t off = tc::tile_offset(m, k);
			*reinterpret_cast<float*>(sa + off) = hi;
			if (NT == 3) *reinterpret_cast<float*>(sa + kTileABytes + off) = lo;
		}
#pragma unroll
		for (int j = 0; j < BE; ++j) {
			const int e = tid + j * kTcThreads;
			const int n = b_kfast ? (e >> 5) : (e & (kTcN - 1));
			const int k = b_kfast ? (e & 31) : (e >> 6);
			float hi, lo;
			split_tf32(vb[j], hi, lo);
			const uint32_t off = tc::tile_offset(n, k);
			*reinterpret_cast<float*>(sb + off) = hi;
			if (NT == 3) *reinterpret_cast<float*>(sb + kTileBBytes + off) = lo;
		}
		tc::fence_async_smem();
		__syncthreads();
		if (tid == 0 && s_ok) {
			tc::fence_after_sync();
			const uint32_t a_hi = base + st * SB, b_hi = a_hi + (NT == 3 ? 2 : 1) * kTileABytes;
#pragma unroll
			for (int s = 0; s < tc::kTileK / 8; ++s) {
				const uint32_t ko = uint32_t(s) * 2 * tc::kCoreBytes;
				const bool first = (kc == 0 && s == 0);
				tc::mma_tf32(tmem, tc::smem_desc(a_hi + ko), tc::smem_desc(b_hi + ko), idesc, !first);
				if (NT == 3) {
					tc::mma_tf32(tmem, tc::smem_desc(a_hi + ko), tc::smem_desc(b_hi + kTileBBytes + ko), idesc, true);
					tc::mma_tf32(tmem, tc::smem_desc(a_hi + kTileABytes + ko), tc::smem_desc(b_hi + ko), idesc, true);
				}
			}
			tc::mma_commit(&bar[st]);
			s_last = kc;
		}
	}
	if (tid == 0 && s_ok && nk > 0 && !tc::mbar_wait(&bar[(nk - 1) & 1], uint32_t(((nk - 1) >> 1) & 1))) s_ok = 0;
	__syncthreads();
	tc::fence_after_sync();
	const bool ok = s_ok != 0;
	if (ok) {
		const int m = m0 + warp * 32 + lane;
		const long long om = moffC[warp * 32 + lane];
		const T* C0 = g.C + b * g.sCb;
		T* C = g.C + b * g.sCb;
		// split K: raw partial sums, dense (batch, M, N) per split, summed by k_tc_reduce
		float* P = part ? part + ((size_t)blockIdx.y * g.batch + b) * (size_t)g.M * g.N : nullptr;
#pragma unroll
		for (int c = 0; c < kTcN; c += 16) {
			float v[16];
			if (nk > 0) {
				tc::tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
			} else {
#pragma unroll
				for (int i = 0; i < 16; ++i) v[i] = 0.f;
			}
			if (m < g.M) {
#pragma unroll
				for (int i = 0; i < 16; ++i) {
					const int n = n0 + c + i;
					if (n < g.N) {
						if (P) {
							P[(size_t)m * g.N + n] = v[i];
						} else {
							const long long o = om + noffC[c + i];
							const T r = g.alpha * T(v[i]);
							C[o] = g.beta == T(0) ? r : r + g.beta * C0[o];
						}
					}
				}
			}
		}
	} else if (tid == 0) {
		record_status(status, DEV_TIMEOUT);
		// a wait gave up: wait (bounded) once more for the MMAs in flight before freeing TMEM
		if (s_last >= 0) tc::mbar_wait(&bar[s_last & 1], uint32_t((s_last >> 1) & 1));
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::fence_after_sync();
		tc::tmem_dealloc(tmem, kTcN);
	}
}

// C = alpha sum_s part[s] + beta C over the S split-K partials, added in split order.
template <class T>
__global__ void k_tc_reduce(Gemm<T> g, int S, const float* part) {
	const long long mn = (long long)g.M * g.N, total = (long long)g.batch * mn;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
	     e += (long long)gridDim.x * blockDim.x) {
		const long long b = e / mn, r = e - b * mn;
		const int m = int(r / g.N), n = int(r - (long long)m * g.N);
		float s = 0.f;
		for (int k = 0; k < S; ++k) s += part[(size_t)k * total + e];
		T* C = g.C + b * g.sCb;
		const long long o = g.offC(m, n);
		const T v = g.alpha * T(s);
		C[o] = g.beta == T(0) ? v : v + g.beta * C[o];
	}
}

template <class T, int NT>
void launch_tc(Context& c, const Gemm<T>& g) {
	constexpr int kMaxChunks = 64;  // K offsets tabulated per CTA: at most 64 chunks (2048 K)
	func_attr_once(k_tc_gemm<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                              2 * stage_bytes<NT>() + int(sizeof(long long)) * (2 * (kTcM + kTcN) + 2 * kMaxChunks * tc::kTileK));
	const long long tiles = (long long)g.batch * ((g.M + kTcM - 1) / kTcM) * ((g.N + kTcN - 1) / kTcN);
	XTT_REQUIRE(tiles < (1ll << 31), "GEMM too large");
	// split K when the tiles alone leave most SMs idle (deterministic: partials reduced in order)
	const int nk = (g.K + tc::kTileK - 1) / tc::kTileK;
	int S = 1;
	const long long partial_elems = (long long)g.batch * g.M * g.N;
	if (tiles < c.num_sms && nk >= 4 && partial_elems <= (1ll << 24))
		S = int(std::min<long long>(std::min<long long>(8, nk / 2), (c.num_sms + tiles - 1) / tiles));
	S = std::max(S, (nk + kMaxChunks - 1) / kMaxChunks);
	const int cpk = (nk + S - 1) / S;
	S = std::max(1, (nk + cpk - 1) / cpk);
	XTT_REQUIRE(S == 1 || S * partial_elems <= (1ll << 27), "tensor-core GEMM: K too long for its split-K workspace");
	const int smem = 2 * stage_bytes<NT>() + int(sizeof(long long)) * (2 * (kTcM + kTcN) + 2 * cpk * tc::kTileK);
	float* part = S > 1 ? c.scratch<float>(S_GEMM_TC_WORK, size_t(S) * partial_elems) : nullptr;
	k_tc_gemm<T, NT><<<dim3(unsigned(tiles), unsigned(S)), kTcThreads, smem, c.stream>>>(g, c.d_status, cpk, part);
	XTT_CUDA(cudaGetLastError());
	if (S > 1) {
		const unsigned blocks = unsigned(std::min<long long>(4ll * c.num_sms, (partial_elems + 255) / 256));
		k_tc_reduce<T><<<blocks, 256, 0, c.stream>>>(g, S, part);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	}
}

}  // namespace

template <class T>
void gemm_tc(Context& c, const Gemm<T>& g, int terms) {
	if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return;
	check_gemm(g);
	XTT_REQUIRE(!g.D, "internal: the tensor-core GEMM has no C.*D epilogue");
	XTT_REQUIRE(terms == 1 || terms == 3 || terms == 6, "internal: tensor-core GEMM terms must be 1, 3 or 6");
	const double mn = double(g.batch) * g.M * g.N, mk = double(g.M) * g.K, kn = double(g.K) * g.N;
	ProfScope ps(c, "gemm_tc", double(sizeof(T)) * (double(g.batch) * (mk + kn) + mn), 2.0 * mn * g.K * terms);
	// TMA-fed tiles (the operands split once into K-major pieces); the per-thread staged
	// kernel where the driver cannot describe them as tensor maps
	if (gemm_tc_tma(c, g, terms)) {
		c.count_launch();
		return;
	}
	XTT_REQUIRE(terms != 6, "the BF16 split form needs the TMA path");
	if (terms == 3) launch_tc<T, 3>(c, g);
	else launch_tc<T, 1>(c, g);
	c.count_launch();
}
template void gemm_tc<double>(Context&, const Gemm<double>&, int);
template void gemm_tc<float>(Context&, const Gemm<float>&, int);

}  // namespace xtt
