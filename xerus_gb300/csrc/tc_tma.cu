// TMA-fed tensor-core GEMM for the precision forms: C = alpha A B + beta C on the
// strided batched Gemm<T> descriptor of the sweep engine, FP64 or FP32 operands.
//
// 1. The operands are split once per call into K-major FP32 (TF32) or BF16 pieces in
//    global memory (k_split_kmajor: a = p0 + p1 [+ p2], each piece exactly
//    representable), padded to 128-byte rows, so every K chunk of a tile is one TMA box.
// 2. k_tma_gemm: one 128 x 64 output tile per CTA, accumulated in 64 tensor-memory
//    columns. Warp 0 (one thread) streams the pieces' boxes with cp.async.bulk.tensor
//    into a ring of shared-memory stages (128-byte swizzle) under mbarrier expect-tx;
//    warp 1 (one thread) issues the tcgen05 MMAs of every piece product and commits
//    each stage back to the producer; all four warps then read the accumulator
//    (tcgen05.ld) and write C. Split K over blockIdx.y when the tiles leave SMs idle,
//    partial sums reduced in split order (deterministic).
//
// Kinds: TF32 (1 product, 11-bit products), TF32x3 (hi hi + hi lo + lo hi: FP32-level
// products), BF16x6 (three BF16 pieces, the six products of weight >= 2^-16: FP32-level
// products on the 16-bit MMA path).
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "engine.cuh"
#include "tc.cuh"

namespace xtt {

namespace {

enum TmaKind : int { KIND_TF32 = 1, KIND_TF32X3 = 3, KIND_BF16X6 = 6 };

constexpr int kTmThreads = 128;
constexpr int kTmM = 128, kTmN = 64;
constexpr int kRowBytes = 128;  // one swizzle row of K: 32 TF32 or 64 BF16 elements

template <int KIND>
struct KindTraits;
template <>
struct KindTraits<KIND_TF32> {
	static constexpr int pieces = 1, esize = 4, kchunk = 32, stages = 4;
};
template <>
struct KindTraits<KIND_TF32X3> {
	static constexpr int pieces = 2, esize = 4, kchunk = 32, stages = 4;
};
template <>
struct KindTraits<KIND_BF16X6> {
	static constexpr int pieces = 3, esize = 2, kchunk = 64, stages = 3;
};

template <int KIND>
__host__ __device__ constexpr int a_piece_bytes() { return kTmM * kRowBytes; }
template <int KIND>
__host__ __device__ constexpr int b_piece_bytes() { return kTmN * kRowBytes; }
template <int KIND>
__host__ __device__ constexpr int stage_bytes() {
	return KindTraits<KIND>::pieces * (a_piece_bytes<KIND>() + b_piece_bytes<KIND>());
}
template <int KIND>
__host__ __device__ constexpr int smem_bytes() {
	return KindTraits<KIND>::stages * stage_bytes<KIND>() + 1024;  // + alignment slack
}

// ---------------------------------------------------------------- operand split
// Piece p of element (row, k) of operand `which` (0: A rows = M, 1: B rows = N) of batch b
// at out + ((p * batch + b) * rows + row) * kpad + k; zero beyond K. TF32 pieces are
// FP32 values with their low 13 mantissa bits zero (hi = tf32(v), lo = tf32(v - hi));
// BF16 pieces are bf16(v), bf16(v - p0), bf16(v - p0 - p1) (FP32 arithmetic for FP32
// operands, FP64 for FP64 ones so that the remainders keep every bit).
template <class T, int KIND>
__global__ void k_split_kmajor(Gemm<T> g, int which, void* out, int rows, int kpad) {
	const long long per = (long long)rows * kpad, total = (long long)g.batch * per;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
	     e += (long long)gridDim.x * blockDim.x) {
		const long long b = e / per, r = e - b * per;
		const int row = int(r / kpad), k = int(r - (long long)row * kpad);
		T v = T(0);
		if (k < g.K) v = which == 0 ? g.A[b * g.sAb + g.offA(row, k)] : g.B[b * g.sBb + g.offB(k, row)];
		const long long pstride = (long long)g.batch * per;
		if constexpr (KIND == KIND_BF16X6) {
			__nv_bfloat16* o = static_cast<__nv_bfloat16*>(out);
			const __nv_bfloat16 p0 = __float2bfloat16_rn(float(v));
			const T r1 = v - T(__bfloat162float(p0));
			const __nv_bfloat16 p1 = __float2bfloat16_rn(float(r1));
			const T r2 = r1 - T(__bfloat162float(p1));
			o[e] = p0;
			o[pstride + e] = p1;
			o[2 * pstride + e] = __float2bfloat16_rn(float(r2));
		} else {
			float* o = static_cast<float*>(out);
			const float hi = tc::to_tf32(float(v));
			o[e] = hi;
			if (KIND == KIND_TF32X3) o[pstride + e] = tc::to_tf32(float(v - T(hi)));
		}
	}
}

// ---------------------------------------------------------------- the GEMM
struct TmaMaps {
	CUtensorMap a[3], b[3];  // one map per piece
};

template <class T, int KIND>
__global__ void __launch_bounds__(kTmThreads, 1)
    k_tma_gemm(const __grid_constant__ TmaMaps maps, Gemm<T> g, int cpk, float* part, int* status) {
	using KT = KindTraits<KIND>;
	constexpr int ST = KT::stages, NP = KT::pieces;
	constexpr int AB = a_piece_bytes<KIND>(), BB = b_piece_bytes<KIND>(), SB = stage_bytes<KIND>();
	extern __shared__ unsigned char tm_raw[];
	__shared__ __align__(8) uint64_t full[ST], empty[ST], done;
	__shared__ uint32_t s_tmem;
	__shared__ int s_ok, s_issued;
	unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tm_raw) + 1023) & ~uintptr_t(1023));
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const long long tn = (g.N + kTmN - 1) / kTmN, tm = (g.M + kTmM - 1) / kTmM;
	const long long bb = blockIdx.x / (tm * tn), rem = blockIdx.x - bb * tm * tn;
	const int m0 = int(rem / tn) * kTmM, n0 = int(rem % tn) * kTmN;
	const int nk_all = (g.K + KT::kchunk - 1) / KT::kchunk;
	const int kc0 = blockIdx.y * cpk, nk = max(0, min(nk_all, kc0 + cpk) - kc0);
	if (warp == 0) tc::tmem_alloc(&s_tmem, kTmN);
	if (tid == 32) {
		for (int s = 0; s < ST; ++s) {
			tc::mbar_init(&full[s], 1);
			tc::mbar_init(&empty[s], 1);
		}
		tc::mbar_init(&done, 1);
		tc::mbar_fence_init();
		s_ok = 1;
		s_issued = 0;
	}
	if (tid == 0)
		for (int p = 0; p < NP; ++p) {
			tc::tma_prefetch_desc(&maps.a[p]);
			tc::tma_prefetch_desc(&maps.b[p]);
		}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = s_tmem;
	const uint32_t base = tc::smem_u32(sm);
	if (warp == 0 && lane == 0) {
		// producer: every piece's A and B boxes of chunk kc into stage kc % ST
		for (int kc = 0; kc < nk; ++kc) {
			const int s = kc % ST;
			const uint32_t round = uint32_t(kc / ST);
			if (!tc::mbar_wait(&empty[s], (round & 1u) ^ 1u)) {
				atomicExch(&s_ok, 0);
				break;
			}
			if (!s_ok) break;
			tc::mbar_arrive_expect_tx(&full[s], uint32_t(SB));
			unsigned char* st = sm + s * SB;
			const int kx = (kc0 + kc) * KT::kchunk;  // innermost coordinate: a multiple of 128 bytes
			for (int p = 0; p < NP; ++p) {
				tc::tma_load_3d(st + p * AB, &maps.a[p], &full[s], kx, m0, int(bb));
				tc::tma_load_3d(st + NP * AB + p * BB, &maps.b[p], &full[s], kx, n0, int(bb));
			}
		}
	} else if (warp == 1 && lane == 0) {
		// MMA issuer
		constexpr uint32_t idesc = KIND == KIND_BF16X6 ? tc::idesc_bf16(kTmM, kTmN) : tc::idesc_tf32(kTmM, kTmN);
		int issued = 0;
		for (int kc = 0; kc < nk; ++kc) {
			const int s = kc % ST;
			if (!tc::mbar_wait(&full[s], uint32_t(kc / ST) & 1u)) {
				atomicExch(&s_ok, 0);
				break;
			}
			if (!s_ok) break;
			tc::fence_after_sync();
			const uint32_t a0 = base + uint32_t(s * SB), b0 = a0 + uint32_t(NP * AB);
#pragma unroll
			for (int kk = 0; kk < 4; ++kk) {
				const uint32_t ko = uint32_t(kk * 32);
				const bool first = kc == 0 && kk == 0;
				if constexpr (KIND == KIND_BF16X6) {
					// products p_i q_j with i + j <= 2
#pragma unroll
					for (int i = 0; i < 3; ++i)
#pragma unroll
						for (int j = 0; j < 3 - i; ++j)
							tc::mma_bf16(tmem, tc::smem_desc_sw128(a0 + uint32_t(i * AB) + ko),
							             tc::smem_desc_sw128(b0 + uint32_t(j * BB) + ko), idesc, !(first && i == 0 && j == 0));
				} else {
					tc::mma_tf32(tmem, tc::smem_desc_sw128(a0 + ko), tc::smem_desc_sw128(b0 + ko), idesc, !first);
					if constexpr (KIND == KIND_TF32X3) {
						tc::mma_tf32(tmem, tc::smem_desc_sw128(a0 + ko), tc::smem_desc_sw128(b0 + uint32_t(BB) + ko), idesc,
						             true);
						tc::mma_tf32(tmem, tc::smem_desc_sw128(a0 + uint32_t(AB) + ko), tc::smem_desc_sw128(b0 + ko), idesc,
						             true);
					}
				}
			}
			tc::mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
			issued = kc + 1;
		}
		s_issued = issued;
		tc::mma_commit(&done);  // arrives when every MMA issued above has completed
	}
	__syncthreads();
	// every thread: the accumulator is complete (bounded wait)
	bool ok = true;
	if (nk > 0) ok = tc::mbar_wait(&done, 0u);
	if (!ok && tid == 0) atomicExch(&s_ok, 0);
	__syncthreads();
	tc::fence_after_sync();
	ok = s_ok != 0 && s_issued == nk;
	if (ok) {
		const int ml = warp * 32 + lane, m = m0 + ml;
		T* C = g.C + bb * g.sCb;
		float* P = part ? part + ((size_t)blockIdx.y * g.batch + bb) * (size_t)g.M * g.N : nullptr;
		const long long om = m < g.M ? g.offC(m, 0) : 0;
#pragma unroll
		for (int c = 0; c < kTmN; c += 16) {
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
							const long long o = om + g.offC(0, n);
							const T r = g.alpha * T(v[i]);
							C[o] = g.beta == T(0) ? r : r + g.beta * C[o];
						}
					}
				}
			}
		}
	} else if (tid == 0) {
		record_status(status, DEV_TIMEOUT);
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::fence_after_sync();
		tc::tmem_dealloc(tmem, kTmN);
	}
}

template <class T>
__global__ void k_tma_reduce(Gemm<T> g, int S, const float* part) {
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

// ---------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
	static std::once_flag once;
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	std::call_once(once, [] {
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
		cudaGetLastError();
	});
	return fn;
}

// 3-D map over pieces laid out [batch][rows][kpad] (elements), box {kchunk, box_rows, 1},
// 128-byte swizzle. False if the driver refuses it.
bool encode_piece(CUtensorMap* m, const void* ptr, bool bf16, int kpad, int rows, int batch, int box_rows) {
	auto fn = encode_tiled();
	if (!fn) return false;
	const int es = bf16 ? 2 : 4;
	const cuuint64_t dims[3] = {cuuint64_t(kpad), cuuint64_t(rows), cuuint64_t(batch)};
	const cuuint64_t strides[2] = {cuuint64_t(kpad) * es, cuuint64_t(kpad) * es * cuuint64_t(rows)};
	const cuuint32_t box[3] = {cuuint32_t(kRowBytes / es), cuuint32_t(box_rows), 1};
	const cuuint32_t estr[3] = {1, 1, 1};
	const CUresult r = fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
	                      const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
	                      CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
	                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS;
}

template <class T, int KIND>
bool launch_tma(Context& c, const Gemm<T>& g) {
	using KT = KindTraits<KIND>;
	constexpr bool bf = KIND == KIND_BF16X6;
	const int kpad = (g.K + KT::kchunk - 1) / KT::kchunk * KT::kchunk;
	const long long elems_a = (long long)g.batch * g.M * kpad, elems_b = (long long)g.batch * g.N * kpad;
	XTT_REQUIRE(elems_a < (1ll << 31) && elems_b < (1ll << 31), "tensor-core GEMM operands too large");
	const size_t es = bf ? 2 : 4;
	unsigned char* wa = c.scratch<unsigned char>(S_TMA_A, size_t(KT::pieces) * size_t(elems_a) * es);
	unsigned char* wb = c.scratch<unsigned char>(S_TMA_B, size_t(KT::pieces) * size_t(elems_b) * es);
	TmaMaps maps;
	for (int p = 0; p < KT::pieces; ++p) {
		if (!encode_piece(&maps.a[p], wa + size_t(p) * size_t(elems_a) * es, bf, kpad, g.M, g.batch, kTmM) ||
		    !encode_piece(&maps.b[p], wb + size_t(p) * size_t(elems_b) * es, bf, kpad, g.N, g.batch, kTmN))
			return false;
	}
	const unsigned sa = unsigned(std::min<long long>((elems_a + 255) / 256, 8ll * c.num_sms));
	const unsigned sbk = unsigned(std::min<long long>((elems_b + 255) / 256, 8ll * c.num_sms));
	k_split_kmajor<T, KIND><<<std::max(1u, sa), 256, 0, c.stream>>>(g, 0, wa, g.M, kpad);
	k_split_kmajor<T, KIND><<<std::max(1u, sbk), 256, 0, c.stream>>>(g, 1, wb, g.N, kpad);
	XTT_CUDA(cudaGetLastError());
	c.count_launch(2);
	const long long tiles = (long long)g.batch * ((g.M + kTmM - 1) / kTmM) * ((g.N + kTmN - 1) / kTmN);
	XTT_REQUIRE(tiles < (1ll << 31), "GEMM too large");
	const int nk = kpad / KT::kchunk;
	int S = 1;
	const long long partial = (long long)g.batch * g.M * g.N;
	if (tiles < c.num_sms && nk >= 4 && partial <= (1ll << 24))
		S = int(std::min<long long>(std::min<long long>(8, nk / 2), (c.num_sms + tiles - 1) / tiles));
	const int cpk = (nk + S - 1) / S;
	S = std::max(1, (nk + cpk - 1) / cpk);
	float* part = S > 1 ? c.scratch<float>(S_GEMM_TC_WORK, size_t(S) * size_t(partial)) : nullptr;
	func_attr_once(k_tma_gemm<T, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes<KIND>());
	k_tma_gemm<T, KIND><<<dim3(unsigned(tiles), unsigned(S)), kTmThreads, smem_bytes<KIND>(), c.stream>>>(
	    maps, g, cpk, part, c.d_status);
	XTT_CUDA(cudaGetLastError());
	if (S > 1) {
		const unsigned blocks = unsigned(std::min<long long>(4ll * c.num_sms, (partial + 255) / 256));
		k_tma_reduce<T><<<blocks, 256, 0, c.stream>>>(g, S, part);
		XTT_CUDA(cudaGetLastError());
		c.count_launch();
	}
	return true;
}

}  // namespace

// The TMA-fed form of gemm_tc; false when the driver cannot describe the operands as
// tensor maps (the caller then stages them itself).
template <class T>
bool gemm_tc_tma(Context& c, const Gemm<T>& g, int terms) {
	if (terms == 6) return launch_tma<T, KIND_BF16X6>(c, g);
	if (terms == 3) return launch_tma<T, KIND_TF32X3>(c, g);
	return launch_tma<T, KIND_TF32>(c, g);
}
template bool gemm_tc_tma<double>(Context&, const Gemm<double>&, int);
template bool gemm_tc_tma<float>(Context&, const Gemm<float>&, int);

}  // namespace xtt
