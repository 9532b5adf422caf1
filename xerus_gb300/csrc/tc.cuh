// Fifth-generation tensor core (tcgen05) building blocks for sm_103a, written as
// inline PTX: tensor-memory allocation, shared-memory matrix descriptors, the
// TF32 MMA with FP32 accumulation in tensor memory, completion through an
// mbarrier (bounded wait), and the accumulator read-back.
//
// Operand layout in shared memory: no swizzle, K-major "core matrices" of 8 rows
// x 16 bytes (8 x 4 TF32 elements) stored as 128 contiguous bytes. A tile of R
// rows and 32 K-elements holds its core matrices K-group-fastest: core (g_r, g_k)
// at byte (g_r * 8 + g_k) * 128, so the K-direction core stride (LBO) is 128 bytes
// and the 8-row-group stride (SBO) is 1024 bytes. One MMA consumes K = 8 (two
// K-groups); the k-th MMA of a 32-deep chunk starts 256 * k bytes into the tile.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace xtt {
namespace tc {

constexpr int kTileK = 32;             // K elements per staged chunk
constexpr int kCoreBytes = 128;        // one 8 x 16-byte core matrix
constexpr uint32_t kLbo = 128;         // K-direction core-matrix stride
constexpr uint32_t kSbo = 8 * 128;     // 8-row-group stride (8 K-groups of a 32-deep chunk)
constexpr long long kWaitLimit = 1ll << 22;  // bounded mbarrier polls (seconds at most)

// Byte offset of element (r, k) (0 <= k < 32) inside a staged tile.
__device__ __forceinline__ uint32_t tile_offset(int r, int k) {
	return uint32_t((((r >> 3) << 3) + (k >> 2)) * kCoreBytes + ((r & 7) << 4) + ((k & 3) << 2));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, LBO and SBO (all >> 4), the
// fixed version field (bits 46-48 = 1), no base offset, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
	uint64_t d = 0;
	d |= uint64_t((addr & 0x3FFFF) >> 4);
	d |= uint64_t(kLbo >> 4) << 16;
	d |= uint64_t(kSbo >> 4) << 32;
	d |= uint64_t(1) << 46;
	return d;
}

// Instruction descriptor of kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
	return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Round an FP32 value to TF32 (nearest, ties away), low 13 mantissa bits zero.
__device__ __forceinline__ float to_tf32(float x) {
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return __uint_as_float(r);
}

// Tensor memory: one warp allocates `cols` columns (a power of two >= 32) and
// writes the base address to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t cols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(cols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory stores become visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Waits for phase `parity` of the barrier to complete; false after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
	const uint32_t a = smem_u32(bar);
	for (long long i = 0; i < kWaitLimit; ++i) {
		uint32_t done;
		asm volatile(
		    "{\n\t.reg .pred p;\n\t"
		    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}"
		    : "=r"(done)
		    : "r"(a), "r"(parity)
		    : "memory");
		if (done) return true;
	}
	return false;
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 8 TF32 (one thread issues).
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
	    : "memory");
}

// The barrier's next phase completes when every MMA this thread issued so far has.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
	    "%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr)
	    : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ TMA-fed operands
// Shared-memory matrix descriptor for a K-major operand tile written by TMA with the
// 128-byte swizzle: rows of 128 bytes (32 TF32 or 64 BF16 elements of K), 8-row groups
// 1024 bytes apart (SBO), the leading offset unused for swizzled K-major tiles (1),
// version 1 (bits 46-48), swizzle mode 2 = 128B (bits 61-63). The tile must start on a
// 1024-byte boundary; the k-th 32-byte K step of a row starts `32 k` bytes in.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
	uint64_t d = 0;
	d |= uint64_t((addr & 0x3FFFF) >> 4);
	d |= uint64_t(1) << 16;
	d |= uint64_t(1024 >> 4) << 32;
	d |= uint64_t(1) << 46;
	d |= uint64_t(2) << 61;
	return d;
}

// Instruction descriptor of kind::f16 with BF16 operands: D = F32 (bits 4-5 = 1),
// A = B = BF16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 16 BF16 (one thread issues).
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
	    : "memory");
}

// The barrier's current phase also waits for `bytes` of asynchronous copies (this
// thread's arrival counts as one).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// A 3-D tile of a tensor map (coordinates innermost first) into shared memory; the
// copy's bytes complete on `bar`. The innermost coordinate times the element size must
// be a multiple of 16 bytes (callers pass multiples of the 128-byte box row).
__device__ __forceinline__ void tma_load_3d(void* dst, const void* tmap, uint64_t* bar, int c0, int c1, int c2) {
	asm volatile(
	    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
	    "[%5];" ::"r"(smem_u32(dst)),
	    "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
	    : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const void* tmap) {
	asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

}  // namespace tc
}  // namespace xtt
