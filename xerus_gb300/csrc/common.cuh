// Shared definitions of the GB300 TT sweep engine: status codes, launch checks,
// warp/block reductions and a bounded grid-wide barrier for persistent kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

#include "../../include/xtt.h"

namespace xtt {

// Exception carrying an xtt_status; the C ABI turns it into a return code.
struct Error : std::runtime_error {
	int code;
	Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define XTT_REQUIRE(cond, msg)                                                                       \
	do {                                                                                             \
		if (!(cond)) throw ::xtt::Error(XTT_ERR_ARGUMENT, std::string("requirement failed: ") + msg); \
	} while (0)

#define XTT_CUDA(call)                                                                                        \
	do {                                                                                                      \
		cudaError_t e_ = (call);                                                                              \
		if (e_ != cudaSuccess)                                                                                \
			throw ::xtt::Error(XTT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " at " +   \
			                                     __FILE__ + ":" + std::to_string(__LINE__));                  \
	} while (0)

// Makes `device` current for the scope's lifetime and restores the previous device
// afterwards (device < 0: no change). Every entry point switches to the device of the
// context it works on, so one host thread can drive contexts on several GPUs.
struct DeviceScope {
	int prev = -1;
	explicit DeviceScope(int device) {
		if (device < 0) return;
		int cur = -1;
		XTT_CUDA(cudaGetDevice(&cur));
		if (cur != device) {
			XTT_CUDA(cudaSetDevice(device));
			prev = cur;
		}
	}
	~DeviceScope() {
		if (prev >= 0) cudaSetDevice(prev);
	}
	DeviceScope(const DeviceScope&) = delete;
	DeviceScope& operator=(const DeviceScope&) = delete;
};

// cudaFuncSetAttribute acts on the current device only: applies (kernel, attribute,
// value) once per device, thread-safe (defined in ops.cu).
void func_attr_once(const void* kernel, cudaFuncAttribute attr, int value);
template <class K>
inline void func_attr_once(K* kernel, cudaFuncAttribute attr, int value) {
	func_attr_once(reinterpret_cast<const void*>(kernel), attr, value);
}

// Device-side status word of a context: kernels record the first failure here
// instead of trapping, the host reads it after synchronising.
enum DeviceStatus : int {
	DEV_OK = 0,
	DEV_TIMEOUT = 1,        // a bounded spin in a grid barrier gave up
	DEV_NOT_CONVERGED = 2,  // CG / Jacobi iteration cap
	DEV_BREAKDOWN = 3,      // CG breakdown (p^T A p <= 0: operator not SPD) or NaN
	DEV_CAPACITY = 4,       // a launch got a size beyond what it was built for
};

// Conjugate gradients on an SPD system whose tolerance lies below its rounding
// floor stagnate, and p^T M p can then round to <= 0. Both are the floor, not
// an indefinite operator, once the relative residual is small: a breakdown is
// an error only while ||r|| > 1e-6 ||b||.
__host__ __device__ __forceinline__ bool cg_breakdown_is_error(double rr, double bb) { return rr > 1e-12 * bb; }

// Stagnation test: every 256 iterations the smallest ||r||^2 of the window must
// improve on the best of the earlier windows by 1%, else the solve stops at its
// floor (slow but genuine convergence, condition numbers up to ~1e8, passes).
struct CgFloor {
	double best = 1e300, window = 1e300;
	__host__ __device__ bool stalled(double rr, int it) {
		if (rr < window) window = rr;
		if (it % 256 != 0) return false;
		const bool stop = !(window < 0.99 * best);
		best = window < best ? window : best;
		window = 1e300;
		return stop;
	}
};

__device__ __forceinline__ void record_status(int* status, int code) {
	if (status) atomicCAS(status, DEV_OK, code);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// Sum over the block; every thread gets the result. `scratch` holds >= 32 T.
template <class T>
__device__ T block_sum(T v, T* scratch) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
	v = warp_sum(v);
	__syncthreads();
	if (lane == 0) scratch[warp] = v;
	__syncthreads();
	T s = T(0);
	for (int i = 0; i < nw; ++i) s += scratch[i];  // fixed order: deterministic
	__syncthreads();
	return s;
}

// Grid barrier for a cooperative (co-resident) launch: a sense-reversing
// counter with an iteration limit. On timeout it records DEV_TIMEOUT and
// returns false; callers then leave their loops, so the kernel always ends.
struct GridBarrier {
	unsigned int* count;   // zero-initialised
	unsigned int* phase;   // zero-initialised
	int* status;
};

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
	unsigned int v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
	int v;
	asm volatile("ld.volatile.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

constexpr long long kBarrierSpinLimit = 20000000;  // ~ seconds of spinning at most

__device__ __forceinline__ bool grid_sync(const GridBarrier& b) {
	__syncthreads();
	__shared__ int ok;
	if (threadIdx.x == 0) {
		ok = 1;
		const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
		const unsigned int my_phase = ld_acquire_u32(b.phase);
		__threadfence();
		const unsigned int arrived = atomicAdd(b.count, 1u);
		if (arrived == nb - 1) {
			*b.count = 0;
			__threadfence();
			atomicAdd(b.phase, 1u);
		} else {
			long long spins = 0;
			while (ld_acquire_u32(b.phase) == my_phase) {
				if (++spins > kBarrierSpinLimit || ld_volatile_i32(b.status) == DEV_TIMEOUT) {
					record_status(b.status, DEV_TIMEOUT);
					ok = 0;
					break;
				}
				__nanosleep(20);
			}
		}
		__threadfence();
	}
	__syncthreads();
	return ok != 0;
}

inline int ceil_div(long long a, long long b) { return int((a + b - 1) / b); }

}  // namespace xtt
