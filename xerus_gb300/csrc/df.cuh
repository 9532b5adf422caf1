// Double-float arithmetic: an FP64 value carried as an FP32 pair hi + lo (hi its
// leading 24 significand bits, lo the next 29 rounded to 24: relative error ~2^-47),
// products formed error-free by FMA and summed by TwoSum, so FP64-accurate inner
// products run on the FP32 pipe (on GB300 one DFMA costs the issue of ~64 FFMAs). The
// intrinsics keep the compiler from contracting the error-free steps into FMAs.
#pragma once

#include <cuda_runtime.h>

namespace xtt {

__device__ __forceinline__ float2 df_split(double d) {
	const unsigned long long u = (unsigned long long)__double_as_longlong(d);
	const int e = int((u >> 52) & 0x7ffu) - 1023;
	if (e >= -74 && e <= 127) {  // hi and the scale of lo are normal FP32 numbers
		const unsigned sign = unsigned(u >> 32) & 0x80000000u;
		const float hi = __uint_as_float(sign | (unsigned(e + 127) << 23) | unsigned((u >> 29) & 0x7fffffu));
		const float scale = __uint_as_float(sign | (unsigned(e + 75) << 23));  // +-2^(e-52)
		return make_float2(hi, __fmul_rn(__uint2float_rn(unsigned(u & 0x1fffffffu)), scale));
	}
	return make_float2(__double2float_rn(d), 0.f);  // zero, and magnitudes FP32 cannot split
}

__device__ __forceinline__ void df_fma(float2 a, float2 b, float& s, float& c) {
	const float p = __fmul_rn(a.x, b.x);
	float e = __fmaf_rn(a.x, b.x, -p);
	e = __fmaf_rn(a.x, b.y, e);
	e = __fmaf_rn(a.y, b.x, e);
	const float t = __fadd_rn(s, p);
	const float bp = __fsub_rn(t, s);
	const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
	s = t;
	c = __fadd_rn(c, __fadd_rn(err, e));
}

// s + c -> s + c with |c| <= ulp(s) / 2 (Fast2Sum); keeps the low part's own rounding small
__device__ __forceinline__ void df_renorm(float& s, float& c) {
	const float t = __fadd_rn(s, c);
	c = __fsub_rn(c, __fsub_rn(t, s));
	s = t;
}

}  // namespace xtt
