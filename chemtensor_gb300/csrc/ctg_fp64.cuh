// ctg_fp64.cuh - FP64 reciprocal and square root without the FP64 division / square-root
// sequences, for device code on GB300 (whose FP64 pipe makes those cost over a thousand cycles).
// Both start from FP32 hardware approximations on the mantissa and finish with cubically
// convergent corrections in FP64 (textbook Newton / Halley-type iterations), accurate to about one
// unit in the last place; exponents are handled exactly with integer operations.
#pragma once

#include <cuda_runtime.h>

namespace ctg {

// 1 / x for a normal double: FP32 estimate on the mantissa, one cubically convergent Newton step
// d (1 + e + e^2), e = 1 - m d (error ~e^3, below FP64 rounding), exponent negated exactly. An FP64
// division costs over a thousand cycles of GB300's FP64 pipe; this is six FP64 instructions.
__device__ __forceinline__ double rcp64(double x)
{
	const int hi = __double2hiint(x), lo = __double2loint(x);
	const int ex = ((hi >> 20) & 0x7ff) - 1023;
	const double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, lo);       // sign kept, |m| in [1, 2)
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)m));
	const double d = (double)r;
	const double e = fma(-m, d, 1.0);
	const double y = fma(d, fma(e, e, e), d);
	return y * __hiloint2double((1023 - ex) << 20, 0);
}

// sqrt(x) for a positive normal double: reciprocal square root of the mantissa (scaled into [1, 4)
// with an even exponent) from FP32, one cubically convergent correction y (1 + e/2 + 3 e^2 / 8),
// e = 1 - m y^2, then one Newton step for the square root itself, s + y (m - s^2) / 2.
__device__ __forceinline__ double sqrt64(double x)
{
	const int hi = __double2hiint(x), lo = __double2loint(x);
	int ex = ((hi >> 20) & 0x7ff) - 1023;
	double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);             // [1, 2)
	if (ex & 1)
	{
		m *= 2.0;                                                                 // [2, 4)
		ex -= 1;
	}
	float r;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)m));
	const double y0 = (double)r;
	const double e = fma(-m * y0, y0, 1.0);
	const double y = y0 * fma(e, fma(e, 0.375, 0.5), 1.0);
	double sroot = m * y;
	sroot = fma(0.5 * y, fma(-sroot, sroot, m), sroot);
	return sroot * __hiloint2double((1023 + ex / 2) << 20, 0);
}


// sqrt(x) and 1 / sqrt(x) together for a positive normal double (the reciprocal comes with the
// square root: one Newton sequence for both, accurate to about one unit in the last place)
__device__ __forceinline__ void sqrt_rsqrt64(double x, double& sq, double& rsq)
{
	const int hi = __double2hiint(x), lo = __double2loint(x);
	int ex = ((hi >> 20) & 0x7ff) - 1023;
	double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);             // [1, 2)
	if (ex & 1)
	{
		m *= 2.0;                                                                 // [2, 4)
		ex -= 1;
	}
	float r;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)m));
	const double y0 = (double)r;
	const double e = fma(-m * y0, y0, 1.0);
	const double y = y0 * fma(e, fma(e, 0.375, 0.5), 1.0);
	double sroot = m * y;
	sroot = fma(0.5 * y, fma(-sroot, sroot, m), sroot);
	sq = sroot * __hiloint2double((1023 + ex / 2) << 20, 0);
	rsq = y * __hiloint2double((1023 - ex / 2) << 20, 0);
}

// ---- double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits. Built from the error-free transformations of
// Knuth (two-sum) and Dekker (two-product, here with a hardware FMA); see D. H. Bailey's
// double-double / double-float libraries for the scheme. GB300 issues FP32 at 64 times the FP64
// rate, so a df64 operation of about a dozen FP32 instructions is several times cheaper than one
// FP64 instruction. Stored as float2 (x = hi, y = lo): the same 8 bytes as a double.

__device__ __forceinline__ float2 df_make(float hi, float lo) { return make_float2(hi, lo); }

// exact split of a double into hi + lo (rounding only below the 48th bit)
__device__ __forceinline__ float2 df_from_double(double x)
{
	const float hi = __double2float_rn(x);
	return make_float2(hi, __double2float_rn(x - (double)hi));
}

__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// s + e = a + b exactly
__device__ __forceinline__ float2 two_sum(float a, float b)
{
	const float s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
	return make_float2(s, e);
}

// s + e = a + b exactly, for |a| >= |b|
__device__ __forceinline__ float2 quick_two_sum(float a, float b)
{
	const float s = __fadd_rn(a, b);
	return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
	const float2 s = two_sum(a.x, b.x);
	const float2 t = two_sum(a.y, b.y);
	float2 r = quick_two_sum(s.x, __fadd_rn(s.y, t.x));
	return quick_two_sum(r.x, __fadd_rn(r.y, t.y));
}

// a * b (both df64)
__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
	const float p = __fmul_rn(a.x, b.x);
	float e = __fmaf_rn(a.x, b.x, -p);
	e = __fmaf_rn(a.x, b.y, e);
	e = __fmaf_rn(a.y, b.x, e);
	return quick_two_sum(p, e);
}

// a * b for a float a (exactly representable coefficient) and df64 b
__device__ __forceinline__ float2 df_mul_f(float a, float2 b)
{
	const float p = __fmul_rn(a, b.x);
	float e = __fmaf_rn(a, b.x, -p);
	e = __fmaf_rn(a, b.y, e);
	return quick_two_sum(p, e);
}

// acc + a * b, the product formed exactly in its leading part (inner products)
__device__ __forceinline__ float2 df_fma(float2 a, float2 b, float2 acc)
{
	return df_add(acc, df_mul(a, b));
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

}  // namespace ctg
