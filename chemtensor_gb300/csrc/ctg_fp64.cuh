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

}  // namespace ctg
