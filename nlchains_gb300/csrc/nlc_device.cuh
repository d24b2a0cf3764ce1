// Device-side helpers shared by the nlchains sm_103a kernels.
//
// Every FP64 operation on the hot path is written with an explicit round-to-nearest intrinsic, so
// that the operation sequence (and therefore every rounding) is fixed by this source rather than by
// the compiler's contraction choices; the CPU oracle replays the same sequence in C.  On GB300 the
// FP64 pipe is the bottleneck of every integrator (600 G DFMA lane-ops/s for the whole GPU, ~1/58
// of FP32), so these kernels are written to minimise FP64 instructions: integer and FP32 work,
// shuffles and shared-memory traffic are comparatively free.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nlc_internal.h"

namespace nlc {

__device__ __forceinline__ double dfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// On GB300 the FP64 pipe issues DFMA at 600 G lane-ops/s but DADD / DMUL at 506 G (measured with
// runtime operands, independent of the values).  Adds, subtractions and multiplications on the hot
// paths are therefore issued as FMAs with the exact same result: a + b = fma(a, 1, b),
// a - b = fma(b, -1, a), a * b = fma(a, b, -0) (the -0 addend keeps the sign of a zero product).
// The constants reach the kernels as parameters (FpOnes in nlc_internal.h), so the compiler cannot
// fold them back into DADD / DMUL, and they are parameter-bank operands rather than registers.
__device__ __forceinline__ double fadd(double a, double b, const FpOnes &k) { return __fma_rn(a, k.one, b); }
__device__ __forceinline__ double fsub(double a, double b, const FpOnes &k) { return __fma_rn(b, k.mone, a); }
__device__ __forceinline__ double fmul(double a, double b, const FpOnes &k) { return __fma_rn(a, b, k.mzero); }

// Table-driven exp (Tang, ACM TOMS 15(2) 1989): x = (n/2048) ln2 + r, |r| <= ln2/4096,
// scale*exp(x) = 2^(n>>11) * T[n&2047] * (1 + r + r^2/2 + r^3/6), T[j] = scale * 2^(j/2048); the
// dropped r^4/24 is below 2^-54.  Eight FP64 operations (all issued as FMAs) on the fast path
// against ~22 DFMA-equivalents for the library exp; the 16 KB table sits in shared memory.  The
// range checks use the integer high word of x, which costs no FP64 issue slot.
__device__ __forceinline__ double exp_scaled(double x, const double *__restrict__ table, const FpOnes &k1,
                                             const ExpConsts &c) {
	const int hi = __double2hiint(x);
	if ((hi & 0x7fffffff) >= 0x40f00000) {   // |x| >= 65536, inf or NaN
		if (x != x) return x;
		return hi > 0 ? dmul(table[0], __longlong_as_double(0x7ff0000000000000LL)) : dmul(table[0], 0.);
	}
	const double t = dfma(x, c.inv_l, c.shifter);
	const int n = __double2loint(t);
	const double nf = fsub(t, c.shifter, k1);
	double r = dfma(-nf, c.l1, x);
	r = dfma(-nf, c.l2, r);
	double q = dfma(r, c.c3, c.c2);
	q = dfma(q, r, k1.one);
	const double p = fmul(q, r, k1);
	const double tj = table[n & (kExpTable - 1)];
	double v = dfma(tj, p, tj);
	const int k = n >> 11;
	long long vb = __double_as_longlong(v);
	const int e = int((vb >> 52) & 0x7ff);
	if (k > -1000 && k < 1000 && e + k > 0 && e + k < 0x7ff) {
		vb += (long long) k << 52;
		return __longlong_as_double(vb);
	}
	return ldexp(v, k);
}

// sin(th), cos(th) from a 1024-entry table (S. Gal, "Computing elementary functions: a new approach
// for achieving high accuracy and good performance", LNCS 235, 1986; P. T. P. Tang's table-driven
// method): th = j 2 pi/1024 + r with j = round(th 1024 / (2 pi)) by the shifter trick and r reduced
// in two FMAs against pi/512 split into two doubles, |r| <= pi/1024; sin r and cos r - 1 by their
// Taylor series to r^5 / r^4 (next terms below 2^-59 relative), then
//   cos th = C_j + C_j (cos r - 1) - S_j sin r,  sin th = S_j + S_j (cos r - 1) + C_j sin r.
// 14 FP64 operations; the 16 KB table is read through the read-only cache.  Angles below 2^-4 (the
// DNLS phase rotation's usual range, beta dt c_k |psi|^2) skip the reduction and the table: their
// Taylor series to th^9 / th^8, 10 operations.  |th| >= 2^20, inf and NaN go to the library sincos.
__device__ __forceinline__ void sincos_table(double th, const double2 *__restrict__ tab, const SinCosConsts &C,
                                             const FpOnes &k, double *s, double *c) {
	const int hi = __double2hiint(th) & 0x7fffffff;
	if (hi < 0x3fb00000) {   // |th| < 2^-4
		const double t2 = fmul(th, th, k);
		const double ps = dfma(t2, dfma(t2, dfma(t2, C.q9, C.q7), C.q5), C.q3);
		*s = dfma(fmul(th, t2, k), ps, th);
		*c = dfma(t2, dfma(t2, dfma(t2, dfma(t2, C.w8, C.w6), C.w4), C.w2), k.one);
		return;
	}
	if (hi >= 0x41300000) {
		sincos(th, s, c);
		return;
	}
	const double t = dfma(th, C.inv, C.shifter);
	const double kd = fsub(t, C.shifter, k);
	const double r = dfma(-kd, C.p2, dfma(-kd, C.p1, th));
	const double2 e = __ldg(tab + (__double2loint(t) & (kSinCosTable - 1)));
	const double r2 = fmul(r, r, k);
	const double sr = dfma(fmul(r, r2, k), dfma(r2, C.s5, C.s3), r);
	const double cm1 = fmul(r2, dfma(r2, C.c4, C.c2), k);
	*c = dfma(e.x, cm1, dfma(-e.y, sr, e.x));
	*s = dfma(e.y, cm1, dfma(e.x, sr, e.y));
}

}  // namespace nlc
