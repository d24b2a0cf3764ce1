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

namespace nlc {

__device__ __forceinline__ double dfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Table-driven exp (Tang, ACM TOMS 15(2) 1989): x = (n/256) ln2 + r, |r| <= ln2/512,
// scale*exp(x) = 2^(n>>8) * T[n&255] * (1 + r + r^2/2 + r^3/6 + r^4/24), T[j] = scale * 2^(j/256).
// Nine FP64 operations on the fast path against ~22 DFMA-equivalents for the library exp.  The
// range checks use the integer high word of x, which costs no FP64 issue slot.
__device__ __forceinline__ double exp_scaled(double x, const double *__restrict__ table) {
	const double shifter = 0x1.8p52, inv_l = 256. / 0x1.62e42fefa39efp-1;
	const double l1 = 0x1.62e42fefa39efp-9, l2 = 0x1.abc9e3b39803fp-64;
	const int hi = __double2hiint(x);
	if ((hi & 0x7fffffff) >= 0x40f00000) {   // |x| >= 65536, inf or NaN
		if (x != x) return x;
		return hi > 0 ? dmul(table[0], __longlong_as_double(0x7ff0000000000000LL)) : dmul(table[0], 0.);
	}
	const double t = dfma(x, inv_l, shifter);
	const int n = __double2loint(t);
	const double nf = dsub(t, shifter);
	double r = dfma(-nf, l1, x);
	r = dfma(-nf, l2, r);
	double q = dfma(r, 1. / 24, 1. / 6);
	q = dfma(q, r, 0.5);
	q = dfma(q, r, 1.);
	const double p = dmul(q, r);
	const double tj = table[n & 255];
	double v = dfma(tj, p, tj);
	const int k = n >> 8;
	long long vb = __double_as_longlong(v);
	const int e = int((vb >> 52) & 0x7ff);
	if (k > -1000 && k < 1000 && e + k > 0 && e + k < 0x7ff) {
		vb += (long long) k << 52;
		return __longlong_as_double(vb);
	}
	return ldexp(v, k);
}

}  // namespace nlc
