// Batched FP64 complex FFT in shared memory, one chain per team of threads (a warp or a block).
//
// Stockham autosort, decimation in frequency (C. Van Loan, "Computational Frameworks for the Fast
// Fourier Transform", SIAM 1992, sec. 1.7): for each radix p of n = p_1 p_2 ... with the current
// sub-length L (L = n before the first stage) and stride s (s = 1), every butterfly (q, t),
// q < L/p, t < s, reads a_u = x[t + s (q + u L/p)], forms the p-point DFT, multiplies output v by
// exp(-+2 pi i q v / L) and writes y[t + s (p q + v)]; then L /= p, s *= p.  The result lands in
// natural order after the last stage, with no bit reversal.  Radices 4, 2, 3 have dedicated
// butterflies; any other prime radix uses a direct p-point DFT (the linear-energy diagnostics are
// the only users of those, and they run once per sample).
//
// Forward = exp(-2 pi i jk/n), unnormalised, as cuFFT / FFTW forward transforms in the reference.
#pragma once

#include "nlc_device.cuh"
#include "nlc_internal.h"

namespace nlc {

template <bool BLOCK>
__device__ __forceinline__ void team_sync() {
	if (BLOCK) __syncthreads();
	else __syncwarp();
}

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(dadd(a.x, b.x), dadd(a.y, b.y)); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(dsub(a.x, b.x), dsub(a.y, b.y)); }
// a * w
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
	return make_double2(dfma(a.x, w.x, -dmul(a.y, w.y)), dfma(a.x, w.y, dmul(a.y, w.x)));
}
// twiddle exp(-+2 pi i e / n) from the forward table
template <bool INV>
__device__ __forceinline__ double2 twiddle(const double2 *__restrict__ tw, int e) {
	const double2 w = tw[e];
	return INV ? make_double2(w.x, -w.y) : w;
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ double2 rot_mi(double2 a) {
	return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// In-place transform of one chain held in x (shared memory, n complex), y the ping-pong buffer.
// t / T: this thread's index / size of the team.  Returns the buffer holding the result.
template <bool BLOCK, bool INV>
__device__ double2 *fft_team(const FftPlanDev &P, double2 *x, double2 *y, int t, int T) {
	const int n = P.n;
	const double2 *__restrict__ tw = P.tw;
	int L = n, s = 1;
	for (int r = 0; r < P.nradix; r++) {
		const int p = P.radix[r];
		const int m = L / p;
		const int tws = n / L;
		const int nb = n / p;
		if (p == 4) {
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)], a2 = x[tt + s * (q + 2 * m)],
				              a3 = x[tt + s * (q + 3 * m)];
				const double2 b0 = cadd(a0, a2), b1 = csub(a0, a2), b2 = cadd(a1, a3), b3 = rot_mi<INV>(csub(a1, a3));
				double2 *o = y + tt + s * 4 * q;
				o[0] = cadd(b0, b2);
				if (q == 0) {
					o[s] = cadd(b1, b3);
					o[2 * s] = csub(b0, b2);
					o[3 * s] = csub(b1, b3);
				} else {
					o[s] = cmul(cadd(b1, b3), twiddle<INV>(tw, q * tws));
					o[2 * s] = cmul(csub(b0, b2), twiddle<INV>(tw, 2 * q * tws));
					o[3 * s] = cmul(csub(b1, b3), twiddle<INV>(tw, 3 * q * tws));
				}
			}
		} else if (p == 2) {
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)];
				double2 *o = y + tt + s * 2 * q;
				o[0] = cadd(a0, a1);
				o[s] = q == 0 ? csub(a0, a1) : cmul(csub(a0, a1), twiddle<INV>(tw, q * tws));
			}
		} else if (p == 3) {
			const double sn = 0.86602540378443864676;   // sin(2 pi / 3)
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)], a2 = x[tt + s * (q + 2 * m)];
				const double2 t1 = cadd(a1, a2);
				const double2 t2 = make_double2(dfma(t1.x, -0.5, a0.x), dfma(t1.y, -0.5, a0.y));
				const double2 d = csub(a1, a2);
				const double2 u = make_double2(dmul(sn, d.x), dmul(sn, d.y));
				// forward: X1 = t2 - i u, X2 = t2 + i u
				const double2 x1 = INV ? make_double2(dsub(t2.x, u.y), dadd(t2.y, u.x)) : make_double2(dadd(t2.x, u.y), dsub(t2.y, u.x));
				const double2 x2 = INV ? make_double2(dadd(t2.x, u.y), dsub(t2.y, u.x)) : make_double2(dsub(t2.x, u.y), dadd(t2.y, u.x));
				double2 *o = y + tt + s * 3 * q;
				o[0] = cadd(a0, t1);
				o[s] = q == 0 ? x1 : cmul(x1, twiddle<INV>(tw, q * tws));
				o[2 * s] = q == 0 ? x2 : cmul(x2, twiddle<INV>(tw, 2 * q * tws));
			}
		} else {
			// direct p-point DFT: X_v = sum_u a_u W_p^{uv}, W_p^e = tw[(e mod p) n/p]
			const int np = n / p;
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				for (int v = 0; v < p; v++) {
					double re = 0., im = 0.;
					for (int u = 0; u < p; u++) {
						const double2 a = x[tt + s * (q + u * m)];
						const double2 w = twiddle<INV>(tw, (u * v) % p * np);
						re = dfma(a.x, w.x, dfma(-a.y, w.y, re));
						im = dfma(a.x, w.y, dfma(a.y, w.x, im));
					}
					double2 out = make_double2(re, im);
					if (q != 0 && v != 0) out = cmul(out, twiddle<INV>(tw, q * v * tws));
					y[tt + s * (p * q + v)] = out;
				}
			}
		}
		team_sync<BLOCK>();
		double2 *sw = x;
		x = y, y = sw;
		L = m, s *= p;
	}
	return x;
}

}  // namespace nlc
