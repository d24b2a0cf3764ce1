// Batched FP64 complex FFT in shared memory, one chain per team of threads (a warp or a block).
//
// Stockham autosort, decimation in frequency (C. Van Loan, "Computational Frameworks for the Fast
// Fourier Transform", SIAM 1992, sec. 1.7): for each radix p of n = p_1 p_2 ... with the current
// sub-length L (L = n before the first stage) and stride s (s = 1), every butterfly (q, t),
// q < L/p, t < s, reads a_u = x[t + s (q + u L/p)], forms the p-point DFT, multiplies output v by
// exp(-+2 pi i q v / L) and writes y[t + s (p q + v)]; then L /= p, s *= p.  The result lands in
// natural order after the last stage, with no bit reversal.  Radices 4, 2, 3, 5 have dedicated
// butterflies; any other prime radix uses a direct p-point DFT.
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

// complex add / subtract / multiply, every FP64 operation issued as an FMA (nlc_device.cuh)
__device__ __forceinline__ double2 cadd(double2 a, double2 b, const FpOnes &k) {
	return make_double2(fadd(a.x, b.x, k), fadd(a.y, b.y, k));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b, const FpOnes &k) {
	return make_double2(fsub(a.x, b.x, k), fsub(a.y, b.y, k));
}
// a * w
__device__ __forceinline__ double2 cmul(double2 a, double2 w, const FpOnes &k) {
	return make_double2(dfma(a.x, w.x, -fmul(a.y, w.y, k)), dfma(a.x, w.y, fmul(a.y, w.x, k)));
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

// Stockham pass of length P.len on x (shared memory), y the ping-pong buffer.  t / T: this
// thread's index / size of the team.  Returns the buffer holding the result.
template <bool BLOCK, bool INV>
__device__ double2 *stockham_team(const FftPlanDev &P, double2 *x, double2 *y, int t, int T) {
	const int n = P.len;
	const double2 *__restrict__ tw = P.tw;
	const FpOnes &k = P.k1;
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
				const double2 b0 = cadd(a0, a2, k), b1 = csub(a0, a2, k), b2 = cadd(a1, a3, k), b3 = rot_mi<INV>(csub(a1, a3, k));
				double2 *o = y + tt + s * 4 * q;
				o[0] = cadd(b0, b2, k);
				if (q == 0) {
					o[s] = cadd(b1, b3, k);
					o[2 * s] = csub(b0, b2, k);
					o[3 * s] = csub(b1, b3, k);
				} else {
					o[s] = cmul(cadd(b1, b3, k), twiddle<INV>(tw, q * tws), k);
					o[2 * s] = cmul(csub(b0, b2, k), twiddle<INV>(tw, 2 * q * tws), k);
					o[3 * s] = cmul(csub(b1, b3, k), twiddle<INV>(tw, 3 * q * tws), k);
				}
			}
		} else if (p == 2) {
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)];
				double2 *o = y + tt + s * 2 * q;
				o[0] = cadd(a0, a1, k);
				o[s] = q == 0 ? csub(a0, a1, k) : cmul(csub(a0, a1, k), twiddle<INV>(tw, q * tws), k);
			}
		} else if (p == 3) {
			const double sn = P.sin60;   // sin(2 pi / 3), a parameter-bank operand
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)], a2 = x[tt + s * (q + 2 * m)];
				const double2 t1 = cadd(a1, a2, k);
				const double2 t2 = make_double2(dfma(t1.x, -P.half, a0.x), dfma(t1.y, -P.half, a0.y));
				const double2 d = csub(a1, a2, k);
				const double2 u = make_double2(fmul(sn, d.x, k), fmul(sn, d.y, k));
				// forward: X1 = t2 - i u, X2 = t2 + i u
				const double2 x1 = INV ? make_double2(fsub(t2.x, u.y, k), fadd(t2.y, u.x, k))
				                       : make_double2(fadd(t2.x, u.y, k), fsub(t2.y, u.x, k));
				const double2 x2 = INV ? make_double2(fadd(t2.x, u.y, k), fsub(t2.y, u.x, k))
				                       : make_double2(fsub(t2.x, u.y, k), fadd(t2.y, u.x, k));
				double2 *o = y + tt + s * 3 * q;
				o[0] = cadd(a0, t1, k);
				o[s] = q == 0 ? x1 : cmul(x1, twiddle<INV>(tw, q * tws), k);
				o[2 * s] = q == 0 ? x2 : cmul(x2, twiddle<INV>(tw, 2 * q * tws), k);
			}
		} else if (p == 5) {
			// t1 = a1 + a4, t2 = a2 + a3, t3 = a1 - a4, t4 = a2 - a3;
			// X1,4 = a0 + c1 t1 + c2 t2 -+ i (s1 t3 + s2 t4), X2,3 = a0 + c2 t1 + c1 t2 -+ i (s2 t3 - s1 t4)
			// (forward; the inverse swaps the signs of i), c_j = cos(2 pi j/5), s_j = sin(2 pi j/5)
			for (int b = t; b < nb; b += T) {
				const int q = b / s, tt = b - q * s;
				const double2 a0 = x[tt + s * q], a1 = x[tt + s * (q + m)], a2 = x[tt + s * (q + 2 * m)],
				              a3 = x[tt + s * (q + 3 * m)], a4 = x[tt + s * (q + 4 * m)];
				const double2 t1 = cadd(a1, a4, k), t2 = cadd(a2, a3, k), t3 = csub(a1, a4, k), t4 = csub(a2, a3, k);
				const double2 b1 = make_double2(dfma(P.c52, t2.x, dfma(P.c51, t1.x, a0.x)),
				                                dfma(P.c52, t2.y, dfma(P.c51, t1.y, a0.y)));
				const double2 b2 = make_double2(dfma(P.c51, t2.x, dfma(P.c52, t1.x, a0.x)),
				                                dfma(P.c51, t2.y, dfma(P.c52, t1.y, a0.y)));
				const double2 u1 = make_double2(dfma(P.s52, t4.x, fmul(P.s51, t3.x, k)),
				                                dfma(P.s52, t4.y, fmul(P.s51, t3.y, k)));
				const double2 u2 = make_double2(dfma(-P.s51, t4.x, fmul(P.s52, t3.x, k)),
				                                dfma(-P.s51, t4.y, fmul(P.s52, t3.y, k)));
				// b -+ i u: forward X1 = b1 - i u1 = (b1.x + u1.y, b1.y - u1.x)
				const double2 x1 = INV ? make_double2(fsub(b1.x, u1.y, k), fadd(b1.y, u1.x, k))
				                       : make_double2(fadd(b1.x, u1.y, k), fsub(b1.y, u1.x, k));
				const double2 x4 = INV ? make_double2(fadd(b1.x, u1.y, k), fsub(b1.y, u1.x, k))
				                       : make_double2(fsub(b1.x, u1.y, k), fadd(b1.y, u1.x, k));
				const double2 x2 = INV ? make_double2(fsub(b2.x, u2.y, k), fadd(b2.y, u2.x, k))
				                       : make_double2(fadd(b2.x, u2.y, k), fsub(b2.y, u2.x, k));
				const double2 x3 = INV ? make_double2(fadd(b2.x, u2.y, k), fsub(b2.y, u2.x, k))
				                       : make_double2(fsub(b2.x, u2.y, k), fadd(b2.y, u2.x, k));
				double2 *o = y + tt + s * 5 * q;
				o[0] = cadd(a0, cadd(t1, t2, k), k);
				if (q == 0) {
					o[s] = x1, o[2 * s] = x2, o[3 * s] = x3, o[4 * s] = x4;
				} else {
					o[s] = cmul(x1, twiddle<INV>(tw, q * tws), k);
					o[2 * s] = cmul(x2, twiddle<INV>(tw, 2 * q * tws), k);
					o[3 * s] = cmul(x3, twiddle<INV>(tw, 3 * q * tws), k);
					o[4 * s] = cmul(x4, twiddle<INV>(tw, 4 * q * tws), k);
				}
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
					if (q != 0 && v != 0) out = cmul(out, twiddle<INV>(tw, q * v * tws), k);
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

__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }

// Transform of one chain of length P.n held in x[0, n); x and y hold P.len elements each.
// Lengths whose padded form costs fewer operations (large prime factors; the plan decides) go
// through Bluestein's chirp-z identity
//   X_k = w_k sum_j (x_j w_j) conj(w)_{k-j},  w_j = exp(-i pi j^2 / n)
// (L. Bluestein, IEEE Trans. Audio Electroacoust. 18, 1970), the convolution evaluated as a cyclic
// convolution of smooth length m >= 2n - 1 by two Stockham passes; the backward transform uses the
// conjugate chirp.  Returns the buffer holding X[0, n).
template <bool BLOCK, bool INV>
__device__ double2 *fft_team(const FftPlanDev &P, double2 *x, double2 *y, int t, int T) {
	if (!P.bluestein) return stockham_team<BLOCK, INV>(P, x, y, t, T);
	const int n = P.n, m = P.len;
	const FpOnes &k = P.k1;
	for (int j = t; j < m; j += T) {
		if (j < n) {
			const double2 w = P.chirp[j];
			y[j] = cmul(x[j], INV ? conj2(w) : w, k);
		} else {
			y[j] = make_double2(0., 0.);
		}
	}
	team_sync<BLOCK>();
	double2 *r = stockham_team<BLOCK, false>(P, y, x, t, T);
	double2 *o = r == y ? x : y;
	const double2 *__restrict__ b = INV ? P.bi : P.bf;
	for (int j = t; j < m; j += T) r[j] = cmul(r[j], b[j], k);
	team_sync<BLOCK>();
	double2 *c = stockham_team<BLOCK, true>(P, r, o, t, T);
	for (int j = t; j < n; j += T) {
		const double2 w = P.chirp[j];
		c[j] = cmul(c[j], INV ? conj2(w) : w, k);
	}
	team_sync<BLOCK>();
	return c;
}

}  // namespace nlc
