// Batched FP64 complex FFT in shared memory, one chain per team of threads (a warp or a block).
//
// Stockham autosort, decimation in time (C. Van Loan, "Computational Frameworks for the Fast
// Fourier Transform", SIAM 1992, sec. 1.7): for each radix p of len = p_1 p_2 ..., with Ns the
// product of the radices already applied (1 before the first pass) and m = len / p, butterfly
// b < m, q = b / Ns, k = b mod Ns, reads a_u = x[b + u m], forms the p-point DFT of a_u w^{uk},
// w = exp(-+2 pi i / (Ns p)), and writes output v to y[q Ns p + k + v Ns]; then Ns *= p.  The
// result lands in natural order after the last pass, with no bit reversal.
//
// Twiddled radix-4, -3 and -2 butterflies use the FMA factorisation of S. Goedecker ("Fast radix
// 2, 3, 4, and 5 kernels for fast Fourier transformations on computers with overlapping
// multiply-add instructions", SIAM J. Sci. Comput. 18(6), 1997): with w_u = c_u (1 + i t_u),
// a_u w_u = c_u Z_u where Z_u = (x - t_u y, y + t_u x) takes two FMAs, and the c_u become the
// multipliers of the FMAs that form the butterfly's sums.  A twiddled radix-4 butterfly takes 22
// FP64 operations instead of 28 (three complex products and eight complex additions), radix 3 16
// instead of 22, radix 2 6 instead of 8.  The per-pass tables of t_u, c_u and their ratios are
// built on the host (fma_twiddle_entry).  Radix 5 multiplies its inputs by the twiddles and forms
// the DFT with its own butterfly; any other prime radix forms the direct DFT with the twiddles
// folded into the DFT's table index.
//
// Forward = exp(-2 pi i jk/n), unnormalised, as cuFFT / FFTW forward transforms in the reference.
#pragma once

#include <type_traits>

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

// a (1 + i t) (forward) or a (1 - i t) (inverse): two FMAs
template <bool INV>
__device__ __forceinline__ double2 ztan(double2 a, double t) {
	return INV ? make_double2(dfma(a.y, t, a.x), dfma(-a.x, t, a.y)) : make_double2(dfma(-a.y, t, a.x), dfma(a.x, t, a.y));
}
// a + c z, a - c z
__device__ __forceinline__ double2 fma2(double c, double2 z, double2 a) {
	return make_double2(dfma(c, z.x, a.x), dfma(c, z.y, a.y));
}

// Elementwise maps fused into a transform: `Pre` is applied to every element as the first pass
// reads it, `Post` to every element as the last pass writes it (index in [0, len)); each element
// passes through each exactly once, so the result equals a separate pass over the buffer.
struct NoMap {
	__device__ __forceinline__ double2 operator()(int, double2 v) const { return v; }
};

// One Stockham pass r (radix P.radix[r], Ns points already combined) from x to y.  PRE / POST: the
// pass applies `pre` to its inputs (the first pass) / `post` to its outputs (the last pass); they
// are template flags so that the other passes carry no trace of the maps.
template <bool BLOCK, bool INV, bool PRE, bool POST, class Pre, class Post>
__device__ __forceinline__ void stockham_pass(const FftPlanDev &P, int r, int Ns, double2 *x, double2 *y, int t, int T,
                                              const Pre &pre, const Post &post) {
	const int n = P.len;
	const double2 *__restrict__ tw = P.tw;
	const FpOnes &k = P.k1;
	const int p = P.radix[r];
	const int m = n / p;
	const double2 *__restrict__ g = P.gw + P.gw_off[r];
	// input u of butterfly b, and output v of the butterfly at base o (stride Ns)
	auto in = [&](int b, int u) {
		if constexpr (PRE) return pre(b + u * m, x[b + u * m]);
		else return x[b + u * m];
	};
	auto out = [&](int o, int v, double2 val) {
		if constexpr (POST) y[o + v * Ns] = post(o + v * Ns, val);
		else y[o + v * Ns] = val;
	};
	if (PRE && p != 4 && p != 2 && p != 3 && p != 5) {
		// a direct DFT reads each input p times: map the inputs once, in place, first
		for (int j = t; j < n; j += T) x[j] = pre(j, x[j]);
		team_sync<BLOCK>();
	}
	// the four outputs of a radix-4 butterfly, stored in an order rotated by b / max(Ns, 2): with
	// Ns < 8 the natural order puts the 8 threads of a 128-byte store phase on the same banks (Ns = 1:
	// a 64-byte stride, 4-way; Ns = 4: runs of four 256 bytes apart, 2-way), the rotated one on 8
	// different 16-byte bank groups.  The addresses written are the same.
	auto store4 = [&](int o, int b, double2 X0, double2 X1, double2 X2, double2 X3) {
		if (Ns >= 8) {
			out(o, 0, X0), out(o, 1, X1), out(o, 2, X2), out(o, 3, X3);
			return;
		}
		const int r = b / (Ns < 2 ? 2 : Ns);
#pragma unroll
		for (int i = 0; i < 4; i++) {
			const int v = (i + r) & 3;
			out(o, v, v == 0 ? X0 : v == 1 ? X1 : v == 2 ? X2 : X3);
		}
	};
	if (p == 4) {
		if (Ns == 1) {
			for (int b = t; b < m; b += T) {
				const double2 a0 = in(b, 0), a1 = in(b, 1), a2 = in(b, 2), a3 = in(b, 3);
				const double2 b0 = cadd(a0, a2, k), b1 = csub(a0, a2, k), b2 = cadd(a1, a3, k), b3 = rot_mi<INV>(csub(a1, a3, k));
				store4(4 * b, b, cadd(b0, b2, k), cadd(b1, b3, k), csub(b0, b2, k), csub(b1, b3, k));
			}
		} else {
			for (int b = t; b < m; b += T) {
				const int q = b / Ns, kk = b - q * Ns;
				const double2 a0 = x[b], a1 = x[b + m], a2 = x[b + 2 * m], a3 = x[b + 3 * m];
				const double2 e0 = g[3 * kk], e1 = g[3 * kk + 1], e2 = g[3 * kk + 2];   // {t1,t2} {t3,c1} {c2,c3/c1}
				const double2 z1 = ztan<INV>(a1, e0.x), z2 = ztan<INV>(a2, e0.y), z3 = ztan<INV>(a3, e1.x);
				const double c1 = e1.y, c2 = e2.x, rho = e2.y;
				// A_u = a_u w_u: A0 +- A2 = a0 +- c2 Z2, A1 +- A3 = c1 (Z1 +- (c3/c1) Z3)
				const double2 b0 = fma2(c2, z2, a0), b1 = fma2(-c2, z2, a0);
				const double2 p2 = fma2(rho, z3, z1), p3 = fma2(-rho, z3, z1);
				// X1 = (A0 - A2) -+ i (A1 - A3), X3 = (A0 - A2) +- i (A1 - A3) (forward / inverse)
				const double2 bm = make_double2(dfma(c1, p3.y, b1.x), dfma(-c1, p3.x, b1.y));   // b1 - i c1 p3
				const double2 bp = make_double2(dfma(-c1, p3.y, b1.x), dfma(c1, p3.x, b1.y));   // b1 + i c1 p3
				store4(q * 4 * Ns + kk, b, fma2(c1, p2, b0), INV ? bp : bm, fma2(-c1, p2, b0), INV ? bm : bp);
			}
		}
	} else if (p == 2) {
		for (int b = t; b < m; b += T) {
			const int q = b / Ns, kk = b - q * Ns;
			const double2 a0 = in(b, 0), a1 = in(b, 1);
			const int o = q * 2 * Ns + kk;
			if (Ns == 1) {
				out(o, 0, cadd(a0, a1, k));
				out(o, 1, csub(a0, a1, k));
			} else {
				const double2 e = g[kk];   // {t1, c1}
				const double2 z = ztan<INV>(a1, e.x);
				out(o, 0, fma2(e.y, z, a0));
				out(o, 1, fma2(-e.y, z, a0));
			}
		}
	} else if (p == 3) {
		for (int b = t; b < m; b += T) {
			const int q = b / Ns, kk = b - q * Ns;
			const double2 a0 = in(b, 0), a1 = in(b, 1), a2 = in(b, 2);
			double2 x0, xm, xp;   // X0, t2 - i u, t2 + i u
			if (Ns == 1) {
				const double sn = P.sin60;   // sin(2 pi / 3), a parameter-bank operand
				const double2 t1 = cadd(a1, a2, k);
				const double2 t2 = make_double2(dfma(t1.x, -P.half, a0.x), dfma(t1.y, -P.half, a0.y));
				const double2 d = csub(a1, a2, k);
				const double2 u = make_double2(fmul(sn, d.x, k), fmul(sn, d.y, k));
				x0 = cadd(a0, t1, k);
				xm = make_double2(fadd(t2.x, u.y, k), fsub(t2.y, u.x, k));
				xp = make_double2(fsub(t2.x, u.y, k), fadd(t2.y, u.x, k));
			} else {
				const double2 e0 = g[3 * kk], e1 = g[3 * kk + 1], e2 = g[3 * kk + 2];   // {t1,t2} {c1,c2/c1} {c1/2, c1 sin60}
				const double2 z1 = ztan<INV>(a1, e0.x), z2 = ztan<INV>(a2, e0.y);
				// A1 +- A2 = c1 (Z1 +- (c2/c1) Z2)
				const double2 ts = fma2(e1.y, z2, z1), d = fma2(-e1.y, z2, z1);
				x0 = fma2(e1.x, ts, a0);
				const double2 t2 = fma2(-e2.x, ts, a0);
				xm = make_double2(dfma(e2.y, d.y, t2.x), dfma(-e2.y, d.x, t2.y));
				xp = make_double2(dfma(-e2.y, d.y, t2.x), dfma(e2.y, d.x, t2.y));
			}
			// forward: X1 = t2 - i u, X2 = t2 + i u; the inverse the other way round
			const int o = q * 3 * Ns + kk;
			out(o, 0, x0);
			out(o, 1, INV ? xp : xm);
			out(o, 2, INV ? xm : xp);
		}
	} else if (p == 5) {
		// t1 = a1 + a4, t2 = a2 + a3, t3 = a1 - a4, t4 = a2 - a3;
		// X1,4 = a0 + c1 t1 + c2 t2 -+ i (s1 t3 + s2 t4), X2,3 = a0 + c2 t1 + c1 t2 -+ i (s2 t3 - s1 t4)
		// (forward; the inverse swaps the signs of i), c_j = cos(2 pi j/5), s_j = sin(2 pi j/5),
		// on the twiddled inputs a_u w^{uk}
		const int stride = n / (Ns * 5);
		for (int b = t; b < m; b += T) {
			const int q = b / Ns, kk = b - q * Ns;
			double2 a0 = in(b, 0), a1 = in(b, 1), a2 = in(b, 2), a3 = in(b, 3), a4 = in(b, 4);
			if (Ns > 1) {
				const int e = kk * stride;
				a1 = cmul(a1, twiddle<INV>(tw, e), k);
				a2 = cmul(a2, twiddle<INV>(tw, 2 * e), k);
				a3 = cmul(a3, twiddle<INV>(tw, 3 * e), k);
				a4 = cmul(a4, twiddle<INV>(tw, 4 * e), k);
			}
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
			const int o = q * 5 * Ns + kk;
			out(o, 0, cadd(a0, cadd(t1, t2, k), k));
			out(o, 1, x1), out(o, 2, x2), out(o, 3, x3), out(o, 4, x4);
		}
	} else {
		// direct p-point DFT of the twiddled inputs: X_v = sum_u a_u w^{uk} W_p^{uv}
		// = sum_u a_u tw[u (k + v Ns) n / (Ns p) mod n]
		const int stride = n / (Ns * p);
		for (int b = t; b < m; b += T) {
			const int q = b / Ns, kk = b - q * Ns;
			for (int v = 0; v < p; v++) {
				const int step = int((long long) (kk + v * Ns) * stride % n);
				double re = 0., im = 0.;
				int e = 0;
				for (int u = 0; u < p; u++) {
					const double2 a = x[b + u * m];
					const double2 w = twiddle<INV>(tw, e);
					re = dfma(a.x, w.x, dfma(-a.y, w.y, re));
					im = dfma(a.x, w.y, dfma(a.y, w.x, im));
					e += step;
					if (e >= n) e -= n;
				}
				out(q * p * Ns + kk, v, make_double2(re, im));
			}
		}
	}
}

// Stockham transform of length P.len on x (shared memory), y the ping-pong buffer.  t / T: this
// thread's index / size of the team.  Returns the buffer holding the result.
template <bool BLOCK, bool INV, class Pre = NoMap, class Post = NoMap>
__device__ double2 *stockham_team(const FftPlanDev &P, double2 *x, double2 *y, int t, int T, Pre pre = Pre(),
                                  Post post = Post()) {
	constexpr bool kPre = !std::is_same<Pre, NoMap>::value, kPost = !std::is_same<Post, NoMap>::value;
	int Ns = 1;
	for (int r = 0; r < P.nradix; r++) {
		const bool first = r == 0, last = r == P.nradix - 1;
		if (kPre && kPost && first && last) stockham_pass<BLOCK, INV, kPre, kPost>(P, r, Ns, x, y, t, T, pre, post);
		else if (kPre && first) stockham_pass<BLOCK, INV, kPre, false>(P, r, Ns, x, y, t, T, pre, post);
		else if (kPost && last) stockham_pass<BLOCK, INV, false, kPost>(P, r, Ns, x, y, t, T, pre, post);
		else stockham_pass<BLOCK, INV, false, false>(P, r, Ns, x, y, t, T, pre, post);
		team_sync<BLOCK>();
		double2 *sw = x;
		x = y, y = sw;
		Ns *= P.radix[r];
	}
	return x;
}

// FP32 forward transform for the FP32 diagnostics: the same decimation-in-time passes, with plain
// complex products by the twiddles of a float table tw[e] = exp(-2 pi i e / len) and FP32 sums.
// Only for direct passes (the plan keeps FP64 diagnostics for padded lengths).
__device__ __forceinline__ float2 cmulf(float2 a, float2 w) {
	return make_float2(fmaf(a.x, w.x, -(a.y * w.y)), fmaf(a.x, w.y, a.y * w.x));
}

template <bool BLOCK>
__device__ float2 *stockham32_team(const FftPlanDev &P, const float2 *__restrict__ tw, float2 *x, float2 *y, int t,
                                   int T) {
	const int n = P.len;
	int Ns = 1;
	for (int r = 0; r < P.nradix; r++) {
		const int p = P.radix[r];
		const int m = n / p;
		const int stride = n / (Ns * p);   // twiddle w^{uk} = tw[u k stride]
		if (p == 4) {
			for (int b = t; b < m; b += T) {
				const int q = b / Ns, kk = b - q * Ns;
				float2 a0 = x[b], a1 = x[b + m], a2 = x[b + 2 * m], a3 = x[b + 3 * m];
				if (Ns > 1) {
					const int e = kk * stride;
					a1 = cmulf(a1, tw[e]), a2 = cmulf(a2, tw[2 * e]), a3 = cmulf(a3, tw[3 * e]);
				}
				const float2 b0 = make_float2(a0.x + a2.x, a0.y + a2.y), b1 = make_float2(a0.x - a2.x, a0.y - a2.y);
				const float2 b2 = make_float2(a1.x + a3.x, a1.y + a3.y);
				const float2 b3 = make_float2(a1.y - a3.y, a3.x - a1.x);   // -i (a1 - a3)
				float2 *o = y + q * 4 * Ns + kk;
				o[0] = make_float2(b0.x + b2.x, b0.y + b2.y);
				o[Ns] = make_float2(b1.x + b3.x, b1.y + b3.y);
				o[2 * Ns] = make_float2(b0.x - b2.x, b0.y - b2.y);
				o[3 * Ns] = make_float2(b1.x - b3.x, b1.y - b3.y);
			}
		} else if (p == 2) {
			for (int b = t; b < m; b += T) {
				const int q = b / Ns, kk = b - q * Ns;
				float2 a0 = x[b], a1 = x[b + m];
				if (Ns > 1) a1 = cmulf(a1, tw[kk * stride]);
				float2 *o = y + q * 2 * Ns + kk;
				o[0] = make_float2(a0.x + a1.x, a0.y + a1.y);
				o[Ns] = make_float2(a0.x - a1.x, a0.y - a1.y);
			}
		} else {
			// direct p-point DFT of the twiddled inputs: X_v = sum_u a_u tw[u (k + v Ns) stride mod n]
			for (int b = t; b < m; b += T) {
				const int q = b / Ns, kk = b - q * Ns;
				for (int v = 0; v < p; v++) {
					const int step = int((long long) (kk + v * Ns) * stride % n);
					float re = 0.f, im = 0.f;
					int e = 0;
					for (int u = 0; u < p; u++) {
						const float2 a = x[b + u * m], w = tw[e];
						re = fmaf(a.x, w.x, fmaf(-a.y, w.y, re));
						im = fmaf(a.x, w.y, fmaf(a.y, w.x, im));
						e += step;
						if (e >= n) e -= n;
					}
					y[q * p * Ns + kk + v * Ns] = make_float2(re, im);
				}
			}
		}
		team_sync<BLOCK>();
		float2 *sw = x;
		x = y, y = sw;
		Ns *= p;
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
