/*
 * nlc_oracle.c -- TEST INFRASTRUCTURE ONLY (see nlc_oracle.h).  CPU restatement of the nlchains
 * hot path.  Built twice by oracle/build.py: a strict checker (-O2 -ffp-contract=off, the one the
 * tests compare against) and the timed CPU baseline (-Ofast -ffp-contract=fast -fopenmp, as the
 * reference's CPU build is -Ofast; one OpenMP thread per core over copies, the moral equivalent of
 * `mpirun -n <cores> nlchains <model>-cpu`).
 *
 * Parity: pinned to the reference's own CPU program, compiled in place from its sources (see
 * nlc_oracle.h and tests/test_reference_pin.py), and by analytic known answers in tests/
 * (test_oracle.py, test_known_answers.py).
 */
#include "nlc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* common/symplectic.hpp:5-8 */
static const double yoshida_c[8] = {0.392256805238780, 0.510043411918458, -0.471053385409757,
                                    0.068753168252518, 0.068753168252518, -0.471053385409757,
                                    0.510043411918458, 0.392256805238780};
static const double yoshida_d[8] = {0.784513610477560, 0.235573213359357, -1.177679984178870,
                                    1.315186320683906, -1.177679984178870, 0.235573213359357,
                                    0.784513610477560, 0};

void nlo_coefficients(double c[8], double d[8]) {
	for (int i = 0; i < 8; i++) c[i] = yoshida_c[i], d[i] = yoshida_d[i];
}

/* ------------------------------------------------------------------------------------------------
 * Table-driven exp (Tang, "Table-driven implementation of the exponential function in IEEE
 * floating-point arithmetic", ACM TOMS 15(2), 1989): x = (n/256) ln2 + r, exp(x) = 2^(n>>8) *
 * 2^((n&255)/256) * exp(r), |r| <= ln2/512, exp(r) - 1 by its degree-4 Taylor polynomial.  The
 * table is generated in double-double arithmetic so that every IEEE platform builds the same bits.
 * ----------------------------------------------------------------------------------------------*/

typedef struct { double hi, lo; } dd;

static dd dd_two_sum(double a, double b) {
	double s = a + b, bb = s - a, e = (a - (s - bb)) + (b - bb);
	dd r = {s, e};
	return r;
}

static dd dd_renorm(double hi, double lo) {
	double s = hi + lo, e = lo - (s - hi);
	dd r = {s, e};
	return r;
}

static dd dd_add(dd a, dd b) {
	dd s = dd_two_sum(a.hi, b.hi);
	return dd_renorm(s.hi, s.lo + a.lo + b.lo);
}

static dd dd_mul(dd a, dd b) {
	double p = a.hi * b.hi, e = fma(a.hi, b.hi, -p);
	e += a.hi * b.lo + a.lo * b.hi;
	return dd_renorm(p, e);
}

static dd dd_div_u(dd a, unsigned k) {
	double q1 = a.hi / k;
	/* remainder a - q1*k, exact product by fma */
	double p = q1 * k, pe = fma(q1, (double) k, -p);
	double rem = ((a.hi - p) - pe) + a.lo;
	double q2 = rem / k;
	return dd_renorm(q1, q2);
}

/* exp(y) for 0 <= y < 1 in double-double by its Taylor series */
static dd dd_exp_small(dd y) {
	dd sum = {1., 0.}, term = {1., 0.};
	for (unsigned k = 1; k < 40; k++) {
		term = dd_div_u(dd_mul(term, y), k);
		sum = dd_add(sum, term);
		if (fabs(term.hi) < 1e-40) break;
	}
	return sum;
}

void nlo_exp_table(double scale, double table[NLO_EXP_TABLE]) {
	const dd ln2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
	for (unsigned j = 0; j < NLO_EXP_TABLE; j++) {
		dd frac = {(double) j / NLO_EXP_TABLE, 0.};
		dd v = dd_exp_small(dd_mul(ln2, frac));
		dd s = {scale, 0.};
		v = dd_mul(v, s);
		table[j] = v.hi + v.lo;
	}
}

/* The exact FP64 sequence of the device exp (nlchains_gb300/csrc/nlc_device.cuh, exp_scaled). */
double nlo_exp_scaled(double x, const double table[NLO_EXP_TABLE]) {
	const double shifter = 0x1.8p52, inv_l = 2048. / 0x1.62e42fefa39efp-1;
	const double l1 = 0x1.62e42fefa39efp-12, l2 = 0x1.abc9e3b39803fp-67;
	int64_t xb;
	memcpy(&xb, &x, 8);
	const int32_t hi = (int32_t) (xb >> 32);
	if ((hi & 0x7fffffff) >= 0x40f00000) { /* |x| >= 65536, inf or NaN */
		if (x != x) return x;
		return hi > 0 ? table[0] * INFINITY : table[0] * 0.;
	}
	double t = fma(x, inv_l, shifter);
	int64_t tb;
	memcpy(&tb, &t, 8);
	int32_t n = (int32_t) (uint32_t) tb;
	double nf = t - shifter;
	double r = fma(-nf, l1, x);
	r = fma(-nf, l2, r);
	double q = fma(r, 1. / 6, 0.5);
	q = fma(q, r, 1.);
	double p = q * r;
	double tj = table[n & (NLO_EXP_TABLE - 1)];
	double v = fma(tj, p, tj);
	int32_t k = n >> 11;   /* arithmetic shift: floor(n / 2048) */
	if (k > -1000 && k < 1000) {
		int64_t vb;
		memcpy(&vb, &v, 8);
		/* the table entries are normal numbers; only fold the scale in when it stays normal */
		int64_t e = (vb >> 52) & 0x7ff;
		if (e + k > 0 && e + k < 0x7ff) {
			vb += (int64_t) k << 52;
			memcpy(&v, &vb, 8);
			return v;
		}
	}
	return ldexp(v, k);
}

/* ------------------------------------------------------------------------------------------------
 * Real models: DNKG, FPUT, Toda, dDNKG
 * ----------------------------------------------------------------------------------------------*/

typedef struct {
	double dtc[8], dtd[8], dtc0x2;
	double mp2;            /* DNKG: m + 2 */
	double alpha2, alpha2_inv;
	double exptab[NLO_EXP_TABLE];   /* Toda device order: alpha2_inv * 2^(j/2048) */
} consts;

static void make_consts(const nlo_model *M, consts *K) {
	for (int i = 0; i < 8; i++) K->dtc[i] = yoshida_c[i] * M->dt, K->dtd[i] = yoshida_d[i] * M->dt;
	K->dtc0x2 = K->dtc[0] * 2;
	K->mp2 = M->m + 2;
	K->alpha2 = 2 * M->alpha;
	K->alpha2_inv = 1 / K->alpha2;
	if (M->model == NLO_TODA) nlo_exp_table(K->alpha2_inv, K->exptab);
}

/* Reference CPU arithmetic: DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp:23-40 and
 * dDNKG/cpu-implementation/dDNKG.cpp:160-162, one rounding per C operator (no contraction). */
static inline double rhs_reference(int model, const nlo_model *M, const consts *K, double left,
                                   double center, double right, double mp2_x) {
	switch (model) {
		case NLO_DNKG:
			return -(center * (M->m + 2 + M->beta * center * center) - left - right);
		case NLO_FPUT: {
			double ret = (left + right - 2 * center);
			ret *= (1 + M->alpha * (right - left));
			double dright = right - center, dleft = center - left;
			return ret + M->beta * (dright * dright * dright - dleft * dleft * dleft);
		}
		case NLO_TODA:
			return K->alpha2_inv * (exp(K->alpha2 * (right - center)) - exp(K->alpha2 * (center - left)));
		default: /* dDNKG */
			return -(center * (mp2_x + M->beta * center * center) - left - right);
	}
}

/* One launch of `batching` steps on one chain, reference CPU loop structure
 * (DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp:121-142): phi carries two ghost sites. */
static void move_chain_reference(const nlo_model *M, const consts *K, double *restrict phi,
                                 double *restrict pi, uint32_t batching) {
	const uint32_t n = M->n;
	const double *mp2 = M->mp2;
	for (uint32_t i = 0; i < batching; i++) {
		for (int k = 0; k < 7; k++) {
			double dt_c_k = K->dtc[k];
			if (i && !k) dt_c_k *= 2;
			for (uint32_t s = 0; s < n; s++) phi[s + 1] += dt_c_k * pi[s];
			phi[0] = phi[n], phi[n + 1] = phi[1];
			const double dt_d_k = K->dtd[k];
			for (uint32_t s = 0; s < n; s++)
				pi[s] += dt_d_k * rhs_reference(M->model, M, K, phi[s], phi[s + 1], phi[s + 2],
				                                mp2 ? mp2[s] : 0.);
		}
	}
	for (uint32_t s = 0; s < n; s++) phi[s + 1] += K->dtc[7] * pi[s];
}

/* One launch of `batching` steps on one chain in the device operation order (nlchains_gb300/csrc/nlc_real.cuh):
 *   drift   q = fma(cd, p, q)
 *   DNKG    t = fma(beta*c, c, mp2); u = fma(c, t, -l); v = u - r; p = fma(-ck, v, p)
 *   FPUT    bond d = q[s+1]-q[s]; g = d*fma(fma(beta, d, alpha), d, 1); p = fma(ck, g[s]-g[s-1], p)
 *   Toda    bond d; g = exp_scaled(alpha2*d) (= exp(2 alpha d)/(2 alpha)); p = fma(ck, g[s]-g[s-1], p)
 * Forces are the reference GPU's (DNKG_FPUT_Toda.cu:32-74, dDNKG.cu:17-19) written per bond. */
static void move_chain_device(const nlo_model *M, const consts *K, double *restrict q,
                              double *restrict p, double *restrict g, uint32_t batching) {
	const uint32_t n = M->n;
	const double beta = M->beta, alpha = M->alpha;
	for (uint32_t i = 0; i < batching; i++) {
		for (int k = 0; k < 7; k++) {
			const double cd = (i && !k) ? K->dtc0x2 : K->dtc[k];
			for (uint32_t s = 0; s < n; s++) q[s] = fma(cd, p[s], q[s]);
			const double ck = K->dtd[k];
			switch (M->model) {
				case NLO_DNKG:
				case NLO_DDNKG:
					for (uint32_t s = 0; s < n; s++) {
						double l = q[s ? s - 1 : n - 1], c = q[s], r = q[s + 1 < n ? s + 1 : 0];
						double mp2 = M->model == NLO_DDNKG ? M->mp2[s] : K->mp2;
						double bc = beta * c;
						double t = fma(bc, c, mp2);
						double u = fma(c, t, -l);
						double v = u - r;
						p[s] = fma(-ck, v, p[s]);
					}
					break;
				case NLO_FPUT:
					for (uint32_t s = 0; s < n; s++) {
						double d = q[s + 1 < n ? s + 1 : 0] - q[s];
						double h = fma(beta, d, alpha);
						double w = fma(h, d, 1.);
						g[s] = d * w;
					}
					for (uint32_t s = 0; s < n; s++) p[s] = fma(ck, g[s] - g[s ? s - 1 : n - 1], p[s]);
					break;
				case NLO_TODA:
					for (uint32_t s = 0; s < n; s++) {
						double d = q[s + 1 < n ? s + 1 : 0] - q[s];
						g[s] = nlo_exp_scaled(K->alpha2 * d, K->exptab);
					}
					for (uint32_t s = 0; s < n; s++) p[s] = fma(ck, g[s] - g[s ? s - 1 : n - 1], p[s]);
					break;
			}
		}
	}
	for (uint32_t s = 0; s < n; s++) q[s] = fma(K->dtc[7], p[s], q[s]);
}

/* ------------------------------------------------------------------------------------------------
 * FFT: mixed radix decimation in time, twiddles from one table of length n
 * ----------------------------------------------------------------------------------------------*/

static uint32_t smallest_factor(uint32_t n) {
	if (n % 4 == 0) return 4;
	if (n % 2 == 0) return 2;
	for (uint32_t f = 3; f * f <= n; f += 2)
		if (n % f == 0) return f;
	return n;
}

/* out[0..n) = DFT of in[0], in[stride], ... ; tw[e] = exp(sign 2 pi i e / ntop), ntop = n * twstride */
static void fft_rec(uint32_t n, const double *in, size_t stride, double *out, const double *tw,
                    size_t twstride, double *scratch) {
	if (n == 1) {
		out[0] = in[0], out[1] = in[1];
		return;
	}
	uint32_t pf = smallest_factor(n), m = n / pf;
	for (uint32_t r = 0; r < pf; r++) fft_rec(m, in + 2 * r * stride, stride * pf, out + 2 * r * m, tw, twstride * pf, scratch);
	/* combine: X[k + q m] = sum_r W_n^{r (k + q m)} Y_r[k] */
	double *y = scratch; /* pf complex values: column k is read completely before it is rewritten */
	for (uint32_t k = 0; k < m; k++) {
		for (uint32_t r = 0; r < pf; r++) {
			size_t e = (size_t) r * k % n * twstride;
			double wr = tw[2 * e], wi = tw[2 * e + 1];
			double ar = out[2 * (r * m + k)], ai = out[2 * (r * m + k) + 1];
			y[2 * r] = ar * wr - ai * wi;
			y[2 * r + 1] = ar * wi + ai * wr;
		}
		for (uint32_t qq = 0; qq < pf; qq++) {
			double sr = 0, si = 0;
			for (uint32_t r = 0; r < pf; r++) {
				size_t e = (size_t) r * qq % pf * m * twstride;
				double wr = tw[2 * e], wi = tw[2 * e + 1];
				sr += y[2 * r] * wr - y[2 * r + 1] * wi;
				si += y[2 * r] * wi + y[2 * r + 1] * wr;
			}
			out[2 * (k + qq * m)] = sr, out[2 * (k + qq * m) + 1] = si;
		}
	}
}

/* The sub-transforms read a strided copy of the input, so the top level runs out of place. */
static void fft_any(uint32_t n, double *z, int sign) {
	double *tw = malloc(sizeof(double) * 2 * n), *in = malloc(sizeof(double) * 2 * n),
	       *scr = malloc(sizeof(double) * 2 * n);
	for (uint32_t e = 0; e < n; e++) {
		double a = 2 * M_PI * e / n;
		tw[2 * e] = cos(a), tw[2 * e + 1] = sign * sin(a);
	}
	memcpy(in, z, sizeof(double) * 2 * n);
	fft_rec(n, in, 1, z, tw, 1, scr);
	free(tw), free(in), free(scr);
}

void nlo_fft(uint32_t n, double *z, int sign) {
	if (n <= 1) return;
	fft_any(n, z, sign);
}

void nlo_dispersion(int32_t model, uint32_t n, double m, double *omega) {
	for (uint32_t k = 0; k < n; k++) {
		double s2 = 2 * sin(k * M_PI / n);
		omega[k] = model == NLO_DNLS ? s2 * s2 : sqrt(m + s2 * s2);
	}
}

/* ------------------------------------------------------------------------------------------------
 * DNLS: split step, DNLS/cpu-implementation/DNLS.cpp:75-127 with sincos in place of the
 * |sin| = sqrt(1 - cos^2) shortcut of :85-95 (which loses accuracy at small angles)
 * ----------------------------------------------------------------------------------------------*/

static void dnls_nonlinear_sincos(uint32_t n, double *psi, double beta_dt_symplectic) {
	for (uint32_t s = 0; s < n; s++) {
		double r1 = psi[2 * s], i1 = psi[2 * s + 1];
		double norm = r1 * r1 + i1 * i1, angle = -beta_dt_symplectic * norm;
		double er = cos(angle), ei = sin(angle);
		psi[2 * s] = r1 * er - i1 * ei;
		psi[2 * s + 1] = ei * r1 + i1 * er;
	}
}

/* The reference CPU rotation itself (DNLS/cpu-implementation/DNLS.cpp:77-98): cos(angle), then
 * |sin| = sqrt(1 - cos^2) with the sign of sin recovered from the half-turn count of the angle.
 * Used by NLO_ORDER_REFERENCE to pin the oracle to the reference's CPU program; its sine is off by
 * up to eps / angle^2 relative at small angles, so the sincos form above is the checker. */
static void dnls_nonlinear_reference(uint32_t n, double *psi, double beta_dt_symplectic) {
	for (uint32_t s = 0; s < n; s++) {
		double r1 = psi[2 * s], i1 = psi[2 * s + 1];
		double norm = r1 * r1 + i1 * i1, angle = -beta_dt_symplectic * norm;
		double er = cos(angle), ei = sqrt(1 - er * er);
		int32_t invert_sign = (int32_t) (angle / M_PI) & 1;
		ei *= (1. - 2. * invert_sign) * copysign(1., angle);
		psi[2 * s] = r1 * er - i1 * ei;
		psi[2 * s + 1] = ei * r1 + i1 * er;
	}
}

static void dnls_tables(uint32_t n, double dt, double *tables /* [7][n][2] */) {
	double *omega = malloc(sizeof(double) * n);
	nlo_dispersion(NLO_DNLS, n, 0, omega);
	double normalization = 1. / n;
	for (int i = 0; i < 7; i++)
		for (uint32_t j = 0; j < n; j++) {
			/* exp(complex(0, -dt) * d_i * omega_j) / n  (DNLS/dispersion.cpp:19-26) */
			double im = (-dt * yoshida_d[i]) * omega[j];
			tables[2 * (i * n + j)] = cos(im) * normalization;
			tables[2 * (i * n + j) + 1] = sin(im) * normalization;
		}
	free(omega);
}

static void move_chain_dnls(const nlo_model *M, const double *tables, double *psi, uint32_t batching) {
	const uint32_t n = M->n;
	void (*const dnls_nonlinear)(uint32_t, double *, double) =
			M->order == NLO_ORDER_REFERENCE ? dnls_nonlinear_reference : dnls_nonlinear_sincos;
	for (uint32_t i = 0; i < batching; i++)
		for (int k = 0; k < 7; k++) {
			dnls_nonlinear(n, psi, M->beta * M->dt * (!k && i ? 2. : 1.) * yoshida_c[k]);
			nlo_fft(n, psi, -1);
			const double *t = tables + 2 * (size_t) k * n;
			for (uint32_t s = 0; s < n; s++) {
				double r1 = psi[2 * s], i1 = psi[2 * s + 1], r2 = t[2 * s], i2 = t[2 * s + 1];
				psi[2 * s] = r1 * r2 - i1 * i2;
				psi[2 * s + 1] = i2 * r1 + i1 * r2;
			}
			nlo_fft(n, psi, +1);
		}
	dnls_nonlinear(n, psi, M->beta * M->dt * yoshida_c[7]);
}

/* ------------------------------------------------------------------------------------------------
 * DNLS, the engine's stencil form (NLO_ORDER_STENCIL): each linear sub-step as the propagator's
 * real-space kernel exp(-2 i tau) i^|x| J_|x|(2 tau) (Jacobi-Anger), replayed operation for
 * operation from nlchains_gb300/csrc/nlc_dnls_stencil.cu, with the device's table sincos
 * (nlc_device.cuh sincos_table) and its table (nlc_tables.cpp sincos_table).
 * ----------------------------------------------------------------------------------------------*/

#define NLO_SINCOS_TABLE 1024

/* sin and cos of x in [0, pi/4] by their Taylor series in double-double */
static void dd_sincos_small(dd x, dd *s, dd *c) {
	const dd x2 = dd_mul(x, x);
	dd term = x;
	*s = x;
	for (unsigned k = 1; k < 40; k++) {
		term = dd_div_u(dd_mul(term, x2), (2 * k) * (2 * k + 1));
		term.hi = -term.hi, term.lo = -term.lo;
		*s = dd_add(*s, term);
		if (fabs(term.hi) < 1e-40) break;
	}
	term.hi = 1., term.lo = 0.;
	*c = term;
	for (unsigned k = 1; k < 40; k++) {
		term = dd_div_u(dd_mul(term, x2), (2 * k - 1) * (2 * k));
		term.hi = -term.hi, term.lo = -term.lo;
		*c = dd_add(*c, term);
		if (fabs(term.hi) < 1e-40) break;
	}
}

/* (cos, sin)(2 pi j / 1024): octant values m pi / 512, m = 0..128, then the quarter-turn symmetries */
static void sincos_table_1024(double *table /* [1024][2] */) {
	const unsigned Q = NLO_SINCOS_TABLE / 4, O = NLO_SINCOS_TABLE / 8;
	const dd pi = {3.141592653589793116, 1.2246467991473532072e-16};
	double cs[NLO_SINCOS_TABLE / 8 + 1], sn[NLO_SINCOS_TABLE / 8 + 1];
	for (unsigned m = 0; m <= O; m++) {
		dd s, c, mm = {(double) m, 0.};
		dd_sincos_small(dd_div_u(dd_mul(pi, mm), NLO_SINCOS_TABLE / 2), &s, &c);
		sn[m] = s.hi + s.lo, cs[m] = c.hi + c.lo;
	}
	for (unsigned j = 0; j < NLO_SINCOS_TABLE; j++) {
		const unsigned q = j / Q, jj = j % Q;
		const double c0 = jj <= O ? cs[jj] : sn[Q - jj], s0 = jj <= O ? sn[jj] : cs[Q - jj];
		table[2 * j] = q == 0 ? c0 : q == 1 ? -s0 : q == 2 ? -c0 : s0;
		table[2 * j + 1] = q == 0 ? s0 : q == 1 ? c0 : q == 2 ? -s0 : -c0;
	}
}

/* the device's sincos: Taylor series below 2^-4, the table method below 2^20, libm beyond */
static void sincos_device(double th, const double *tab, double *s, double *c) {
	int64_t b;
	memcpy(&b, &th, 8);
	const int32_t hi = (int32_t) (b >> 32) & 0x7fffffff;
	if (hi < 0x3fb00000) {
		const double t2 = th * th;
		const double ps = fma(t2, fma(t2, fma(t2, 1. / 362880, -1. / 5040), 1. / 120), -1. / 6);
		*s = fma(th * t2, ps, th);
		*c = fma(t2, fma(t2, fma(t2, fma(t2, 1. / 40320, -1. / 720), 1. / 24), -1. / 2), 1.);
		return;
	}
	if (hi >= 0x41300000) {
		*s = sin(th), *c = cos(th);
		return;
	}
	const double shifter = 0x1.8p52, inv = 512. / 3.141592653589793116;
	const double p1 = 3.141592653589793116 / 512, p2 = 1.2246467991473532072e-16 / 512;
	const double t = fma(th, inv, shifter);
	const double kd = t - shifter;
	const double r = fma(-kd, p2, fma(-kd, p1, th));
	int64_t tb;
	memcpy(&tb, &t, 8);
	const double *e = tab + 2 * ((uint32_t) tb & (NLO_SINCOS_TABLE - 1));
	const double r2 = r * r;
	const double sr = fma(r * r2, fma(r2, 1. / 120, -1. / 6), r);
	const double cm1 = r2 * fma(r2, 1. / 24, -1. / 2);
	*c = fma(e[0], cm1, fma(-e[1], sr, e[0]));
	*s = fma(e[1], cm1, fma(e[0], sr, e[1]));
}

/* psi exp(i (neg_coef |psi|^2 + neg_phase)) in the device's order */
static void rotate_device(double *v, double neg_coef, double neg_phase, const double *tab) {
	const double norm = fma(v[0], v[0], v[1] * v[1]);
	double s, c;
	sincos_device(fma(neg_coef, norm, neg_phase), tab, &s, &c);
	const double re = fma(v[0], c, -(v[1] * s)), im = fma(v[0], s, v[1] * c);
	v[0] = re, v[1] = im;
}

/* J_x(2t) = sum_m (-1)^m t^(2m + x) / (m! (m + x)!) in double-double; minus_one (x = 0): without
 * the leading 1 */
static dd bessel_j_2t(unsigned x, dd t, int minus_one) {
	const dd t2 = dd_mul(t, t);
	dd term = {1., 0.};
	for (unsigned i = 1; i <= x; i++) term = dd_div_u(dd_mul(term, t), i);
	unsigned m = 0;
	if (minus_one) {
		const dd mone = {-1., 0.};
		term = dd_mul(t2, mone);
		m = 1;
	}
	dd sum = {0., 0.};
	for (; m < 60; m++) {
		sum = dd_add(sum, term);
		term = dd_div_u(dd_mul(term, t2), (m + 1) * (m + 1 + x));
		term.hi = -term.hi, term.lo = -term.lo;
		if (fabs(term.hi) < 1e-40 * fabs(sum.hi) || term.hi == 0.) break;
	}
	return sum;
}

int nlo_dnls_stencil_coefficients(double dt, int max_radius, double *c0m1, double *taps, double *phase) {
	const double limit = 0x1p-64;
	int radius = 0;
	for (int k = 0; k < 7; k++) {
		const dd a = {dt, 0.}, d = {yoshida_d[k], 0.}, m2 = {-2., 0.};
		const dd tau = dd_mul(a, d);
		const dd c = bessel_j_2t(0, tau, 1);
		c0m1[k] = c.hi + c.lo;
		const dd ph = dd_mul(tau, m2);
		phase[k] = ph.hi + ph.lo;
		int r = 0;
		for (int x = 1; x <= max_radius + 1; x++) {
			const dd j = bessel_j_2t((unsigned) x, tau, 0);
			const double v = j.hi + j.lo;
			if (x <= max_radius) taps[k * max_radius + x - 1] = (x & 2) ? -v : v;
			if (fabs(v) > limit) r = x;
		}
		if (r > radius) radius = r;
	}
	return radius;
}

#define NLO_STENCIL_MAX 11

typedef struct {
	int radius;   /* the instantiated radius the engine runs: 7, or 11 */
	double c0m1[7], taps[7 * NLO_STENCIL_MAX], phase[7];
	double tab[2 * NLO_SINCOS_TABLE];
} stencil_consts;

/* 0 when the engine's stencil form does not apply to this dt (taps beyond radius 11) */
static int make_stencil(double dt, stencil_consts *S) {
	const int need = nlo_dnls_stencil_coefficients(dt, NLO_STENCIL_MAX, S->c0m1, S->taps, S->phase);
	S->radius = need <= 7 ? 7 : need <= NLO_STENCIL_MAX ? NLO_STENCIL_MAX : 0;
	sincos_table_1024(S->tab);
	return S->radius;
}

/* One launch of `batching` steps on one chain (psi: n interleaved complex), w: 2 n scratch */
static void move_chain_dnls_stencil(const nlo_model *M, const stencil_consts *S, double *psi, double *w,
                                    uint32_t batching) {
	const int64_t n = M->n;
	const int R = S->radius;
	const double bdt = M->beta * M->dt;
	for (uint32_t i = 0; i < batching; i++)
		for (int k = 0; k < 7; k++) {
			const double nc = -(k == 0 && i ? bdt * 2. * yoshida_c[0] : bdt * 1. * yoshida_c[k]);
			for (int64_t s = 0; s < n; s++) rotate_device(psi + 2 * s, nc, S->phase[k], S->tab);
			memcpy(w, psi, sizeof(double) * 2 * n);
			const double c0 = S->c0m1[k];
			const double *tp = S->taps + k * NLO_STENCIL_MAX;
			for (int64_t s = 0; s < n; s++) {
				const double *c = w + 2 * s;
				double yr = fma(c0, c[0], c[0]), yi = fma(c0, c[1], c[1]);
				for (int x = 1; x <= R; x++) {
					const double *a = w + 2 * ((s + x) % n), *b = w + 2 * ((s - x + n) % n);
					const double sr = a[0] + b[0], si = a[1] + b[1];
					if (x & 1) {
						yr = fma(-tp[x - 1], si, yr);
						yi = fma(tp[x - 1], sr, yi);
					} else {
						yr = fma(tp[x - 1], sr, yr);
						yi = fma(tp[x - 1], si, yi);
					}
				}
				psi[2 * s] = yr, psi[2 * s + 1] = yi;
			}
		}
	for (int64_t s = 0; s < n; s++) rotate_device(psi + 2 * s, -(bdt * yoshida_c[7]), 0., S->tab);
}

/* ------------------------------------------------------------------------------------------------
 * Driver
 * ----------------------------------------------------------------------------------------------*/

int nlo_advance(const nlo_model *M, double *state, uint64_t steps, uint32_t batching) {
	if (!M || !state || M->n < 2 || !batching || steps % batching) return -1;
	if (M->model == NLO_DDNKG && !M->mp2) return -1;
	const uint32_t n = M->n;
	consts *K = malloc(sizeof(consts));
	make_consts(M, K);
	double *tables = 0;
	stencil_consts *S = 0;
	if (M->model == NLO_DNLS && M->order == NLO_ORDER_STENCIL) {
		S = malloc(sizeof(stencil_consts));
		if (!make_stencil(M->dt, S) || n < (uint32_t) (2 * S->radius + 2)) {
			free(S), free(K);
			return -1;
		}
	} else if (M->model == NLO_DNLS) {
		tables = malloc(sizeof(double) * 2 * 7 * n);
		dnls_tables(n, M->dt, tables);
	}
	const int64_t copies = M->copies;
#ifdef _OPENMP
	int nthreads = M->threads > 0 ? M->threads : 1;
#pragma omp parallel num_threads(nthreads)
#endif
	{
		double *a = malloc(sizeof(double) * (n + 2)), *b = malloc(sizeof(double) * n),
		       *g = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * 2 * n),
		       *zw = malloc(sizeof(double) * 2 * n);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
		for (int64_t c = 0; c < copies; c++) {
			double *chain = state + 2 * (size_t) c * n;
			if (M->model == NLO_DNLS) {
				memcpy(z, chain, sizeof(double) * 2 * n);
				for (uint64_t t = 0; t < steps; t += batching)
					if (S) move_chain_dnls_stencil(M, S, z, zw, batching);
					else move_chain_dnls(M, tables, z, batching);
				memcpy(chain, z, sizeof(double) * 2 * n);
				continue;
			}
			if (M->order == NLO_ORDER_REFERENCE) {
				for (uint32_t s = 0; s < n; s++) a[s + 1] = chain[2 * s], b[s] = chain[2 * s + 1];
				for (uint64_t t = 0; t < steps; t += batching) move_chain_reference(M, K, a, b, batching);
				for (uint32_t s = 0; s < n; s++) chain[2 * s] = a[s + 1], chain[2 * s + 1] = b[s];
			} else {
				for (uint32_t s = 0; s < n; s++) a[s] = chain[2 * s], b[s] = chain[2 * s + 1];
				for (uint64_t t = 0; t < steps; t += batching) move_chain_device(M, K, a, b, g, batching);
				for (uint32_t s = 0; s < n; s++) chain[2 * s] = a[s], chain[2 * s + 1] = b[s];
			}
		}
		free(a), free(b), free(g), free(z), free(zw);
	}
	free(K);
	free(tables);
	free(S);
	return 0;
}

int nlo_linenergies(const nlo_model *M, const double *state, const double *eigvecs,
                    const double *omegas, double *out) {
	const uint32_t n = M->n;
	const uint64_t copies = M->copies;
	if (!M || !state || !out || n < 2 || !copies) return -1;
	for (uint32_t k = 0; k < n; k++) out[k] = 0;
	double *omega = malloc(sizeof(double) * n), *zphi = malloc(sizeof(double) * 2 * n),
	       *zpi = malloc(sizeof(double) * 2 * n);
	nlo_dispersion(M->model, n, M->m, omega);
	double norm;
	int a0is0;
	if (M->model == NLO_DDNKG) {
		if (!eigvecs || !omegas) return -1;
		/* dDNKG/cpu-implementation/dDNKG.cpp:201-213 */
		for (uint64_t c = 0; c < copies; c++) {
			const double *chain = state + 2 * c * n;
			const double *eigen = eigvecs;
			for (uint32_t i = 0; i < n; i++) {
				double dotphi = 0, dotpi = 0;
				for (uint32_t s = 0; s < n; s++, eigen++) dotphi += chain[2 * s] * *eigen, dotpi += chain[2 * s + 1] * *eigen;
				double od = omegas[i] * dotphi;
				out[i] += od * od + dotpi * dotpi;
			}
		}
		norm = 0.5 / copies;
		a0is0 = 0;
	} else if (M->model == NLO_DNLS) {
		/* DNLS.cu:70-81 */
		for (uint64_t c = 0; c < copies; c++) {
			memcpy(zphi, state + 2 * c * n, sizeof(double) * 2 * n);
			nlo_fft(n, zphi, -1);
			for (uint32_t k = 0; k < n; k++) out[k] += zphi[2 * k] * zphi[2 * k] + zphi[2 * k + 1] * zphi[2 * k + 1];
		}
		for (uint32_t k = 0; k < n; k++) out[k] *= omega[k];
		norm = 1. / ((double) copies * n);
		a0is0 = 1;
	} else {
		/* DNKG_FPUT_Toda.cu:304-321: expanded |omega Phi + i Pi|^2 */
		for (uint64_t c = 0; c < copies; c++) {
			const double *chain = state + 2 * c * n;
			for (uint32_t s = 0; s < n; s++) {
				zphi[2 * s] = chain[2 * s], zphi[2 * s + 1] = 0;
				zpi[2 * s] = chain[2 * s + 1], zpi[2 * s + 1] = 0;
			}
			nlo_fft(n, zphi, -1);
			nlo_fft(n, zpi, -1);
			for (uint32_t k = 0; k < n; k++) {
				double fx = zphi[2 * k], fy = zphi[2 * k + 1], px = zpi[2 * k], py = zpi[2 * k + 1];
				double energy = (fx * fx + fy * fy) * omega[k];
				energy += 2 * (fy * px - fx * py);
				energy *= omega[k];
				energy += px * px + py * py;
				out[k] += energy;
			}
		}
		norm = (0.5 / copies) / n;
		a0is0 = M->m == 0.;
	}
	/* results_entropy.cpp:11-19 */
	if (a0is0) out[0] = 0;
	for (uint32_t k = 0; k < n; k++) out[k] *= norm;
	free(omega), free(zphi), free(zpi);
	return 0;
}

int nlo_entropies(const double *e, uint32_t n, int a0is0, const uint8_t *mask, double *wt, double *inf) {
	double totale = 0, totalloge = 0, totaleloge = 0;
	uint32_t modes = 0;
	for (uint32_t k = 0; k < n; k++) {
		if (mask ? !mask[k] : 0) continue;
		if (a0is0 && k == 0) continue;
		double x = e[k], lx = log(x);
		totale += x, totalloge += lx, totaleloge += x * lx;
		modes++;
	}
	/* like results::calc_entropies, any mode count is accepted (the < 2 check is the mask's) */
	double normalization = modes / totale, lognormalization = log(normalization);
	*wt = -(totalloge + modes * lognormalization);
	*inf = normalization * (totaleloge + lognormalization * totale);
	return 0;
}

double nlo_energy(const nlo_model *M, const double *chain) {
	const uint32_t n = M->n;
	double h = 0;
	for (uint32_t s = 0; s < n; s++) {
		uint32_t s1 = s + 1 < n ? s + 1 : 0;
		if (M->model == NLO_DNLS) {
			double dr = chain[2 * s1] - chain[2 * s], di = chain[2 * s1 + 1] - chain[2 * s + 1];
			double a2 = chain[2 * s] * chain[2 * s] + chain[2 * s + 1] * chain[2 * s + 1];
			h += dr * dr + di * di + M->beta / 2 * a2 * a2;
			continue;
		}
		double q = chain[2 * s], p = chain[2 * s + 1], d = chain[2 * s1] - q;
		h += p * p / 2;
		switch (M->model) {
			case NLO_DNKG:
				h += d * d / 2 + M->m * q * q / 2 + M->beta * q * q * q * q / 4;
				break;
			case NLO_DDNKG:
				h += d * d / 2 + (M->mp2[s] - 2) * q * q / 2 + M->beta * q * q * q * q / 4;
				break;
			case NLO_FPUT:
				h += d * d / 2 + M->alpha * d * d * d / 3 + M->beta * d * d * d * d / 4;
				break;
			case NLO_TODA: {
				double a2 = 2 * M->alpha;
				h += (exp(a2 * d) - a2 * d - 1) / (4 * M->alpha * M->alpha);
				break;
			}
		}
	}
	return h;
}

/* Cyclic Jacobi with threshold on a symmetric column-major matrix `a` (overwritten), then ascending
 * sort (LAPACK dsyev order): eigenvalues in w, eigenvectors as the columns of v. */
int nlo_eig_sym(uint32_t n, double *a, double *w, double *v) {
#define A(i, j) a[(size_t) (j) * n + (i)]
#define V(i, j) v[(size_t) (j) * n + (i)]
	for (uint32_t i = 0; i < n; i++)
		for (uint32_t j = 0; j < n; j++) V(i, j) = i == j;
	for (int sweep = 0; sweep < 100; sweep++) {
		double off = 0, diag = 0;
		for (uint32_t j = 0; j < n; j++)
			for (uint32_t i = 0; i < n; i++) {
				if (i == j) diag += A(i, j) * A(i, j);
				else off += A(i, j) * A(i, j);
			}
		if (off <= 1e-34 * diag) break;
		for (uint32_t p = 0; p < n; p++)
			for (uint32_t q = p + 1; q < n; q++) {
				double apq = A(p, q);
				if (apq == 0) continue;
				double theta = (A(q, q) - A(p, p)) / (2 * apq);
				double t = (theta >= 0 ? 1. : -1.) / (fabs(theta) + sqrt(theta * theta + 1));
				double c = 1 / sqrt(t * t + 1), s = t * c;
				for (uint32_t k = 0; k < n; k++) {
					double akp = A(k, p), akq = A(k, q);
					A(k, p) = c * akp - s * akq;
					A(k, q) = s * akp + c * akq;
				}
				for (uint32_t k = 0; k < n; k++) {
					double apk = A(p, k), aqk = A(q, k);
					A(p, k) = c * apk - s * aqk;
					A(q, k) = s * apk + c * aqk;
				}
				for (uint32_t k = 0; k < n; k++) {
					double vkp = V(k, p), vkq = V(k, q);
					V(k, p) = c * vkp - s * vkq;
					V(k, q) = s * vkp + c * vkq;
				}
			}
	}
	/* selection sort ascending, moving eigenvector columns along */
	double *ev = malloc(sizeof(double) * n), *col = malloc(sizeof(double) * n);
	for (uint32_t i = 0; i < n; i++) ev[i] = A(i, i);
	for (uint32_t i = 0; i < n; i++) {
		uint32_t best = i;
		for (uint32_t j = i + 1; j < n; j++)
			if (ev[j] < ev[best]) best = j;
		if (best != i) {
			double te = ev[i];
			ev[i] = ev[best], ev[best] = te;
			memcpy(col, &V(0, i), sizeof(double) * n);
			memcpy(&V(0, i), &V(0, best), sizeof(double) * n);
			memcpy(&V(0, best), col, sizeof(double) * n);
		}
	}
	for (uint32_t i = 0; i < n; i++) w[i] = ev[i];
#undef A
#undef V
	free(ev), free(col);
	return 0;
}

/* eigensystem.cpp:13-22: the periodic operator diag(mp2) - shift(+-1), its eigenvectors, and
 * omegas = sqrt(eigenvalues). */
int nlo_eigensystem(uint32_t n, const double *mp2, double *omegas, double *v) {
	double *a = calloc((size_t) n * n, sizeof(double));
	if (!a) return -1;
	/* eigensystem.cpp:15-18: the corner entries are assigned, not added (n = 2 keeps -1) */
	for (uint32_t i = 0; i < n; i++) {
		a[(size_t) i * n + i] = mp2[i];
		uint32_t j = i + 1 < n ? i + 1 : 0;
		a[(size_t) j * n + i] = a[(size_t) i * n + j] = -1.;
	}
	int rc = nlo_eig_sym(n, a, omegas, v);
	for (uint32_t i = 0; !rc && i < n; i++) omegas[i] = sqrt(omegas[i]);
	free(a);
	return rc;
}
