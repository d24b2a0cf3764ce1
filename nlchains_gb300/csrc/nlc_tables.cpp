// Host-side constant tables of the engine: exp table, dispersion, FFT radices and twiddles (the
// dDNKG eigensystem is in nlc_eig_host.cpp).  Compiled with -ffp-contract=off so that every
// rounding is the one written here on both x86-64 and aarch64 hosts.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <thread>

#include "nlc_host.h"

namespace nlc {

const double kYoshidaC[8] = {0.392256805238780, 0.510043411918458, -0.471053385409757, 0.068753168252518,
                             0.068753168252518, -0.471053385409757, 0.510043411918458, 0.392256805238780};
const double kYoshidaD[8] = {0.784513610477560, 0.235573213359357, -1.177679984178870, 1.315186320683906,
                             -1.177679984178870, 0.235573213359357, 0.784513610477560, 0};

namespace {

struct DD {
	double hi, lo;
};

DD renorm(double hi, double lo) {
	const double s = hi + lo;
	return {s, lo - (s - hi)};
}

DD dd_add(DD a, DD b) {
	const double s = a.hi + b.hi, bb = s - a.hi, e = (a.hi - (s - bb)) + (b.hi - bb);
	return renorm(s, e + a.lo + b.lo);
}

DD dd_mul(DD a, DD b) {
	const double p = a.hi * b.hi;
	double e = std::fma(a.hi, b.hi, -p);
	e += a.hi * b.lo + a.lo * b.hi;
	return renorm(p, e);
}

DD dd_div_u(DD a, unsigned k) {
	const double q1 = a.hi / k;
	const double p = q1 * k, pe = std::fma(q1, (double) k, -p);
	const double rem = ((a.hi - p) - pe) + a.lo;
	return renorm(q1, rem / k);
}

DD dd_exp_small(DD y) {
	DD sum{1., 0.}, term{1., 0.};
	for (unsigned k = 1; k < 40; k++) {
		term = dd_div_u(dd_mul(term, y), k);
		sum = dd_add(sum, term);
		if (std::fabs(term.hi) < 1e-40) break;
	}
	return sum;
}

// sin and cos of x in [0, pi/4] by their Taylor series in double-double
void dd_sincos_small(DD x, DD &s, DD &c) {
	const DD x2 = dd_mul(x, x);
	DD term = x;
	s = x;
	for (unsigned k = 1; k < 40; k++) {   // term_k = (-1)^k x^(2k+1) / (2k+1)!
		term = dd_div_u(dd_mul(term, x2), (2 * k) * (2 * k + 1));
		term = {-term.hi, -term.lo};
		s = dd_add(s, term);
		if (std::fabs(term.hi) < 1e-40) break;
	}
	term = {1., 0.};
	c = term;
	for (unsigned k = 1; k < 40; k++) {   // (-1)^k x^(2k) / (2k)!
		term = dd_div_u(dd_mul(term, x2), (2 * k - 1) * (2 * k));
		term = {-term.hi, -term.lo};
		c = dd_add(c, term);
		if (std::fabs(term.hi) < 1e-40) break;
	}
}

}  // namespace

void sincos_table(double table[2 * kSinCosTable]) {
	// octant values m pi/512, m = 0..128, then quarter-turn symmetries (exact sign and swap)
	constexpr unsigned Q = kSinCosTable / 4, O = kSinCosTable / 8;
	const DD pi{3.141592653589793116, 1.2246467991473532072e-16};
	double cs[O + 1], sn[O + 1];
	for (unsigned m = 0; m <= O; m++) {
		DD s, c;
		dd_sincos_small(dd_div_u(dd_mul(pi, DD{double(m), 0.}), kSinCosTable / 2), s, c);
		sn[m] = s.hi + s.lo, cs[m] = c.hi + c.lo;
	}
	for (unsigned j = 0; j < unsigned(kSinCosTable); j++) {
		const unsigned q = j / Q, jj = j % Q;
		const double c0 = jj <= O ? cs[jj] : sn[Q - jj], s0 = jj <= O ? sn[jj] : cs[Q - jj];
		const double c = q == 0 ? c0 : q == 1 ? -s0 : q == 2 ? -c0 : s0;
		const double s = q == 0 ? s0 : q == 1 ? c0 : q == 2 ? -s0 : -c0;
		table[2 * j] = c, table[2 * j + 1] = s;
	}
}

namespace {

// J_x(2t) = sum_m (-1)^m t^(2m + x) / (m! (m + x)!) in double-double (|t| well below 1 here); with
// minus_one and x = 0 the series without its leading 1, i.e. J_0(2t) - 1 to full relative precision
DD bessel_j_2t(unsigned x, DD t, bool minus_one) {
	const DD t2 = dd_mul(t, t);
	DD term{1., 0.};
	for (unsigned i = 1; i <= x; i++) term = dd_div_u(dd_mul(term, t), i);   // t^x / x!
	unsigned m = 0;
	if (minus_one) {   // start at m = 1: -t^2
		term = dd_mul(t2, DD{-1., 0.});
		m = 1;
	}
	DD sum{0., 0.};
	for (; m < 60; m++) {
		sum = dd_add(sum, term);
		term = dd_div_u(dd_mul(term, t2), (m + 1) * (m + 1 + x));
		term = {-term.hi, -term.lo};
		if (std::fabs(term.hi) < 1e-40 * std::fabs(sum.hi) || term.hi == 0.) break;
	}
	return sum;
}

}  // namespace

int dnls_stencil_coefficients(double dt, int max_radius, double c0m1[7], double *taps, double phase[7]) {
	const double limit = 0x1p-64;
	int radius = 0;
	for (int k = 0; k < 7; k++) {
		const DD tau = dd_mul(DD{dt, 0.}, DD{kYoshidaD[k], 0.});
		const DD c = bessel_j_2t(0, tau, true);
		c0m1[k] = c.hi + c.lo;
		const DD ph = dd_mul(tau, DD{-2., 0.});
		phase[k] = ph.hi + ph.lo;
		int r = 0;
		for (int x = 1; x <= max_radius + 1; x++) {
			const DD j = bessel_j_2t(unsigned(x), tau, false);
			const double v = j.hi + j.lo;
			if (x <= max_radius) taps[k * max_radius + x - 1] = (x & 2) ? -v : v;   // the sign of i^x
			if (std::fabs(v) > limit) r = x;
		}
		radius = std::max(radius, r);
	}
	return radius;
}

void exp_table(double scale, double table[kExpTable]) {
	const DD ln2{0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
	for (unsigned j = 0; j < unsigned(kExpTable); j++) {
		DD v = dd_exp_small(dd_mul(ln2, DD{double(j) / kExpTable, 0.}));
		v = dd_mul(v, DD{scale, 0.});
		table[j] = v.hi + v.lo;
	}
}

std::vector<double> dispersion_real(uint32_t n, double m) {
	std::vector<double> omega(n);
	for (uint32_t k = 0; k < n; k++) {
		const double s2 = 2 * std::sin(k * M_PI / n);
		omega[k] = std::sqrt(m + s2 * s2);
	}
	return omega;
}

std::vector<double> dispersion_dnls(uint32_t n) {
	std::vector<double> omega(n);
	for (uint32_t k = 0; k < n; k++) {
		const double s2 = 2 * std::sin(k * M_PI / n);
		omega[k] = s2 * s2;
	}
	return omega;
}

std::vector<int> fft_radices(uint32_t n) {
	std::vector<int> r;
	if (n < 2) return r;
	while (n % 4 == 0) r.push_back(4), n /= 4;
	while (n % 2 == 0) r.push_back(2), n /= 2;
	for (uint32_t f = 3; f * f <= n; f += 2)
		while (n % f == 0) r.push_back(int(f)), n /= f;
	if (n > 1) r.push_back(int(n));
	return r;
}

std::vector<double> fft_twiddles(uint32_t n) {
	std::vector<double> tw(2 * size_t(n));
	for (uint32_t e = 0; e < n; e++) {
		const double a = 2 * M_PI * e / n;
		tw[2 * e] = std::cos(a);
		tw[2 * e + 1] = -std::sin(a);
	}
	return tw;
}

void fft_fma_twiddles(const std::vector<int> &radices, std::vector<double> &gw, std::vector<int> &off) {
	gw.clear();
	off.assign(radices.size(), 0);
	uint64_t ns = 1;
	for (size_t r = 0; r < radices.size(); r++) {
		const int p = radices[r];
		off[r] = int(gw.size() / 2);
		const int per = fma_twiddle_double2s(p);
		if (ns > 1 && per) {
			const uint64_t span = ns * uint64_t(p);
			for (uint64_t k = 0; k < ns; k++) {
				double c[4] = {1., 1., 1., 1.}, s[4] = {0., 0., 0., 0.}, e[6];
				for (int u = 1; u < p; u++) {
					// theta_u = 2 pi (u k mod span) / span, the argument reduced exactly
					const double a = 2 * M_PI * double((uint64_t(u) * k) % span) / double(span);
					c[u] = std::cos(a), s[u] = std::sin(a);
				}
				fma_twiddle_entry(p, c, s, e);
				gw.insert(gw.end(), e, e + 2 * per);
			}
		}
		ns *= uint64_t(p);
	}
}


namespace {

uint32_t largest_prime_factor(uint32_t n) {
	uint32_t p = 1;
	for (uint32_t f = 2; f * f <= n; f++)
		while (n % f == 0) p = f, n /= f;
	return n > 1 ? std::max(p, n) : p;
}

// FP64 operations per element of one Stockham pass of radix r (nlc_fft.cuh): the radix-4 butterfly
// (16 for the additions and 12 for three twiddle products per 4 points), radix 2, 3 and 5, and the
// direct p-point DFT of any other radix (4p for the sums plus a twiddle product)
double pass_cost(int r) {
	switch (r) {
		case 4: return 22. / 4;
		case 2: return 6. / 2;
		case 3: return 16. / 3;
		case 5: return 52. / 5;
		default: return 4. * r;
	}
}

// The length in [x, max_len] of the form 2^a 3^b 5^c 7^d whose transform takes the fewest FP64
// operations (length x sum of pass costs), not merely the smallest: 384 = 4^3 2 3 costs less than
// 360 = 4 2 3^2 5.  0 when there is none.
uint32_t cheapest_length(uint32_t x, uint32_t max_len) {
	uint32_t best = 0;
	double best_cost = 0;
	for (uint64_t a = 1; a <= max_len; a *= 2)
		for (uint64_t b = a; b <= max_len; b *= 3)
			for (uint64_t c = b; c <= max_len; c *= 5)
				for (uint64_t d = c; d <= max_len; d *= 7) {
					if (d < x) continue;
					double cost = 0;
					for (int r : fft_radices(uint32_t(d))) cost += pass_cost(r);
					cost *= double(d);
					if (!best || cost < best_cost) best = uint32_t(d), best_cost = cost;
				}
	return best;
}

// in-place recursive mixed-radix DFT (sign -1 forward), for host table set-up only
void host_dft(std::vector<std::complex<double>> &z, int sign) {
	const size_t n = z.size();
	if (n <= 1) return;
	size_t p = 2;
	while (n % p) p++;
	if (p == n) {
		std::vector<std::complex<double>> w(n), out(n);
		for (size_t e = 0; e < n; e++) w[e] = std::polar(1., sign * 2 * M_PI * double(e) / n);
		for (size_t k = 0; k < n; k++) {
			std::complex<double> acc = 0;
			for (size_t j = 0, e = 0; j < n; j++, e = e + k < n ? e + k : e + k - n) acc += z[j] * w[e];
			out[k] = acc;
		}
		z = out;
		return;
	}
	const size_t m = n / p;
	std::vector<std::vector<std::complex<double>>> sub(p, std::vector<std::complex<double>>(m));
	for (size_t r = 0; r < p; r++) {
		for (size_t j = 0; j < m; j++) sub[r][j] = z[j * p + r];
		host_dft(sub[r], sign);
	}
	for (size_t k = 0; k < n; k++) {
		std::complex<double> acc = 0;
		for (size_t r = 0; r < p; r++) acc += sub[r][k % m] * std::polar(1., sign * 2 * M_PI * double(r * k % n) / n);
		z[k] = acc;
	}
}

}  // namespace

// host_dft for any length: lengths with a prime factor above 7 through Bluestein's identity on a
// 2^a 3^b 5^c length >= 2n - 1 (O(n log n) instead of the O(n^2) direct prime pass)
void host_fft_any(std::vector<std::complex<double>> &z, int sign) {
	const uint32_t n = uint32_t(z.size());
	if (n < 2 || largest_prime_factor(n) <= 7) return host_dft(z, sign);
	uint32_t m = 1u << 31;
	for (uint64_t a = 1; a < 4ull * n; a *= 2)
		for (uint64_t b = a; b < 4ull * n; b *= 3)
			for (uint64_t c = b; c < 4ull * n; c *= 5)
				if (c >= 2ull * n - 1 && c < m) m = uint32_t(c);
	std::vector<std::complex<double>> w(n), a(m, 0.), b(m, 0.);
	for (uint32_t j = 0; j < n; j++) {
		const double ang = M_PI * double((uint64_t(j) * j) % (2ull * n)) / n;
		w[j] = std::polar(1., sign * ang);   // exp(sign i pi j^2 / n)
		a[j] = z[j] * w[j];
		b[j] = std::conj(w[j]);
		if (j) b[m - j] = b[j];
	}
	host_dft(a, -1);
	host_dft(b, -1);
	for (uint32_t k = 0; k < m; k++) a[k] *= b[k] / double(m);
	host_dft(a, +1);
	for (uint32_t k = 0; k < n; k++) z[k] = w[k] * a[k];
}

std::vector<double> dnls_conv_tables(const std::vector<double> &lin, uint32_t n, uint32_t m) {
	std::vector<double> out(2 * 7 * size_t(m));
	for (int k = 0; k < 7; k++) {
		std::vector<std::complex<double>> h(n), g(m, 0.);
		for (uint32_t q = 0; q < n; q++) h[q] = {lin[2 * (k * size_t(n) + q)], lin[2 * (k * size_t(n) + q) + 1]};
		host_fft_any(h, +1);   // h[t] = sum_q L_k[q] exp(+2 pi i q t / n): the propagator's kernel in site space
		for (uint32_t t = 0; t < n; t++) g[t] = h[t];
		for (uint32_t t = 1; t < n; t++) g[m - t] = h[n - t];   // g[-t mod m] = h[-t mod n]
		host_dft(g, -1);
		for (uint32_t j = 0; j < m; j++) {
			out[2 * (k * size_t(m) + j)] = g[j].real() / m;
			out[2 * (k * size_t(m) + j) + 1] = g[j].imag() / m;
		}
	}
	return out;
}

FftTables fft_tables(uint32_t n, uint32_t smem_len, uint32_t max_len, bool convolution) {
	FftTables T;
	T.n = n;
	T.len = n;
	if (n >= 2 && largest_prime_factor(n) > 5) {
		// FP64 operations of the direct form against the padded form of length m; a transform whose
		// two buffers do not fit shared memory (len > smem_len) runs from global memory at about half
		// the rate.  DNLS (convolution): two passes of n and the propagator product, or two passes of
		// m, the kernel product and the zero padding.  Diagnostics: one pass of n, or Bluestein's two
		// passes of m with the kernel and chirp products.
		auto cost = [](uint32_t len) {
			double c = 0;
			for (int r : fft_radices(len)) c += pass_cost(r);
			return c * len;
		};
		auto slow = [&](uint32_t len) { return len > smem_len ? 2. : 1.; };
		const uint32_t m = cheapest_length(2 * n - 1, max_len);
		if (m) {
			const double direct = convolution ? (2 * cost(n) + 4. * n) * slow(n) : cost(n) * slow(n);
			const double padded = convolution ? (2 * cost(m) + 6. * m) * slow(m) : (2 * cost(m) + 4. * m + 8. * n) * slow(m);
			if (padded < direct) T.bluestein = true, T.len = m;
		}
	}
	T.radices = fft_radices(T.len);
	T.tw = fft_twiddles(T.len);
	fft_fma_twiddles(T.radices, T.gw, T.gw_off);
	if (!T.bluestein) return T;
	const uint32_t m = T.len;
	T.chirp.resize(2 * size_t(n));
	std::vector<std::complex<double>> b(m, 0.), bc(m, 0.);
	for (uint32_t j = 0; j < n; j++) {
		// exp(-i pi j^2 / n) with j^2 reduced mod 2n exactly
		const double ang = M_PI * double((uint64_t(j) * j) % (2ull * n)) / n;
		T.chirp[2 * j] = std::cos(ang), T.chirp[2 * j + 1] = -std::sin(ang);
		const std::complex<double> bj(std::cos(ang), std::sin(ang));   // exp(+i pi j^2 / n)
		b[j] = bj, bc[j] = std::conj(bj);
		if (j) b[m - j] = bj, bc[m - j] = std::conj(bj);
	}
	host_dft(b, -1);
	host_dft(bc, -1);
	T.bf.resize(2 * size_t(m));
	T.bi.resize(2 * size_t(m));
	for (uint32_t k = 0; k < m; k++) {
		T.bf[2 * k] = b[k].real() / m, T.bf[2 * k + 1] = b[k].imag() / m;
		T.bi[2 * k] = bc[k].real() / m, T.bi[2 * k + 1] = bc[k].imag() / m;
	}
	return T;
}

namespace {
thread_local unsigned t_host_threads = 0;
}

void set_host_setup_threads(unsigned threads) { t_host_threads = threads; }

unsigned host_setup_threads() {
	if (t_host_threads) return t_host_threads;
	unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
	if (const char *e = std::getenv("NLC_HOST_THREADS"); e && std::atoi(e) > 0) hw = unsigned(std::atoi(e));
	return hw;
}

}  // namespace nlc
