/*
 * TEST INFRASTRUCTURE ONLY -- bodies of the third-party stand-ins (fftw3.h, armadillo) that let
 * the reference's CPU sources compile and run in place (oracle/build.py, build_ref_cpu).  Written
 * for this repository from the published definitions, not from FFTW's, LAPACK's or Armadillo's
 * code:
 *
 *   - the discrete Fourier transform by its definition, in long double: a radix-2 decimation in
 *     time (Cooley and Tukey, 1965) for power-of-two lengths, the direct sum otherwise, with the
 *     twiddles cos/sin(2 pi m / n) evaluated in long double;
 *   - the symmetric eigenproblem by cyclic Jacobi rotations (Jacobi 1846; Golub and Van Loan,
 *     "Matrix Computations", section 8.5), in long double, eigenvalues sorted ascending.
 *
 * Compiled with -DREF_SHIM_ORACLE_MATH, the transform and the eigensolver are the oracle's own
 * (nlo_fft, nlo_eig_sym) instead: the second build of the reference's program, in which the
 * third-party arithmetic rounds exactly as the oracle's does, so that everything else can be
 * compared bit for bit.
 */
#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "armadillo"
#include "fftw3.h"

namespace {

struct split_ptrs {
	double *ri, *ii, *ro, *io;
	int stride_in, stride_out;   /* in doubles between consecutive elements of one component */
};

#ifdef REF_SHIM_ORACLE_MATH
}  // namespace
extern "C" void nlo_fft(uint32_t n, double *z, int sign);
extern "C" int nlo_eig_sym(uint32_t n, double *a, double *w, double *v);
namespace {

/* The variant that hands every transform to the oracle's own FFT (nlo_fft), so that the
 * reference's program and the oracle round every transform identically and the rest of their
 * arithmetic can be compared bit for bit. */
void dft(int n, int sign, std::vector<long double> &re, std::vector<long double> &im) {
	std::vector<double> z(2 * size_t(n));
	for (int j = 0; j < n; j++) z[2 * j] = (double) re[j], z[2 * j + 1] = (double) im[j];
	nlo_fft((uint32_t) n, z.data(), sign);
	for (int j = 0; j < n; j++) re[j] = z[2 * j], im[j] = z[2 * j + 1];
}
#else
/* Forward (sign -1) or backward (sign +1) DFT of n complex numbers, long double throughout. */
void dft(int n, int sign, std::vector<long double> &re, std::vector<long double> &im) {
	const long double two_pi = 6.283185307179586476925286766559005768L;
	std::vector<long double> cw(n), sw(n);
	for (int m = 0; m < n; m++) {
		long double a = two_pi * (long double) m / (long double) n;
		cw[m] = cosl(a), sw[m] = sign * sinl(a);
	}
	if ((n & (n - 1)) == 0) {
		/* bit reversal, then log2(n) butterfly passes */
		for (int i = 1, j = 0; i < n; i++) {
			int bit = n >> 1;
			for (; j & bit; bit >>= 1) j ^= bit;
			j ^= bit;
			if (i < j) std::swap(re[i], re[j]), std::swap(im[i], im[j]);
		}
		for (int len = 2; len <= n; len <<= 1) {
			int step = n / len;
			for (int s = 0; s < n; s += len)
				for (int k = 0; k < len / 2; k++) {
					long double wr = cw[k * step], wi = sw[k * step];
					int a = s + k, b = s + k + len / 2;
					long double tr = re[b] * wr - im[b] * wi, ti = re[b] * wi + im[b] * wr;
					re[b] = re[a] - tr, im[b] = im[a] - ti;
					re[a] += tr, im[a] += ti;
				}
		}
		return;
	}
	std::vector<long double> outr(n), outi(n);
	for (int k = 0; k < n; k++) {
		long double sr = 0, si = 0;
		for (int j = 0; j < n; j++) {
			int m = (int) (((long long) j * k) % n);
			sr += re[j] * cw[m] - im[j] * sw[m];
			si += re[j] * sw[m] + im[j] * cw[m];
		}
		outr[k] = sr, outi[k] = si;
	}
	re.swap(outr), im.swap(outi);
}
#endif

}  // namespace

struct fftw_plan_s {
	int n, sign;
	bool split;
	fftw_complex *in, *out;   /* interleaved plans */
	split_ptrs sp;            /* split plans */
};

extern "C" {

fftw_complex *fftw_alloc_complex(size_t n) {
	void *p = nullptr;
	if (posix_memalign(&p, 64, sizeof(fftw_complex) * (n ? n : 1))) return nullptr;
	return static_cast<fftw_complex *>(p);
}

void fftw_free(void *p) { std::free(p); }

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned) {
	if (n < 1) return nullptr;
	auto *p = new fftw_plan_s();
	p->n = n, p->sign = sign, p->split = false, p->in = in, p->out = out;
	return p;
}

fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim *dims, int howmany_rank, const fftw_iodim *,
                                   double *ri, double *ii, double *ro, double *io, unsigned) {
	/* the reference plans one transform of rank 1 (DNLS/cpu-implementation/DNLS.cpp:58-61) */
	if (rank != 1 || howmany_rank != 0 || dims[0].n < 1) return nullptr;
	auto *p = new fftw_plan_s();
	p->n = dims[0].n, p->sign = FFTW_FORWARD, p->split = true;
	p->sp = split_ptrs{ri, ii, ro, io, dims[0].is, dims[0].os};
	return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
	std::vector<long double> re(p->n), im(p->n);
	for (int j = 0; j < p->n; j++) re[j] = in[j][0], im[j] = in[j][1];
	dft(p->n, p->sign, re, im);
	for (int k = 0; k < p->n; k++) out[k][0] = (double) re[k], out[k][1] = (double) im[k];
}

void fftw_execute(const fftw_plan p) {
	if (!p->split) {
		fftw_execute_dft(p, p->in, p->out);
		return;
	}
	const split_ptrs &s = p->sp;
	std::vector<long double> re(p->n), im(p->n);
	for (int j = 0; j < p->n; j++) re[j] = s.ri[j * s.stride_in], im[j] = s.ii[j * s.stride_in];
	dft(p->n, p->sign, re, im);
	for (int k = 0; k < p->n; k++) s.ro[k * s.stride_out] = (double) re[k], s.io[k * s.stride_out] = (double) im[k];
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

void fftw_cleanup(void) {}

void fftw_forget_wisdom(void) {}

int fftw_import_wisdom_from_string(const char *) { return 1; }

int fftw_import_wisdom_from_filename(const char *) { return 1; }

char *fftw_export_wisdom_to_string(void) {
	char *s = static_cast<char *>(std::malloc(1));
	if (s) s[0] = 0;
	return s;
}

}  // extern "C"

namespace arma {

bool eig_sym(Col &eigval, Mat &eigvec, const Mat &X) {
	const uword n = X.n_rows;
	if (n != X.n_cols || !n) return false;
#ifdef REF_SHIM_ORACLE_MATH
	{
		std::vector<double> a(X.d);
		eigval.resize(n);
		eigvec = Mat(n, n);
		return nlo_eig_sym((uint32_t) n, a.data(), eigval.memptr(), eigvec.memptr()) == 0;
	}
#endif
	std::vector<long double> a(n * n), v(n * n, 0.L);
	for (uword j = 0; j < n; j++)
		for (uword i = 0; i < n; i++) a[j * n + i] = (X(i, j) + X(j, i)) / 2;
	for (uword i = 0; i < n; i++) v[i * n + i] = 1;
	auto A = [&](uword i, uword j) -> long double & { return a[j * n + i]; };
	auto V = [&](uword i, uword j) -> long double & { return v[j * n + i]; };
	for (int sweep = 0; sweep < 60; sweep++) {
		long double off = 0, total = 0;
		for (uword j = 0; j < n; j++)
			for (uword i = 0; i < n; i++) {
				long double x = A(i, j) * A(i, j);
				total += x;
				if (i != j) off += x;
			}
		if (off <= 1e-40L * total) break;
		for (uword p = 0; p + 1 < n; p++)
			for (uword q = p + 1; q < n; q++) {
				long double apq = A(p, q);
				if (apq == 0) continue;
				long double theta = (A(q, q) - A(p, p)) / (2 * apq);
				long double t = (theta >= 0 ? 1.L : -1.L) / (fabsl(theta) + sqrtl(theta * theta + 1));
				long double c = 1 / sqrtl(t * t + 1), s = t * c;
				for (uword k = 0; k < n; k++) {
					long double akp = A(k, p), akq = A(k, q);
					A(k, p) = c * akp - s * akq, A(k, q) = s * akp + c * akq;
				}
				for (uword k = 0; k < n; k++) {
					long double apk = A(p, k), aqk = A(q, k);
					A(p, k) = c * apk - s * aqk, A(q, k) = s * apk + c * aqk;
				}
				for (uword k = 0; k < n; k++) {
					long double vkp = V(k, p), vkq = V(k, q);
					V(k, p) = c * vkp - s * vkq, V(k, q) = s * vkp + c * vkq;
				}
			}
	}
	std::vector<uword> order(n);
	std::iota(order.begin(), order.end(), 0);
	std::stable_sort(order.begin(), order.end(), [&](uword x, uword y) { return A(x, x) < A(y, y); });
	eigval.resize(n);
	eigvec = Mat(n, n);
	for (uword c = 0; c < n; c++) {
		eigval[c] = (double) A(order[c], order[c]);
		for (uword i = 0; i < n; i++) eigvec(i, c) = (double) V(i, order[c]);
	}
	return true;
}

}  // namespace arma
