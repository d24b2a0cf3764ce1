// dDNKG eigensystem on the host: the periodic operator A = diag(mp2) - S - S^T, S the cyclic shift
// (eigensystem.cpp:13-22), with ascending eigenvalues and orthonormal eigenvectors, what Armadillo's
// eig_sym (LAPACK's divide and conquer) returns there.
//
// From 64 sites: divide and conquer (Cuppen, Numer. Math. 36, 1981; the eigenvectors by Gu and
// Eisenstat, SIAM J. Matrix Anal. Appl. 16(1), 1995).  A bond of coupling b between sites x and y
// is b (e_x + e_y)(e_x + e_y)^T minus b on the two diagonal entries, so cutting two bonds of the
// ring leaves two open chains (symmetric tridiagonal matrices) plus two rank-one terms, and each
// chain is cut in the middle the same way down to 24 sites, solved there by the implicit QR
// iteration.  Merging a rank-one term costs one secular equation and one product of the
// eigenvector matrix with an m x m matrix, m the pairs that do not deflate.  The result is checked
// (residuals, norms, orthogonality) and the dense Householder + QR path below is the fallback; it
// also serves chains shorter than 64 sites.  NLC_HOST_EIGEN_QR=1 selects it at every length;
// NLC_HOST_EIGEN_DC_ONLY=1 turns the fallback off (a failed check is then an error).
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "nlc_host.h"

namespace nlc {
namespace {

// Fork-join pool for the O(n^3) loops of the eigensolver: the calling thread plus helpers, each
// call splits [0, count) into contiguous chunks, one per thread.
class Pool {
public:
	explicit Pool(unsigned threads) {
		for (unsigned t = 1; t < threads; t++) helpers_.emplace_back([this, t] { run(t); });
		size_ = threads;
	}
	~Pool() {
		{
			std::lock_guard<std::mutex> lk(mu_);
			stop_ = true;
			gen_++;
		}
		cv_.notify_all();
		for (auto &h : helpers_) h.join();
	}
	void parallel_for(size_t count, const std::function<void(size_t, size_t)> &fn) {
		if (size_ == 1 || count < 64) {
			fn(0, count);
			return;
		}
		{
			std::lock_guard<std::mutex> lk(mu_);
			fn_ = &fn, count_ = count, pending_ = size_ - 1;
			gen_++;
		}
		cv_.notify_all();
		chunk(0, fn, count);
		std::unique_lock<std::mutex> lk(mu_);
		done_.wait(lk, [&] { return pending_ == 0; });
	}

private:
	void chunk(unsigned t, const std::function<void(size_t, size_t)> &fn, size_t count) {
		const size_t b = count * t / size_, e = count * (t + 1) / size_;
		if (b < e) fn(b, e);
	}
	void run(unsigned t) {
		uint64_t seen = 0;
		for (;;) {
			const std::function<void(size_t, size_t)> *fn;
			size_t count;
			{
				std::unique_lock<std::mutex> lk(mu_);
				cv_.wait(lk, [&] { return gen_ != seen; });
				seen = gen_;
				if (stop_) return;
				fn = fn_, count = count_;
			}
			chunk(t, *fn, count);
			std::lock_guard<std::mutex> lk(mu_);
			if (--pending_ == 0) done_.notify_one();
		}
	}
	std::vector<std::thread> helpers_;
	unsigned size_ = 1;
	std::mutex mu_;
	std::condition_variable cv_, done_;
	const std::function<void(size_t, size_t)> *fn_ = nullptr;
	size_t count_ = 0;
	unsigned pending_ = 0;
	uint64_t gen_ = 0;
	bool stop_ = false;
};

constexpr double kEps = 2.220446049250313e-16;

// Implicit symmetric QR iteration with Wilkinson shifts (Golub and Van Loan, Matrix Computations,
// algorithm 8.3.3) on the tridiagonal (d[0..k), e[0..k-1)), deflating from the bottom.  The
// rotations of one sweep are recorded and then applied to the k columns of Z (rows x k,
// column-major), by row blocks in parallel when a pool is given.  On return d holds the
// eigenvalues, unsorted; false if it does not converge.
bool tridiag_qr(double *d, double *e, size_t k, double *Z, size_t rows, Pool *pool) {
	std::vector<double> rc(k), rs(k);
	size_t iter = 0, hi = k - 1;
	while (hi > 0) {
		if (std::fabs(e[hi - 1]) <= kEps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) {
			e[hi - 1] = 0.;
			hi--;
			continue;
		}
		size_t lo = hi - 1;
		while (lo > 0 && std::fabs(e[lo - 1]) > kEps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) lo--;
		if (++iter > 60 * k) return false;
		const double delta = (d[hi - 1] - d[hi]) / 2, b2 = e[hi - 1] * e[hi - 1];
		const double den = delta + (delta >= 0 ? 1. : -1.) * std::hypot(delta, e[hi - 1]);
		const double mu = den != 0. ? d[hi] - b2 / den : d[hi] - std::fabs(e[hi - 1]);
		double x = d[lo] - mu, z = e[lo];
		for (size_t j = lo; j < hi; j++) {
			const double r = std::hypot(x, z);
			const double c = r != 0. ? x / r : 1., s = r != 0. ? z / r : 0.;
			if (j > lo) e[j - 1] = r;
			// rotate rows/cols j, j+1 of the tridiagonal: T' = P T P^T, P = [c s; -s c]
			const double aj = d[j], aj1 = d[j + 1], bj = e[j];
			d[j] = c * c * aj + 2 * c * s * bj + s * s * aj1;
			d[j + 1] = s * s * aj - 2 * c * s * bj + c * c * aj1;
			e[j] = c * s * (aj1 - aj) + (c * c - s * s) * bj;
			if (j + 1 < hi) {
				z = s * e[j + 1];        // bulge T(j, j+2)
				e[j + 1] = c * e[j + 1];
				x = e[j];
			}
			rc[j] = c, rs[j] = s;
		}
		// Z <- Z P^T on columns (j, j+1), j = lo .. hi-1 in order
		auto apply = [&](size_t b, size_t e2) {
			for (size_t j = lo; j < hi; j++) {
				const double c = rc[j], s = rs[j];
				double *zj = &Z[j * rows], *zj1 = &Z[(j + 1) * rows];
				for (size_t i = b; i < e2; i++) {
					const double x0 = zj[i], x1 = zj1[i];
					zj[i] = c * x0 + s * x1;
					zj1[i] = -s * x0 + c * x1;
				}
			}
		};
		if (pool)
			pool->parallel_for(rows, apply);
		else
			apply(0, rows);
	}
	return true;
}

// Sort the eigenpairs (w[k], columns of V: rows x k) by ascending eigenvalue.
void sort_pairs(std::vector<double> &w, std::vector<double> &V, size_t rows) {
	const size_t k = w.size();
	std::vector<size_t> idx(k);
	std::iota(idx.begin(), idx.end(), size_t(0));
	std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return w[a] < w[b]; });
	std::vector<double> w2(k), V2(rows * k);
	for (size_t j = 0; j < k; j++) {
		w2[j] = w[idx[j]];
		std::memcpy(&V2[j * rows], &V[idx[j] * rows], rows * sizeof(double));
	}
	w.swap(w2);
	V.swap(V2);
}

// The dense path for short chains and as the fallback: Householder tridiagonalisation of the
// periodic operator (Golub and Van Loan, algorithm 8.3.1) with the reflections accumulated into Q,
// then the QR iteration above.
bool eigensystem_periodic_qr(const std::vector<double> &mp2, std::vector<double> &omegas, std::vector<double> &eigvec) {
	const size_t n = mp2.size();
	if (n < 2) return false;
	Pool pool(n >= 512 ? host_setup_threads() : 1);
	// dense symmetric matrix, column-major A[j*n + i]
	std::vector<double> A(n * n, 0.), Q(n * n, 0.);
	auto a = [&](size_t i, size_t j) -> double & { return A[j * n + i]; };
	auto q = [&](size_t i, size_t j) -> double & { return Q[j * n + i]; };
	for (size_t i = 0; i < n; i++) {
		a(i, i) = mp2[i];
		const size_t j = (i + 1) % n;
		a(i, j) = a(j, i) = -1.;   // assignment: for n = 2 the corner entry stays -1 (eigensystem.cpp:16-18)
		q(i, i) = 1.;
	}
	// Householder tridiagonalisation: for column k, reflect x = A[k+1:, k] onto alpha e_1.
	std::vector<double> v(n), p(n), w(n);
	for (size_t k = 0; k + 2 < n; k++) {
		double norm2 = 0.;
		for (size_t i = k + 1; i < n; i++) norm2 += a(i, k) * a(i, k);
		const double norm = std::sqrt(norm2);
		if (norm == 0.) continue;
		const double x0 = a(k + 1, k);
		const double alpha = x0 > 0 ? -norm : norm;
		// v = x - alpha e1, normalised
		std::fill(v.begin(), v.end(), 0.);
		for (size_t i = k + 1; i < n; i++) v[i] = a(i, k);
		v[k + 1] -= alpha;
		double vn2 = 0.;
		for (size_t i = k + 1; i < n; i++) vn2 += v[i] * v[i];
		if (vn2 == 0.) continue;
		const double vinv = 1. / std::sqrt(vn2);
		for (size_t i = k + 1; i < n; i++) v[i] *= vinv;
		// p = A v over the trailing block; A is symmetric, so p[i] = sum_j A(j, i) v[j] reads column i
		pool.parallel_for(n - k, [&](size_t b, size_t e) {
			for (size_t i = k + b; i < k + e; i++) {
				const double *col = &A[i * n];
				double s = 0.;
				for (size_t j = k + 1; j < n; j++) s += col[j] * v[j];
				p[i] = s;
			}
		});
		double K = 0.;
		for (size_t i = k + 1; i < n; i++) K += v[i] * p[i];
		// A <- A - v w^T - w v^T with w = 2 (p - K v)
		for (size_t i = k; i < n; i++) w[i] = 2. * (p[i] - K * v[i]);
		pool.parallel_for(n - k, [&](size_t b, size_t e) {
			for (size_t j = k + b; j < k + e; j++) {
				double *col = &A[j * n];
				const double vj = v[j], wj = w[j];
				for (size_t i = k; i < n; i++) col[i] -= v[i] * wj + w[i] * vj;
			}
		});
		// exact zeros below the subdiagonal of column k
		a(k + 1, k) = a(k, k + 1) = alpha;
		for (size_t i = k + 2; i < n; i++) a(i, k) = a(k, i) = 0.;
		// Q <- Q H, H = I - 2 v v^T: s = Q v (rows in parallel), then a rank-1 update (columns)
		pool.parallel_for(n, [&](size_t b, size_t e) {
			for (size_t i = b; i < e; i++) p[i] = 0.;
			for (size_t j = k + 1; j < n; j++) {
				const double *col = &Q[j * n];
				const double vj = v[j];
				for (size_t i = b; i < e; i++) p[i] += col[i] * vj;
			}
		});
		pool.parallel_for(n - k - 1, [&](size_t b, size_t e) {
			for (size_t j = k + 1 + b; j < k + 1 + e; j++) {
				double *col = &Q[j * n];
				const double vj2 = 2. * v[j];
				for (size_t i = 0; i < n; i++) col[i] -= p[i] * vj2;
			}
		});
	}
	std::vector<double> d(n), e(n, 0.);
	for (size_t i = 0; i < n; i++) d[i] = a(i, i);
	for (size_t i = 0; i + 1 < n; i++) e[i] = a(i + 1, i);

	if (!tridiag_qr(d.data(), e.data(), n, Q.data(), n, &pool)) return false;
	sort_pairs(d, Q, n);
	omegas.assign(n, 0.);
	for (size_t k = 0; k < n; k++) omegas[k] = std::sqrt(d[k]);
	eigvec.swap(Q);
	return true;
}

// C[r, j] = sum_{l in [l0, l1)} col[l][r] U[l + j m] for the rows r in [r0, r1) and every j < m (C
// column-major with k rows).  The rows' slice of the columns is first packed into tiles of 12 rows
// (contiguous in l, so that the product reads one stream instead of one page per column); then
// register tiles of 12 rows x 4 columns, with the columns of U in panels of 64 that stay in cache
// while the row tiles pass over them.
void product_rows(const double *const *col, const double *U, size_t m, size_t l0, size_t l1, double *C, size_t k,
                  size_t r0, size_t r1) {
	constexpr size_t kR = 12, kC = 4, kPanel = 64;
	const size_t nl = l1 - l0, tiles = (r1 - r0 + kR - 1) / kR;
	std::vector<double> pack(tiles * nl * kR, 0.);
	for (size_t t = 0; t < tiles; t++) {
		const size_t rb = r0 + t * kR, nr = std::min(kR, r1 - rb);
		double *dst = &pack[t * nl * kR];
		for (size_t l = 0; l < nl; l++) {
			const double *a = col[l0 + l] + rb;
			for (size_t r = 0; r < nr; r++) dst[l * kR + r] = a[r];
		}
	}
	for (size_t jb = 0; jb < m; jb += kPanel) {
		const size_t je = std::min(m, jb + kPanel);
		for (size_t t = 0; t < tiles; t++) {
			const size_t rb = r0 + t * kR, nr = std::min(kR, r1 - rb);
			const double *ap = &pack[t * nl * kR];
			for (size_t j = jb; j < je; j += kC) {
				const size_t nc = std::min(kC, je - j);
				double acc[kC][kR] = {};
				if (nc == kC) {
					const double *u0 = U + j * m + l0, *u1 = u0 + m, *u2 = u1 + m, *u3 = u2 + m;
					for (size_t l = 0; l < nl; l++) {
						const double *a = ap + l * kR;
						const double x0 = u0[l], x1 = u1[l], x2 = u2[l], x3 = u3[l];
						for (size_t r = 0; r < kR; r++) {
							acc[0][r] += a[r] * x0;
							acc[1][r] += a[r] * x1;
							acc[2][r] += a[r] * x2;
							acc[3][r] += a[r] * x3;
						}
					}
				} else {
					for (size_t l = 0; l < nl; l++) {
						const double *a = ap + l * kR;
						for (size_t c = 0; c < nc; c++) {
							const double x = U[(j + c) * m + l0 + l];
							for (size_t r = 0; r < kR; r++) acc[c][r] += a[r] * x;
						}
					}
				}
				for (size_t c = 0; c < nc; c++) std::memcpy(C + (j + c) * k + rb, acc[c], nr * sizeof(double));
			}
		}
	}
}

// Rank-one update of an eigen-decomposition (Cuppen; Gu and Eisenstat): V (k x k, column-major)
// holds orthonormal eigenvectors of a symmetric M with eigenvalues w (any order).  On return (w, V)
// is the ascending eigen-decomposition of M + rho u u^T, u = V z.
//   1. Work with s M, s = sign(rho), so that the update is positive; sort the poles d = s w.
//   2. Deflation (as LAPACK's dlaed2): a component with r |z_i| <= tol keeps its pair; two poles
//      closer than tol / |c s| are rotated so that one component of z vanishes.
//   3. The secular equation 1 + r sum z_i^2 / (d_i - lambda) = 0 has one root in each gap of the
//      remaining poles and one above the last.  Each root is found as lambda = d_o + tau with the
//      origin d_o the nearer end of its gap, by Newton's method kept inside a shrinking bracket,
//      until the step or the bracket is at rounding level or the secular function is zero within
//      its own rounding error; every lambda - d_i = (d_o - d_i) + tau keeps full relative accuracy.
//   4. z is recomputed from the roots by Loewner's formula (Gu and Eisenstat), which makes the
//      eigenvectors (D - lambda_j)^-1 z numerically orthogonal, and V <- V U.  When V is block
//      diagonal over rows [0, split) and [split, k) (a merge of two halves), a column that is zero
//      in one block skips it in the product (as LAPACK's dlaed3), halving the work.
bool rank_one_update(std::vector<double> &w, std::vector<double> &V, const std::vector<double> &z, double rho,
                     size_t split, Pool &pool) {
	const size_t k = w.size();
	double zn2 = 0.;
	for (double v : z) zn2 += v * v;
	if (rho == 0. || zn2 == 0.) {
		sort_pairs(w, V, k);
		return true;
	}
	const double sgn = rho > 0 ? 1. : -1.;
	const double r = std::fabs(rho) * zn2, zn = std::sqrt(zn2);
	// 1. position i holds the pole d[i] and the column ord[i] of V
	std::vector<size_t> ord(k);
	std::iota(ord.begin(), ord.end(), size_t(0));
	std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return sgn * w[a] < sgn * w[b]; });
	std::vector<double> d(k), zz(k);
	double dmax = 0.;
	for (size_t i = 0; i < k; i++) {
		d[i] = sgn * w[ord[i]];
		zz[i] = z[ord[i]] / zn;
		dmax = std::max(dmax, std::fabs(d[i]));
	}
	const double tol = 8. * kEps * std::max(dmax, r);

	// 2. deflation
	std::vector<size_t> K;
	K.reserve(k);
	long pj = -1;
	for (size_t i = 0; i < k; i++) {
		if (r * std::fabs(zz[i]) <= tol) {
			zz[i] = 0.;
			continue;
		}
		if (pj >= 0) {
			const double t = std::hypot(zz[pj], zz[i]);
			const double c = zz[i] / t, s = zz[pj] / t;
			if (std::fabs((d[i] - d[pj]) * c * s) <= tol) {
				// G = [c -s; s c] on (pj, i): z_pj -> 0, z_i -> t; V <- V G^T
				const double dp = d[pj], di = d[i];
				d[pj] = c * c * dp + s * s * di;
				d[i] = s * s * dp + c * c * di;
				zz[pj] = 0., zz[i] = t;
				double *qp = &V[ord[pj] * k], *qi = &V[ord[i] * k];
				for (size_t x = 0; x < k; x++) {
					const double a = qp[x], b = qi[x];
					qp[x] = c * a - s * b;
					qi[x] = s * a + c * b;
				}
				pj = long(i);
				continue;
			}
			K.push_back(size_t(pj));
		}
		pj = long(i);
	}
	if (pj >= 0) K.push_back(size_t(pj));
	const size_t m = K.size();

	// 3. the secular equation over the m remaining poles
	std::vector<double> dk(m), zk(m), z2(m), tau(m);
	std::vector<size_t> org(m);
	double zsum = 0.;
	for (size_t j = 0; j < m; j++) {
		dk[j] = d[K[j]], zk[j] = zz[K[j]], z2[j] = zk[j] * zk[j];
		zsum += z2[j];
	}
	std::vector<char> found(m, 1);
	pool.parallel_for(m, [&](size_t b, size_t e) {
		std::vector<double> delta(m);
		for (size_t j = b; j < e; j++) {
			size_t o;
			double lo, hi;
			if (j + 1 < m) {
				const double half = (dk[j + 1] - dk[j]) / 2;
				double f = 1.;
				for (size_t i = 0; i < m; i++) f += r * z2[i] / ((dk[i] - dk[j]) - half);
				if (f >= 0.)
					o = j, lo = 0., hi = half;
				else
					o = j + 1, lo = -half, hi = 0.;
			} else {
				o = m - 1, lo = 0., hi = r * zsum;
			}
			for (size_t i = 0; i < m; i++) delta[i] = dk[i] - dk[o];
			double t = (lo + hi) / 2;
			bool done = false;
			for (int it = 0; it < 400 && !done; it++) {
				double f = 1., fp = 0., fabs_sum = 1.;
				for (size_t i = 0; i < m; i++) {
					const double q = 1. / (delta[i] - t), v = r * z2[i] * q;
					f += v, fp += v * q, fabs_sum += std::fabs(v);
				}
				// f is zero within its own rounding error (its terms can be large and cancel)
				if (std::fabs(f) <= 16. * kEps * fabs_sum) {
					done = true;
					break;
				}
				if (f > 0.)
					hi = t;
				else
					lo = t;
				double tn = t - f / fp;
				if (!(tn > lo && tn < hi)) tn = (lo + hi) / 2;
				done = std::fabs(tn - t) <= 2. * kEps * std::fabs(tn) ||
				       hi - lo <= 2. * kEps * std::max(std::fabs(lo), std::fabs(hi));
				t = tn;
			}
			// a root that converged on the last iteration counts; only an exhausted search fails
			if (!done) found[j] = 0;
			org[j] = o, tau[j] = t;
		}
	});
	for (char f : found)
		if (!f) return false;

	// 4. Loewner's z and the eigenvectors of D + r z z^T; the poles reordered for the product as
	// [zero below split | dense | zero above split]
	std::vector<size_t> top, dense, bottom;
	for (size_t i = 0; i < m; i++) {
		const double *v = &V[ord[K[i]] * k];
		bool up = false, down = false;
		for (size_t x = 0; x < split && !up; x++) up = v[x] != 0.;
		for (size_t x = split; x < k && !down; x++) down = v[x] != 0.;
		(up && down ? dense : up ? top : bottom).push_back(i);
	}
	std::vector<size_t> perm;   // product order -> pole
	perm.reserve(m);
	perm.insert(perm.end(), top.begin(), top.end());
	perm.insert(perm.end(), dense.begin(), dense.end());
	perm.insert(perm.end(), bottom.begin(), bottom.end());
	std::vector<const double *> col(m);
	for (size_t l = 0; l < m; l++) col[l] = &V[ord[K[perm[l]]] * k];

	auto gap = [&](size_t j, size_t i) { return (dk[org[j]] - dk[i]) + tau[j]; };   // lambda_j - d_i
	std::vector<double> zh(m), U(m * m);
	pool.parallel_for(m, [&](size_t b, size_t e) {
		for (size_t i = b; i < e; i++) {
			double p = gap(m - 1, i) / r;
			for (size_t j = 0; j < i; j++) p *= gap(j, i) / (dk[j] - dk[i]);
			for (size_t j = i; j + 1 < m; j++) p *= gap(j, i) / (dk[j + 1] - dk[i]);
			zh[i] = std::copysign(std::sqrt(std::max(p, 0.)), zk[i]);
		}
	});
	pool.parallel_for(m, [&](size_t b, size_t e) {
		for (size_t j = b; j < e; j++) {
			double *u = &U[j * m], nrm = 0.;
			for (size_t l = 0; l < m; l++) {
				const size_t i = perm[l];
				u[l] = -zh[i] / gap(j, i);
				nrm += u[l] * u[l];
			}
			nrm = 1. / std::sqrt(nrm);
			for (size_t l = 0; l < m; l++) u[l] *= nrm;
		}
	});
	std::vector<double> C(k * m);
	const size_t upper = top.size() + dense.size(), lower0 = top.size();
	pool.parallel_for(k, [&](size_t b, size_t e) {
		if (b < split) product_rows(col.data(), U.data(), m, 0, upper, C.data(), k, b, std::min(e, split));
		if (e > split) product_rows(col.data(), U.data(), m, lower0, m, C.data(), k, std::max(b, split), e);
	});

	// every pair, back in the eigenvalues of M + rho u u^T, ascending
	std::vector<char> in_k(k, 0);
	for (size_t j = 0; j < m; j++) in_k[K[j]] = 1;
	std::vector<double> val;
	std::vector<const double *> src;
	val.reserve(k), src.reserve(k);
	for (size_t i = 0; i < k; i++)
		if (!in_k[i]) val.push_back(sgn * d[i]), src.push_back(&V[ord[i] * k]);
	for (size_t j = 0; j < m; j++) val.push_back(sgn * (dk[org[j]] + tau[j])), src.push_back(&C[j * k]);
	std::vector<size_t> idx(k);
	std::iota(idx.begin(), idx.end(), size_t(0));
	std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return val[a] < val[b]; });
	std::vector<double> w2(k), V2(k * k);
	pool.parallel_for(k, [&](size_t b, size_t e) {
		for (size_t j = b; j < e; j++) {
			w2[j] = val[idx[j]];
			std::memcpy(&V2[j * k], src[idx[j]], k * sizeof(double));
		}
	});
	w.swap(w2);
	V.swap(V2);
	return true;
}

// (w, V) of diag(M1, M2) from the halves' decompositions (w1, V1: m1 x m1) and (w2, V2: m2 x m2).
void block_diag(const std::vector<double> &w1, const std::vector<double> &V1, const std::vector<double> &w2,
                const std::vector<double> &V2, std::vector<double> &w, std::vector<double> &V) {
	const size_t m1 = w1.size(), m2 = w2.size(), k = m1 + m2;
	w.assign(k, 0.);
	V.assign(k * k, 0.);
	for (size_t j = 0; j < m1; j++) {
		w[j] = w1[j];
		std::memcpy(&V[j * k], &V1[j * m1], m1 * sizeof(double));
	}
	for (size_t j = 0; j < m2; j++) {
		w[m1 + j] = w2[j];
		std::memcpy(&V[(m1 + j) * k + m1], &V2[j * m2], m2 * sizeof(double));
	}
}

// A bond of coupling rho between x and y, rho (e_x + e_y)(e_x + e_y)^T, added to (w, V); split as
// in rank_one_update (k where V has no block structure).
bool add_bond(std::vector<double> &w, std::vector<double> &V, size_t x, size_t y, double rho, size_t split,
              Pool &pool) {
	const size_t k = w.size();
	std::vector<double> z(k);
	for (size_t j = 0; j < k; j++) z[j] = V[j * k + x] + V[j * k + y];
	return rank_one_update(w, V, z, rho, split, pool);
}

// Ascending eigen-decomposition of the symmetric tridiagonal (d[0..k), e[0..k-1)): Cuppen's split
// at the middle bond b = e[m-1], T = diag(T1 - b e_last e_last^T, T2 - b e_0 e_0^T)
// + b (e_{m-1} + e_m)(e_{m-1} + e_m)^T, each half solved the same way down to 24 rows (QR).
constexpr size_t kLeaf = 24;

bool tridiag_dc(const double *d, const double *e, size_t k, std::vector<double> &w, std::vector<double> &V,
                Pool &pool) {
	if (k <= kLeaf) {
		std::vector<double> dd(d, d + k), ee(k, 0.);
		for (size_t i = 0; i + 1 < k; i++) ee[i] = e[i];
		V.assign(k * k, 0.);
		for (size_t i = 0; i < k; i++) V[i * k + i] = 1.;
		if (!tridiag_qr(dd.data(), ee.data(), k, V.data(), k, nullptr)) return false;
		w = dd;
		sort_pairs(w, V, k);
		return true;
	}
	const size_t m = k / 2;
	const double b = e[m - 1];
	std::vector<double> d1(d, d + m), d2(d + m, d + k);
	d1[m - 1] -= b, d2[0] -= b;
	std::vector<double> w1, V1, w2, V2;
	if (!tridiag_dc(d1.data(), e, m, w1, V1, pool) || !tridiag_dc(d2.data(), e + m, k - m, w2, V2, pool))
		return false;
	block_diag(w1, V1, w2, V2, w, V);
	return add_bond(w, V, m - 1, m, b, m, pool);
}

// The eigenpairs of the periodic operator satisfy A v = w v to rounding and V is orthogonal:
// residual of every pair, unit norms, and |V^T x| = |x| for two fixed vectors x.
bool check_periodic(const std::vector<double> &mp2, const std::vector<double> &w, const std::vector<double> &V,
                    Pool &pool) {
	const size_t n = mp2.size();
	double anorm = 0.;
	for (double v : mp2) anorm = std::max(anorm, std::fabs(v) + 2.);
	std::vector<char> bad(n, 0);
	std::vector<double> x1(n), x2(n), y1(n), y2(n);
	for (size_t i = 0; i < n; i++) x1[i] = std::sin(0.7 * double(i) + 0.3), x2[i] = 1. / (1. + double(i));
	pool.parallel_for(n, [&](size_t b, size_t e) {
		for (size_t j = b; j < e; j++) {
			const double *v = &V[j * n];
			double res = 0., nrm = 0., p1 = 0., p2 = 0.;
			for (size_t s = 0; s < n; s++) {
				const double av = mp2[s] * v[s] - v[s ? s - 1 : n - 1] - v[s + 1 < n ? s + 1 : 0];
				res = std::max(res, std::fabs(av - w[j] * v[s]));
				nrm += v[s] * v[s], p1 += v[s] * x1[s], p2 += v[s] * x2[s];
			}
			y1[j] = p1, y2[j] = p2;
			bad[j] = !(res <= 1e-10 * anorm) || !(std::fabs(nrm - 1.) <= 1e-10);
		}
	});
	for (char f : bad)
		if (f) return false;
	double a1 = 0., a2 = 0., b1 = 0., b2 = 0.;
	for (size_t i = 0; i < n; i++) a1 += x1[i] * x1[i], a2 += x2[i] * x2[i], b1 += y1[i] * y1[i], b2 += y2[i] * y2[i];
	return std::fabs(b1 - a1) <= 1e-10 * a1 && std::fabs(b2 - a2) <= 1e-10 * a2;
}

// The ring cut into the open paths [0, m) and [m, n) at the bonds (m-1, m) and (n-1, 0), each
// solved by divide and conquer; the two bonds (coupling -1) added back as rank-one updates, their
// diagonal part taken from the paths' diagonals.
bool eigensystem_periodic_dc(const std::vector<double> &mp2, std::vector<double> &omegas,
                             std::vector<double> &eigvec) {
	const size_t n = mp2.size();
	if (n < 3) return false;
	Pool pool(n >= 256 ? host_setup_threads() : 1);
	const size_t m = n / 2;
	std::vector<double> d(mp2), e(n, -1.);
	d[m - 1] += 1., d[m] += 1., d[n - 1] += 1., d[0] += 1.;
	std::vector<double> w1, V1, w2, V2, w, V;
	if (!tridiag_dc(d.data(), e.data(), m, w1, V1, pool) ||
	    !tridiag_dc(d.data() + m, e.data() + m, n - m, w2, V2, pool))
		return false;
	block_diag(w1, V1, w2, V2, w, V);
	if (!add_bond(w, V, m - 1, m, -1., m, pool) || !add_bond(w, V, n - 1, 0, -1., n, pool)) return false;
	if (!check_periodic(mp2, w, V, pool)) return false;
	omegas.assign(n, 0.);
	for (size_t k = 0; k < n; k++) omegas[k] = std::sqrt(w[k]);
	eigvec.swap(V);
	return true;
}

constexpr size_t kDcMinSites = 64;

}  // namespace

bool eigensystem_periodic(const std::vector<double> &mp2, std::vector<double> &omegas, std::vector<double> &eigvec) {
	const size_t n = mp2.size();
	if (n < 2) return false;
	auto flag = [](const char *name) {
		const char *v = std::getenv(name);
		return v && *v && *v != '0';
	};
	if (n >= kDcMinSites && !flag("NLC_HOST_EIGEN_QR")) {
		if (eigensystem_periodic_dc(mp2, omegas, eigvec)) return true;
		if (flag("NLC_HOST_EIGEN_DC_ONLY")) return false;   // tests: no silent fallback
	}
	return eigensystem_periodic_qr(mp2, omegas, eigvec);
}

}  // namespace nlc
