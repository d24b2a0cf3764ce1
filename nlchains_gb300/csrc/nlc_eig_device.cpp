// dDNKG eigensystem on the GPU: the symmetric eigenproblem of the periodic operator
// diag(mp2) - shift(+-1) (eigensystem.cpp:13-22) solved by cuSOLVER's divide-and-conquer
// cusolverDnDsyevd (LAPACK's dsyevd algorithm, the family of Armadillo's eig_sym that the reference
// calls).  A set-up step, not the hot path: the host solver (nlc_eig_host.cpp) costs O(n^3) on the
// CPU, and a dDNKG plan of 1024 sites is made in ~70 ms with this one.
//
// cuSOLVER is loaded at run time (dlopen), so the library has no link dependency on it: where it is
// missing, or any step fails, the caller keeps the host solver.
#include <dlfcn.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>
#include <cusolverDn.h>

#include "nlc_host.h"

namespace nlc {
namespace {

struct Cusolver {
	bool loaded = false, tried = false;
	cusolverStatus_t (*create)(cusolverDnHandle_t *) = nullptr;
	cusolverStatus_t (*destroy)(cusolverDnHandle_t) = nullptr;
	cusolverStatus_t (*set_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
	cusolverStatus_t (*buffer_size)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, const double *, int,
	                                const double *, int *) = nullptr;
	cusolverStatus_t (*syevd)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, double *, int, double *,
	                          double *, int, int *) = nullptr;
};

std::mutex g_mu;
Cusolver g_cs;
// one handle per device, created on first use (its start-up is most of a small solve's time) and
// used by one solve at a time
constexpr int kMaxDevices = 64;
std::mutex g_solve_mu;
cusolverDnHandle_t g_handle[kMaxDevices] = {};

const Cusolver *cusolver() {
	std::lock_guard<std::mutex> lk(g_mu);
	if (g_cs.tried) return g_cs.loaded ? &g_cs : nullptr;
	g_cs.tried = true;
	void *h = nullptr;
	for (const char *name : {"libcusolver.so.12", "libcusolver.so.11", "libcusolver.so"})
		if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
	if (!h) return nullptr;
	g_cs.create = reinterpret_cast<decltype(g_cs.create)>(dlsym(h, "cusolverDnCreate"));
	g_cs.destroy = reinterpret_cast<decltype(g_cs.destroy)>(dlsym(h, "cusolverDnDestroy"));
	g_cs.set_stream = reinterpret_cast<decltype(g_cs.set_stream)>(dlsym(h, "cusolverDnSetStream"));
	g_cs.buffer_size = reinterpret_cast<decltype(g_cs.buffer_size)>(dlsym(h, "cusolverDnDsyevd_bufferSize"));
	g_cs.syevd = reinterpret_cast<decltype(g_cs.syevd)>(dlsym(h, "cusolverDnDsyevd"));
	g_cs.loaded = g_cs.create && g_cs.destroy && g_cs.set_stream && g_cs.buffer_size && g_cs.syevd;
	return g_cs.loaded ? &g_cs : nullptr;
}

thread_local bool t_eigen_on_host = false;

}  // namespace

void set_eigen_on_host(bool host) { t_eigen_on_host = host; }

bool eigensystem_periodic_device(const std::vector<double> &mp2, std::vector<double> &omegas,
                                 std::vector<double> &eigvec) {
	const size_t n = mp2.size();
	if (n < 3 || t_eigen_on_host) return false;   // the n = 2 corner rule is the host solver's
	if (const char *e = std::getenv("NLC_HOST_EIGEN"); e && *e && *e != '0') return false;
	const Cusolver *cs = cusolver();
	if (!cs) return false;
	// the dense operator, column-major (symmetric: the layout does not matter)
	std::vector<double> A(n * n, 0.);
	for (size_t i = 0; i < n; i++) {
		A[i * n + i] = mp2[i];
		const size_t j = (i + 1) % n;
		A[j * n + i] = A[i * n + j] = -1.;
	}
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return false;
	std::lock_guard<std::mutex> lk(g_solve_mu);
	if (!g_handle[dev] && cs->create(&g_handle[dev]) != CUSOLVER_STATUS_SUCCESS) {
		g_handle[dev] = nullptr;
		return false;
	}
	cusolverDnHandle_t handle = g_handle[dev];
	cudaStream_t st = nullptr;
	double *d_a = nullptr, *d_w = nullptr, *d_work = nullptr;
	int *d_info = nullptr;
	bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
	          cs->set_stream(handle, st) == CUSOLVER_STATUS_SUCCESS &&
	          cudaMallocAsync(&d_a, n * n * sizeof(double), st) == cudaSuccess &&
	          cudaMallocAsync(&d_w, n * sizeof(double), st) == cudaSuccess &&
	          cudaMallocAsync(&d_info, sizeof(int), st) == cudaSuccess &&
	          cudaMemcpyAsync(d_a, A.data(), n * n * sizeof(double), cudaMemcpyHostToDevice, st) == cudaSuccess;
	int lwork = 0, info = -1;
	ok = ok && cs->buffer_size(handle, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, int(n), d_a, int(n), d_w,
	                           &lwork) == CUSOLVER_STATUS_SUCCESS;
	ok = ok && cudaMallocAsync(&d_work, size_t(std::max(lwork, 1)) * sizeof(double), st) == cudaSuccess;
	ok = ok && cs->syevd(handle, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, int(n), d_a, int(n), d_w, d_work,
	                     lwork, d_info) == CUSOLVER_STATUS_SUCCESS;
	std::vector<double> w(n);
	ok = ok && cudaMemcpyAsync(A.data(), d_a, n * n * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
	     cudaMemcpyAsync(w.data(), d_w, n * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
	     cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
	     cudaStreamSynchronize(st) == cudaSuccess && info == 0;
	if (st) {
		cudaFreeAsync(d_a, st), cudaFreeAsync(d_w, st), cudaFreeAsync(d_info, st), cudaFreeAsync(d_work, st);
		cudaStreamSynchronize(st);
		cudaStreamDestroy(st);
	}
	if (!ok) {
		cudaGetLastError();
		return false;
	}
	// ascending eigenvalues, eigenvector k in column k: the host solver's (and eig_sym's) layout
	omegas.assign(n, 0.);
	for (size_t k = 0; k < n; k++) {
		if (!(w[k] >= 0.)) return false;
		omegas[k] = std::sqrt(w[k]);
	}
	eigvec.swap(A);
	return true;
}

}  // namespace nlc
