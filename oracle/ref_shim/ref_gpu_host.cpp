/*
 * TEST INFRASTRUCTURE ONLY -- launches the reference's own GPU kernels (compiled unmodified from the
 * reference's sources into oracle/_ref/ref_gpu_n<N>.fatbin by oracle/build.py) on ensembles that
 * the tests and the bench's plain-reference line hand over as device pointers.  The host logic
 * restates the reference's drivers, which cannot be compiled where the fatbin runs:
 *
 *   refgpu_advance      move<model> (DNKG_FPUT_Toda/DNKG_FPUT_Toda.cu:254-289) and dDNKG::move
 *                       (dDNKG/dDNKG.cu:199-234): the thread kernel below 32 sites, the warp kernel
 *                       at the optimised length, otherwise plane2split (common/utilities_cuda.cu:
 *                       213-248) and move_split; constants as DNKG_FPUT_Toda.cpp:76-84 and
 *                       dDNKG.cpp:56-60,94-97 upload them;
 *   refgpu_linenergies  the real-model FFT preparation (DNKG_FPUT_Toda.cpp:68-73,113-122) with cuFFT
 *                       and make_linenergies_kernel; the dDNKG projection (dDNKG.cpp:61-69,118-141)
 *                       with two cublasDgemm and the warp-reduce kernel; the DNLS forward transform
 *                       and make_linenergies_kernel (DNLS.cpp:142-150); normalised as
 *                       results::calc_linenergies does (results_entropy.cpp:11-19);
 *   refgpu_dnls_advance the DNLS split step without cuFFT callbacks (DNLS.cpp:159-175 with
 *                       --no_linear_callback --no_nonlinear_callback), tables as
 *                       DNLS/dispersion.cpp:10-26 build them.
 *
 * Kernels are found by their demangled names in the loaded module (cuModuleEnumerateFunctions), the
 * reference's __constant__ symbols by their mangled names (cuModuleGetGlobal).  Every launch is
 * checked against the reference's own limits (16-bit copy counts, 2^30 sites) before it is made.
 */
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <cxxabi.h>
#include <map>
#include <string>
#include <vector>

#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

namespace {

enum { M_DNKG = 0, M_FPUT = 1, M_TODA = 2, M_DDNKG = 3, M_DNLS = 4 };

}  // namespace

struct refgpu {
	CUmodule mod = nullptr;
	int n_opt = 0;
	double c[8], d[8];
	std::map<std::string, CUfunction> kernels;   /* demangled name without a leading "void " */
	cublasHandle_t cublas = nullptr;
	std::map<std::pair<uint32_t, uint32_t>, cufftHandle> dnls_plans;   /* (n, copies): as DNLS.cpp:73-126 keeps them */
	std::map<std::pair<uint32_t, double>, double2 *> dnls_tables;      /* (n, dt): the 7 linear tables */
	std::string err;
};

namespace {

int fail(refgpu *r, const std::string &msg) {
	r->err = msg;
	return -1;
}

bool cu_ok(refgpu *r, CUresult e, const char *what) {
	if (e == CUDA_SUCCESS) return true;
	const char *s = nullptr;
	cuGetErrorString(e, &s);
	r->err = std::string(what) + ": " + (s ? s : "CUDA driver error");
	return false;
}

bool rt_ok(refgpu *r, cudaError_t e, const char *what) {
	if (e == cudaSuccess) return true;
	r->err = std::string(what) + ": " + cudaGetErrorString(e);
	return false;
}

CUfunction find_kernel(refgpu *r, const std::string &prefix) {
	CUfunction hit = nullptr;
	for (auto &kv: r->kernels)
		if (kv.first.compare(0, prefix.size(), prefix) == 0) {
			if (hit) {
				r->err = "ambiguous kernel name prefix " + prefix;
				return nullptr;
			}
			hit = kv.second;
		}
	if (!hit) {
		r->err = "no kernel " + prefix + " in the reference module; it has:";
		int shown = 0;
		for (auto &kv: r->kernels)
			if (shown++ < 40) r->err += "\n  " + kv.first;
	}
	return hit;
}

bool set_global(refgpu *r, const char *mangled, const void *src, size_t bytes) {
	CUdeviceptr p = 0;
	size_t size = 0;
	if (!cu_ok(r, cuModuleGetGlobal(&p, &size, r->mod, mangled), mangled)) return false;
	if (bytes > size) {
		r->err = std::string("reference symbol ") + mangled + " is smaller than the value written";
		return false;
	}
	return cu_ok(r, cuMemcpyHtoD(p, src, bytes), mangled);
}

bool launch(refgpu *r, CUfunction f, unsigned blocks, unsigned threads, cudaStream_t s, void **args) {
	if (!blocks) return true;
	return cu_ok(r, cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, 0, (CUstream) s, args, nullptr), "cuLaunchKernel");
}

unsigned grid_for(uint64_t elements, unsigned threads) { return unsigned((elements + threads - 1) / threads); }

/* plane2split::split / plane (common/utilities_cuda.cu:219-248): planar double2[copies][n] <->
 * transposed double2[n][copies] by cublasZgeam, then split_kernel / unsplit_kernel between that and
 * the double[n][copies] phi and pi arrays.  beta = 0: the B operand is not read; it is given as the
 * output itself (cuBLAS's in-place form) instead of a null pointer. */
bool split(refgpu *r, cudaStream_t s, double2 *planar, double2 *transposed, double *phi, double *pi, uint32_t n,
           uint32_t copies) {
	cuDoubleComplex one{1., 0.}, zero{0., 0.};
	if (cublasSetStream(r->cublas, s) != CUBLAS_STATUS_SUCCESS ||
	    cublasZgeam(r->cublas, CUBLAS_OP_T, CUBLAS_OP_N, (int) copies, (int) n, &one, (cuDoubleComplex *) planar, (int) n,
	                &zero, (cuDoubleComplex *) transposed, (int) copies, (cuDoubleComplex *) transposed, (int) copies) !=
	    CUBLAS_STATUS_SUCCESS)
		return fail(r, "cublasZgeam (split)"), false;
	CUfunction k = find_kernel(r, "split_kernel(");
	if (!k) return false;
	uint32_t elements = n * copies;
	void *args[] = {&elements, &transposed, &phi, &pi};
	return launch(r, k, grid_for(elements, 256), 256, s, args);
}

bool plane(refgpu *r, cudaStream_t s, double2 *planar, double2 *transposed, double *phi, double *pi, uint32_t n,
           uint32_t copies) {
	CUfunction k = find_kernel(r, "unsplit_kernel(");
	if (!k) return false;
	uint32_t elements = n * copies;
	const double *cphi = phi, *cpi = pi;
	void *args[] = {&elements, &cphi, &cpi, &transposed};
	if (!launch(r, k, grid_for(elements, 256), 256, s, args)) return false;
	cuDoubleComplex one{1., 0.}, zero{0., 0.};
	if (cublasSetStream(r->cublas, s) != CUBLAS_STATUS_SUCCESS ||
	    cublasZgeam(r->cublas, CUBLAS_OP_T, CUBLAS_OP_N, (int) n, (int) copies, &one, (cuDoubleComplex *) transposed,
	                (int) copies, &zero, (cuDoubleComplex *) planar, (int) n, (cuDoubleComplex *) planar, (int) n) !=
	    CUBLAS_STATUS_SUCCESS)
		return fail(r, "cublasZgeam (plane)"), false;
	return true;
}

bool check_sizes(refgpu *r, uint32_t n, uint32_t copies) {
	/* common/configuration.hpp:24 (16-bit lengths and per-process copies), common/main.cpp:86,102 */
	if (n < 2 || n > 65535 || copies < 1 || copies > 65535 || uint64_t(n) * copies >= 0x40000000ULL)
		return fail(r, "sizes outside the reference's limits (2 <= n <= 65535, 1 <= copies <= 65535, n copies < 2^30)"),
				false;
	return true;
}

const char *real_ns(int model) { return model == M_DDNKG ? "dDNKG" : "DNKG_FPUT_Toda"; }

}  // namespace

extern "C" {

/* Load one fatbin (built with optimized_chain_length = n_opt) into the calling thread's current
 * context (the runtime's primary context of the current device). c, d: the Yoshida tables. */
int refgpu_open(const char *fatbin_path, int n_opt, const double *c, const double *d, refgpu **out) {
	*out = nullptr;
	auto *r = new refgpu();
	r->n_opt = n_opt;
	std::memcpy(r->c, c, sizeof r->c);
	std::memcpy(r->d, d, sizeof r->d);
	if (!rt_ok(r, cudaFree(nullptr), "cudaFree(0)") || !cu_ok(r, cuModuleLoad(&r->mod, fatbin_path), fatbin_path)) {
		*out = r;
		return -1;
	}
	unsigned count = 0;
	if (!cu_ok(r, cuModuleGetFunctionCount(&count, r->mod), "cuModuleGetFunctionCount")) return *out = r, -1;
	std::vector<CUfunction> fns(count);
	if (!cu_ok(r, cuModuleEnumerateFunctions(fns.data(), count, r->mod), "cuModuleEnumerateFunctions")) return *out = r, -1;
	for (auto f: fns) {
		const char *name = nullptr;
		if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
		int status = 0;
		char *dem = abi::__cxa_demangle(name, nullptr, nullptr, &status);
		std::string s = status == 0 && dem ? dem : name;
		std::free(dem);
		if (s.compare(0, 5, "void ") == 0) s = s.substr(5);
		r->kernels[s] = f;
	}
	if (cublasCreate(&r->cublas) != CUBLAS_STATUS_SUCCESS) return *out = r, fail(r, "cublasCreate");
	*out = r;
	return 0;
}

void refgpu_close(refgpu *r) {
	if (!r) return;
	for (auto &kv: r->dnls_plans) cufftDestroy(kv.second);
	for (auto &kv: r->dnls_tables) cudaFree(kv.second);
	if (r->cublas) cublasDestroy(r->cublas);
	if (r->mod) cuModuleUnload(r->mod);
	delete r;
}

const char *refgpu_error(refgpu *r) { return r ? r->err.c_str() : "no handle"; }

int refgpu_kernel_count(refgpu *r) { return (int) r->kernels.size(); }

/* Advance a planar double2[copies][n] device ensemble of a real model by `steps` steps in launches
 * of `batching` steps (one move<model> call per launch).  mp2_host: dDNKG m_x + 2 (n values).
 * force_split: the reference's --split_kernel.  Synchronous. */
int refgpu_advance(refgpu *r, int model, void *state_dev, uint32_t n, uint32_t copies, double dt, double m, double alpha,
                   double beta, const double *mp2_host, uint64_t steps, uint32_t batching, int force_split,
                   void *stream) {
	if (model < M_DNKG || model > M_DDNKG) return fail(r, "not a real model");
	if (!check_sizes(r, n, copies) || !batching || steps % batching) return fail(r, "bad sizes or batching");
	if (model == M_DDNKG && !mp2_host) return fail(r, "dDNKG needs mp2");
	cudaStream_t s = (cudaStream_t) stream;
	if (!rt_ok(r, cudaStreamSynchronize(s), "sync")) return -1;
	/* constants, DNKG_FPUT_Toda.cpp:76-84 / dDNKG.cpp:94-97 */
	double dtc[8], dtd[8];
	for (int i = 0; i < 8; i++) dtc[i] = r->c[i] * dt, dtd[i] = r->d[i] * dt;
	double *mp2_dev = nullptr;
	if (model == M_DDNKG) {
		if (!set_global(r, "_ZN5dDNKG4dt_cE", dtc, sizeof dtc) || !set_global(r, "_ZN5dDNKG4dt_dE", dtd, sizeof dtd) ||
		    !set_global(r, "_ZN5dDNKG4betaE", &beta, sizeof beta) ||
		    !set_global(r, "_ZN5dDNKG3mp2E", mp2_host, sizeof(double) * (n < 2048 ? n : 2048)))
			return -1;
		if (!rt_ok(r, cudaMalloc(&mp2_dev, sizeof(double) * n), "cudaMalloc mp2") ||
		    !rt_ok(r, cudaMemcpy(mp2_dev, mp2_host, sizeof(double) * n, cudaMemcpyHostToDevice), "mp2 upload"))
			return -1;
	} else {
		double alpha2 = 2 * alpha, alpha2_inv = 1 / alpha2;
		if (!set_global(r, "_ZN14DNKG_FPUT_Toda4dt_cE", dtc, sizeof dtc) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda4dt_dE", dtd, sizeof dtd) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda1mE", &m, sizeof m) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda5alphaE", &alpha, sizeof alpha) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda4betaE", &beta, sizeof beta) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda6alpha2E", &alpha2, sizeof alpha2) ||
		    !set_global(r, "_ZN14DNKG_FPUT_Toda10alpha2_invE", &alpha2_inv, sizeof alpha2_inv))
			return -1;
	}
	const std::string ns = real_ns(model);
	const std::string tmodel = model == M_DDNKG ? "" : "(DNKG_FPUT_Toda::Model)" + std::to_string(model);
	double2 *planar = (double2 *) state_dev;
	uint32_t steps_grouping = batching;
	uint16_t copies16 = (uint16_t) copies;
	int rc = 0;
	bool use_split = force_split || (n >= 32 && (int) n != r->n_opt);
	if (!use_split && n < 32) {
		std::string name = ns + "::move_chain_in_thread<" + (tmodel.empty() ? "" : tmodel + ", ") + "(unsigned short)" +
		                   std::to_string(n) + ">(";
		CUfunction k = find_kernel(r, name);
		if (!k) rc = -1;
		for (uint64_t t = 0; !rc && t < steps; t += batching) {
			void *args[] = {&planar, &steps_grouping, &copies16};
			if (!launch(r, k, grid_for(copies, 128), 128, s, args)) rc = -1;
		}
	} else if (!use_split) {
		std::string name = ns + "::move_chain_in_warp" + (tmodel.empty() ? "(" : "<" + tmodel + ">(");
		CUfunction k = find_kernel(r, name);
		if (!k) rc = -1;
		for (uint64_t t = 0; !rc && t < steps; t += batching) {
			const double *cmp2 = mp2_dev;
			void *args_real[] = {&planar, &steps_grouping, &copies16};
			void *args_dd[] = {&planar, &cmp2, &steps_grouping, &copies16};
			if (!launch(r, k, grid_for(uint64_t(copies) * 32, 256), 256, s, model == M_DDNKG ? args_dd : args_real))
				rc = -1;
		}
	} else {
		double2 *transposed = nullptr;
		double *phi = nullptr;
		size_t elements = size_t(n) * copies;
		if (!rt_ok(r, cudaMalloc(&transposed, sizeof(double2) * elements), "cudaMalloc transposed") ||
		    !rt_ok(r, cudaMalloc(&phi, sizeof(double2) * elements), "cudaMalloc split"))
			rc = -1;
		double *pi = phi + elements;
		std::string name = ns + "::move_split" + (tmodel.empty() ? "(" : "<" + tmodel + ">(");
		CUfunction k = rc ? nullptr : find_kernel(r, name);
		if (!k) rc = -1;
		if (!rc && !split(r, s, planar, transposed, phi, pi, n, copies)) rc = -1;
		const double *mp2_arg = mp2_dev;
		if (!rc && model == M_DDNKG && n <= 2048) {
			/* dDNKG.cu:203-204: the constant-memory copy of mp2 when it fits */
			CUdeviceptr p = 0;
			size_t size = 0;
			if (!cu_ok(r, cuModuleGetGlobal(&p, &size, r->mod, "_ZN5dDNKG3mp2E"), "mp2 symbol")) rc = -1;
			mp2_arg = (const double *) p;
		}
		for (uint64_t t = 0; !rc && t < steps; t += batching) {
			uint32_t chainlen = n, shard_copies = copies;
			void *args_real[] = {&phi, &pi, &chainlen, &shard_copies, &steps_grouping};
			void *args_dd[] = {&phi, &pi, &mp2_arg, &chainlen, &shard_copies, &steps_grouping};
			if (!launch(r, k, grid_for(copies, 128), 128, s, model == M_DDNKG ? args_dd : args_real)) rc = -1;
		}
		if (!rc && !plane(r, s, planar, transposed, phi, pi, n, copies)) rc = -1;
		cudaStreamSynchronize(s);
		cudaFree(transposed);
		cudaFree(phi);
	}
	if (!rt_ok(r, cudaStreamSynchronize(s), "reference move")) rc = -1;
	if (mp2_dev) cudaFree(mp2_dev);
	return rc;
}

/* Launch only the integration kernel of a warp-resident real-model ensemble, `launches` times, on
 * `stream` without synchronising (the bench's plain-reference timing; constants as refgpu_advance
 * set them last, sizes as there).  mp2_dev: dDNKG's m_x + 2 in device memory (n values). */
int refgpu_move_warp_async(refgpu *r, int model, void *state_dev, uint32_t n, uint32_t copies, uint32_t batching,
                           uint32_t launches, const double *mp2_dev, void *stream) {
	if (model < M_DNKG || model > M_DDNKG || (int) n != r->n_opt || !check_sizes(r, n, copies) ||
	    (model == M_DDNKG && !mp2_dev))
		return fail(r, "the warp kernel needs a real model at the optimised length (dDNKG: with its masses)");
	CUfunction k = find_kernel(r, model == M_DDNKG ? std::string("dDNKG::move_chain_in_warp(")
	                                               : std::string("DNKG_FPUT_Toda::move_chain_in_warp<(DNKG_FPUT_Toda::Model)") +
	                                                 std::to_string(model) + ">(");
	if (!k) return -1;
	double2 *planar = (double2 *) state_dev;
	uint32_t steps_grouping = batching;
	uint16_t copies16 = (uint16_t) copies;
	for (uint32_t l = 0; l < launches; l++) {
		void *args_real[] = {&planar, &steps_grouping, &copies16};
		void *args_dd[] = {&planar, &mp2_dev, &steps_grouping, &copies16};
		if (!launch(r, k, grid_for(uint64_t(copies) * 32, 256), 256, (cudaStream_t) stream,
		            model == M_DDNKG ? args_dd : args_real))
			return -1;
	}
	return 0;
}

/* Normalised linear-mode energies (results::calc_linenergies) of a device ensemble.  eigvecs_host
 * (column-major, eigenvector k = column k) and omegas_host are read for dDNKG only.  Synchronous. */
int refgpu_linenergies(refgpu *r, int model, const void *state_dev, uint32_t n, uint32_t copies, double m,
                       const double *eigvecs_host, const double *omegas_host, double *out_host, void *stream) {
	if (!check_sizes(r, n, copies)) return -1;
	cudaStream_t s = (cudaStream_t) stream;
	size_t elements = size_t(n) * copies;
	double *lin_dev = nullptr, *omega_dev = nullptr;
	int rc = 0;
	if (!rt_ok(r, cudaMalloc(&lin_dev, sizeof(double) * n), "cudaMalloc linenergies") ||
	    !rt_ok(r, cudaMalloc(&omega_dev, sizeof(double) * n), "cudaMalloc omega"))
		return -1;
	uint16_t n16 = (uint16_t) n, c16 = (uint16_t) copies;
	double norm;
	bool a0is0;
	if (model == M_DDNKG) {
		if (!eigvecs_host || !omegas_host) return fail(r, "dDNKG needs the eigensystem");
		/* dDNKG.cpp:61-69: E and E diag(omega) on the device; split; two DGEMMs; warp reduce */
		std::vector<double> ew(eigvecs_host, eigvecs_host + size_t(n) * n);
		for (uint32_t i = 0; i < n; i++)
			for (uint32_t j = 0; j < n; j++) ew[size_t(i) * n + j] *= omegas_host[i];
		double *E = nullptr, *EW = nullptr, *phi = nullptr, *proj = nullptr;
		double2 *transposed = nullptr;
		if (!rt_ok(r, cudaMalloc(&E, sizeof(double) * n * n), "cudaMalloc E") ||
		    !rt_ok(r, cudaMalloc(&EW, sizeof(double) * n * n), "cudaMalloc EW") ||
		    !rt_ok(r, cudaMalloc(&phi, sizeof(double2) * elements), "cudaMalloc split") ||
		    !rt_ok(r, cudaMalloc(&proj, sizeof(double2) * elements), "cudaMalloc projection") ||
		    !rt_ok(r, cudaMalloc(&transposed, sizeof(double2) * elements), "cudaMalloc transposed"))
			rc = -1;
		double *pi = phi + elements, *proj_phi = proj, *proj_pi = proj + elements;
		if (!rc && (!rt_ok(r, cudaMemcpy(E, eigvecs_host, sizeof(double) * n * n, cudaMemcpyHostToDevice), "E") ||
		            !rt_ok(r, cudaMemcpy(EW, ew.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice), "EW")))
			rc = -1;
		if (!rc && !split(r, s, (double2 *) state_dev, transposed, phi, pi, n, copies)) rc = -1;
		double one = 1, zero = 0;
		if (!rc && (cublasSetStream(r->cublas, s) != CUBLAS_STATUS_SUCCESS ||
		            cublasDgemm(r->cublas, CUBLAS_OP_N, CUBLAS_OP_N, (int) copies, (int) n, (int) n, &one, phi, (int) copies,
		                        EW, (int) n, &zero, proj_phi, (int) copies) != CUBLAS_STATUS_SUCCESS ||
		            cublasDgemm(r->cublas, CUBLAS_OP_N, CUBLAS_OP_N, (int) copies, (int) n, (int) n, &one, pi, (int) copies,
		                        E, (int) n, &zero, proj_pi, (int) copies) != CUBLAS_STATUS_SUCCESS))
			rc = fail(r, "cublasDgemm");
		CUfunction k = rc ? nullptr : find_kernel(r, "dDNKG::make_linenergies_kernel(");
		if (!k) rc = -1;
		if (!rc) {
			const double *cphi = proj_phi, *cpi = proj_pi;
			void *args[] = {&cphi, &cpi, &n16, &c16, &lin_dev};
			if (!launch(r, k, grid_for(uint64_t(n) * 32, 256), 256, s, args)) rc = -1;
		}
		cudaStreamSynchronize(s);
		cudaFree(E), cudaFree(EW), cudaFree(phi), cudaFree(proj), cudaFree(transposed);
		norm = 0.5 / copies;   /* dDNKG.cpp:141 */
		a0is0 = false;
	} else {
		/* dispersion: DNKG_FPUT_Toda/dispersion.cpp:9-16, DNLS/dispersion.cpp:10-17 */
		std::vector<double> omega(n);
		for (size_t k = 0; k < n; k++) {
			auto s2 = 2 * sin(k * M_PI / n);
			omega[k] = model == M_DNLS ? s2 * s2 : sqrt(m + s2 * s2);
		}
		if (!rt_ok(r, cudaMemcpy(omega_dev, omega.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "omega")) rc = -1;
		double2 *fft = nullptr;
		cufftHandle plan = 0;
		int batch = model == M_DNLS ? (int) copies : 2 * (int) copies;
		if (!rc && !rt_ok(r, cudaMalloc(&fft, sizeof(double2) * elements * (model == M_DNLS ? 1 : 2)), "cudaMalloc fft"))
			rc = -1;
		if (!rc && (cufftPlan1d(&plan, (int) n, CUFFT_Z2Z, batch) != CUFFT_SUCCESS || cufftSetStream(plan, s) != CUFFT_SUCCESS))
			rc = fail(r, "cufftPlan1d");
		const double2 *st = (const double2 *) state_dev;
		if (!rc && model == M_DNLS) {
			if (cufftExecZ2Z(plan, (cufftDoubleComplex *) st, fft, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = fail(r, "cufftExecZ2Z");
			CUfunction k = rc ? nullptr : find_kernel(r, "DNLS::make_linenergies_kernel(");
			if (!k) rc = -1;
			if (!rc) {
				const double2 *cfft = fft;
				const double *com = omega_dev;
				void *args[] = {&c16, &n16, &cfft, &com, &lin_dev};
				if (!launch(r, k, grid_for(n, 256), 256, s, args)) rc = -1;
			}
			norm = 1. / (uint32_t(n) * copies);   /* DNLS.cpp:150, 1 / shard_elements */
			a0is0 = true;
		} else if (!rc) {
			/* DNKG_FPUT_Toda.cpp:113-122: phi and pi as real parts of two batches of complex chains */
			double2 *fft_pi = fft + elements;
			if (!rt_ok(r, cudaMemsetAsync(fft, 0, sizeof(double2) * elements * 2, s), "memset") ||
			    !rt_ok(r, cudaMemcpy2DAsync(fft, sizeof(double2), st, sizeof(double2), sizeof(double), elements,
			                                cudaMemcpyDeviceToDevice, s), "interleave phi") ||
			    !rt_ok(r, cudaMemcpy2DAsync(fft_pi, sizeof(double2), &st[0].y, sizeof(double2), sizeof(double), elements,
			                                cudaMemcpyDeviceToDevice, s), "interleave pi"))
				rc = -1;
			if (!rc && cufftExecZ2Z(plan, fft, fft, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = fail(r, "cufftExecZ2Z");
			CUfunction k = rc ? nullptr : find_kernel(r, "DNKG_FPUT_Toda::make_linenergies_kernel(");
			if (!k) rc = -1;
			if (!rc) {
				const double2 *cphi = fft, *cpi = fft_pi;
				const double *com = omega_dev;
				void *args[] = {&n16, &c16, &lin_dev, &cphi, &cpi, &com};
				if (!launch(r, k, grid_for(n, 256), 256, s, args)) rc = -1;
			}
			norm = (0.5 / copies) / n;   /* DNKG_FPUT_Toda.cpp:129 */
			a0is0 = m == 0.;
		}
		cudaStreamSynchronize(s);
		if (plan) cufftDestroy(plan);
		cudaFree(fft);
	}
	if (!rc && !rt_ok(r, cudaMemcpy(out_host, lin_dev, sizeof(double) * n, cudaMemcpyDeviceToHost), "read-back")) rc = -1;
	cudaFree(lin_dev), cudaFree(omega_dev);
	if (rc) return rc;
	/* results_entropy.cpp:11-19 (one process) */
	if (a0is0) out_host[0] = 0;
	for (uint32_t i = 0; i < n; i++) out_host[i] *= norm;
	return 0;
}

/* Advance a DNLS complex128[copies][n] device ensemble (DNLS.cpp:159-175, no callbacks).  The cuFFT
 * plan and the linear tables are made on first use and kept, as the reference's main keeps them;
 * sync = 0 returns with the launches queued on `stream`. */
int refgpu_dnls_advance(refgpu *r, void *state_dev, uint32_t n, uint32_t copies, double dt, double beta, uint64_t steps,
                        uint32_t batching, void *stream, int sync) {
	if (!check_sizes(r, n, copies) || !batching || steps % batching) return fail(r, "bad sizes or batching");
	cudaStream_t s = (cudaStream_t) stream;
	double2 *&table_dev = r->dnls_tables[{n, dt}];
	if (!table_dev) {
		using namespace std::complex_literals;
		/* DNLS/dispersion.cpp:10-26 */
		std::vector<double> omega(n);
		for (size_t k = 0; k < n; k++) {
			auto s2 = 2 * sin(k * M_PI / n);
			omega[k] = s2 * s2;
		}
		std::vector<std::complex<double>> table(size_t(7) * n);
		auto normalization = 1. / n;
		std::complex<double> complexdt = -1i * dt;
		for (size_t i = 0; i < 7; i++)
			for (size_t j = 0; j < n; j++) table[i * n + j] = exp(complexdt * r->d[i] * omega[j]) * normalization;
		if (!rt_ok(r, cudaMalloc(&table_dev, sizeof(double2) * table.size()), "cudaMalloc tables") ||
		    !rt_ok(r, cudaMemcpy(table_dev, table.data(), sizeof(double2) * table.size(), cudaMemcpyHostToDevice),
		           "tables")) {
			cudaFree(table_dev);
			table_dev = nullptr;
			return -1;
		}
	}
	int rc = 0;
	cufftHandle &plan = r->dnls_plans[{n, copies}];
	if (!plan && cufftPlan1d(&plan, (int) n, CUFFT_Z2Z, (int) copies) != CUFFT_SUCCESS) {
		plan = 0;
		rc = fail(r, "cufftPlan1d");
	}
	if (!rc && cufftSetStream(plan, s) != CUFFT_SUCCESS) rc = fail(r, "cufftSetStream");
	CUfunction knl = rc ? nullptr : find_kernel(r, "DNLS::evolve_nonlinear_kernel(");
	CUfunction kl = rc ? nullptr : find_kernel(r, "DNLS::evolve_linear_kernel(");
	if (!knl || !kl) rc = -1;
	uint32_t elements = n * copies;
	uint16_t n16 = (uint16_t) n;
	double2 *psis = (double2 *) state_dev;
	auto nonlinear = [&](double bds) {
		void *args[] = {&elements, &psis, &bds};
		return launch(r, knl, grid_for(elements, 256), 256, s, args);
	};
	for (uint64_t t = 0; !rc && t < steps; t += batching) {
		for (uint32_t i = 0; !rc && i < batching; i++)
			for (int k = 0; !rc && k < 7; k++) {
				if (!nonlinear(beta * dt * (!k && i ? 2. : 1.) * r->c[k]) ||
				    cufftExecZ2Z(plan, (cufftDoubleComplex *) psis, (cufftDoubleComplex *) psis, CUFFT_FORWARD) != CUFFT_SUCCESS) {
					rc = r->err.empty() ? fail(r, "cufftExecZ2Z") : -1;
					break;
				}
				/* the load_ldg iterator argument is one pointer (cub CacheModifiedInputIterator) */
				double2 *tk = table_dev + size_t(k) * n;
				void *args[] = {&elements, &n16, &psis, &tk};
				if (!launch(r, kl, grid_for(elements, 256), 256, s, args) ||
				    cufftExecZ2Z(plan, (cufftDoubleComplex *) psis, (cufftDoubleComplex *) psis, CUFFT_INVERSE) != CUFFT_SUCCESS)
					rc = r->err.empty() ? fail(r, "cufftExecZ2Z") : -1;
			}
		if (!rc && !nonlinear(beta * dt * r->c[7])) rc = -1;
	}
	if (!sync) return rc;
	if (!rt_ok(r, cudaStreamSynchronize(s), "reference DNLS")) rc = -1;
	return rc;
}

}  // extern "C"
