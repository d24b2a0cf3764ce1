// DNLS split-step integrator, fused: one launch advances every chain by `steps` Yoshida steps with
// the chain resident in shared memory.
//
// The reference drives this from the host: per step and sub-step k it launches (or sets a cuFFT
// load callback for) the nonlinear phase rotation, a forward cuFFT, the linear propagator and an
// inverse cuFFT over the whole ensemble -- 14 FFT launches and ~14 tiny H2D/memset operations per
// time step, each a full round trip of the state through HBM (DNLS.cpp:159-175, DNLS.cu:11-67).
// Here a team of threads owns one chain for the whole launch:
//   psi <- psi exp(-i beta dt c_k |psi|^2)       (DNLS.cu:11-17; c_0 doubled when merged, DNLS.cpp:162)
//   psi_k <- FFT(psi) * exp(-i dt d_k omega_k)/n  (DNLS/dispersion.cpp:19-26, DNLS.cu:19-25)
//   psi <- IFFT(psi_k)
// (for a length whose direct passes cost more, i.e. with large prime factors, the last two lines
// are one zero-padded cyclic convolution of smooth length len >= 2n - 1: the propagator is
// circulant, nlc_host.h), and finally psi <- psi exp(-i beta dt c_7 |psi|^2) (DNLS.cpp:175).  The
// FFTs are the Stockham transforms of nlc_fft.cuh, in shared memory (beyond it, in per-block global
// scratch); the state is read once and written once per launch.
#include "nlc_fft.cuh"

namespace nlc {

__device__ __forceinline__ double2 nonlinear_rotate(double2 v, double neg_coef, const double2 *__restrict__ sctab,
                                                    const SinCosConsts &sc, const FpOnes &k) {
	const double norm = dfma(v.x, v.x, fmul(v.y, v.y, k));
	double s, c;
	sincos_table(fmul(neg_coef, norm, k), sctab, sc, k, &s, &c);
	return make_double2(dfma(v.x, c, -fmul(v.y, s, k)), dfma(v.x, s, fmul(v.y, c, k)));
}

// BLOCK: one chain per block.  Otherwise teams of a.team lanes (a power of two, 4 .. 32) inside each
// warp, 32 / a.team chains per warp: short chains keep every lane busy.  A warp takes its chains as
// one unit from the self-resetting counter, so all its teams run the same control flow (a team
// past the last chain repeats the last one and does not store).
// 64 registers a thread: four 256-thread chains (or eight 128-thread team blocks) per SM; the block
// variant also runs with 512 threads when the chain's buffers live in global memory
template <bool BLOCK>
__global__ void __launch_bounds__(BLOCK ? 512 : 128, BLOCK ? 2 : 8) dnls_move_kernel(double2 *__restrict__ psi, const DnlsArgs a) {
	extern __shared__ double2 sm[];
	__shared__ unsigned long long s_chain[32];
	const int n = int(a.n);
	const int T = BLOCK ? blockDim.x : a.team;
	const int t = BLOCK ? threadIdx.x : (threadIdx.x & (T - 1));
	const int team = BLOCK ? 0 : (threadIdx.x / T);
	const int per_warp = BLOCK ? 1 : 32 / T;
	const int len = a.fft.len;
	double2 *buf0 = BLOCK && a.gscratch ? a.gscratch + (size_t) blockIdx.x * 2 * len : sm + (size_t) team * 2 * len;
	double2 *buf1 = buf0 + len;
	const unsigned long long units = (a.copies + per_warp - 1) / per_warp;

	for (;;) {
		// the next unit from the self-resetting counter: a chain (BLOCK) or a warp's chains
		unsigned long long u;
		if (BLOCK) {
			__syncthreads();
			if (t == 0) s_chain[0] = atomicAdd(&a.work_counter[0], 1ull);
			__syncthreads();
			u = s_chain[0];
		} else {
			unsigned long long c = 0;
			if ((threadIdx.x & 31) == 0) c = atomicAdd(&a.work_counter[0], 1ull);
			u = __shfl_sync(0xffffffffu, c, 0);
		}
		if (u >= units) break;
		unsigned long long chain = u * per_warp + (BLOCK ? 0 : (threadIdx.x & 31) / T);
		const bool active = chain < a.copies;
		if (!active) chain = a.copies - 1;

		double2 *g = psi + chain * (unsigned long long) n;
		double2 *x = buf0, *y = buf1;
		for (int j = t; j < n; j += T) x[j] = g[j];
		team_sync<BLOCK>();

		for (uint32_t i = 0; i < a.steps; i++) {
			for (int k = 0; k < 7; k++) {
				const double coef = (k == 0 && (i != 0 || (a.seg & NLC_SEG_CONTINUE))) ? a.nl[7] : a.nl[k];
				// the phase rotation is applied as the forward transform's first pass reads each
				// element (beyond n: the zero padding of the convolution form), the propagator (or
				// the convolution kernel's spectrum) as its last pass writes each element
				auto rotate = [&](int j, double2 v) {
					return j < n ? nonlinear_rotate(v, -coef, a.sctab, a.sc, a.fft.k1) : make_double2(0., 0.);
				};
				const double2 *tab = a.conv_tables ? a.conv_tables + (size_t) k * len : a.lin_tables + (size_t) k * n;
				auto propagate = [&](int j, double2 v) { return cmul(v, tab[j], a.fft.k1); };
				double2 *r = stockham_team<BLOCK, false>(a.fft, x, y, t, T, rotate, propagate);
				double2 *o = r == x ? y : x;
				x = stockham_team<BLOCK, true>(a.fft, r, o, t, T);
				y = x == buf0 ? buf1 : buf0;
			}
		}
		if (active) {
			if (a.seg & NLC_SEG_OPEN)
				for (int j = t; j < n; j += T) g[j] = x[j];
			else
				for (int j = t; j < n; j += T) g[j] = nonlinear_rotate(x[j], -a.nl_final, a.sctab, a.sc, a.fft.k1);
		}
		team_sync<BLOCK>();
	}

	if (!BLOCK) __syncthreads();
	if (threadIdx.x == 0) {
		__threadfence();
		const unsigned long long done = atomicAdd(&a.work_counter[1], 1ull);
		if (done == gridDim.x - 1) {
			a.work_counter[0] = 0;
			a.work_counter[1] = 0;
			__threadfence();
		}
	}
}

cudaError_t launch_dnls_move(const DnlsArgs &a, double2 *psi, int blocks, int threads, size_t smem,
                             int team_block, cudaStream_t stream) {
	count_launch();
	if (team_block) dnls_move_kernel<true><<<blocks, threads, smem, stream>>>(psi, a);
	else dnls_move_kernel<false><<<blocks, threads, smem, stream>>>(psi, a);
	return cudaGetLastError();
}

// Elementwise operators with the reference's semantics (DNLS.cu:11-25), for callers that keep
// their own FFT loop.
__global__ void dnls_nonlinear_kernel(double2 *psi, unsigned long long elements, double neg_coef,
                                      const double2 *sctab, const SinCosConsts sc, const FpOnes k) {
	const unsigned long long i = (unsigned long long) blockIdx.x * blockDim.x + threadIdx.x;
	if (i < elements) psi[i] = nonlinear_rotate(psi[i], neg_coef, sctab, sc, k);
}

__global__ void dnls_linear_kernel(double2 *psi, unsigned long long elements, uint32_t n, const double2 *table,
                                   const FpOnes k) {
	const unsigned long long i = (unsigned long long) blockIdx.x * blockDim.x + threadIdx.x;
	if (i < elements) psi[i] = cmul(psi[i], table[i % n], k);
}

cudaError_t launch_dnls_nonlinear(double2 *psi, uint64_t elements, double coef, const double2 *sctab,
                                  cudaStream_t stream) {
	count_launch();
	const unsigned long long blocks = (elements + 255) / 256;
	dnls_nonlinear_kernel<<<(unsigned) blocks, 256, 0, stream>>>(psi, elements, -coef, sctab, SinCosConsts{}, FpOnes{});
	return cudaGetLastError();
}

cudaError_t launch_dnls_linear(double2 *psi, uint64_t elements, uint32_t n, const double2 *table,
                               cudaStream_t stream) {
	count_launch();
	const unsigned long long blocks = (elements + 255) / 256;
	dnls_linear_kernel<<<(unsigned) blocks, 256, 0, stream>>>(psi, elements, n, table, FpOnes{});
	return cudaGetLastError();
}

}  // namespace nlc

namespace nlc {
const void *dnls_kernel_ptr(int team_block) {
	return team_block ? (const void *) dnls_move_kernel<true> : (const void *) dnls_move_kernel<false>;
}
}  // namespace nlc
