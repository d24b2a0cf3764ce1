// DNLS split step with the linear sub-steps as a real-space stencil; chains resident in registers.
//
// The linear sub-step of the reference, psi <- IFFT(FFT(psi) exp(-i tau omega_j) / n) with
// tau = dt d_k and omega_j = 4 sin^2(pi j / n) = 2 - 2 cos(2 pi j / n) (DNLS.cpp:166-172,
// DNLS.cu:19-25, dispersion.cpp:19-26), is a circulant operator.  Its kernel follows from the
// Jacobi-Anger expansion exp(i z cos phi) = sum_m i^m J_m(z) exp(i m phi):
//
//   psi'_s = exp(-2 i tau) sum_x i^|x| J_|x|(2 tau) psi_{s+x}
//
// plus periodic images J_{|x| + l n}, l != 0.  J_x(2 tau) ~ tau^x / x! is below 2^-64 beyond a
// radius R (7 for dt = 0.01 with the Yoshida coefficients), and for n >= 2R + 2 the images are too,
// so a linear sub-step is a (2R + 1)-point stencil with real coefficients and the factors i^x, which
// only swap and negate real and imaginary parts.  The common phase exp(-2 i tau) is folded into the
// angle of the nonlinear rotation that precedes the sub-step (both are diagonal in real space and
// commute with |psi|).  FP64 operations per site and sub-step: the rotation 17 (norm 2, angle 1,
// sincos 10 below 2^-4, product 4) and the stencil 4R + 2 (R symmetric sums psi_{s+x} + psi_{s-x},
// R + 1 FMAs per component): 47 at R = 7, against 73 with the two shared-memory transforms at
// n = 1024 (nlc_dnls.cu) and about twice that for a length with a large prime factor.  The centre
// term is psi + (J_0 - 1) psi in one FMA, with J_0 - 1 held to full relative precision, so no
// coefficient rounded near 1 scales the smooth modes the same way at every sub-step.
//
// Layout: a chain of n sites on G lanes (any G up to 256), each lane holding E or E - 1 consecutive
// sites (E in {8, 12, 16}, the first n - G (E - 1) lanes holding E) plus R halo sites on each side.
// G <= 32: floor(32 / G) chains per warp, halos by shuffles from explicit lanes, no barrier;
// G > 32: one chain per block, halos by shuffles inside warps and through shared memory across
// them, one barrier per sub-step.  The grid is persistent (self-resetting work counter) as for the
// real models.
//
// Chains longer than one block holds (WIN): windows of G E sites of the periodic chain (every lane
// full), advanced a few steps per launch as if the window were a ring.  A sub-step moves
// information R sites, so after s steps only the 7 R s sites at each end of the window have seen
// the false wrap-around; the interior between them is exact and is written to the second buffer,
// and the windows' interiors tile the chain.
#include "nlc_device.cuh"
#include "nlc_internal.h"

namespace nlc {

namespace {

__device__ __forceinline__ double2 shfl2(double2 v, int src) {
	return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// psi exp(i (neg_coef |psi|^2 + neg_phase)): the nonlinear rotation with the propagator's phase
__device__ __forceinline__ double2 rotate_phase(double2 v, double neg_coef, double neg_phase,
                                                const double2 *__restrict__ sctab, const SinCosConsts &sc,
                                                const FpOnes &k) {
	const double norm = dfma(v.x, v.x, fmul(v.y, v.y, k));
	double s, c;
	sincos_table(dfma(neg_coef, norm, neg_phase), sctab, sc, k, &s, &c);
	return make_double2(dfma(v.x, c, -fmul(v.y, s, k)), dfma(v.x, s, fmul(v.y, c, k)));
}

}  // namespace

// TEAM: G <= 32, 128-thread blocks; otherwise one chain (WIN: one window) per block of ceil(G / 32)
// warps
template <int E, int R, bool TEAM, bool WIN>
__global__ void __launch_bounds__(TEAM ? 128 : 256) dnls_stencil_kernel(double2 *__restrict__ psi, const DnlsStencilArgs a) {
	static_assert(E - 1 >= R, "a lane's halo comes from one neighbour: E - 1 >= R sites");
	static_assert(!(WIN && TEAM), "windows are block-wide");
	// G > 32: the halos crossing warps, [2 parities][2 directions][warps][R]
	extern __shared__ double2 xb[];
	__shared__ unsigned long long s_unit;
	const int G = a.lanes, n = int(a.n), tid = threadIdx.x;
	const int wl = tid & 31, warp = tid >> 5;
	const int per_warp = TEAM ? 32 / G : 1;
	const int cw = TEAM ? wl / G : 0;                    // chain of this lane within its warp
	const bool spare = TEAM && cw >= per_warp;           // lanes past the warp's last whole chain
	const int lane = TEAM ? (spare ? 0 : wl - cw * G) : tid;
	const int gpb = TEAM ? per_warp * int(blockDim.x >> 5) : 1;   // chains per block
	const int gib = TEAM ? warp * per_warp + cw : 0;
	const int W = TEAM ? 1 : (G + 31) >> 5;
	const bool idle = spare || lane >= G;                // lanes that hold no sites (never stored)
	// neighbour lanes (within the warp; G > 32: the warp-edge and wrap-around pairs go through
	// shared memory)
	const int src_left = TEAM ? (spare ? wl : cw * G + (lane + G - 1) % G) : ((wl + 31) & 31);
	const int src_right = TEAM ? (spare ? wl : cw * G + (lane + 1) % G) : ((wl + 1) & 31);
	const bool left_smem = !TEAM && !idle && (wl == 0 || lane == 0);
	const bool right_smem = !TEAM && !idle && (wl == 31 || lane == G - 1);
	const int left_warp = lane == 0 ? ((G - 1) >> 5) : warp - 1;   // warp of lane - 1 (mod G)
	const int right_warp = lane == G - 1 ? 0 : warp + 1;            // warp of lane + 1 (mod G)

	const int full = WIN ? G : n - G * (E - 1);
	const bool fl = lane < full;
	const int ne = fl ? E : E - 1;
	const int first = fl ? lane * E : full * E + (lane - full) * (E - 1);
	const FpOnes &k1 = a.k1;
	int parity = 0;

	const unsigned long long units =
	    WIN ? (unsigned long long) a.copies * a.win_count : (a.copies + gpb - 1) / gpb;
	for (;;) {
		__syncthreads();
		if (tid == 0) s_unit = atomicAdd(&a.work_counter[0], 1ull);
		__syncthreads();
		const unsigned long long u = s_unit;
		if (u >= units) break;
		unsigned long long chain = WIN ? u / a.win_count : u * gpb + gib;
		const uint32_t win = WIN ? uint32_t(u - chain * a.win_count) : 0;
		// WIN: the chain site of this lane's first site (the window starts win_halo sites before its
		// interior)
		const uint32_t wsite = WIN ? uint32_t((win * (unsigned long long) a.win_inner + n - a.win_halo + first) % n) : 0;
		const bool active = chain < a.copies && !idle;
		if (chain >= a.copies) chain = a.copies - 1;   // redundant work keeps shuffles and barriers convergent
		double2 *g = psi + chain * (unsigned long long) n + (idle || WIN ? 0 : first);

		// w: [0, R) left halo, [R, R + E) this lane's sites, [R + E, R + E + R) right halo; a short
		// lane's slot R + E - 1 is inert (zero) between sub-steps
		double2 w[E + 2 * R];
#pragma unroll
		for (int j = 0; j < E; j++) {
			uint32_t sj = j;
			if (WIN) {
				sj = wsite + j;
				if (sj >= uint32_t(n)) sj -= n;
			}
			w[R + j] = (!idle && j < ne) ? g[sj] : make_double2(0., 0.);
		}

		for (uint32_t i = 0; i < a.steps; i++) {
#pragma unroll 1
			for (int k = 0; k < 7; k++) {
				const double nc = -((k == 0 && (i != 0 || (a.seg & NLC_SEG_CONTINUE))) ? a.nl[7] : a.nl[k]);
				const double ph = a.phase[k];
#pragma unroll
				for (int j = 0; j < E; j++) w[R + j] = rotate_phase(w[R + j], nc, ph, a.sctab, a.sc, k1);

				// halos: the left one is lane - 1's last R sites, the right one lane + 1's first R
				double2 rl[R], rr[R];
#pragma unroll
				for (int x = 0; x < R; x++) {
					const double2 last = fl ? w[E + x] : w[E - 1 + x];   // site ne - R + x
					rl[x] = shfl2(last, src_left);
					rr[x] = shfl2(w[R + x], src_right);
				}
				if (!TEAM) {
					double2 *buf = xb + parity * 2 * W * R;
					if (right_smem) {
#pragma unroll
						for (int x = 0; x < R; x++) buf[warp * R + x] = fl ? w[E + x] : w[E - 1 + x];
					}
					if (left_smem) {
#pragma unroll
						for (int x = 0; x < R; x++) buf[(W + warp) * R + x] = w[R + x];
					}
					__syncthreads();
					if (left_smem) {
#pragma unroll
						for (int x = 0; x < R; x++) rl[x] = buf[left_warp * R + x];
					}
					if (right_smem) {
#pragma unroll
						for (int x = 0; x < R; x++) rr[x] = buf[(W + right_warp) * R + x];
					}
					parity ^= 1;
				}
#pragma unroll
				for (int x = 0; x < R; x++) w[x] = rl[x];
				// the right halo follows the lane's last site: slot R + E on a full lane, R + E - 1 on a
				// short one (its inert slot)
				w[R + E - 1] = fl ? w[R + E - 1] : rr[0];
#pragma unroll
				for (int x = 0; x < R - 1; x++) w[R + E + x] = fl ? rr[x] : rr[x + 1];
				w[R + E + R - 1] = rr[R - 1];

				// the stencil: psi + (J_0 - 1) psi + sum_x J_x i^x (psi_{s+x} + psi_{s-x}), the sign of
				// i^x folded into taps (x = 2, 3 mod 4 negative), the factor i of odd x as a swap
				const double c0 = a.c0m1[k];
				double tp[R];
#pragma unroll
				for (int x = 0; x < R; x++) tp[x] = a.taps[k][x];
				double2 y[E];
#pragma unroll
				for (int j = 0; j < E; j++) {
					const double2 c = w[R + j];
					double yr = dfma(c0, c.x, c.x), yi = dfma(c0, c.y, c.y);
#pragma unroll
					for (int x = 1; x <= R; x++) {
						const double sr = fadd(w[R + j + x].x, w[R + j - x].x, k1);
						const double si = fadd(w[R + j + x].y, w[R + j - x].y, k1);
						if (x & 1) {
							yr = dfma(-tp[x - 1], si, yr);
							yi = dfma(tp[x - 1], sr, yi);
						} else {
							yr = dfma(tp[x - 1], sr, yr);
							yi = dfma(tp[x - 1], si, yi);
						}
					}
					y[j] = make_double2(yr, yi);
				}
#pragma unroll
				for (int j = 0; j < E; j++) w[R + j] = y[j];
				if (!fl) w[R + E - 1] = make_double2(0., 0.);
			}
		}
		if (active) {
			const bool open = a.seg & NLC_SEG_OPEN;
			double2 *dst = g;
			// WIN: the interior's window positions [lo, hi) relative to this lane's first site, and the
			// chain site of this lane's first site, written to win_out
			int lo = 0, hi = E;
			long long site0 = 0;
			if (WIN) {
				const uint32_t base = win * a.win_inner;   // chain site of the interior's first site
				const uint32_t inner = min(a.win_inner, uint32_t(n) - base);
				dst = a.win_out + chain * (unsigned long long) n;
				lo = int(a.win_halo) - first;
				hi = int(a.win_halo + inner) - first;
				site0 = (long long) base - a.win_halo + first;
			}
#pragma unroll
			for (int j = 0; j < E; j++)
				if (j < ne && j >= lo && j < hi)
					dst[site0 + j] = open ? w[R + j] : rotate_phase(w[R + j], -a.nl_final, 0., a.sctab, a.sc, k1);
		}
	}

	// the last block out resets the work counters for the next launch on this plan
	if (tid == 0) {
		__threadfence();
		const unsigned long long done = atomicAdd(&a.work_counter[1], 1ull);
		if (done == gridDim.x - 1) {
			a.work_counter[0] = 0;
			a.work_counter[1] = 0;
			__threadfence();
		}
	}
}

namespace {

using StencilKernel = void (*)(double2 *, const DnlsStencilArgs);

StencilKernel stencil_kernel(int sites, int radius, bool team, bool win) {
	if (win) {   // windows: 16 sites per lane
		if (sites != 16 || team) return nullptr;
		return radius == 7 ? dnls_stencil_kernel<16, 7, false, true>
		                   : radius == 11 ? dnls_stencil_kernel<16, 11, false, true> : nullptr;
	}
	if (radius == 7) {
		switch (sites) {
			case 8: return team ? dnls_stencil_kernel<8, 7, true, false> : dnls_stencil_kernel<8, 7, false, false>;
			case 12: return team ? dnls_stencil_kernel<12, 7, true, false> : dnls_stencil_kernel<12, 7, false, false>;
			case 16: return team ? dnls_stencil_kernel<16, 7, true, false> : dnls_stencil_kernel<16, 7, false, false>;
		}
	} else if (radius == 11) {
		switch (sites) {
			case 12: return team ? dnls_stencil_kernel<12, 11, true, false> : dnls_stencil_kernel<12, 11, false, false>;
			case 16: return team ? dnls_stencil_kernel<16, 11, true, false> : dnls_stencil_kernel<16, 11, false, false>;
		}
	}
	return nullptr;
}

}  // namespace

const void *dnls_stencil_kernel_ptr(int sites, int radius, bool team, bool windowed) {
	return (const void *) stencil_kernel(sites, radius, team, windowed);
}

size_t dnls_stencil_smem(int lanes, int radius) {
	return lanes > 32 ? size_t(4) * ((lanes + 31) / 32) * radius * sizeof(double2) : 0;
}

cudaError_t launch_dnls_stencil(const DnlsStencilArgs &a, double2 *psi, int sites, int radius, int blocks,
                                cudaStream_t stream) {
	const bool team = a.lanes <= 32;
	const StencilKernel k = stencil_kernel(sites, radius, team, a.win_len != 0);
	if (!k || a.lanes < 1 || a.lanes > 256 || !a.copies || blocks < 1) return cudaErrorInvalidConfiguration;
	if (a.win_len) {
		// a window fills every lane, lies inside the chain, and keeps a non-empty interior
		if (a.win_len != uint32_t(a.lanes) * uint32_t(sites) || a.n <= a.win_len || !a.win_inner ||
		    2ull * a.win_halo + a.win_inner > a.win_len || !a.win_out ||
		    a.win_count != (a.n + a.win_inner - 1) / a.win_inner)
			return cudaErrorInvalidConfiguration;
	} else if (uint64_t(a.lanes) * (sites - 1) >= a.n || uint64_t(a.lanes) * sites < a.n || a.n < uint32_t(2 * radius + 2)) {
		return cudaErrorInvalidConfiguration;   // every lane holds sites or sites - 1 >= radius sites
	}
	count_launch();
	const int threads = team ? 128 : (a.lanes + 31) / 32 * 32;
	k<<<blocks, threads, dnls_stencil_smem(a.lanes, radius), stream>>>(psi, a);
	return cudaGetLastError();
}

}  // namespace nlc
