// Linear-mode energy diagnostics and entropies.
//
// Real models (DNKG, FPUT, Toda): the reference transforms phi and pi as two zero-padded complex
// sequences (DNKG_FPUT_Toda.cpp:113-122) and sums |omega_k Phi_k + i Pi_k|^2 over copies with one
// thread per mode (DNKG_FPUT_Toda.cu:304-321).  Here one complex FFT of z = phi + i pi per chain
// gives both: Phi_k = (Z_k + conj Z_{n-k})/2, Pi_k = (Z_k - conj Z_{n-k})/(2i), hence
//     omega Phi_k + i Pi_k = a_k Z_k + b_k conj(Z_{n-k}),  a_k = (omega_k + 1)/2, b_k = (omega_k - 1)/2,
// and the planar double2 (phi, pi) state already *is* z, so no interleaving copies are needed.
// DNLS: |FFT(psi)_k|^2 summed, times omega_k (DNLS.cu:70-81).  dDNKG: explicit eigenbasis
// projection (the reference's two cublasDgemm calls, dDNKG.cpp:118-133, plus dDNKG.cu:237-256).
//
// The sum over copies (the reference's MPI all_reduce, results_entropy.cpp:13) runs on the device
// in a fixed order: each team (or, for dDNKG, each block) accumulates its chains into its own
// partial row, and a single-block finish kernel sums the rows in row order, normalises, and
// computes the WT / information entropies (results_entropy.cpp:21-46).  Results are therefore
// identical from run to run on a given GPU.
#include <algorithm>

#include "nlc_fft.cuh"

namespace nlc {

// One team (warp, or whole block when BLOCK) per chain; shared memory per team: 2 n complex
// (ping-pong).  Each team accumulates its chains into its own row of `partials` (row = block *
// teams + team), so no two threads ever add into the same element.
template <bool BLOCK>
__global__ void lin_fft_kernel(const double2 *__restrict__ state, const DiagArgs a) {
	extern __shared__ double2 sm[];
	const int n = int(a.n);
	const int T = BLOCK ? blockDim.x : 32;
	const int t = BLOCK ? threadIdx.x : (threadIdx.x & 31);
	const int team = BLOCK ? 0 : (threadIdx.x >> 5);
	const int teams = BLOCK ? 1 : (blockDim.x >> 5);
	const int len = a.fft.len;
	double2 *x = BLOCK && a.gscratch ? a.gscratch + (size_t) blockIdx.x * 2 * len : sm + (size_t) team * 2 * len;
	double2 *y = x + len;
	double *acc = a.partials + ((size_t) blockIdx.x * teams + team) * n;
	for (int k = t; k < n; k += T) acc[k] = 0.;

	const bool dnls = a.model == NLC_DNLS;
	const FpOnes &k1 = a.fft.k1;
	for (unsigned long long chain = (unsigned long long) blockIdx.x * teams + team; chain < a.copies;
	     chain += (unsigned long long) gridDim.x * teams) {
		const double2 *src = state + chain * (unsigned long long) n;
		for (int k = t; k < n; k += T) x[k] = src[k];
		team_sync<BLOCK>();
		const double2 *Z = fft_team<BLOCK, false>(a.fft, x, y, t, T);
		if (dnls) {
			for (int k = t; k < n; k += T) {
				const double2 z = Z[k];
				acc[k] = fadd(acc[k], dfma(z.x, z.x, fmul(z.y, z.y, k1)), k1);
			}
		} else {
			for (int k = t; k < n; k += T) {
				const double2 zk = Z[k], zm = Z[k ? n - k : 0];
				const double ak = a.coef_a[k], bk = a.coef_b[k];
				const double re = dfma(ak, zk.x, fmul(bk, zm.x, k1));
				const double im = dfma(ak, zk.y, -fmul(bk, zm.y, k1));
				acc[k] = fadd(acc[k], dfma(re, re, fmul(im, im, k1)), k1);
			}
		}
		team_sync<BLOCK>();
	}
}

// The FP32 diagnostics (NLC_FLAG_FP32_DIAGNOSTICS): the same teams and partial rows, each chain
// transformed in FP32 in shared memory (half the bytes of the FP64 buffers) and its mode energies
// formed in FP32; the sum over chains stays in the FP64 partial rows.  The error against the FP64
// path is that of an FP32 transform, ~1e-7 of the largest mode energies.
template <bool BLOCK>
__global__ void lin_fft32_kernel(const double2 *__restrict__ state, const DiagArgs a) {
	extern __shared__ float2 smf[];
	const int n = int(a.n);
	const int T = BLOCK ? blockDim.x : 32;
	const int t = BLOCK ? threadIdx.x : (threadIdx.x & 31);
	const int team = BLOCK ? 0 : (threadIdx.x >> 5);
	const int teams = BLOCK ? 1 : (blockDim.x >> 5);
	const int len = a.fft.len;
	float2 *x = smf + (size_t) team * 2 * len;
	float2 *y = x + len;
	double *acc = a.partials + ((size_t) blockIdx.x * teams + team) * n;
	for (int k = t; k < n; k += T) acc[k] = 0.;
	const bool dnls = a.model == NLC_DNLS;
	for (unsigned long long chain = (unsigned long long) blockIdx.x * teams + team; chain < a.copies;
	     chain += (unsigned long long) gridDim.x * teams) {
		const double2 *src = state + chain * (unsigned long long) n;
		for (int k = t; k < n; k += T) {
			const double2 v = src[k];
			x[k] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
		}
		team_sync<BLOCK>();
		const float2 *Z = stockham32_team<BLOCK>(a.fft, a.tw32, x, y, t, T);
		for (int k = t; k < n; k += T) {
			const float2 zk = Z[k];
			float e;
			if (dnls) {
				e = fmaf(zk.x, zk.x, zk.y * zk.y);
			} else {
				const float2 zm = Z[k ? n - k : 0];
				const float ak = a.coef32[k], bk = a.coef32[n + k];
				const float re = fmaf(ak, zk.x, bk * zm.x), im = fmaf(ak, zk.y, -(bk * zm.y));
				e = fmaf(re, re, im * im);
			}
			acc[k] += (double) e;
		}
		team_sync<BLOCK>();
	}
}

// dDNKG projection: a block takes CH chains at a time; thread k of a block of modes accumulates
// sum_c (omega_k e_k.phi_c)^2 + (e_k.pi_c)^2 over its chains.  The chains' sites pass through shared
// memory in chunks of a.proj_chunk (whole chains when they fit), the eigenvector matrix is read
// site-major (a warp reads 32 consecutive modes of one site), and each block accumulates into its
// own row of partial sums in global memory.  Sums over sites run in site order for every length.
constexpr int kProjChains = 8;

__global__ void lin_ddnkg_kernel(const double2 *__restrict__ state, const DiagArgs a) {
	extern __shared__ double2 sm[];
	const int n = int(a.n), SC = a.proj_chunk;
	double2 *tile = sm;   // [CH][SC]
	double *acc = a.partials + (size_t) blockIdx.x * n;
	for (int k = threadIdx.x; k < n; k += blockDim.x) acc[k] = 0.;
	for (unsigned long long base = (unsigned long long) blockIdx.x * kProjChains; base < a.copies;
	     base += (unsigned long long) gridDim.x * kProjChains) {
		for (int kb = 0; kb < n; kb += blockDim.x) {
			const int k = kb + threadIdx.x;
			double dphi[kProjChains], dpi[kProjChains];
#pragma unroll
			for (int c = 0; c < kProjChains; c++) dphi[c] = 0., dpi[c] = 0.;
			for (int s0 = 0; s0 < n; s0 += SC) {
				const int cs = min(SC, n - s0);
				__syncthreads();
				for (int i = threadIdx.x; i < kProjChains * cs; i += blockDim.x) {
					const int c = i / cs, sl = i - c * cs;
					const unsigned long long ch = base + c;
					tile[c * SC + sl] = ch < a.copies ? state[ch * n + s0 + sl] : make_double2(0., 0.);
				}
				__syncthreads();
				if (k < n) {
					for (int sl = 0; sl < cs; sl++) {
						const double e = a.eigT[(size_t) (s0 + sl) * n + k];
#pragma unroll
						for (int c = 0; c < kProjChains; c++) {
							const double2 v = tile[c * SC + sl];
							dphi[c] = dfma(v.x, e, dphi[c]);
							dpi[c] = dfma(v.y, e, dpi[c]);
						}
					}
				}
			}
			if (k < n) {
				const double om = a.omega[k];
				double s = acc[k];
#pragma unroll
				for (int c = 0; c < kProjChains; c++) {
					const double v = fmul(om, dphi[c], a.fft.k1);
					s = fadd(s, dfma(v, v, fmul(dpi[c], dpi[c], a.fft.k1)), a.fft.k1);
				}
				acc[k] = s;
			}
		}
	}
}

// Seeded initial ensembles on the device, the recipes of nlchains_gb300/ic.py: uniform phases from
// SplitMix64 counters keyed by (seed, stream, copy, mode) (G. Steele, D. Lea, C. Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014), amplitudes from the energy (or norm)
// density spread equally over the excited modes, then one inverse transform per chain:
//   real models: z_k = A e^{i theta}, Phi_k = (z_k + conj z_{n-k}) / (2 omega_k), Pi_k =
//     (z_k - conj z_{n-k}) / (2i); both have Hermitian spectra, so the inverse transform of
//     Phi + i Pi is phi + i pi, the planar state itself;
//   DNLS: psi_hat_k = A e^{i theta}, psi = inverse transform;
//   dDNKG: phi = sum_k A cos(theta) / omega_k e_k, pi = sum_k A sin(theta) e_k over the excited
//     eigenmodes (eigenvectors read site-major from the diagnostics tables).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
	unsigned long long z = x + 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

// uniform [0, 1) of counter (key, copy, index) with `count` indices per copy, as ic.uniform
__device__ __forceinline__ double ic_uniform(unsigned long long key, unsigned long long copy, unsigned int count,
                                             unsigned int index) {
	return double(splitmix64(key + copy * count + index) >> 11) * (1.0 / 9007199254740992.0);
}

template <bool BLOCK>
__global__ void ic_kernel(double2 *__restrict__ state, const DiagArgs a, const IcArgs c) {
	extern __shared__ double2 sm[];
	const int n = int(a.n);
	const int T = BLOCK ? blockDim.x : 32;
	const int t = BLOCK ? threadIdx.x : (threadIdx.x & 31);
	const int team = BLOCK ? 0 : (threadIdx.x >> 5);
	const int teams = BLOCK ? 1 : (blockDim.x >> 5);
	const int len = a.fft.len;
	double2 *x = BLOCK && a.gscratch ? a.gscratch + (size_t) blockIdx.x * 2 * len : sm + (size_t) team * 2 * len;
	double2 *y = x + len;
	for (unsigned long long chain = (unsigned long long) blockIdx.x * teams + team; chain < a.copies;
	     chain += (unsigned long long) gridDim.x * teams) {
		const unsigned long long copy = c.first_copy + chain;
		double2 *dst = state + chain * (unsigned long long) n;
		if (a.model == NLC_DDNKG) {
			// the excited eigenmodes' amplitudes into the team's nmodes slots, then each site sums them
			double2 *amp = sm + (size_t) team * c.nmodes;
			for (int j = t; j < int(c.nmodes); j += T) {
				const int k = c.modes[j];
				double s, co;
				sincospi(2. * ic_uniform(c.key, copy, n, k), &s, &co);
				amp[j] = make_double2(c.amp * co / a.omega[k], c.amp * s);
			}
			team_sync<BLOCK>();
			for (int site = t; site < n; site += T) {
				double p = 0., q = 0.;
				for (int j = 0; j < int(c.nmodes); j++) {
					const double e = a.eigT[(size_t) site * n + c.modes[j]];
					p = fma(amp[j].x, e, p), q = fma(amp[j].y, e, q);
				}
				dst[site] = make_double2(p, q);
			}
			team_sync<BLOCK>();
			continue;
		}
		for (int k = t; k < n; k += T) x[k] = make_double2(0., 0.);
		team_sync<BLOCK>();
		for (int j = t; j < int(c.nmodes); j += T) {
			const int k = c.modes[j];
			double s, co;
			sincospi(2. * ic_uniform(c.key, copy, n, k), &s, &co);
			x[k] = make_double2(c.amp * co, c.amp * s);
		}
		team_sync<BLOCK>();
		double2 *w = x;
		if (a.model != NLC_DNLS) {
			// Phi + i Pi from z: Phi_k = (z_k + conj z_{n-k}) / (2 omega_k), Pi_k = (z_k - conj z_{n-k}) / (2i)
			for (int k = t; k < n; k += T) {
				const double2 zk = x[k], zc = make_double2(x[k ? n - k : 0].x, -x[k ? n - k : 0].y);
				const double om = a.omega[k];
				const double2 ph = om > 0 ? make_double2((zk.x + zc.x) / (2 * om), (zk.y + zc.y) / (2 * om))
				                          : make_double2(0., 0.);
				const double2 pk = make_double2((zk.y - zc.y) / 2, -(zk.x - zc.x) / 2);   // (z - zc) / (2i)
				y[k] = make_double2(ph.x - pk.y, ph.y + pk.x);                           // Phi + i Pi
			}
			team_sync<BLOCK>();
			w = y;
		}
		double2 *o = w == x ? y : x;
		const double2 *r = fft_team<BLOCK, true>(a.fft, w, o, t, T);
		const double inv_n = 1. / n;
		for (int k = t; k < n; k += T) dst[k] = make_double2(r[k].x * inv_n, r[k].y * inv_n);
		team_sync<BLOCK>();
	}
}

cudaError_t launch_initial_state(const DiagArgs &a, const IcArgs &c, double2 *state, int blocks, int threads,
                                 size_t smem, int team_block, cudaStream_t stream) {
	// dDNKG: warp teams, shared memory for the excited modes' amplitudes; otherwise the transform's
	// teams and buffers of the diagnostics
	const bool block = a.model != NLC_DDNKG && team_block;
	if (a.model == NLC_DDNKG) threads = 128, smem = 4 * size_t(c.nmodes) * sizeof(double2);
	const void *k = block ? (const void *) ic_kernel<true> : (const void *) ic_kernel<false>;
	if (smem > 48 * 1024) {
		const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
		if (e != cudaSuccess) return e;
	}
	count_launch();
	if (block) ic_kernel<true><<<blocks, threads, smem, stream>>>(state, a, c);
	else ic_kernel<false><<<blocks, threads, smem, stream>>>(state, a, c);
	return cudaGetLastError();
}

cudaError_t launch_linenergies_partials(const DiagArgs &a, const void *state, int blocks, int threads,
                                        size_t smem, int team_block, cudaStream_t stream) {
	const double2 *st = static_cast<const double2 *>(state);
	count_launch();
	if (a.model == NLC_DDNKG) {
		lin_ddnkg_kernel<<<blocks, threads, smem, stream>>>(st, a);
	} else if (a.tw32) {
		if (team_block) lin_fft32_kernel<true><<<blocks, threads, smem / 2, stream>>>(st, a);
		else lin_fft32_kernel<false><<<blocks, threads, smem / 2, stream>>>(st, a);
	} else if (team_block) {
		lin_fft_kernel<true><<<blocks, threads, smem, stream>>>(st, a);
	} else {
		lin_fft_kernel<false><<<blocks, threads, smem, stream>>>(st, a);
	}
	return cudaGetLastError();
}

// Single block: sum the partial rows in a fixed order, normalise, entropies.  For n <= 1024 the
// rows are split into 1024/n interleaved slices (thread t: mode t % n, slice t / n, coalesced
// reads), the slices are then added in slice order; the result is identical on every run.
constexpr int kFinishThreads = 1024;

__device__ __forceinline__ void finish_mode(const FinishArgs &a, int k, double v, double &se, double &sl,
                                            double &sel, int &cnt) {
	if (a.model == NLC_DNLS) v = dmul(v, a.omega[k]);
	if (a.a0is0 && k == 0) v = 0.;
	v = dmul(v, a.norm);
	a.lin[k] = v;
	if ((!a.mask || a.mask[k]) && !(a.a0is0 && k == 0)) {
		const double lv = log(v);
		se = dadd(se, v), sl = dadd(sl, lv), sel = dfma(v, lv, sel);
		cnt++;
	}
}

__global__ void __launch_bounds__(kFinishThreads) lin_finish_kernel(const FinishArgs a) {
	__shared__ double r_e[kFinishThreads], r_l[kFinishThreads], r_el[kFinishThreads];
	__shared__ int r_c[kFinishThreads];
	const int t = threadIdx.x;
	const int n = int(a.n);
	double se = 0., sl = 0., sel = 0.;
	int cnt = 0;
	if (n <= kFinishThreads) {
		const int slices = kFinishThreads / n;
		const int k = t % n, sidx = t / n;
		double v = 0.;
		if (sidx < slices)
			for (int r = sidx; r < a.nblocks; r += slices) v = dadd(v, a.partials[(size_t) r * n + k]);
		r_e[t] = v;
		__syncthreads();
		if (t < n) {
			double tot = 0.;
			for (int q = 0; q < slices; q++) tot = dadd(tot, r_e[q * n + t]);
			finish_mode(a, t, tot, se, sl, sel, cnt);
		}
		__syncthreads();
	} else {
		for (int k = t; k < n; k += kFinishThreads) {
			double v = 0.;
			for (int r = 0; r < a.nblocks; r++) v = dadd(v, a.partials[(size_t) r * n + k]);
			finish_mode(a, k, v, se, sl, sel, cnt);
		}
	}
	r_e[t] = se, r_l[t] = sl, r_el[t] = sel, r_c[t] = cnt;
	__syncthreads();
	for (int w = kFinishThreads / 2; w > 0; w >>= 1) {
		if (t < w) {
			r_e[t] = dadd(r_e[t], r_e[t + w]);
			r_l[t] = dadd(r_l[t], r_l[t + w]);
			r_el[t] = dadd(r_el[t], r_el[t + w]);
			r_c[t] += r_c[t + w];
		}
		__syncthreads();
	}
	if (t == 0 && a.entropies) {
		const double modes = r_c[0];
		const double normalization = modes / r_e[0], lognorm = log(normalization);
		a.entropies[0] = -(r_l[0] + modes * lognorm);
		a.entropies[1] = normalization * (r_el[0] + lognorm * r_e[0]);
	}
}

// Long chains: the row sums of 256 modes per block (coalesced over the modes, rows in order), the
// normalisation and the block's entropy sums {sum e, sum log e, sum e log e, count} in a fixed
// tree; then one block adds the blocks' sums in order and forms the entropies.
__global__ void __launch_bounds__(kFinishModesPerBlock) lin_finish_modes_kernel(const FinishArgs a) {
	__shared__ double r_e[kFinishModesPerBlock], r_l[kFinishModesPerBlock], r_el[kFinishModesPerBlock];
	__shared__ int r_c[kFinishModesPerBlock];
	const int t = threadIdx.x, k = blockIdx.x * kFinishModesPerBlock + t;
	double se = 0., sl = 0., sel = 0.;
	int cnt = 0;
	if (k < (int) a.n) {
		double v = 0.;
		for (int r = 0; r < a.nblocks; r++) v = dadd(v, a.partials[(size_t) r * a.n + k]);
		finish_mode(a, k, v, se, sl, sel, cnt);
	}
	r_e[t] = se, r_l[t] = sl, r_el[t] = sel, r_c[t] = cnt;
	__syncthreads();
	for (int w = kFinishModesPerBlock / 2; w > 0; w >>= 1) {
		if (t < w) {
			r_e[t] = dadd(r_e[t], r_e[t + w]);
			r_l[t] = dadd(r_l[t], r_l[t + w]);
			r_el[t] = dadd(r_el[t], r_el[t + w]);
			r_c[t] += r_c[t + w];
		}
		__syncthreads();
	}
	if (t == 0) {
		double *o = a.block_sums + 4 * (size_t) blockIdx.x;
		o[0] = r_e[0], o[1] = r_l[0], o[2] = r_el[0], o[3] = r_c[0];
	}
}

__global__ void lin_finish_entropy_kernel(const FinishArgs a, int blocks) {
	if (threadIdx.x != 0 || !a.entropies) return;
	double se = 0., sl = 0., sel = 0., modes = 0.;
	for (int b = 0; b < blocks; b++) {
		const double *o = a.block_sums + 4 * (size_t) b;
		se = dadd(se, o[0]), sl = dadd(sl, o[1]), sel = dadd(sel, o[2]), modes = dadd(modes, o[3]);
	}
	const double normalization = modes / se, lognorm = log(normalization);
	a.entropies[0] = -(sl + modes * lognorm);
	a.entropies[1] = normalization * (sel + lognorm * se);
}

// Pre-reduction of many partial rows: block (x, y) adds rows [y per_slice, (y + 1) per_slice) of
// the modes of tile x in row order, so that the finish reads one row per slice.  Every sum keeps a
// fixed order: the result is identical on every run.
__global__ void lin_rows_kernel(const double *__restrict__ partials, int rows, uint32_t n, int per_slice,
                                double *__restrict__ out) {
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	const int r0 = int(blockIdx.y) * per_slice, r1 = min(rows, r0 + per_slice);
	double v = 0.;
	for (int r = r0; r < r1; r++) v = dadd(v, partials[(size_t) r * n + k]);
	out[(size_t) blockIdx.y * n + k] = v;
}

constexpr int kRowsPerSliceMin = 8;

int finish_row_slices(uint32_t n, int rows, int sms) {
	if (rows < 8 * kRowsPerSliceMin) return 0;
	const int tiles = int((n + kFinishModesPerBlock - 1) / kFinishModesPerBlock);
	const int want = (2 * sms + tiles - 1) / tiles;   // about two blocks per SM
	const int slices = std::min(want, (rows + kRowsPerSliceMin - 1) / kRowsPerSliceMin);
	return slices >= 2 ? slices : 0;
}

cudaError_t launch_linenergies_finish(const FinishArgs &in, cudaStream_t stream) {
	FinishArgs a = in;
	if (a.row_slices && a.row_slice_cap >= 2 && a.nblocks >= 8 * kRowsPerSliceMin) {
		const int per_slice = (a.nblocks + a.row_slice_cap - 1) / a.row_slice_cap;
		const int slices = (a.nblocks + per_slice - 1) / per_slice;
		const int threads = int(std::min<uint32_t>(kFinishModesPerBlock, (a.n + 31) / 32 * 32));
		count_launch();
		lin_rows_kernel<<<dim3((a.n + threads - 1) / threads, slices), threads, 0, stream>>>(a.partials, a.nblocks, a.n,
		                                                                                   per_slice, a.row_slices);
		a.partials = a.row_slices;
		a.nblocks = slices;
	}
	if (a.block_sums && a.n > (uint32_t) kFinishModesPerBlock) {
		const int blocks = int((a.n + kFinishModesPerBlock - 1) / kFinishModesPerBlock);
		count_launch(2);
		lin_finish_modes_kernel<<<blocks, kFinishModesPerBlock, 0, stream>>>(a);
		lin_finish_entropy_kernel<<<1, 32, 0, stream>>>(a, blocks);
		return cudaGetLastError();
	}
	count_launch();
	lin_finish_kernel<<<1, kFinishThreads, 0, stream>>>(a);
	return cudaGetLastError();
}

// FP64 FMA probe: 8 independent chains per thread, 4x unrolled; one FMA = 2 flops.
__global__ void fp64_probe_kernel(double *out, int iters, double a, double b) {
	double x[8];
#pragma unroll
	for (int j = 0; j < 8; j++) x[j] = threadIdx.x * 1e-3 + j;
#pragma unroll 4
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int j = 0; j < 8; j++) x[j] = dfma(x[j], a, b);
	}
	double s = 0.;
#pragma unroll
	for (int j = 0; j < 8; j++) s += x[j];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream) {
	count_launch();
	fp64_probe_kernel<<<blocks, threads, 0, stream>>>(out, iters, 0.999999, 1e-7);
	return cudaGetLastError();
}

}  // namespace nlc

namespace nlc {
const void *lin32_kernel_ptr(int team_block) {
	return team_block ? (const void *) lin_fft32_kernel<true> : (const void *) lin_fft32_kernel<false>;
}
const void *lin_kernel_ptr(int model, int team_block) {
	if (model == NLC_DDNKG) return (const void *) lin_ddnkg_kernel;
	return team_block ? (const void *) lin_fft_kernel<true> : (const void *) lin_fft_kernel<false>;
}
}  // namespace nlc
