// Register-resident Yoshida integrator for the real-valued models (DNKG, FPUT, Toda, dDNKG).
//
// Replaces the reference's three GPU tiers (move_chain_in_thread / move_chain_in_warp / move_split,
// DNKG_FPUT_Toda.cu:82-259, dDNKG.cu:25-196) with one kernel family:
//
// * a chain of n sites is spread over G lanes (G a power of two, 1 .. 1024), each lane holding E or
//   E - 1 consecutive sites in registers (E a compile-time constant 2..16, so arrays index
//   statically), the first n - G(E - 1) lanes holding E -- the reference's warp layout
//   (DNKG_FPUT_Toda.cu:94-106) generalised to any group width;
// * groups of G <= 32 lanes exchange halos with width-G shuffles; for G > 32 one block holds one
//   chain and warp-boundary halos go through double-buffered shared memory, one barrier per exchange;
// * the grid is persistent: each block takes units of work (one chain per group) from a
//   self-resetting device counter, which balances the FP64 pipes of all SMs to within one unit;
// * a batched launch packs several ensembles of one kernel class (model, constants, G, E) into the
//   same persistent grid through a device table (BatchJob): units are numbered across the table and
//   each block looks up the ensemble of its unit, so small requests share the GPU without extra
//   launches and every chain still sees exactly the arithmetic of a launch of its own;
// * bond-based forces (FPUT, Toda) compute each bond once: a lane computes its own right bonds and
//   receives the left bond of its first site from its left neighbour by shuffle, instead of
//   recomputing it as the reference's RHS constructor does;
// * every FP64 operation is an explicit round-to-nearest intrinsic in the order the CPU oracle
//   replays (oracle/nlc_oracle.c, move_chain_device); adds and products are issued as FMAs with
//   parameter-bank constants (bit-identical, faster issue on GB300, see nlc_device.cuh).
//
// FP64 operations per site and sub-step (GB300 is FP64-pipe bound, see nlc_device.cuh):
//   DNKG / dDNKG 6 (5 with beta == 1), FPUT 7 (6 with alpha == 0 and beta == 1),
//   Toda 13 (12 with 2 alpha == 1) including the 8-operation table exp.
#pragma once

#include <type_traits>

#include "nlc_device.cuh"
#include "nlc_internal.h"

namespace nlc {

// Halo exchange around the ring of G lanes that hold one chain.  SHFL: G <= 32, the whole ring in
// one warp (width-G shuffles); otherwise warp-boundary halos go through shared memory.  The kernel
// picks the form once per launch, outside the step loop, so that for SHFL the seven sub-steps of a
// step are one straight-line block the compiler can schedule across.
struct Ring {
	int G;          // lanes per chain
	int lane;       // lane index within the chain
	int wl;         // lane index within the warp
	int warp;       // warp index within the block (G > 32 only)
	int W;          // warps per chain (G > 32 only)
	double *xbuf;   // 2 parities x 2 directions x W doubles (G > 32 only)
	int parity;

	// value of lane (lane - 1) mod G
	template <bool SHFL>
	__device__ __forceinline__ double from_left(double v) {
		if constexpr (SHFL) return __shfl_sync(0xffffffffu, v, (lane + G - 1) & (G - 1), G);
		double a = __shfl_sync(0xffffffffu, v, (wl + 31) & 31);
		double *buf = xbuf + parity * 2 * W;
		if (wl == 31) buf[warp] = v;
		__syncthreads();
		if (wl == 0) a = buf[(warp + W - 1) % W];
		parity ^= 1;
		return a;
	}

	// value of lane (lane + 1) mod G
	template <bool SHFL>
	__device__ __forceinline__ double from_right(double v) {
		if constexpr (SHFL) return __shfl_sync(0xffffffffu, v, (lane + 1) & (G - 1), G);
		double a = __shfl_sync(0xffffffffu, v, (wl + 1) & 31);
		double *buf = xbuf + parity * 2 * W + W;
		if (wl == 0) buf[warp] = v;
		__syncthreads();
		if (wl == 31) a = buf[(warp + 1) % W];
		parity ^= 1;
		return a;
	}

	// both directions with a single barrier: left <- lane-1's `to_right`, right <- lane+1's `to_left`
	template <bool SHFL>
	__device__ __forceinline__ void both(double to_right, double to_left, double &left, double &right) {
		if constexpr (SHFL) {
			left = __shfl_sync(0xffffffffu, to_right, (lane + G - 1) & (G - 1), G);
			right = __shfl_sync(0xffffffffu, to_left, (lane + 1) & (G - 1), G);
			return;
		}
		left = __shfl_sync(0xffffffffu, to_right, (wl + 31) & 31);
		right = __shfl_sync(0xffffffffu, to_left, (wl + 1) & 31);
		double *buf = xbuf + parity * 2 * W;
		if (wl == 31) buf[warp] = to_right;
		if (wl == 0) buf[W + warp] = to_left;
		__syncthreads();
		if (wl == 0) left = buf[(warp + W - 1) % W];
		if (wl == 31) right = buf[W + (warp + 1) % W];
		parity ^= 1;
	}
};

// Bond force term V'(d) of the bond-based models.
template <int MODEL, int VAR>
__device__ __forceinline__ double bond_force(double d, const RealArgs &a, const double *tab) {
	if constexpr (MODEL == NLC_FPUT) {
		// d + alpha d^2 + beta d^3 = d * (1 + d * (alpha + beta d))
		const double h = VAR ? d : dfma(a.beta, d, a.alpha);
		const double w = dfma(h, d, a.k1.one);
		return fmul(d, w, a.k1);
	} else {
		// (exp(2 alpha d) - 1) / (2 alpha) up to the constant, which cancels in g[s] - g[s-1]
		return exp_scaled(VAR ? d : fmul(a.alpha2, d, a.k1), tab, a.k1, a.ek);
	}
}

template <int MODEL, int E, int VAR, bool WIN>
__global__ void real_move_kernel_t(double2 *__restrict__ state, const RealArgs a) {
	__shared__ double xbuf[4 * 32];
	__shared__ double s_tab[MODEL == NLC_TODA ? kExpTable : 1];
	__shared__ unsigned long long s_unit;
	__shared__ int s_job;

	const int G = a.lanes;
	const int tid = threadIdx.x;
	const int lane = tid & (G - 1);
	const int gib = tid / G;                 // group (chain) in block
	const int gpb = blockDim.x / G;          // groups per block

	Ring ring{G, lane, tid & 31, tid >> 5, G > 32 ? G >> 5 : 1, xbuf, 0};

	if constexpr (MODEL == NLC_TODA) {
		for (int i = tid; i < kExpTable; i += blockDim.x) s_tab[i] = a.exptab[i];
	}

	// the ensemble of the current unit: the launch's own, or one entry of the batch table
	int cur_job = -1;
	double2 *st = state;
	uint32_t n = a.n, copies = a.copies, steps = a.steps, seg = a.seg;
	const double *mp2_site = a.mp2_site;
	unsigned long long unit_base = 0;
	int full = 0, ne = 0, first = 0;
	bool fl = false;
	double mv[MODEL == NLC_DDNKG ? E : 1];
	constexpr bool windowed = WIN;
	auto layout = [&]() {
		// lanes [0, full) hold E sites, the others E - 1 (a window: G E sites, every lane E)
		full = int(windowed ? a.win_len : n) - G * (E - 1);
		fl = lane < full;
		ne = fl ? E : E - 1;
		first = fl ? lane * E : full * E + (lane - full) * (E - 1);
		if constexpr (MODEL == NLC_DDNKG) {
			if (!windowed) {
#pragma unroll
				for (int j = 0; j < E; j++) mv[j] = j < ne ? mp2_site[first + j] : 2.;
			}
		}
	};
	if (!a.batch) layout();

	const unsigned long long units =
	    a.batch ? a.batch_units
	            : ((windowed ? (unsigned long long) copies * a.win_count : (unsigned long long) copies) + gpb - 1) / gpb;
	for (;;) {
		__syncthreads();
		if (tid == 0) {
			const unsigned long long u = atomicAdd(&a.work_counter[0], 1ull);
			s_unit = u;
			if (a.batch && u < units) {
				// last table entry whose first unit is <= u
				int lo = 0, hi = a.nbatch - 1;
				while (lo < hi) {
					const int mid = (lo + hi + 1) >> 1;
					if (a.batch[mid].unit_begin <= u) lo = mid;
					else hi = mid - 1;
				}
				s_job = lo;
			}
		}
		__syncthreads();
		const unsigned long long u = s_unit;
		if (u >= units) break;
		if (a.batch && s_job != cur_job) {
			cur_job = s_job;
			const BatchJob &J = a.batch[cur_job];
			st = J.state, n = J.n, copies = J.copies, steps = J.steps, mp2_site = J.mp2_site, seg = J.seg;
			unit_base = J.unit_begin;
			layout();
		}

		unsigned long long chain = (u - unit_base) * gpb + gib;
		uint32_t win = 0, wsite = 0;   // windowed: window index, chain site of this lane's first site
		if (windowed) {
			const unsigned long long item = chain;
			chain = item / a.win_count;
			win = uint32_t(item - chain * a.win_count);
			// the window starts win_halo sites before its interior; n > win_len >= first + E
			wsite = uint32_t((win * (unsigned long long) a.win_inner + n - a.win_halo + first) % n);
		}
		const bool active = chain < copies;
		if (!active) chain = copies - 1;   // redundant work keeps shuffles and barriers convergent
		double2 *cp = st + chain * (unsigned long long) n + (windowed ? 0 : first);

		double x[E + 2], p[E];
#pragma unroll
		for (int j = 0; j < E; j++) {
			uint32_t sj = j;
			if (windowed) {
				sj = wsite + j;
				if (sj >= n) sj -= n;
				if constexpr (MODEL == NLC_DDNKG) mv[j] = mp2_site[sj];
			}
			if (j < ne) {
				const double2 v = cp[sj];
				x[j + 1] = v.x, p[j] = v.y;
			} else {
				x[j + 1] = 0., p[j] = 0.;
			}
		}

		const double cd_lead = (seg & NLC_SEG_CONTINUE) ? a.cd0_merged : a.cd[0];
		auto integrate = [&](auto shfl_tag) {
		constexpr bool SHFL = decltype(shfl_tag)::value;
		uint32_t rpos = 0;   // steps of the current round done (fused rounds, a.round_steps)
		for (uint32_t i = 0; i < steps; i++) {
			// a round boundary inside the launch: the closing drift of the round just done, then the
			// next round's leading drift unmerged, as between two launches
			const bool boundary = a.round_steps && rpos == a.round_steps;
			if (boundary) {
				rpos = 0;
#pragma unroll
				for (int j = 0; j < E; j++) x[j + 1] = dfma(a.cd_final, p[j], x[j + 1]);
			}
			rpos++;
#pragma unroll
			for (int k = 0; k < 7; k++) {
				// the trailing drift of step i-1 (c[7]) merged with the leading drift of step i (c[0])
				const double cd = k == 0 ? (i == 0 ? cd_lead : boundary ? a.cd[0] : a.cd0_merged) : a.cd[k];
#pragma unroll
				for (int j = 0; j < E; j++) x[j + 1] = dfma(cd, p[j], x[j + 1]);

				if constexpr (MODEL == NLC_DNKG || MODEL == NLC_DDNKG) {
					double l, r;
					ring.template both<SHFL>(fl ? x[E] : x[E - 1], x[1], l, r);
					x[0] = l, x[E + 1] = r;
					if (!fl) x[E] = r;
#pragma unroll
					for (int j = 1; j <= E; j++) {
						const double c = x[j];
						const double bc = VAR ? c : fmul(a.beta, c, a.k1);
						double mp2x;
						if constexpr (MODEL == NLC_DDNKG) mp2x = mv[j - 1];
						else mp2x = a.mp2;
						const double t = dfma(bc, c, mp2x);
						const double uu = dfma(c, t, -x[j - 1]);
						const double v = fsub(uu, x[j + 1], a.k1);
						p[j - 1] = dfma(a.nck[k], v, p[j - 1]);
					}
				} else {
					const double r = ring.template from_right<SHFL>(x[1]);
					x[E + 1] = r;
					if (!fl) x[E] = r;
					double g[E + 1];
#pragma unroll
					for (int j = 1; j <= E; j++) g[j] = bond_force<MODEL, VAR>(fsub(x[j + 1], x[j], a.k1), a, s_tab);
					g[0] = ring.template from_left<SHFL>(fl ? g[E] : g[E - 1]);
#pragma unroll
					for (int j = 1; j <= E; j++) p[j - 1] = dfma(a.ck[k], fsub(g[j], g[j - 1], a.k1), p[j - 1]);
				}
				if (!fl) p[E - 1] = 0.;   // the slot past a short lane's last site stays inert
			}
		}
		};
		if (G <= 32) integrate(std::true_type{});
		else integrate(std::false_type{});

		if (active) {
			const bool open = seg & NLC_SEG_OPEN;
			double2 *dst = cp;
			uint32_t lo = 0, hi = E;   // window offsets of the interior, relative to this lane's first site
			if (windowed) {
				dst = a.win_out + chain * (unsigned long long) n;
				const uint32_t inner = min(a.win_inner, n - win * a.win_inner);
				lo = a.win_halo > uint32_t(first) ? a.win_halo - first : 0;
				hi = a.win_halo + inner > uint32_t(first) ? a.win_halo + inner - first : 0;
			}
#pragma unroll
			for (int j = 0; j < E; j++) {
				uint32_t sj = j;
				if (windowed) {
					sj = wsite + j;
					if (sj >= n) sj -= n;
				}
				if (j < ne && uint32_t(j) >= lo && uint32_t(j) < hi)
					dst[sj] = make_double2(open ? x[j + 1] : dfma(a.cd_final, p[j], x[j + 1]), p[j]);
			}
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

// Kernel table of one model: [variant][E], and the windowed tier's kernels for a few E (the window
// bookkeeping costs registers, so it has its own instantiations)
template <int MODEL>
struct RealKernels {
	using K = void (*)(double2 *, const RealArgs);
	template <int E, bool WIN = false>
	static constexpr K get(int variant) {
		return variant ? real_move_kernel_t<MODEL, E, 1, WIN> : real_move_kernel_t<MODEL, E, 0, WIN>;
	}
	// Two halves of about equal compile time, so that a model whose kernels take long to compile can
	// build them in two translation units: lanes of 2..13 sites and 4-site windows; lanes of 14..16
	// sites and the wider windows
	static bool is_short(int e, bool win) { return win ? e == 4 : e <= 13; }
	static K lookup_short(int variant, int e, bool win) {
		if (win) return e == 4 ? get<4, true>(variant) : nullptr;
		switch (e) {
			case 2: return get<2>(variant);
			case 3: return get<3>(variant);
			case 4: return get<4>(variant);
			case 5: return get<5>(variant);
			case 6: return get<6>(variant);
			case 7: return get<7>(variant);
			case 8: return get<8>(variant);
			case 9: return get<9>(variant);
			case 10: return get<10>(variant);
			case 11: return get<11>(variant);
			case 12: return get<12>(variant);
			case 13: return get<13>(variant);
			default: return nullptr;
		}
	}
	static K lookup_long(int variant, int e, bool win) {
		if (win) {
			switch (e) {
				case 8: return get<8, true>(variant);
				case 12: return get<12, true>(variant);
				case 14: return get<14, true>(variant);
				case 16: return get<16, true>(variant);
				default: return nullptr;
			}
		}
		switch (e) {
			case 14: return get<14>(variant);
			case 15: return get<15>(variant);
			case 16: return get<16>(variant);
			default: return nullptr;
		}
	}
	static K lookup(int variant, int e, bool win) {
		return is_short(e, win) ? lookup_short(variant, e, win) : lookup_long(variant, e, win);
	}
};

}  // namespace nlc
