// dDNKG linear-mode projection on the tensor cores (tcgen05, sm_103a), FP64-accurate.
//
// The projection is a matrix product: with X the 2C x n matrix whose rows are the chains' phi and
// pi (row 2c = phi_c, 2c + 1 = pi_c) and E the eigenvector matrix (E[k][s] = component s of mode
// k), P = X E^T and e_k = sum_c (omega_k P[2c][k])^2 + P[2c+1][k]^2 (the reference: two
// cublasDgemm + a reduction kernel, dDNKG.cpp:120-141, dDNKG.cu:237-256).  GB300's FP64 rate is a
// small fraction of its BF16 tensor rate, so the product runs as an Ozaki-type split (K. Ozaki,
// T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of matrix multiplication by using
// fast routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012):
//
//   each row of X and of E is scaled by a power of two 2^e so that |x 2^-e| < 1, then written as
//   7 slices  x 2^-e = sum_i sigma_i 2^(-8i),  sigma_i integers with |sigma_i| <= 256 (exact in
//   BF16).  P = 2^(e_r + f_k) sum_{t = 2..8} 2^(-8t) G_t,  G_t = sum_{i + j = t} A_i B_j^T.
//
// Every G_t is a sum of integer products below 2^16, accumulated in FP32 in tensor memory; it is
// read out every 256 sites of K, while the partial sums that matter are still exact (below 2^24),
// and the groups are combined exactly in integers and added in FP64.  The slices beyond t = 8 and the residual of the 7-slice truncation are
// below 2^-56 of the row and column maxima, so P carries FP64-level error.  The squares, the omega
// weights and the sum over the tile's 128 rows are fused into the epilogue; a block's column sums
// go to its row of partial sums, which the linenergies finish kernel adds in a fixed order.
//
// With 3 slices instead of 7 (NLC_FLAG_BF16X3_PROJECTION: 6 slice products, t = 2..4) the same
// kernels give P to ~2^-24 of the maxima: the precision of a three-way BF16 split, faster.
//
// One CTA: 128 rows (64 chains) x 64 modes; 8 warps.  Thread 0 drives a TMA pipeline of 5 stages
// (S = 3: 8), each 16 sites of K (32-byte swizzle: S A tiles of 128 x 16 and S B tiles of 64 x 16),
// and issues S (S + 1) / 2 tcgen05.mma (M = 128, N = 64, K = 16, BF16 in, FP32 in TMEM) per stage into
// eight accumulators: G_t, t = 2..8, with the (2,2) product of G_4 apart (8 x 64 = all 512 TMEM
// columns).  A stage is refilled one stage late (once the MMAs of the stage before the current one
// are done), so the tensor pipe always holds the current stage's MMAs queued while thread 0 waits,
// and the loads run four stages ahead.  Tiles are numbered with the 64-mode columns fastest: the
// CTAs resident at one time share row tiles, so the slices of X come from DRAM once and the
// eigenvector slices stay in L2.  Every wait is bounded: on a timeout the block records a status,
// writes NaN into its partial row (the host then sees a non-finite entropy) and returns after
// freeing its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>

#include "nlc_device.cuh"

namespace nlc {

namespace {

constexpr int kSlicesFull = 7;   // FP64-accurate; 3: the BF16x3 option (~2^-24 of the maxima)
constexpr int kBM = 128, kBN = 64, kBK = 16;
// sites of K between two read-outs of the accumulators.  With 256, G_2 <= 256 x 256^2, G_3 <= 256 x
// 2 x 256 x 128 and, the (2,2) product kept in an accumulator of its own, both parts of G_4 stay
// within 2^24, so the FP32 accumulation in tensor memory is exact for every group the result
// depends on above 2^-40; the groups t >= 5 may round in their last bit, 2^-40 below the maxima.
constexpr int kChunkK = 256;
constexpr uint32_t kTmemCols = 512;
template <int S>
__host__ __device__ constexpr uint32_t stage_a() { return S * kBM * kBK * 2; }
template <int S>
__host__ __device__ constexpr uint32_t stage_bytes() { return S * (kBM + kBN) * kBK * 2; }
// pipeline depth: 5 x 42 KB (S = 7) or 8 x 18 KB (S = 3) of dynamic shared memory
template <int S>
__host__ __device__ constexpr int stages() { return S == 3 ? 8 : 5; }
constexpr int kNonFiniteRow = 0x7fff;   // row exponent of a row holding inf or NaN

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

// Every mbarrier wait gives up after limit_ns of wall clock (%globaltimer), with an iteration cap
// as a second bound.
constexpr long long kWaitTriesMax = 1ll << 30;

__device__ __forceinline__ unsigned long long global_ns() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
	const unsigned long long t0 = global_ns();
	for (long long i = 0; i < kWaitTriesMax; i++) {
		uint32_t ok;
		asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
		             : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
		if (ok) return true;
		if (global_ns() - t0 > limit_ns) return false;
	}
	return false;
}

// The same wait with a suspend-time hint (1 us): the thread sleeps in the barrier until it completes
// or the hint elapses, leaving the issue slots to the thread that issues the loads and MMAs.
constexpr uint32_t kSleepHintNs = 1000;
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
	const unsigned long long t0 = global_ns();
	for (long long i = 0; i < kWaitTriesMax; i++) {
		uint32_t ok;
		asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
		             : "=r"(ok) : "r"(bar), "r"(parity), "r"(kSleepHintNs) : "memory");
		if (ok) return true;
		if (global_ns() - t0 > limit_ns) return false;
	}
	return false;
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the 32-byte swizzle (one
// 16-site row of BF16 per 32 bytes): 8-row atoms of 256 bytes (stride byte offset), descriptor
// version 1, layout type 6.  The tiles start on 1024-byte boundaries, so the base offset is 0 and a
// tile's descriptor is the stage's plus its byte offset / 16 (addresses stay below 2^18).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
	return (uint64_t) ((saddr & 0x3FFFF) >> 4) | ((uint64_t) 1 << 16) | ((uint64_t) (256 >> 4) << 32) |
	       ((uint64_t) 1 << 46) | ((uint64_t) 6 << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N = 64, M = 128.
constexpr uint32_t kIdesc =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (kBN >> 3) << 17) | ((uint32_t) (kBM >> 4) << 24);

__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
	             ::"r"(dst), "l"((uint64_t) map), "r"(x), "r"(y), "r"(bar) : "memory");
}

// 8 columns of this warp's 32 TMEM lanes; tmem_wait_ld() completes every load issued before it
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
	             : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// One stage's slice products: for t = 2..S + 1 the products A_i B_j^T with i + j = t into
// accumulator t - 2, the (2,2) product into accumulator S.  `first`: the chunk's first stage, whose
// first product into each accumulator overwrites it.  Unrolled: every descriptor is the stage's
// plus a constant.
template <int S>
__device__ __forceinline__ void issue_stage_mmas(uint32_t tmem, uint64_t da, uint64_t db, bool first, uint32_t idesc) {
#pragma unroll
	for (int t = 2; t <= S + 1; t++) {
		const int ilo = t - S > 1 ? t - S : 1, ihi = t - 1 < S ? t - 1 : S;
#pragma unroll
		for (int i = ilo; i <= ihi; i++) {
			const int j = t - i;
			const bool own = t == 4 && i == 2;
			const uint32_t d = tmem + (uint32_t) (own ? S : t - 2) * kBN;
			const uint64_t ad = da + (uint64_t) (((i - 1) * kBM * kBK * 2) >> 4);
			const uint64_t bd = db + (uint64_t) (((j - 1) * kBN * kBK * 2) >> 4);
			const uint32_t accum = (first && (own || i == ilo)) ? 0u : 1u;
			asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }"
			             ::"r"(d), "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
		}
	}
}

// an int64 of magnitude below 2^51 as a double, exactly: added to the bit pattern of 1.5 * 2^52 it
// lands in the low mantissa bits, and one FP64 subtraction removes the offset
__device__ __forceinline__ double i64_to_double(long long x) {
	return __longlong_as_double(x + 0x4338000000000000ll) - 0x1.8p52;
}

// 2^k for a normal-range k, built from its bit pattern (an exact scaling, no library call)
__device__ __forceinline__ double pow2i(int k) {
	return k >= -1022 && k <= 1023 ? __longlong_as_double((long long) (k + 1023) << 52) : ldexp(1., k);
}

}  // namespace

// 7 balanced base-256 digits of x 2^(56 - e) (e: the row exponent, |x| < 2^e), in integer
// arithmetic on the FP64 bit pattern: F = round(x 2^(56 - e)) is a 57-bit signed integer, and
// F = sum_i sigma_i 2^(8 (7 - i)) with sigma_1 = round(F / 2^48), sigma_2 = round((F - sigma_1 2^48)
// / 2^40), ...: |sigma_1| <= 256, the others |sigma_i| <= 128, all exact in BF16.  The slices of
// x 2^-e are sigma_i 2^(-8i): the value to 2^-48 of the row maximum, as the tensor product needs.
__device__ __forceinline__ void split7(double x, int e, uint16_t (&out)[7]) {
	const long long bits = __double_as_longlong(x);
	const int ex = int((bits >> 52) & 0x7ff);
	long long m = bits & ((1ll << 52) - 1);
	int E;
	if (ex) m |= 1ll << 52, E = ex - 1075;
	else E = -1074;
	const int shift = E + 56 - e;   // x 2^(56 - e) = m 2^shift, below 2^56 in magnitude
	long long F;
	if (shift >= 0) F = m << shift;
	else if (shift > -63) F = (m + (1ll << (-shift - 1))) >> (-shift);
	else F = 0;
	if (bits < 0) F = -F;
#pragma unroll
	for (int i = 0; i < 7; i++) {
		const int pos = 8 * (6 - i);
		const long long sg = pos ? (F + (1ll << (pos - 1))) >> pos : F;
		F -= sg << pos;
		// |sg| <= 256: exact in BF16; converted from 32 bits (a 64-bit conversion uses the FP64 pipe)
		out[i] = uint16_t(__float_as_uint(__int2float_rn(int(sg))) >> 16);
	}
}

// Split of X: one warp per chain c (rows 2c = phi, 2c + 1 = pi): the row exponents e_r (max |x| =
// m 2^e_r, 0.5 <= m < 1, from the largest magnitude's bit pattern) and the 7 slices of each row,
// into slices[i][r][s].  Integer arithmetic only (GB300 issues it ~30x faster than FP64), coalesced
// double2 reads of the state.  A row holding inf or NaN gets the exponent kNonFiniteRow, which the
// projection turns into NaN energies: a blown-up chain is reported, not hidden.
template <int S>
__global__ void tc_split_rows_kernel(const double2 *__restrict__ state, TcArgs a) {
	const unsigned long long c = (unsigned long long) blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
	const int lane = threadIdx.x & 31;
	if (c >= a.copies) return;
	const uint32_t n = a.n;
	const double2 *chain = state + c * n;
	unsigned long long mphi = 0, mpi = 0;   // |x| bit patterns: ordered like the magnitudes
	for (uint32_t s = lane; s < n; s += 32) {
		const double2 v = chain[s];
		mphi = max(mphi, (unsigned long long) __double_as_longlong(v.x) & 0x7fffffffffffffffull);
		mpi = max(mpi, (unsigned long long) __double_as_longlong(v.y) & 0x7fffffffffffffffull);
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		mphi = max(mphi, __shfl_xor_sync(0xffffffffu, mphi, o));
		mpi = max(mpi, __shfl_xor_sync(0xffffffffu, mpi, o));
	}
	auto row_exp = [](unsigned long long mb) {
		int e = 0;
		if (mb >= 0x7ff0000000000000ull) e = kNonFiniteRow;   // inf or NaN
		else if (mb >> 52) e = int(mb >> 52) - 1022;          // normal: (1.f) 2^(ex - 1023) = (0.1f) 2^(ex - 1022)
		else if (mb) frexp(__longlong_as_double((long long) mb), &e);
		return e;
	};
	const int ephi = row_exp(mphi), epi = row_exp(mpi);
	const unsigned long long r = 2 * c;
	if (lane == 0) a.row_exp[r] = ephi, a.row_exp[r + 1] = epi;
	for (uint32_t s = lane; s < n; s += 32) {
		const double2 v = chain[s];
		uint16_t sp[7], sq[7];
		split7(v.x, ephi, sp);
		split7(v.y, epi, sq);
#pragma unroll
		for (int i = 0; i < S; i++) {
			a.a_slices[((size_t) i * a.mp + r) * a.kp + s] = sp[i];
			a.a_slices[((size_t) i * a.mp + r + 1) * a.kp + s] = sq[i];
		}
	}
}

// 8 warps: warps w and w + 4 read the same 32 rows of the tile (TMEM lane quarter w mod 4), each
// one half of the 64 columns, so the FP64 read-out and epilogue work of a thread is halved and
// every scheduler has two warps to interleave
constexpr int kThreads = 256, kCols = kBN / 2;

template <int S>
__global__ void __launch_bounds__(kThreads, 1)
tc_projection_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, const TcArgs a) {
	extern __shared__ __align__(1024) unsigned char smem_raw[];
	unsigned char *smem = (unsigned char *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
	constexpr int kS = stages<S>();
	__shared__ __align__(8) unsigned long long bars[2 * kS + 2];   // full[kS], empty[kS], acc, test
	__shared__ uint32_t tmem_slot;
	__shared__ int s_fail;
	__shared__ double s_w[kBN];   // per column of the tile: omega_k^2 (weight of the phi rows)
	__shared__ int s_cexp[kBN];   // per column: the eigenvector's power-of-two exponent
	const int tid = threadIdx.x, warp = tid >> 5;
	const int rl = (warp & 3) * 32 + (tid & 31);   // this thread's row of the tile (its TMEM lane)
	const int half = warp >> 2;                    // its columns: [kCols half, kCols (half + 1))
	// tiles numbered with the column tiles fastest (see the header)
	const int col_tiles = a.np / kBN;
	const int row_tile = (int) (blockIdx.x / col_tiles), col_tile = (int) (blockIdx.x % col_tiles);
	const int row0 = row_tile * kBM, col0 = col_tile * kBN;
	const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kS]), accb = smem_u32(&bars[2 * kS]);
	if (tid == 0) {
		for (int i = 0; i < 2 * kS + 2; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[i])));
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		s_fail = 0;
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
		             "r"(kTmemCols));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
	}
	if (tid < kBN) {
		const int k = col0 + tid;
		s_w[tid] = k < (int) a.n ? a.omega[k] * a.omega[k] : 0.;
		s_cexp[tid] = k < (int) a.n ? a.col_exp[k] : 0;
	}
	// tests only: a wait that runs out (nothing arrives at the test barrier) takes the failure path
	if (a.wait_test && tid == 0 && !mbar_wait(smem_u32(&bars[2 * kS + 1]), 0, a.wait_ns)) s_fail = 1;
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;");
	const uint32_t tmem = tmem_slot;

	const int nk = a.kp / kBK;   // stages of K
	const int per_chunk = kChunkK / kBK;
	constexpr uint32_t kStageA = stage_a<S>(), kStageBytes = stage_bytes<S>();
	auto stage_ptr = [&](int s) { return smem + (size_t) s * kStageBytes; };
	int issued = 0, consumed = 0;    // thread 0: stages loaded / stages whose load has landed
	bool committed = false;          // thread 0: the current chunk's MMAs are committed to accb
	auto load_stage = [&](int it, int s) {
		issued = it + 1;
		const uint32_t full = full0 + 8 * s;
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full), "r"(kStageBytes) : "memory");
		unsigned char *base = stage_ptr(s);
		for (int i = 0; i < S; i++) {
			tma_load(smem_u32(base + (size_t) i * kBM * kBK * 2), &map_a, it * kBK, i * a.mp + row0, full);
			tma_load(smem_u32(base + kStageA + (size_t) i * kBN * kBK * 2), &map_b, it * kBK, i * a.np + col0, full);
		}
	};

	double acc[kCols];
#pragma unroll
	for (int c = 0; c < kCols; c++) acc[c] = 0.;
	const uint32_t lane_base = (uint32_t) ((warp & 3) * 32) << 16;
	int chunks = 0;
	for (int c0 = 0; c0 < nk; c0 += per_chunk, chunks++) {
		const int c1 = min(nk, c0 + per_chunk);
		if (tid == 0 && !s_fail) {
			bool ok = true;
			committed = false;
			if (c0 == 0)
				for (int it = 0; it < kS && it < nk; it++) load_stage(it, it);
			for (int it = c0; it < c1 && ok; it++) {
				const int s = it % kS;
				if (!mbar_wait(full0 + 8 * s, (it / kS) & 1, a.wait_ns)) {
					ok = false;
					break;
				}
				consumed = it + 1;
				asm volatile("tcgen05.fence::after_thread_sync;");
				const uint32_t sa = smem_u32(stage_ptr(s));
				issue_stage_mmas<S>(tmem, smem_desc(sa), smem_desc(sa + kStageA), it == c0, kIdesc);
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(empty0 + 8 * s)
				             : "memory");
				// refill the previous stage once its MMAs are done (this stage's are queued behind them)
				const int prev = it - 1;
				if (prev >= 0 && prev + kS < nk) {
					const int ps = prev % kS;
					if (!mbar_wait(empty0 + 8 * ps, (prev / kS) & 1, a.wait_ns)) {
						ok = false;
						break;
					}
					load_stage(prev + kS, ps);
				}
			}
			if (ok) {
				asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(accb)
				             : "memory");
				committed = true;
			} else {
				s_fail = 1;
			}
		}
		// every thread: wait for the chunk's MMAs, then add its groups into the FP64 row sums
		if (!s_fail && !mbar_wait_sleep(accb, chunks & 1, a.wait_ns)) s_fail = 1;
		__syncthreads();
		if (s_fail) break;
		asm volatile("tcgen05.fence::after_thread_sync;");
		// the exact integer group sums, folded with shifts into two int64 halves (hi: t = 2..4 in units
		// of 2^-32, below 2^41; lo: t = 5..8 in units of 2^-64, below 2^49: both exact in FP64), then
		// two FMAs per column into the FP64 row sums.  Accumulators are read four at a time, one wait
		// for the four loads.
		constexpr int kGroups = S + 1;   // accumulators: G_2..G_{S+1} and the (2,2) part of G_4
#pragma unroll
		for (int sg = 0; sg < kCols / 8; sg++) {
			const int seg = half * (kCols / 8) + sg;   // 8-column segment of the tile
			long long hi[8], lo[8];
#pragma unroll
			for (int j = 0; j < 8; j++) hi[j] = 0, lo[j] = 0;
#pragma unroll
			for (int g0 = 0; g0 < kGroups; g0 += 4) {
				uint32_t v[4][8];
#pragma unroll
				for (int q = 0; q < 4; q++)
					if (g0 + q < kGroups) tmem_ld8(tmem + lane_base + (uint32_t) (g0 + q) * kBN + seg * 8, v[q]);
				tmem_wait_ld();
#pragma unroll
				for (int q = 0; q < 4; q++) {
					const int grp = g0 + q;
					if (grp >= kGroups) break;
					const int tt = grp == S ? 4 : grp + 2;   // accumulator S: the (2,2) part of G_4
#pragma unroll
					for (int j = 0; j < 8; j++) {
						const long long g = __float2int_rn(__uint_as_float(v[q][j]));   // below 2^26: a 32-bit conversion
						if (tt <= 4) hi[j] += g << (8 * (4 - tt));
						else lo[j] += g << (8 * (8 - tt));
					}
				}
			}
#pragma unroll
			for (int j = 0; j < 8; j++) {
				double &x = acc[sg * 8 + j];
				x = fma(i64_to_double(hi[j]), 0x1p-32, x);
				if constexpr (S + 1 > 4) x = fma(i64_to_double(lo[j]), 0x1p-64, x);
			}
		}
		asm volatile("tcgen05.fence::before_thread_sync;");
		__syncthreads();
	}

	// epilogue: this thread's row r of P, squared and weighted, summed over the tile's rows.  The
	// buffer (over the finished stages) is column-major with a padded stride: the rows' stores and
	// the column sums' loads are both free of bank conflicts.
	constexpr int kRedStride = kBM + 1;
	static_assert(kBN * kRedStride * sizeof(double) <= (size_t) kS * kStageBytes, "reduction buffer exceeds the stages");
	static_assert((size_t) kS * kStageBytes + 1024 + 1024 <= 227 * 1024, "shared memory above 227 KB");
	double *red = reinterpret_cast<double *>(smem);   // [64][129]
	const int r = row0 + rl;
	const bool phi = (r & 1) == 0;
	const int er = r < 2 * (int) a.copies ? a.row_exp[r] : 0;
	if (!s_fail) {
#pragma unroll
		for (int c = 0; c < kCols; c++) {
			const int col = half * kCols + c;
			double p = 0., w = 1.;
			if (col0 + col < (int) a.n) {
				p = er == kNonFiniteRow ? __longlong_as_double(0x7ff8000000000000ll) : acc[c] * pow2i(er + s_cexp[col]);
				if (phi) w = s_w[col];
			}
			red[col * kRedStride + rl] = w * p * p;
		}
	}
	__syncthreads();
	if (tid < kBN) {
		const int k = col0 + tid;
		if (k < (int) a.n) {
			// four interleaved partial sums in a fixed order, then added pairwise
			const double *col = red + tid * kRedStride;
			double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
			for (int rr = 0; rr < kBM; rr += 4) s0 += col[rr], s1 += col[rr + 1], s2 += col[rr + 2], s3 += col[rr + 3];
			const double s = (s0 + s1) + (s2 + s3);
			a.partials[(size_t) row_tile * a.n + k] = s_fail ? __longlong_as_double(0x7ff8000000000000ll) : s;
		}
	}
	if (tid == 0 && s_fail) {
		// after a timeout: wait (each wait bounded again) for the loads this block issued and has not
		// consumed, then for every MMA it issued, so that nothing lands in shared memory or TMEM after
		// the block has released them
		for (int it = consumed; it < issued; it++) mbar_wait(full0 + 8 * (it % kS), (it / kS) & 1, a.wait_ns);
		if (!committed)
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(accb)
			             : "memory");
		mbar_wait(accb, chunks & 1, a.wait_ns);
		atomicOr(a.status, 1);
	}
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

size_t tc_projection_smem(int slices) {
	return slices == 3 ? (size_t) stages<3>() * stage_bytes<3>() + 1024
	                   : (size_t) stages<kSlicesFull>() * stage_bytes<kSlicesFull>() + 1024;
}

cudaError_t launch_tc_projection(const TcArgs &a, const void *map_a, const void *map_b, const double2 *state,
                                 cudaStream_t stream) {
	count_launch(2);
	const dim3 grid((unsigned) ((size_t) (a.mp / kBM) * (a.np / kBN)));
	const CUtensorMap &ma = *static_cast<const CUtensorMap *>(map_a), &mb = *static_cast<const CUtensorMap *>(map_b);
	const unsigned split_blocks = (unsigned) ((a.copies + 7) / 8);
	if (a.slices == 3) {
		tc_split_rows_kernel<3><<<split_blocks, 256, 0, stream>>>(state, a);
		tc_projection_kernel<3><<<grid, kThreads, tc_projection_smem(3), stream>>>(ma, mb, a);
	} else {
		tc_split_rows_kernel<kSlicesFull><<<split_blocks, 256, 0, stream>>>(state, a);
		tc_projection_kernel<kSlicesFull><<<grid, kThreads, tc_projection_smem(kSlicesFull), stream>>>(ma, mb, a);
	}
	return cudaGetLastError();
}

const void *tc_projection_kernel_ptr(int slices) {
	return slices == 3 ? (const void *) tc_projection_kernel<3> : (const void *) tc_projection_kernel<kSlicesFull>;
}

}  // namespace nlc
