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
// and added with shifts into two exact int64 sums per element of P: hi (t = 2..4, units of 2^-32)
// and lo (t = 5..8, units of 2^-64).  The slices beyond t = 8 and the residual of the 7-slice
// truncation are below 2^-56 of the row and column maxima, so P carries FP64-level error.  At the
// end each element's square becomes one double by an integer-only conversion (nlc_fixed.h,
// truncated to 53 bits); the omega weights and the sum over the tile's 128 rows are fused into the
// epilogue, and a block's column sums go to its row of partial sums, which the linenergies
// finish kernel adds in a fixed order.
//
// With 3 slices instead of 7 (NLC_FLAG_BF16X3_PROJECTION: 6 slice products, t = 2..4) the same
// kernels give P to ~2^-24 of the maxima: the precision of a three-way BF16 split, faster.
//
// Tile and sweeps.  A tcgen05.mma costs about 80 cycles to issue whatever its width (measured on
// GB300: N = 32 and 64 take as long as N = 128; N = 256 runs at the full tensor rate), so the MMAs
// must be wide.  Eight accumulators of N = 128 columns would need 1024 TMEM columns, twice the 512
// an SM has, so one CTA (128 rows x 128 modes, 16 warps) sweeps K twice with four accumulators:
//   sweep 0: G_2, G_3, G_4 without (2,2), and (2,2): 6 MMAs per 16-site block, slices 1..3;
//   sweep 1: G_5, G_6, G_7, G_8: 22 MMAs per block, slices 1..7.
// Between the sweeps every thread parks its hi sums in a global scratch array and takes them back
// for the conversion.  The slices are stored tiled and pre-swizzled (tc_slice_index), so each
// 16-site block of a pipeline stage is two bulk copies, one for A's slices and one for B's (sweep
// 0: 4 stages of two blocks, 48 KB; sweep 1: 3 stages of one block, 56 KB).  Thread 32 issues the
// copies, refilling a stage's buffer as soon as the MMAs that read it are done; threads 0 and 64
// issue the MMAs (M = 128, N = 128, K = 16, BF16 in, FP32 in TMEM), each for two of the four
// accumulators, as soon as a stage has landed.  Each tcgen05 or bulk-copy instruction costs the
// issuing thread tens of cycles (one thread issues N = 128 MMAs at 0.83 of the tensor rate, two
// at the full rate), so the three streams run on three threads.  Tiles are numbered with the
// 128-mode columns fastest: the CTAs resident at one time share row tiles, so the slices of X come
// from DRAM once per sweep and the eigenvector slices stay in L2.  Every wait is bounded: on a timeout the block records a status, writes NaN
// into its partial row (the host then sees a non-finite entropy) and returns after freeing its
// tensor memory.
#include <cuda_bf16.h>

#include <type_traits>

#include "nlc_device.cuh"
#include "nlc_fixed.h"

namespace nlc {

namespace {

constexpr int kSlicesFull = 7;   // FP64-accurate; 3: the BF16x3 option (~2^-24 of the maxima)
constexpr int kBM = 128, kBN = 128, kBK = 16;
// sites of K between two read-outs of the accumulators.  With 256, G_2 <= 256 x 256^2, G_3 <= 256 x
// 2 x 256 x 128 and, the (2,2) product kept in an accumulator of its own, both parts of G_4 stay
// within 2^24, so the FP32 accumulation in tensor memory is exact for every group the result
// depends on above 2^-40; the groups t >= 5 may round in their last bit, 2^-40 below the maxima.
constexpr int kChunkK = 256;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kTile = kBM * kBK * 2;   // one slice tile of A or B: 128 rows x 16 sites, 4 KB
static_assert(kBN == kBM, "A and B tiles share one size");
// slices a sweep reads, its stage size, and the stages that fit in the stage memory
__host__ __device__ constexpr int sweep_slices(int S, int sweep) { return sweep == 0 ? (S < 3 ? S : 3) : S; }
// 16-site blocks per stage: sweep 0's products are few (6 per block), so its stages hold two blocks
// and the per-stage costs (the wait, the commit) are paid once per 12 MMAs
__host__ __device__ constexpr int sweep_blocks(int sweep) { return sweep == 0 ? 2 : 1; }
__host__ __device__ constexpr uint32_t sweep_stage_bytes(int ns, int kb) { return 2u * (uint32_t) (ns * kb) * kTile; }
constexpr uint32_t kStageMem = 200 * 1024;
__host__ __device__ constexpr int sweep_stages(int ns, int kb) { return (int) (kStageMem / sweep_stage_bytes(ns, kb)); }
static_assert(sweep_stages(3, 2) == 4 && sweep_stages(7, 1) == 3, "stage geometry");
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

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
	uint32_t ok;
	asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
	             : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
	return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
	if (mbar_try(bar, parity)) return true;   // the usual case: no clock read
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
// or the hint elapses, leaving the issue slots to the threads that issue the copies and MMAs.
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

// Shared-memory matrix descriptor of a K-major tile in the 32-byte-swizzled layout that the bulk
// copies bring in (tc_slice_index; one 16-site row of BF16 per 32 bytes): 8-row atoms of 256 bytes
// (stride byte offset), descriptor version 1, layout type 6.  The tiles start on 1024-byte boundaries, so the base offset is 0 and a
// tile's descriptor is the stage's plus its byte offset / 16 (addresses stay below 2^18).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
	return (uint64_t) ((saddr & 0x3FFFF) >> 4) | ((uint64_t) 1 << 16) | ((uint64_t) (256 >> 4) << 32) |
	       ((uint64_t) 1 << 46) | ((uint64_t) 6 << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N = 128, M = 128.
constexpr uint32_t kIdesc =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (kBN >> 3) << 17) | ((uint32_t) (kBM >> 4) << 24);

// one contiguous run of global memory into shared memory (the bulk-copy engine), completing on
// the mbarrier `bar`: both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
	             ::"r"(dst), "l"((uint64_t) src), "r"(bytes), "r"(bar) : "memory");
}

// 8 columns of this warp's 32 TMEM lanes; tmem_wait_ld() completes every load issued before it
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
	             : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// One 16-site block's slice products of a sweep into its four accumulators (128 TMEM columns each):
//   sweep 0: (1,1) -> 0 (G_2), (1,2) (2,1) -> 1 (G_3), (1,3) (3,1) -> 2 (G_4 without (2,2)),
//            (2,2) -> 3;
//   sweep 1: the products of G_t, t = 5..8, into t - 5.
// Two threads issue them, each the products of two accumulators (ISSUER 0: accumulators 0 and 1 in
// sweep 0, 0 and 3 in sweep 1; ISSUER 1 the others: 3 + 3 and 11 + 11 MMAs per block).
// `first`: the chunk's first block, whose first product into each accumulator overwrites it.  In
// shared memory the block is NS A tiles, then NS B tiles (da, db: their descriptors).  Unrolled:
// every descriptor is the block's plus a constant.
template <int SWEEP>
__host__ __device__ constexpr int mma_issuer(int acc) { return SWEEP == 0 ? (acc < 2 ? 0 : 1) : (acc == 0 || acc == 3 ? 0 : 1); }

template <int S, int SWEEP, int ISSUER>
__device__ __forceinline__ void issue_sweep_mmas(uint32_t tmem, uint64_t da, uint64_t db, bool first, uint32_t idesc) {
	constexpr int t0 = SWEEP == 0 ? 2 : 5, t1 = SWEEP == 0 ? 4 : S + 1;
#pragma unroll
	for (int t = t0; t <= t1; t++) {
		const int ilo = t - S > 1 ? t - S : 1, ihi = t - 1 < S ? t - 1 : S;
#pragma unroll
		for (int i = ilo; i <= ihi; i++) {
			const int j = t - i;
			const bool own = SWEEP == 0 && t == 4 && i == 2;
			const int acc = SWEEP == 0 ? (own ? 3 : t - 2) : t - 5;
			if (mma_issuer<SWEEP>(acc) != ISSUER) continue;
			const uint32_t d = tmem + (uint32_t) acc * kBN;
			const uint64_t ad = da + (uint64_t) (((i - 1) * kTile) >> 4);
			const uint64_t bd = db + (uint64_t) (((j - 1) * kTile) >> 4);
			const uint32_t accum = (first && (own || i == ilo)) ? 0u : 1u;
			asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }"
			             ::"r"(d), "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
		}
	}
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
	// |sg| <= 256: exact in BF16; converted from 32 bits (a 64-bit conversion uses the FP64 pipe)
	auto bf16 = [](int sg) { return uint16_t(__float_as_uint(__int2float_rn(sg)) >> 16); };
#pragma unroll
	for (int i = 0; i < 4; i++) {
		const int pos = 8 * (6 - i);
		const long long sg = (F + (1ll << (pos - 1))) >> pos;
		F -= sg << pos;
		out[i] = bf16(int(sg));
	}
	// after four digits the remainder lies in [-2^23, 2^23): the rest in 32-bit arithmetic
	int f = int(F);
#pragma unroll
	for (int i = 4; i < 7; i++) {
		const int pos = 8 * (6 - i);
		const int sg = pos ? (f + (1 << (pos - 1))) >> pos : f;
		f -= sg << pos;
		out[i] = bf16(sg);
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
		// slice i lies 128 x 16 elements after slice i - 1; rows 2c and 2c + 1 share a tile and a
		// swizzle phase, so the pi row is the phi row's position plus one row
		uint16_t *dst = a.a_slices + tc_slice_index(0, (int) (s >> 4), a.mp, r, (int) (s & 15), S);
#pragma unroll
		for (int i = 0; i < S; i++) dst[i * 128 * 16] = sp[i], dst[i * 128 * 16 + 16] = sq[i];
	}
}

// 16 warps: warps w, w + 4, w + 8 and w + 12 read the same 32 rows of the tile (TMEM lane quarter
// w mod 4), each a quarter of the 128 columns: a thread's exact row sums (one int64 per column)
// fit in its 128 registers
constexpr int kWarps = 16, kThreads = 32 * kWarps, kCols = kBN / (kWarps / 4);
// lane 0 of warp 1 issues the copies; lane 0 of warps 0 and 2 issue the MMAs (one tcgen05.mma costs
// its issuing thread about 80 cycles; two issuing threads reach the full tensor rate with N = 128)
constexpr int kProducer = 32, kMma1 = 64;

template <int S>
__global__ void __launch_bounds__(kThreads, 1)
tc_projection_kernel(const TcArgs a) {
	extern __shared__ __align__(1024) unsigned char smem_raw[];
	unsigned char *smem = (unsigned char *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
	constexpr int kS0 = sweep_stages(sweep_slices(S, 0), sweep_blocks(0)), kS1 = sweep_stages(sweep_slices(S, 1), sweep_blocks(1));
	// full and empty barriers of sweep 0, then of sweep 1, then acc, test
	constexpr int kBarFull0 = 0, kBarEmpty0 = kS0, kBarFull1 = 2 * kS0, kBarEmpty1 = 2 * kS0 + kS1;
	constexpr int kBarAcc = 2 * (kS0 + kS1), kBars = kBarAcc + 2;
	__shared__ __align__(8) unsigned long long bars[kBars];
	__shared__ uint32_t tmem_slot;
	__shared__ int s_fail, s_issued;
	__shared__ double s_w[kBN];   // per column of the tile: omega_k^2 (weight of the phi rows)
	__shared__ int s_cexp[kBN];   // per column: the eigenvector's power-of-two exponent
	const int tid = threadIdx.x, warp = tid >> 5;
	const int rl = (warp & 3) * 32 + (tid & 31);   // this thread's row of the tile (its TMEM lane)
	const int part = warp >> 2;                    // its columns: [kCols part, kCols (part + 1))
	// tiles numbered with the column tiles fastest (see the header)
	const int col_tiles = a.np / kBN;
	const int row_tile = (int) (blockIdx.x / col_tiles), col_tile = (int) (blockIdx.x % col_tiles);
	const int row0 = row_tile * kBM, col0 = col_tile * kBN;
	const uint32_t accb = smem_u32(&bars[kBarAcc]);
	if (tid == 0) {
		// a full barrier completes on the producer's arrival (with the bytes); empty and acc barriers on
		// one commit from each MMA thread
		for (int i = 0; i < kBars; i++) {
			const bool two = (i >= kBarEmpty0 && i < kBarFull1) || (i >= kBarEmpty1 && i < kBarAcc) || i == kBarAcc;
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars[i])), "r"(two ? 2 : 1));
		}
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		s_fail = 0, s_issued = 0;
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
	if (a.wait_test && tid == 0 && !mbar_wait(smem_u32(&bars[kBarAcc + 1]), 0, a.wait_ns)) s_fail = 1;
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;");
	const uint32_t tmem = tmem_slot;

	const int nkb = a.kp / kBK;   // 16-site blocks of K
	// the MMA threads' bookkeeping for the failure path: the sweep's barriers and stage count, stages
	// landed (the producer's loads: s_issued), and whether the current chunk's MMAs are committed
	uint32_t cur_full = smem_u32(&bars[kBarFull0]);
	int cur_stages = kS0, consumed = 0;
	bool committed = false;
	int rounds = 0;   // chunks read out so far (both sweeps): the parity of accb's next phase

	// this thread's row of P over its columns: the current sweep's exact group sums (hi: units of
	// 2^-32, below 2^49 over 256 chunks; lo: units of 2^-64, below 2^57)
	long long acc[kCols];
#pragma unroll
	for (int c = 0; c < kCols; c++) acc[c] = 0;
	const uint32_t lane_base = (uint32_t) ((warp & 3) * 32) << 16;

	auto sweep = [&](auto sweep_tag) {
		constexpr int W = decltype(sweep_tag)::value;
		constexpr int NS = sweep_slices(S, W), KS = W == 0 ? kS0 : kS1, KB = sweep_blocks(W);
		constexpr uint32_t kStageBytes = sweep_stage_bytes(NS, KB), kBlockBytes = 2u * NS * kTile;
		const int nk = (nkb + KB - 1) / KB;      // stages of the sweep (the last one may hold one block)
		constexpr int per_chunk = kChunkK / (kBK * KB);
		const uint32_t full0 = smem_u32(&bars[W == 0 ? kBarFull0 : kBarFull1]);
		const uint32_t empty0 = smem_u32(&bars[W == 0 ? kBarEmpty0 : kBarEmpty1]);
		auto stage_ptr = [&](int s) { return smem + (size_t) s * kStageBytes; };
		// a stage: per block, NS A tiles then NS B tiles
		auto load_stage = [&](int it, int s) {   // the producer thread
			s_issued = it + 1;
			const uint32_t full = full0 + 8 * s;
			const int blocks = min(KB, nkb - it * KB);
			asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full), "r"(blocks * kBlockBytes) : "memory");
			unsigned char *base = stage_ptr(s);
			for (int b = 0; b < blocks; b++) {
				const int kb = it * KB + b;
				unsigned char *blk = base + (size_t) b * kBlockBytes;
				bulk_load(smem_u32(blk), a.a_slices + tc_slice_index(0, kb, a.mp, row0, 0, S), NS * kTile, full);
				bulk_load(smem_u32(blk + (size_t) NS * kTile), a.b_slices + tc_slice_index(0, kb, a.np, col0, 0, S), NS * kTile,
				          full);
			}
		};
		if (tid == 0) cur_full = full0, cur_stages = KS, consumed = 0;
		if (tid == kProducer) s_issued = 0;
		for (int c0 = 0; c0 < nk; c0 += per_chunk) {
			const int c1 = min(nk, c0 + per_chunk);
			if (tid == kProducer && !s_fail) {
				// the loads: the first KS stages, then stage it + KS into stage it's buffer once the
				// MMAs that read stage it are done
				bool ok = true;
				if (c0 == 0)
					for (int it = 0; it < KS && it < nk; it++) load_stage(it, it);
				for (int it = c0; it < c1 && it + KS < nk; it++) {
					const int s = it % KS;
					if (!mbar_wait(empty0 + 8 * s, (it / KS) & 1, a.wait_ns)) {
						ok = false;
						break;
					}
					load_stage(it + KS, s);
				}
				if (!ok) s_fail = 1;
			}
			if ((tid == 0 || tid == kMma1) && !s_fail) {
				// the MMAs: each stage as soon as it has landed, then its buffer released to the loads
				bool ok = true;
				committed = false;
				for (int it = c0; it < c1; it++) {
					const int s = it % KS;
					if (!mbar_wait(full0 + 8 * s, (it / KS) & 1, a.wait_ns)) {
						ok = false;
						break;
					}
					consumed = it + 1;
					asm volatile("tcgen05.fence::after_thread_sync;");
					const uint32_t sa = smem_u32(stage_ptr(s));
					const int blocks = min(KB, nkb - it * KB);
#pragma unroll
					for (int b = 0; b < KB; b++) {
						if (b >= blocks) break;
						const uint64_t da = smem_desc(sa + b * kBlockBytes), db = smem_desc(sa + b * kBlockBytes + NS * kTile);
						if (tid == 0) issue_sweep_mmas<S, W, 0>(tmem, da, db, it == c0 && b == 0, kIdesc);
						else issue_sweep_mmas<S, W, 1>(tmem, da, db, it == c0 && b == 0, kIdesc);
					}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(empty0 + 8 * s)
					             : "memory");
				}
				if (ok) {
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(accb)
					             : "memory");
					committed = true;
				} else {
					s_fail = 1;
				}
			}
			// every thread: wait for the chunk's MMAs, then add its four groups into the row sums,
			// shifted to the sweep's unit (no FP64 operation); accumulators read two per wait
			if (!s_fail && !mbar_wait_sleep(accb, rounds & 1, a.wait_ns)) s_fail = 1;
			__syncthreads();
			if (s_fail) return;
			asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
			for (int sg = 0; sg < kCols / 8; sg++) {
				const int seg = part * (kCols / 8) + sg;   // 8-column segment of the tile
#pragma unroll
				for (int g0 = 0; g0 < 4; g0 += 2) {
					uint32_t v[2][8];
					tmem_ld8(tmem + lane_base + (uint32_t) g0 * kBN + seg * 8, v[0]);
					tmem_ld8(tmem + lane_base + (uint32_t) (g0 + 1) * kBN + seg * 8, v[1]);
					tmem_wait_ld();
#pragma unroll
					for (int q = 0; q < 2; q++) {
						const int g = g0 + q;
						// sweep 0: G_2 << 16, G_3 << 8, G_4 parts << 0; sweep 1: G_t << 8 (8 - t)
						const int shift = W == 0 ? (g == 0 ? 16 : g == 1 ? 8 : 0) : 8 * (3 - g);
#pragma unroll
						for (int j = 0; j < 8; j++) {
							const long long gv = __float2int_rn(__uint_as_float(v[q][j]));   // below 2^26: a 32-bit conversion
							acc[sg * 8 + j] += gv << shift;
						}
					}
				}
			}
			rounds++;
			asm volatile("tcgen05.fence::before_thread_sync;");
			__syncthreads();
		}
	};

	// parked hi sums of this thread, column-major within the tile ([col][row]): the 32 threads of a
	// warp, 32 consecutive rows, store and load 256 contiguous bytes per column
	long long *park = a.park + ((size_t) blockIdx.x * kBN + part * kCols) * kBM + rl;
	sweep(std::integral_constant<int, 0>{});
	if constexpr (S == kSlicesFull) {
		if (!s_fail) {
#pragma unroll
			for (int c = 0; c < kCols; c++) park[c * kBM] = acc[c], acc[c] = 0;
			sweep(std::integral_constant<int, 1>{});
		}
	}

	// epilogue: this thread's row r of P, squared, into a column-major buffer with a padded stride
	// (over the finished stages; stores and column loads free of bank conflicts); then every thread
	// sums a quarter of a column's rows, phi rows and pi rows apart, and one thread per column adds
	// the four quarters in a fixed order: e_k = omega_k^2 sum_phi + sum_pi
	constexpr int kRedStride = kBM + 1;
	double *red = reinterpret_cast<double *>(smem);                            // [128][129]
	double2 *quarter = reinterpret_cast<double2 *>(smem + kBN * kRedStride * 8);   // [4][128] {phi, pi}
	static_assert(kBN * kRedStride * 8 + 4 * kBN * 16 <= kStageMem, "reduction buffers exceed the stages");
	static_assert(kStageMem + 1024 + 2048 <= 227 * 1024, "shared memory above 227 KB");
	static_assert(kThreads == 4 * kBN, "four threads per column");
	const int r = row0 + rl;
	const int er = r < 2 * (int) a.copies ? a.row_exp[r] : 0;
	if (!s_fail) {
		// eight columns at a time: their parked sums loaded together, so a warp waits for L2 once per
		// eight columns rather than once per column
#pragma unroll
		for (int c0 = 0; c0 < kCols; c0 += 8) {
			long long hv[8];
#pragma unroll
			for (int j = 0; j < 8; j++) hv[j] = S == kSlicesFull ? __ldcg(park + (c0 + j) * kBM) : acc[c0 + j];
#pragma unroll
			for (int j = 0; j < 8; j++) {
				const int c = c0 + j, col = part * kCols + c;
				double p2 = 0.;
				if (col0 + col < (int) a.n) {
					const long long lo = S == kSlicesFull ? acc[c] : 0;
					p2 = er == kNonFiniteRow ? __longlong_as_double(0x7ff8000000000000ll)
					                         : fixed128_square_to_double(hv[j], lo, er + s_cexp[col]);
				}
				red[col * kRedStride + rl] = p2;
			}
		}
	}
	__syncthreads();
	{
		// rows 32 q .. 32 q + 31 of column tid mod 128; rows 0 and 2 mod 4 are phi rows
		const int cc = tid & (kBN - 1), q = tid >> 7;
		const double *col = red + cc * kRedStride + 32 * q;
		double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
#pragma unroll
		for (int rr = 0; rr < 32; rr += 4) s0 += col[rr], s1 += col[rr + 1], s2 += col[rr + 2], s3 += col[rr + 3];
		quarter[q * kBN + cc] = make_double2(s0 + s2, s1 + s3);
	}
	__syncthreads();
	if (tid < kBN) {
		const int k = col0 + tid;
		if (k < (int) a.n) {
			const double2 q0 = quarter[tid], q1 = quarter[kBN + tid], q2 = quarter[2 * kBN + tid], q3 = quarter[3 * kBN + tid];
			const double e = s_w[tid] * ((q0.x + q1.x) + (q2.x + q3.x)) + ((q0.y + q1.y) + (q2.y + q3.y));
			a.partials[(size_t) row_tile * a.n + k] = s_fail ? __longlong_as_double(0x7ff8000000000000ll) : e;
		}
	}
	if (s_fail) {
		// after a timeout: each MMA thread commits what it issued in the current chunk (if it has not),
		// then thread 0 waits (each wait bounded again) for the loads this block issued in the current
		// sweep and has not consumed, and for every MMA, so that nothing lands in shared memory or TMEM
		// after the block has released them
		if ((tid == 0 || tid == kMma1) && !committed)
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(accb)
			             : "memory");
		if (tid == 0) {
			for (int it = consumed; it < s_issued; it++)
				mbar_wait(cur_full + 8 * (it % cur_stages), (it / cur_stages) & 1, a.wait_ns);
			mbar_wait(accb, rounds & 1, a.wait_ns);
			atomicOr(a.status, 1);
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;");
	__syncthreads();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

size_t tc_projection_smem(int) { return kStageMem + 1024; }

cudaError_t launch_tc_projection(const TcArgs &a, const double2 *state, cudaStream_t stream) {
	count_launch(2);
	const dim3 grid((unsigned) ((size_t) (a.mp / kBM) * (a.np / kBN)));
	const unsigned split_blocks = (unsigned) ((a.copies + 7) / 8);
	if (a.slices == 3) {
		tc_split_rows_kernel<3><<<split_blocks, 256, 0, stream>>>(state, a);
		tc_projection_kernel<3><<<grid, kThreads, tc_projection_smem(3), stream>>>(a);
	} else {
		tc_split_rows_kernel<kSlicesFull><<<split_blocks, 256, 0, stream>>>(state, a);
		tc_projection_kernel<kSlicesFull><<<grid, kThreads, tc_projection_smem(kSlicesFull), stream>>>(a);
	}
	return cudaGetLastError();
}

const void *tc_projection_kernel_ptr(int slices) {
	return slices == 3 ? (const void *) tc_projection_kernel<3> : (const void *) tc_projection_kernel<kSlicesFull>;
}

}  // namespace nlc
