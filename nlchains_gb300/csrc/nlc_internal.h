// Host/device shared declarations of the nlchains engine (not part of the public ABI).
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/nlchains.h"

namespace nlc {

// FP64 constants that reach the kernels as parameters rather than literals: on GB300 an FMA whose
// constant operands come from the parameter bank issues faster than one with literal operands or
// than DADD / DMUL, so the hot paths issue adds and products as FMAs with these (see nlc_device.cuh).
struct FpOnes {
	double one = 1., mone = -1., mzero = -0.;
};
// Constants of the table-driven exp (nlc_device.cuh exp_scaled).
constexpr int kExpTable = 2048;   // entries of the table exp: 2^(j/2048), |r| <= ln 2 / 4096
struct ExpConsts {
	double shifter = 0x1.8p52;                     // 1.5 * 2^52: round-to-integer shifter
	double inv_l = 2048. / 0x1.62e42fefa39efp-1;   // 2048 / ln 2
	double l1 = 0x1.62e42fefa39efp-12;             // ln 2 / 2048, leading part
	double l2 = 0x1.abc9e3b39803fp-67;             // ln 2 / 2048, trailing part
	double c3 = 1. / 6, c2 = 0.5;                  // Taylor coefficients of exp(r) - 1 - r (r^4/24 < 2^-54)
};

// Constants of the table-driven sincos (nlc_device.cuh sincos_table): Cody-Waite reduction by
// 2 pi / 1024 = pi / 512 (split as the double-double value of pi, scaled) and Taylor coefficients
constexpr int kSinCosTable = 1024;
struct SinCosConsts {
	double shifter = 0x1.8p52;                      // 1.5 * 2^52: round-to-integer shifter
	double inv = 512. / 3.141592653589793116;       // 1024 / (2 pi)
	double p1 = 3.141592653589793116 / 512;         // pi / 512, leading part
	double p2 = 1.2246467991473532072e-16 / 512;    // pi / 512, trailing part
	double s3 = -1. / 6, s5 = 1. / 120;             // sin r = r + r^3 (s3 + r^2 s5)   (r^7/5040 < 2^-60 r)
	double c2 = -1. / 2, c4 = 1. / 24;              // cos r - 1 = r^2 (c2 + r^2 c4)  (r^6/720 < 2^-59)
	// |th| < 2^-4, no reduction: sin th = th + th^3 (q3 + th^2 (q5 + th^2 (q7 + th^2 q9))),
	// cos th = 1 + th^2 (w2 + th^2 (w4 + th^2 (w6 + th^2 w8))): the next terms, th^11/11! and
	// th^10/10!, are below 2^-60 of the result
	double q3 = -1. / 6, q5 = 1. / 120, q7 = -1. / 5040, q9 = 1. / 362880;
	double w2 = -1. / 2, w4 = 1. / 24, w6 = -1. / 720, w8 = 1. / 40320;
};

constexpr int kMaxSitesPerLane = 16;   // E: sites of a chain held in registers by one thread
constexpr int kMaxLanesPerChain = 1024;

// One ensemble inside a batched launch of the resident integrator (device table, see RealArgs).
struct BatchJob {
	double2 *state;
	const double *mp2_site;          // dDNKG per-site m_x + 2
	unsigned long long unit_begin;   // first work unit of this ensemble in the launch
	uint32_t n, copies, steps;
	uint32_t seg;                    // NLC_SEG_* of this ensemble's segment
};

// Segments: one round of kernel_batching steps may be integrated by several launches.  A launch
// that continues a round starts with the merged drift (DNLS: merged nonlinear rotation) instead of
// the round's leading c[0] sub-step, and a launch that leaves the round open stores the state
// without the closing c[7] sub-step.  The operations and their order are those of the single
// launch, so a round split into segments gives bit-identical results.
enum : uint32_t { NLC_SEG_CONTINUE = 1, NLC_SEG_OPEN = 2 };

// Kernel arguments of the real-model integrators, passed by value (kernel parameter bank).
struct RealArgs {
	double cd[7];          // drift coefficient of sub-step k: dt * c[k]
	double cd0_merged;     // drift of sub-step 0 for every step but the first of a launch: 2 dt c[0]
	double cd_final;       // closing drift of a launch: dt * c[7]
	double ck[7];          // kick coefficient dt * d[k]
	double nck[7];         // -dt * d[k]
	double mp2;            // DNKG: m + 2
	double alpha, beta;
	double alpha2;         // Toda: 2 alpha
	const double *mp2_site;  // dDNKG: m_x + 2 per site (device)
	const double *exptab;    // Toda: alpha2_inv * 2^(j/2048), kExpTable entries (device)
	unsigned long long *work_counter;  // [0] next unit, [1] finished blocks (device, self-resetting)
	uint32_t n;
	uint32_t copies;
	uint32_t steps;
	int32_t lanes;         // G: lanes per chain (power of two)
	FpOnes k1;
	ExpConsts ek;
	// batched launch: when `batch` is set, the launch integrates every ensemble of the table (same
	// model, constants, lanes and sites per lane; its own state, length, copies and step count);
	// n / copies / steps / mp2_site above are then unused
	const BatchJob *batch;
	int32_t nbatch;
	unsigned long long batch_units;
	uint32_t seg;          // NLC_SEG_* of an unbatched launch (batched: per table entry)
	// rounds fused into one launch (unbatched, unwindowed launches): with round_steps set, the launch
	// is steps / round_steps rounds of round_steps steps, each closed by its own final drift and the
	// next opened by an unmerged leading drift -- the operations of one launch per round
	uint32_t round_steps;
	// windowed tier (chains longer than one block's registers hold): when win_len is set, each unit
	// is one window of win_len = G E consecutive sites (mod n) of one chain, integrated as a ring;
	// the sites that the wrong ring closure can reach, win_halo = 7 x steps at each end, are
	// discarded and the interior (at most win_inner sites) is written to win_out
	uint32_t win_len, win_halo, win_inner, win_count;
	double2 *win_out;
};

// Launch shape of the resident integrator.
struct RealShape {
	int lanes = 0;          // G
	int sites = 0;          // E
	int threads = 0;        // threads per block
	int blocks = 0;         // persistent grid size
	size_t smem = 0;        // dynamic shared memory bytes
};

enum Variant { kGeneric = 0, kSpecial = 1 };

// Real-model integrator: launch by (model, E, variant); returns cudaError_t of the launch.
cudaError_t launch_real_move(int model, int variant, const RealShape &shape, double *state,
                             const RealArgs &args, cudaStream_t stream);
// Function pointer for occupancy / attribute queries of one instantiation.
const void *real_move_kernel(int model, int variant, int sites, bool windowed = false);

// Diagnostics ---------------------------------------------------------------------------------

constexpr int kMaxRadices = 24;

// Device plan of the shared-memory FFT of one chain (nlc_fft.cuh).
struct FftPlanDev {
	int n;                 // transform length
	int len;               // length of the Stockham pass: n, or the Bluestein convolution length m
	int nradix;
	int radix[kMaxRadices];  // radices of len
	const double2 *tw;     // tw[e] = exp(-2 pi i e / len), device
	const double2 *gw;     // FMA-form twiddle entries of the radix-2/3/4 passes (fma_twiddle_entry), device
	int gw_off[kMaxRadices];  // offset of pass r's entries in gw, in double2 units
	int bluestein;         // 1: chirp-z transform through a length-m cyclic convolution
	const double2 *chirp;  // exp(-i pi j^2 / n), j < n
	const double2 *bf;     // FFT_m(b) / m, b_j = exp(+i pi j^2 / n) wrapped (forward transforms)
	const double2 *bi;     // FFT_m(conj b) / m (backward transforms)
	FpOnes k1;
	double half = 0.5, sin60 = 0.86602540378443864676;   // radix-3 butterfly constants
	// radix-5 butterfly constants: cos(2 pi/5), cos(4 pi/5), sin(2 pi/5), sin(4 pi/5)
	double c51 = 0.30901699437494742410, c52 = -0.80901699437494742410;
	double s51 = 0.95105651629515357212, s52 = 0.58778525229247312917;
};

struct DiagArgs {
	FftPlanDev fft;
	uint32_t n, copies;
	int model;
	const double *coef_a;    // real models: (omega_k + 1)/2 ; DNLS: unused
	const double *coef_b;    // real models: (omega_k - 1)/2
	const double *omega;     // DNLS omega_k, dDNKG omegas
	const double *eigT;      // dDNKG: eigenvectors, row-major by site: eigT[s*n + k] = e_k[s]
	double *partials;        // [blocks][n]
	double2 *gscratch;       // block teams whose buffers exceed shared memory: [blocks][2][len]
	int proj_chunk;          // dDNKG: sites per shared-memory chunk of the projection
	const float2 *tw32;      // FP32 diagnostics (NLC_FLAG_FP32_DIAGNOSTICS): twiddles in FP32; NULL: FP64
	const float *coef32;     // FP32 diagnostics, real models: [2][n] the coef_a and coef_b in FP32
};

// FMA-form twiddles of a decimation-in-time pass (nlc_fft.cuh): pass radix p in {2, 3, 4} after Ns
// points, entry k < Ns.  With theta_u = 2 pi u k / (Ns p), c_u = cos theta_u and the forward
// twiddle w_u = exp(-i theta_u) = c_u (1 + i t_u), t_u = -tan theta_u, the entry holds
//   p = 4: {t1, t2}, {t3, c1}, {c2, c3 / c1}
//   p = 3: {t1, t2}, {c1, c2 / c1}, {c1 / 2, c1 sin(2 pi / 3)}
//   p = 2: {t1, c1}
// (fma_twiddle_double2s(p) double2s each), from cu[u] = cos theta_u and s[u] = sin theta_u,
// u = 1 .. p - 1.  A cosine near zero makes t_u large and c_u small; their product still reproduces s_u to rounding,
// so the butterfly's error stays relative to its inputs.  An exactly zero cosine (theta = pi/2) is
// replaced by 2^-60: c t = -s stays exact and the real part left behind, 2^-60, is below rounding.
__host__ __device__ inline int fma_twiddle_double2s(int p) { return p == 2 ? 1 : (p == 3 || p == 4) ? 3 : 0; }
__host__ __device__ inline void fma_twiddle_entry(int p, const double *cu, const double *s, double *out) {
	double c[4];
	for (int u = 0; u < 4; u++) c[u] = (cu[u] < 0x1p-60 && cu[u] > -0x1p-60) ? (cu[u] < 0 ? -0x1p-60 : 0x1p-60) : cu[u];
	if (p == 4) {
		out[0] = -s[1] / c[1], out[1] = -s[2] / c[2], out[2] = -s[3] / c[3], out[3] = c[1];
		out[4] = c[2], out[5] = c[3] / c[1];
	} else if (p == 3) {
		out[0] = -s[1] / c[1], out[1] = -s[2] / c[2], out[2] = c[1], out[3] = c[2] / c[1];
		out[4] = 0.5 * c[1], out[5] = c[1] * 0.86602540378443864676;
	} else if (p == 2) {
		out[0] = -s[1] / c[1], out[1] = c[1];
	}
}

// Seeded initial ensembles on the device (nlc_initial_state)
struct IcArgs {
	unsigned long long key;       // SplitMix64 key of (seed, stream)
	unsigned long long first_copy;
	double amp;                   // amplitude of every excited mode
	const int *modes;             // device: the excited mode indices
	uint32_t nmodes;
};
cudaError_t launch_initial_state(const DiagArgs &a, const IcArgs &c, double2 *state, int blocks, int threads,
                                 size_t smem, int team_block, cudaStream_t stream);

cudaError_t launch_linenergies_partials(const DiagArgs &a, const void *state, int blocks, int threads,
                                        size_t smem, int team_block, cudaStream_t stream);
struct FinishArgs {
	const double *partials;
	int nblocks;
	uint32_t n;
	double norm;
	int a0is0;
	int model;
	const double *omega;      // DNLS: multiply by omega_k after the sum
	const uint8_t *mask;      // device, NULL = all modes
	double *lin;              // out [n]
	double *entropies;        // out [2] or NULL
	double *block_sums;       // [ceil(n / 256)][4] scratch: with it, chains longer than 256 sites
	                          // are finished by a grid over the modes instead of one block
	double *row_slices;       // [row_slice_cap][n] scratch: with it, many partial rows are first
	int row_slice_cap;        // added in slices by a grid over (mode tiles x slices)
};
// slices of the partial rows for a finish of n modes over `rows` rows on `sms` SMs: 0 when the
// rows go to the finish directly
int finish_row_slices(uint32_t n, int rows, int sms);
cudaError_t launch_linenergies_finish(const FinishArgs &a, cudaStream_t stream);
constexpr int kFinishModesPerBlock = 256;

// DNLS ------------------------------------------------------------------------------------------

struct DnlsArgs {
	FftPlanDev fft;
	uint32_t n, copies, steps;
	double nl[8];              // nonlinear coefficient of sub-step k: beta*dt*c[k]; nl[7]: beta*dt*2*c[0] (merged)
	double nl_final;           // beta*dt*c[7]
	const double2 *lin_tables; // [7][n] exp(-i dt d_k omega_j)/n
	const double2 *conv_tables;  // [7][len] when set: the linear sub-steps as length-len cyclic convolutions
	unsigned long long *work_counter;
	int team;                  // lanes per chain of the warp-team variant (power of two, 4 .. 32)
	uint32_t seg;              // NLC_SEG_*
	const double2 *sctab;      // (cos, sin)(2 pi j / 1024), j < 1024 (device)
	SinCosConsts sc;
	double2 *gscratch;         // block teams whose buffers exceed shared memory: [blocks][2][len]
};
cudaError_t launch_dnls_move(const DnlsArgs &a, double2 *psi, int blocks, int threads, size_t smem,
                             int team_block, cudaStream_t stream);
// DNLS with the linear sub-steps as a real-space stencil (nlc_dnls_stencil.cu): chains of n sites on
// `lanes` lanes of E or E - 1 sites in registers, stencil radius R (instantiated: E in {8, 12, 16}
// with R = 7, E in {12, 16} with R = 11)
constexpr int kMaxStencilRadius = 11;
struct DnlsStencilArgs {
	uint32_t n, copies, steps, seg;
	int lanes;
	double nl[8], nl_final;    // as DnlsArgs
	double phase[7];           // -2 dt d_k: the propagator's common phase, added to the rotation angle before it
	double c0m1[7];            // J_0(2 dt d_k) - 1
	double taps[7][kMaxStencilRadius];   // x = 1..R: J_x(2 dt d_k) times the sign of i^x (x = 2, 3 mod 4 negative)
	unsigned long long *work_counter;
	const double2 *sctab;
	SinCosConsts sc;
	FpOnes k1;
	// windowed launches (chains beyond one block, win_len != 0): windows of win_len = lanes x E
	// sites, every lane full, win_halo sites at each end recomputed and discarded, the interiors
	// written to win_out
	uint32_t win_len, win_halo, win_inner, win_count;
	double2 *win_out;
};
cudaError_t launch_dnls_stencil(const DnlsStencilArgs &a, double2 *psi, int sites, int radius, int blocks,
                                cudaStream_t stream);
const void *dnls_stencil_kernel_ptr(int sites, int radius, bool team, bool windowed = false);
size_t dnls_stencil_smem(int lanes, int radius);
cudaError_t launch_dnls_nonlinear(double2 *psi, uint64_t elements, double coef, const double2 *sctab,
                                  cudaStream_t stream);
cudaError_t launch_dnls_linear(double2 *psi, uint64_t elements, uint32_t n, const double2 *table,
                               cudaStream_t stream);

// FP64 probe
cudaError_t launch_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream);

// bookkeeping
void count_launch(uint64_t k = 1);
void uncount_launch(uint64_t k);   // launches recorded during a stream capture did not run
uint64_t launch_count();

// dDNKG projection on the tensor cores (nlc_tc.cu): 7 (or 3) BF16 slices of X (rows 2c, 2c + 1 = phi_c,
// pi_c of chain c) and of the eigenvector matrix E, each padded with zeros to mp / np rows (multiples
// of 128 / 64) and kp sites (a multiple of 32), slice i at rows [i mp, (i + 1) mp)
#ifdef __CUDACC__
#define NLC_HD_INLINE __host__ __device__ inline
#else
#define NLC_HD_INLINE inline
#endif
// BF16 slices of the tensor-core projection, laid out as the kernel's shared memory wants them:
// [16-site block][128-row tile][slice][row in tile][16 sites].  The slices of one tile and block
// are one contiguous run (4 KB a slice), so a pipeline stage is two bulk copies (A's slices, B's
// slices), and a sweep that reads slices 1..3 reads a prefix of the run.  Within a row (32 bytes)
// the two 16-byte halves trade places on rows 4..7 of every 8: the 32-byte swizzle of the MMA's
// shared-memory descriptor.
NLC_HD_INLINE size_t tc_slice_index(int slice, int kb, size_t rows, size_t row, int site_in_block, int slices) {
	const int e = site_in_block;
	const size_t tiles = rows / 128, tile = row / 128, r = row % 128;
	return ((((size_t) kb * tiles + tile) * slices + slice) * 128 + r) * 16 +
	       (size_t) (((((e >> 3) ^ (int) (r >> 2)) & 1) << 3) | (e & 7));
}

struct TcArgs {
	uint32_t n, copies;
	int mp, np, kp, nkb;       // padded rows of X, of E; padded sites; 16-site blocks (kp / 16)
	int slices;                // 7 (FP64-accurate) or 3 (BF16x3)
	uint16_t *a_slices;        // slices of X (tc_slice_index, mp rows), written per sample by the split kernel
	const uint16_t *b_slices;  // slices of E (tc_slice_index, np rows), written once at set-up
	int *row_exp;              // [2 copies] power-of-two exponent of each row of X
	const int *col_exp;        // [n] exponent of each eigenvector (row of E)
	const double *omega;       // [n]
	double *partials;          // [mp / 128][n] weighted squared sums per row tile
	long long *park;           // [mp][np] the hi sums of the first sweep (7 slices only)
	int *status;               // set on a bounded-wait timeout
	unsigned long long wait_ns;  // limit of every mbarrier wait (wall clock)
	int wait_test;             // tests only: thread 0 first waits on a barrier nothing arrives at
};
cudaError_t launch_tc_projection(const TcArgs &a, const double2 *state, cudaStream_t stream);
size_t tc_projection_smem(int slices);
const void *tc_projection_kernel_ptr(int slices);

// Per-chain energies (nlc_energy.cu)
struct EnergyArgs {
	int model;
	uint32_t n, copies;
	double m, alpha, beta;
	const double *mp2_site;   // dDNKG: m_s + 2 (device)
};
cudaError_t launch_energies(const EnergyArgs &a, const double2 *state, double *out, cudaStream_t stream);

}  // namespace nlc
