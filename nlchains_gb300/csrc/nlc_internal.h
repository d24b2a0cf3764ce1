// Host/device shared declarations of the nlchains engine (not part of the public ABI).
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/nlchains.h"

namespace nlc {

constexpr int kMaxSitesPerLane = 16;   // E: sites of a chain held in registers by one thread
constexpr int kMaxLanesPerChain = 1024;

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
	const double *exptab;    // Toda: alpha2_inv * 2^(j/256), 256 entries (device)
	unsigned long long *work_counter;  // [0] next unit, [1] finished blocks (device, self-resetting)
	uint32_t n;
	uint32_t copies;
	uint32_t steps;
	int32_t lanes;         // G: lanes per chain (power of two)
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
const void *real_move_kernel(int model, int variant, int sites);

// Diagnostics ---------------------------------------------------------------------------------

constexpr int kMaxRadices = 24;

struct FftPlanDev {
	int n;
	int nradix;
	int radix[kMaxRadices];
	const double2 *tw;     // tw[e] = exp(-2 pi i e / n), device
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
};

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
};
cudaError_t launch_linenergies_finish(const FinishArgs &a, cudaStream_t stream);

// DNLS ------------------------------------------------------------------------------------------

struct DnlsArgs {
	FftPlanDev fft;
	uint32_t n, copies, steps;
	double nl[8];              // nonlinear coefficient of sub-step k: beta*dt*c[k]; nl[7]: beta*dt*2*c[0] (merged)
	double nl_final;           // beta*dt*c[7]
	const double2 *lin_tables; // [7][n] exp(-i dt d_k omega_j)/n
	unsigned long long *work_counter;
};
cudaError_t launch_dnls_move(const DnlsArgs &a, double2 *psi, int blocks, int threads, size_t smem,
                             int team_block, cudaStream_t stream);
cudaError_t launch_dnls_nonlinear(double2 *psi, uint64_t elements, double coef, cudaStream_t stream);
cudaError_t launch_dnls_linear(double2 *psi, uint64_t elements, uint32_t n, const double2 *table,
                               cudaStream_t stream);

// FP64 probe
cudaError_t launch_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream);

// bookkeeping
void count_launch(uint64_t k = 1);

}  // namespace nlc
