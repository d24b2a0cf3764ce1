/*
 * nlchains.h -- C ABI of the GB300-native nlchains engine (libnlchains_gb300.so).
 *
 * The engine integrates ensembles of independent periodic 1-D lattices with the 6th-order Yoshida
 * scheme and computes the ensemble-averaged linear-mode energies and their entropies, for the five
 * nlchains models.  All entry points are plain C: status codes, plain pointers and sizes, no C++
 * exceptions and no CUDA or torch types in the signatures (streams are passed as `void *` holding a
 * cudaStream_t; NULL is the legacy default stream).
 *
 * State layout is the reference's, byte for byte: double[copies][chain_length][2] (phi, pi) for the
 * real models, complex<double>[copies][chain_length] for DNLS (reference README.md:74-82).
 *
 * Three levels:
 *   1. operators on caller-owned device memory, stream ordered (replace the reference's internal
 *      GPU API: move<model>, make_linenergies, DNLS::evolve_*);
 *   2. jobs owned by a context (replace the reference's per-model main loop, its gconf/gres globals
 *      and the results pipeline);
 *   3. nlc_program_run: the reference's `nlchains <model> <options>` command line (common/main.cpp).
 *
 * Errors: every function returns NLC_OK (0) or a negative NLC_E* code; nlc_last_error() gives a
 * thread-local message for the last failure on the calling thread.
 */
#ifndef NLCHAINS_H
#define NLCHAINS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* models, in the order of the reference's DNKG_FPUT_Toda::Model enum (DNKG_FPUT_Toda.hpp:9-11) */
enum {
	NLC_DNKG = 0,
	NLC_FPUT = 1,
	NLC_TODA = 2,
	NLC_DDNKG = 3,
	NLC_DNLS = 4
};

/* status codes */
enum {
	NLC_OK = 0,
	NLC_EINVAL = -1,     /* invalid argument (reference: std::invalid_argument, main.cpp:82-103) */
	NLC_ECUDA = -2,      /* CUDA runtime error (reference: cuda_error, utilities_cuda.cuh:23-37) */
	NLC_ENOMEM = -3,     /* device or host allocation failed */
	NLC_EIO = -4,        /* file I/O (reference: std::ios_base::failure, main.cpp:112-128) */
	NLC_ETIMEDOUT = -5,  /* a bounded wait expired; nothing was left running unbounded */
	NLC_ENOTFOUND = -6,  /* unknown job / request / program */
	NLC_EBLOWUP = -7,    /* non-finite entropy (reference: results::check_entropy, results.cpp:63-68) */
	NLC_EUNSUPPORTED = -8
};

/* flags of nlc_model.flags */
enum {
	NLC_FLAG_SPLIT_KERNEL = 1,    /* --split_kernel (DNKG_FPUT_Toda.cpp:43): accepted; every length runs
	                                 the resident (or, beyond one block, the windowed) integrator */
	NLC_FLAG_NO_TUNE = 2,         /* skip the autotuner, use the heuristic launch shape */
	NLC_FLAG_CANONICAL_SHAPE = 4, /* launch shape from the chain length alone (up to 8 sites per lane, 16
	                                 on a single warp), so ensembles of similar length can share batched
	                                 launches */
	NLC_FLAG_COMPACT_DIAG = 8,    /* fewer partial rows in the diagnostics (less device memory per plan) */
	NLC_FLAG_SHARED_GPU = 16,     /* one work unit per block instead of a persistent grid: blocks retire as
	                                 they finish, so launches on other streams interleave with this plan's */
	NLC_FLAG_TENSOR_PROJECTION = 32, /* dDNKG: the mode projection on the tensor cores (7-slice BF16
	                                    split, FP32 accumulation, FP64 recombination: FP64-level error);
	                                    chosen by default from 128 sites */
	NLC_FLAG_FP64_PROJECTION = 64,   /* dDNKG: the mode projection on the FP64 CUDA cores at any length */
	NLC_FLAG_BF16X3_PROJECTION = 128, /* dDNKG: the tensor-core projection with 3 BF16 slices: faster, with
	                                    mode energies to ~1e-7 relative instead of FP64 level */
	NLC_FLAG_FP32_DIAGNOSTICS = 256, /* DNKG, FPUT, Toda, DNLS: the per-chain transform and mode energies
	                                    in FP32 (the sum over chains in FP64): mode energies to ~1e-7 of
	                                    the largest; lengths that need the padded transform or
	                                    global-memory passes keep the FP64 diagnostics */
	NLC_FLAG_DNLS_FOURIER = 512      /* DNLS: the linear sub-steps through transforms of the chain, as
	                                    the reference does, at every length.  By default, where dt is
	                                    small enough (propagator taps beyond 11 sites below 2^-64, dt up
	                                    to ~0.05) and chain_length >= 2R + 2 (16 at dt = 0.01), each
	                                    linear sub-step is the same operator applied as its real-space
	                                    stencil (nlc_dnls_stencil_coefficients) */
};

/*
 * Model description: the per-model command-line options plus the gconf fields the kernels read
 * (common/configuration.hpp:20-39; DNKG_FPUT_Toda.cpp:26-45; dDNKG.cpp:31-47; DNLS.cpp:34-37).
 */
typedef struct nlc_model {
	int32_t model;             /* NLC_DNKG .. NLC_DNLS */
	uint32_t chain_length;     /* -n, >= 2 */
	uint32_t copies;           /* -c, > 0 */
	double dt;                 /* --dt, > 0 */
	double m;                  /* -m (DNKG) */
	double alpha;              /* --alpha (FPUT cubic term, Toda steepness) */
	double beta;               /* --beta (DNKG, FPUT, dDNKG, DNLS) */
	const double *masses;      /* dDNKG: host array of the chain_length per-site masses m_x (the -m
	                              file content); 2 is added internally as in dDNKG.cpp:47 */
	const uint8_t *entropy_mask; /* optional host array of chain_length bytes, non-zero = mode used
	                              in the entropies (--entropymask, main.cpp:119-128); NULL = all */
	uint32_t flags;            /* NLC_FLAG_* */
} nlc_model;

/* ---------------------------------------------------------------------------------------------
 * Level 1: operators on caller-owned device memory
 * -------------------------------------------------------------------------------------------*/

typedef struct nlc_plan nlc_plan;

/*
 * Validate a model and precompute everything its kernels need on the current CUDA device: Yoshida
 * constants scaled by dt, dispersion, the DNLS propagator tables, the dDNKG eigensystem (the host's
 * divide and conquer, dense QR below 64 sites; from 4096 sites, or NLC_DEVICE_EIGEN_FROM, on the
 * GPU with cuSOLVER's; replacing Armadillo eig_sym in eigensystem.cpp:13-36), twiddle tables, the
 * integrator launch shape (autotuned once per shape unless NLC_FLAG_NO_TUNE) and the scratch used
 * by the diagnostics.  Replaces the setup half of the reference per-model main
 * (DNKG_FPUT_Toda.cpp:47-95, dDNKG.cpp:50-101, DNLS.cpp:39-126).
 */
int nlc_plan_create(const nlc_model *model, nlc_plan **plan);
int nlc_plan_destroy(nlc_plan *plan);

/*
 * A seeded initial ensemble written straight into caller device memory (copies x chain_length in
 * the state layout above), for ensembles too large to build and upload from the host.  The recipes
 * and random numbers are those of nlchains_gb300/ic.py: uniform phases from SplitMix64 counters
 * keyed by (seed, copy first_copy + c, mode), every excited mode with the same energy; to rounding
 * the same ensemble as ic.py's (a different transform).
 *   DNKG, FPUT, Toda: `density` = energy per site, spread over the listed wave numbers (DFT
 *     indices; list +k and n - k for a real standing wave; a zero-frequency mode is skipped);
 *   DNLS: `density` = norm per site, psi_hat equal in modulus over the listed wave numbers;
 *   dDNKG: `density` = energy per site over the listed eigenmodes (indices in ascending order of
 *     frequency).
 * Synchronous with respect to `stream` (it returns once the state is written).
 */
int nlc_initial_state(nlc_plan *plan, uint64_t seed, uint64_t first_copy, double density, const uint32_t *modes,
                      uint32_t nmodes, void *state_dev, void *stream);

/*
 * Advance every chain of the device state by `steps` Yoshida steps in one fused launch (the merged
 * drift inside the launch and the closing drift dt*c[7] as in DNKG_FPUT_Toda.cu:117-146).
 * Replaces `template<Model> completion move(plane2split*&, cudaStream_t)` (DNKG_FPUT_Toda.hpp:22-23,
 * DNKG_FPUT_Toda.cu:262-297), `dDNKG::move` (dDNKG.hpp:12, dDNKG.cu:199-234) and, for DNLS, the
 * host loop of evolve_nonlinear + cuFFT + evolve_linear + cuFFT (DNLS.cpp:159-175).
 */
int nlc_move(nlc_plan *plan, void *state_dev, uint32_t steps, void *stream);

/*
 * Ensemble-averaged linear-mode energies, normalised exactly as results::calc_linenergies leaves
 * them (results_entropy.cpp:11-19), written to lin_dev[chain_length] (device memory), and, when
 * entropies_dev is not NULL, {WT entropy, information entropy} (results_entropy.cpp:21-46) written
 * to entropies_dev[2].  Replaces make_linenergies + its cuFFT / cublasDgemm prelude
 * (DNKG_FPUT_Toda.cpp:113-123, DNKG_FPUT_Toda.cu:304-331; dDNKG.cpp:118-141, dDNKG.cu:237-265;
 * DNLS.cpp:142-144, DNLS.cu:70-90) and the MPI all_reduce, which becomes an on-device reduction
 * over copies in a fixed order (deterministic run to run).
 */
int nlc_linenergies(nlc_plan *plan, const void *state_dev, double *lin_dev, double *entropies_dev,
                    void *stream);

/*
 * Allocation-free variant of nlc_linenergies, for callers that cannot allocate device memory when
 * they need the diagnostics: an application whose device memory is owned by its own pool or
 * framework allocator, or a service that reserves all memory at start-up.  No counterpart in the
 * reference (which allocates its FFT buffers, plans and work areas up front).
 *
 * Inputs and outputs are the caller's: state_dev (reference layout), an optional device mask of
 * chain_length bytes (NULL = all modes; it must select at least two modes), lin_dev[chain_length]
 * and entropies_dev[2] (may be NULL), all device memory, ordered on `stream`.  Models DNKG (m is
 * its -m), FPUT, Toda (m ignored) and DNLS; chain_length <= 4096, larger sizes are rejected with
 * NLC_EINVAL; lengths with a prime factor above 61 are rejected with NLC_EUNSUPPORTED (the
 * transform of such a length needs padded-length tables that the static array does not hold; the
 * regular nlc_linenergies handles every length).  Nothing is allocated: every temporary lives in one 4 MiB static device array that
 * each GPU loading the library holds until exit.  The first call on a device looks up that array's
 * device address and sets kernel attributes, so make the first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU race and must be ordered by the caller.
 */
int nlc_linenergies_noalloc(int32_t model, uint32_t chain_length, uint32_t copies, double m, const void *state_dev,
                            const uint8_t *entropy_mask_dev, double *lin_dev, double *entropies_dev, void *stream);

/*
 * Energy (Hamiltonian) of every chain into energies_dev[copies] (device memory), ordered on
 * `stream`: the definitions of the reference's post-processing (supporting-material/
 * post-processing/nlchains.m:40-48), for energy-drift checks.  The reference C++ has no equivalent.
 */
int nlc_energies(nlc_plan *plan, const void *state_dev, double *energies_dev, void *stream);

/* DNLS elementwise operators with the reference's semantics (DNLS.hpp:16-20, DNLS.cu:11-43), for
 * callers that drive their own FFTs: psi *= exp(-i coef |psi|^2); psi_k *= table[k % n]. */
int nlc_dnls_evolve_nonlinear(nlc_plan *plan, void *psi_dev, double beta_dt_symplectic, void *stream);
int nlc_dnls_evolve_linear(nlc_plan *plan, void *psi_k_dev, const void *table_dev, void *stream);

/* The DNLS linear propagator of sub-step k, psi <- IFFT(FFT(psi) exp(-i dt d_k omega_j) / n) with
 * omega_j = 4 sin^2(pi j / n) (DNLS.cu:19-25, dispersion.cpp:19-26), in real space (Jacobi-Anger):
 * psi'_s = exp(-2 i tau_k) sum_{|x| <= R} i^|x| J_|x|(2 tau_k) psi_{s+x}, tau_k = dt d_k, exact up to
 * terms below 2^-64 for chain_length >= 2R + 2.  Host only (no device is touched): c0m1[7] =
 * J_0(2 tau_k) - 1, taps[7 * max_radius] (row k, x = 1..max_radius) = J_x(2 tau_k) times the sign of
 * i^x (negative for x = 2, 3 mod 4), phase[7] = -2 tau_k; *radius = the R beyond which every tap is
 * below 2^-64 (max_radius + 1 if that is larger than max_radius).  max_radius in 1..32. */
int nlc_dnls_stencil_coefficients(double dt, int32_t max_radius, int32_t *radius, double *c0m1, double *taps,
                                  double *phase);

/* Launch shape chosen for the integrator: lanes per chain, sites per lane, threads per block, and
 * the tier: 1 = register-resident, a chain on G <= 32 lanes of a warp; 2 = register-resident, a
 * chain on one block of G > 32 lanes; 3 = DNLS, chains resident in shared memory (or, beyond it, in
 * per-block global scratch); 4 = windowed, chains longer than one block holds, integrated in
 * overlapping windows of G x E sites (lanes x sites per lane) between two state buffers; 5 = DNLS
 * in registers, G lanes of E or E - 1 sites, the linear sub-steps as real-space stencils; 6 = the
 * same for DNLS chains longer than one block holds, in overlapping windows of G x E sites. */
int nlc_plan_shape(const nlc_plan *plan, int32_t *lanes_per_chain, int32_t *sites_per_lane,
                   int32_t *threads_per_block, int32_t *tier);

/* Linear frequencies omega_k used by the diagnostics, copied to host omegas[chain_length]. */
int nlc_plan_omegas(const nlc_plan *plan, double *omegas);

/*
 * The dDNKG eigensystem on its own, into host buffers: the periodic operator
 * diag(masses[x] + 2) - shift(+-1) (masses = the -m file content), omegas[chain_length] = the
 * square roots of its eigenvalues in ascending order, eigenvectors[chain_length * chain_length]
 * column-major with eigenvector k in column k: the `-omegas` and `-eigenvectors` files of
 * eigensystem.cpp:23-29.  Replaces eigensystem.cpp:13-36 (Armadillo eig_sym) for callers that
 * keep their own plan.  device >= 0 lets cuSOLVER's divide and conquer run on that CUDA device
 * from 4096 sites (or from NLC_DEVICE_EIGEN_FROM sites, the threshold plans use too); device < 0,
 * shorter chains, or no usable GPU solver: the host solver (divide and conquer from 64 sites, dense
 * Householder + QR below), the faster one below about 4096 sites on a GB300 host.  Synchronous.
 */
int nlc_eigensystem(uint32_t chain_length, const double *masses, int32_t device, double *omegas,
                    double *eigenvectors);

/* ---------------------------------------------------------------------------------------------
 * Level 2: jobs (engine-owned device state; the reference main loop)
 * -------------------------------------------------------------------------------------------*/

typedef struct nlc_ctx nlc_ctx;

int nlc_create(nlc_ctx **ctx, int device);
int nlc_destroy(nlc_ctx *ctx);

/* A job owns its plan, device state and stream.  kernel_batching = steps per fused launch (-b). */
int nlc_job_create(nlc_ctx *ctx, const nlc_model *model, uint32_t kernel_batching, uint64_t *job);
int nlc_job_destroy(nlc_ctx *ctx, uint64_t job);
/* host -> device copy of the whole ensemble (reference layout); asynchronous w.r.t. the host when
 * host_state is pinned */
int nlc_job_upload(nlc_ctx *ctx, uint64_t job, const void *host_state);
/* enqueue `steps` steps (a multiple of kernel_batching), asynchronous */
int nlc_job_advance(nlc_ctx *ctx, uint64_t job, uint64_t steps);
/* compute the diagnostics of the current state and copy them to host memory (blocking):
 * lin[chain_length] (may be NULL), wt / inf (may be NULL).  Returns NLC_EBLOWUP when an entropy
 * is not finite (the reference's quit condition, results.cpp:64-68). */
int nlc_job_linenergies(nlc_ctx *ctx, uint64_t job, double *lin, double *wt, double *inf);
int nlc_job_download(nlc_ctx *ctx, uint64_t job, void *host_state);
/* energies of every chain of the job's current state into host_energies[copies] (blocking) */
int nlc_job_energies(nlc_ctx *ctx, uint64_t job, double *host_energies);
/*
 * Pipelined sampling, as the reference's main loop keeps up to two batches in flight
 * (loop_control.hpp, DNKG_FPUT_Toda.cpp:108-151): nlc_job_sample_async enqueues the diagnostics of
 * the job's current state into result slot 0 or 1 (with copy_state, also a copy of the state into
 * the slot's pinned host buffer) and returns at once, so the job can advance before the slot is
 * read.  nlc_job_sample_wait waits for the slot (at most timeout_ms, < 0: no limit; NLC_ETIMEDOUT)
 * and returns what nlc_job_linenergies returns, plus the state copy into host_state when it is not
 * NULL (the slot must have been filled with copy_state).  The `nlchains` command line runs on these.
 */
int nlc_job_sample_async(nlc_ctx *ctx, uint64_t job, int32_t slot, int32_t copy_state);
/* nlc_job_advance(kernel_batching) followed by nlc_job_sample_async(slot, copy_state), replayed as
 * one CUDA graph (captured on the first call for each slot / copy_state pair): one launch per batch
 * instead of the batch's kernels, copies and event, for short batches whose host overhead would
 * otherwise show.  Same results as the two calls. */
int nlc_job_step_async(nlc_ctx *ctx, uint64_t job, int32_t slot, int32_t copy_state);
int nlc_job_sample_wait(nlc_ctx *ctx, uint64_t job, int32_t slot, double *lin, double *wt, double *inf,
                        void *host_state, int32_t timeout_ms);
/* wait for the job's queued work, at most timeout_ms (< 0: no limit); NLC_ETIMEDOUT if not done */
int nlc_job_wait(nlc_ctx *ctx, uint64_t job, int32_t timeout_ms);
/* order two jobs of one context on the device, without blocking the host: work enqueued on `job`
 * after this call starts only once everything enqueued on `after_job` so far has completed.  Two
 * jobs that take turns on one GPU (one uploading or reading back while the other integrates) keep
 * their integrations in sequence this way, so that one job's persistent launch does not take the
 * SMs that the other job's diagnostics are waiting for. */
int nlc_job_after(nlc_ctx *ctx, uint64_t job, uint64_t after_job);
/* device pointer of the job's state, for callers that mix levels 1 and 2 */
int nlc_job_state_ptr(nlc_ctx *ctx, uint64_t job, void **state_dev);

/* ---------------------------------------------------------------------------------------------
 * Serving: continuous batching of ensemble-integration requests
 * -------------------------------------------------------------------------------------------*/

/*
 * A request server on one GPU.  Requests (model, chain length, copies, kernel_batching, steps,
 * initial state) are queued on submit and admitted while the HBM budget and the active-request
 * limit allow.  Once admitted, a request's state stays on the device until it completes, and it
 * advances in rounds of its own kernel_batching steps followed by one diagnostics sample, exactly as
 * the reference's main loop does for one ensemble.  In every round, requests of the same kernel
 * class (model, parameters, launch shape) are packed into one persistent batched launch, and
 * different classes run concurrently on a stream pool.  When a request completes or blows up, its
 * memory is released and queued requests are admitted (continuous batching).  Results are identical
 * to running each request alone.  No counterpart in the reference, which runs one ensemble per
 * process; it covers the served workload of the engine.
 */
typedef struct nlc_server nlc_server;

typedef struct nlc_server_config {
	int32_t device;              /* CUDA device */
	uint64_t hbm_budget_bytes;   /* device memory for admitted requests (0 = 60% of free memory) */
	int32_t max_active;          /* requests integrated at the same time (0 = 256) */
	int32_t streams;             /* CUDA streams in the pool (0 = 16) */
	/* longest wanted block lifetime of one launch: a round of kernel_batching steps is integrated
	   by launches of fewer steps when one block would run longer, so that newly arrived work finds
	   free SMs soon (0 = 3 ms; < 0 = every round in one launch).  Results are bit-identical. */
	double quantum_ms;
} nlc_server_config;

enum { NLC_REQ_QUEUED = 0, NLC_REQ_RUNNING = 1, NLC_REQ_DONE = 2, NLC_REQ_FAILED = 3 };

typedef struct nlc_request_status {
	int32_t state;               /* NLC_REQ_* */
	int32_t error;               /* status code of a failed request (NLC_EBLOWUP: non-finite entropy) */
	uint64_t steps_done;
	uint64_t samples;            /* diagnostics samples taken so far (t = 0 included) */
	double submit_ms;            /* server clock, ms since nlc_server_create: submitted */
	double start_ms;             /* admitted (HBM budget available) */
	double ready_ms;             /* plan, device state and t = 0 sample ready */
	double finish_ms;            /* done or failed */
} nlc_request_status;

int nlc_server_create(const nlc_server_config *config, nlc_server **server);
/* stops admitting, finishes or abandons running work (bounded wait), frees everything */
int nlc_server_destroy(nlc_server *server);
/* queue a request; host_state (reference layout) is copied before return */
int nlc_server_submit(nlc_server *server, const nlc_model *model, uint32_t kernel_batching, uint64_t steps,
                      const void *host_state, uint64_t *request);
/* queue a request whose initial state is generated on the device by nlc_initial_state (seed, density,
 * modes as there; copies counted from 0): large ensembles need no host copy and no upload */
int nlc_server_submit_seeded(nlc_server *server, const nlc_model *model, uint32_t kernel_batching, uint64_t steps,
                             uint64_t seed, double density, const uint32_t *modes, uint32_t nmodes,
                             uint64_t *request);
int nlc_server_poll(nlc_server *server, uint64_t request, nlc_request_status *status);   /* non-blocking */
/* wait until the request is DONE or FAILED, at most timeout_ms (< 0: no limit); NLC_ETIMEDOUT otherwise */
int nlc_server_wait(nlc_server *server, uint64_t request, int32_t timeout_ms);
/*
 * Results of a finished request, then forget it: final state (may be NULL), final linear energies
 * lin[chain_length] (may be NULL), the entropy series {WT, INF} per sample (entropies[2 * samples],
 * may be NULL; samples at t = 0, b, 2b, ...) and the sample count.
 */
int nlc_server_result(nlc_server *server, uint64_t request, void *host_state, double *lin, double *entropies,
                      uint64_t *samples);

/* ---------------------------------------------------------------------------------------------
 * Level 3: the reference command line
 * -------------------------------------------------------------------------------------------*/

/*
 * Run `nlchains <program> <options>` exactly as the reference's main() (common/main.cpp:142-176)
 * with argv[0] = program name among DNKG, FPUT, Toda, dDNKG, DNLS.  Reads -i, writes
 * <prefix>-entropy, <prefix>-linenergies-<t>, <prefix>-<t> (and -omegas / -eigenvectors for dDNKG)
 * in the reference formats.  Returns 0 on success, 1 on error (message on stderr), like the
 * reference executable.
 */
int nlc_program_run(int argc, char **argv);

/* ---------------------------------------------------------------------------------------------
 * Misc
 * -------------------------------------------------------------------------------------------*/

/*
 * The reference's results::calc_entropies (results_entropy.cpp:21-46) on host memory: {WT entropy,
 * information entropy} of the linear energies lin[chain_length] into out[2], over every mode, every
 * mode but 0 when a0is0 (zero-frequency mode 0: m = 0 for DNKG, always for FPUT, Toda and DNLS,
 * never for dDNKG; results.cpp:8), or the modes whose entropy_mask byte is non-zero.  For linear
 * energies combined on the host, e.g. all-reduced over processes that each integrate a shard of the
 * copies, as the reference's MPI ranks do (results_entropy.cpp:13).  NLC_EBLOWUP when a result is
 * not finite (results::check_entropy, results.cpp:63-68); out[] is written either way.  Needs no GPU.
 */
int nlc_entropies(const double *lin, uint32_t chain_length, int32_t a0is0, const uint8_t *entropy_mask,
                  double *out);

const char *nlc_last_error(void);
const char *nlc_version(void);

/* Count of engine kernel launches issued by this process so far (all entry points). */
uint64_t nlc_kernel_launches(void);

/*
 * FP64 throughput probe: runs an FP64 FMA loop kernel of the engine on the current device for
 * roughly `ms` milliseconds and returns the measured FP64 rate in TFLOP/s (FMA = 2 flops).  Used
 * as the roofline denominator for the FP64-bound integrators.
 */
int nlc_fp64_peak(double ms, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
