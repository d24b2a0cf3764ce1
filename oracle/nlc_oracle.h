/*
 * nlc_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the nlchains ensemble integrators and diagnostics, used by the tests, by
 * __graft_entry__.smoke() and by the timed CPU baseline in bench.py as the checker.  The product
 * (libnlchains_gb300.so) never links, loads or calls this code.
 *
 * Parity status: PINNED to the reference's own CPU program.  oracle/build.py compiles the
 * reference's nlchains-cpu sources in place (stand-ins for Boost, MPI, FFTW3 and Armadillo in
 * oracle/ref_shim/); with the oracle's FFT and eigensolver standing in for FFTW and LAPACK, this
 * oracle's NLO_ORDER_REFERENCE reproduces that program bit for bit (states, mode energies and
 * entropies of all five models; tests/golden/reference, tests/test_reference_pin.py).  The
 * reference's GPU kernels, compiled unmodified from its sources, are compared on the GPU
 * (tests/test_gpu_reference.py).
 *
 * Two arithmetic orders are provided for the real models:
 *   NLO_ORDER_REFERENCE  the reference CPU code's expressions, one rounding per C operator
 *                        (DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp:23-40,125-142,
 *                        dDNKG/cpu-implementation/dDNKG.cpp:17-19,91-108), libm exp; for DNLS the
 *                        reference CPU's |sin| = sqrt(1 - cos^2) rotation
 *                        (DNLS/cpu-implementation/DNLS.cpp:77-98);
 *   NLO_ORDER_DEVICE     the exact FP64 operation sequence of the sm_103a kernels (explicit fma,
 *                        bond-cached forces, table-driven exp), so GPU results can be compared
 *                        bit for bit; for DNLS the rotation by sincos (the reference GPU's
 *                        e_pow_I, common/utilities_cuda.cuh:469-473).
 * and for DNLS a third:
 *   NLO_ORDER_STENCIL    the engine's stencil form operation for operation (its table sincos, the
 *                        propagator's real-space taps J_x(2 dt d_k) from the same double-double
 *                        series, the same FMA order), so that form can be compared bit for bit;
 *                        it is tied to the transform form (the reference's) by the tests.
 */
#ifndef NLC_ORACLE_H
#define NLC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { NLO_DNKG = 0, NLO_FPUT = 1, NLO_TODA = 2, NLO_DDNKG = 3, NLO_DNLS = 4 };
enum { NLO_ORDER_REFERENCE = 0, NLO_ORDER_DEVICE = 1, NLO_ORDER_STENCIL = 2 };

typedef struct {
	int32_t model;
	int32_t order;
	uint32_t n;          /* chain length */
	uint32_t copies;
	double dt;
	double m;            /* DNKG linear parameter (dispersion uses it for every real model) */
	double alpha;        /* FPUT cubic term, Toda steepness */
	double beta;         /* quartic term (DNKG, FPUT, dDNKG, DNLS) */
	const double *mp2;   /* dDNKG: m_x + 2, length n */
	int32_t threads;     /* >1: OpenMP over copies (baseline build only) */
} nlo_model;

/* Yoshida 6th-order coefficients, common/symplectic.hpp:5-8. */
void nlo_coefficients(double c[8], double d[8]);

/*
 * Advance every chain of a planar state double2[copies][n] (or complex128[copies][n] for DNLS) by
 * `steps` time steps, in launches of `batching` steps: inside one launch the trailing drift of a
 * step merges with the leading drift of the next (DNKG_FPUT_Toda.cu:121-123), and the final drift
 * dt*c[7] closes the launch (DNKG_FPUT_Toda.cu:138-146).  steps must be a multiple of batching.
 */
int nlo_advance(const nlo_model *mdl, double *state, uint64_t steps, uint32_t batching);

/* The stencil form's coefficients (NLO_ORDER_STENCIL): for the 7 sub-steps, c0m1[k] = J_0(2 tau_k) - 1,
 * taps[k * max_radius + x - 1] = J_x(2 tau_k) times the sign of i^x (x = 1..max_radius), phase[k] =
 * -2 tau_k, tau_k = dt d_k; returns the radius beyond which every tap is below 2^-64 (max_radius + 1
 * if larger). */
int nlo_dnls_stencil_coefficients(double dt, int max_radius, double *c0m1, double *taps, double *phase);

/* Linear dispersion: real models sqrt(m + 4 sin^2(pi k/n)) (DNKG_FPUT_Toda/dispersion.cpp:9-16),
 * DNLS 4 sin^2(pi k/n) (DNLS/dispersion.cpp:10-17). */
void nlo_dispersion(int32_t model, uint32_t n, double m, double *omega);

/* Forward (sign = -1) or backward (sign = +1) unnormalised complex DFT of any length, in place on
 * interleaved re/im doubles.  Mixed radix, naive DFT for prime factors above 5. */
void nlo_fft(uint32_t n, double *z, int sign);

/*
 * Normalised linear-mode energies of the ensemble, as results::calc_linenergies leaves them
 * (results_entropy.cpp:11-19): real models sum |omega_k Phi_k + i Pi_k|^2 * 0.5/(copies n)
 * (DNKG_FPUT_Toda.cu:304-321, DNKG_FPUT_Toda.cpp:129), dDNKG the eigenbasis projection * 0.5/copies
 * (dDNKG/cpu-implementation/dDNKG.cpp:201-213, dDNKG.cpp:141), DNLS omega_k sum |psi_k|^2 /(copies n)
 * (DNLS.cu:70-81, DNLS.cpp:150).  Mode 0 is zeroed when its frequency is 0 (results.cpp:8).
 * eigvecs/omegas are only read for dDNKG (column-major, eigenvector k = column k).
 */
int nlo_linenergies(const nlo_model *mdl, const double *state, const double *eigvecs,
                    const double *omegas, double *out);

/* WT and information entropies, results_entropy.cpp:21-46.  mask may be NULL (all modes). */
int nlo_entropies(const double *linenergies, uint32_t n, int a0is0, const uint8_t *mask,
                  double *wt, double *inf);

/* Total energy of one chain (supporting-material/post-processing/nlchains.m:40-48). */
double nlo_energy(const nlo_model *mdl, const double *chain);

/* Symmetric eigenproblem of the column-major n x n matrix a (overwritten) by cyclic Jacobi:
 * ascending eigenvalues w, eigenvectors as the columns of v (column-major). */
int nlo_eig_sym(uint32_t n, double *a, double *w, double *v);

/* Symmetric eigensystem of the periodic dDNKG operator diag(mp2) - shift(+-1) (eigensystem.cpp:13-22)
 * by cyclic Jacobi: ascending eigenvalues, omegas = sqrt(eigenvalues), column-major eigenvectors. */
int nlo_eigensystem(uint32_t n, const double *mp2, double *omegas, double *eigvecs);

/* Table-driven exp used by the device order (Tang's method, 2048 entries, degree-3 polynomial);
 * the table holds scale * 2^(j/2048) and the function returns scale * exp(x). */
#define NLO_EXP_TABLE 2048
void nlo_exp_table(double scale, double table[NLO_EXP_TABLE]);
double nlo_exp_scaled(double x, const double table[NLO_EXP_TABLE]);

#ifdef __cplusplus
}
#endif
#endif
