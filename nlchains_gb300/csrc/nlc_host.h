// Host-side declarations shared by the engine's C++ translation units.
#pragma once

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "nlc_internal.h"

#include <nvtx3/nvToolsExt.h>

namespace nlc {
// An NVTX range for the life of the object (a stage of an entry point), so that a timeline taken
// with a profiler shows the engine's stages; without a tool attached the calls return at once.
struct NvtxRange {
	explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
	~NvtxRange() { nvtxRangePop(); }
	NvtxRange(const NvtxRange &) = delete;
	NvtxRange &operator=(const NvtxRange &) = delete;
};

// Makes `device` current for the life of the object (one entry point of the C ABI) and restores
// the caller's current device afterwards, so that a process driving several GPUs from one thread
// can call any context or plan whatever device it left current; device < 0: no change.
class DeviceScope {
public:
	explicit DeviceScope(int device) {
		int cur = -1;
		if (device >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != device && cudaSetDevice(device) == cudaSuccess)
			prev_ = cur;
	}
	~DeviceScope() {
		if (prev_ >= 0) cudaSetDevice(prev_);
	}
	DeviceScope(const DeviceScope &) = delete;
	DeviceScope &operator=(const DeviceScope &) = delete;

private:
	int prev_ = -1;
};
}  // namespace nlc

namespace nlc {

// thread-local error message + status helpers
int set_error(int code, const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

// Yoshida 6th-order coefficients (reference common/symplectic.hpp:5-8)
extern const double kYoshidaC[8];
extern const double kYoshidaD[8];

// scale * 2^(j/2048), j < 2048, in double-double arithmetic (identical bits on every IEEE host)
void exp_table(double scale, double table[kExpTable]);

// (cos, sin)(2 pi j / 1024), j < 1024, interleaved, in double-double arithmetic (identical bits on
// every IEEE host): the table of the device's sincos_table
void sincos_table(double table[2 * kSinCosTable]);

// dispersion of the real models, sqrt(m + 4 sin^2(pi k / n)) (DNKG_FPUT_Toda/dispersion.cpp:9-16)
std::vector<double> dispersion_real(uint32_t n, double m);
// dispersion of DNLS, 4 sin^2(pi k / n) (DNLS/dispersion.cpp:10-17)
std::vector<double> dispersion_dnls(uint32_t n);

// FFT radices of n (4s first, then 2, 3, 5, 7, other primes); empty if n < 2
std::vector<int> fft_radices(uint32_t n);
// forward twiddles exp(-2 pi i e / n), e < n, interleaved re/im
std::vector<double> fft_twiddles(uint32_t n);

// Host tables of a chain FFT: Stockham radices/twiddles of the pass length, plus the Bluestein
// chirp and convolution kernels when the padded length m >= 2n - 1 (at most max_len) takes fewer
// FP64 operations than direct passes of n with its prime factors (convolution: the DNLS linear
// sub-step, two transforms; otherwise one transform).  smem_len: the longest pass length whose two
// buffers fit shared memory; longer ones run from global memory.
struct FftTables {
	uint32_t n = 0, len = 0;
	bool bluestein = false;
	std::vector<int> radices;
	std::vector<double> tw, chirp, bf, bi;   // interleaved re/im
	std::vector<double> gw;    // FMA-form twiddle entries of the radix-2/3/4 passes (fma_twiddle_entry)
	std::vector<int> gw_off;   // per pass: offset of its entries in gw, in double2 units
};
// FMA-form twiddle entries of the decimation-in-time passes of `radices`.
void fft_fma_twiddles(const std::vector<int> &radices, std::vector<double> &gw, std::vector<int> &off);
FftTables fft_tables(uint32_t n, uint32_t smem_len, uint32_t max_len, bool convolution);
// the longest padded length of the FFT tables (2^18 >= 2 x 65535 - 1: any chain length of the
// reference's 16-bit --chain_length)
constexpr uint32_t kMaxFftLen = 1u << 18;

// The DNLS linear propagators IFFT_n diag(L_k) FFT_n (lin: 7 tables of n interleaved complex L_k,
// the 1/n included) are circulant: x -> x (*) h_k with h_k = sum_q L_k[q] exp(+2 pi i q t / n).  A
// cyclic convolution of length n equals the first n outputs of a cyclic convolution of length
// m >= 2n - 1 with g_k[t mod m] = h_k[t mod n], |t| < n, and x zero-padded to m.  Returns the 7
// spectra FFT_m(g_k) / m (interleaved), so that x (*) h_k = IFFT_m(FFT_m(x) G_k) on [0, n).
std::vector<double> dnls_conv_tables(const std::vector<double> &lin, uint32_t n, uint32_t m);

// The same propagators in real space (Jacobi-Anger): for n >= 2R + 2, IFFT_n diag(exp(-i tau
// omega_q)) FFT_n = exp(-2 i tau) sum_{|x| <= R} i^|x| J_|x|(2 tau) S^x (S the cyclic shift) up to
// terms below 2^-64, tau = dt d_k.  Fills, for the 7 sub-steps, c0m1[k] = J_0(2 tau_k) - 1,
// taps[k max_radius + x - 1] = J_x(2 tau_k) times the sign of i^x (x = 1..max_radius) and phase[k]
// = -2 tau_k, all from the series in double-double (the same bits on every IEEE host), and returns
// the radius R beyond which every |J_x(2 tau_k)| <= 2^-64 (max_radius + 1 when it is larger).
int dnls_stencil_coefficients(double dt, int max_radius, double c0m1[7], double *taps, double phase[7]);

// The same eigensystem on the GPU (cuSOLVER's divide and conquer, loaded at run time,
// nlc_eig_device.cpp); false when cuSOLVER is missing, any step fails or NLC_HOST_EIGEN is set, and
// the caller then uses the host solver.
bool eigensystem_periodic_device(const std::vector<double> &mp2, std::vector<double> &omegas,
                                 std::vector<double> &eigvec);
// for plans made by the calling thread: the eigensystem on the host even where the GPU solver would
// be used (the request server's preparers: its stream is GPU-bound, and the host solver overlaps)
void set_eigen_on_host(bool host);
// the dDNKG plan's eigenvectors (eigvec layout above), the ones its projection uses; NULL otherwise
const std::vector<double> *plan_eigenvectors(const nlc_plan *plan);

// Host threads of the set-up work (the dDNKG eigensolver): one per core (at most 32, or
// NLC_HOST_THREADS), or what set_host_setup_threads chose for the calling thread (the request
// server's preparers share the cores with each other and with its scheduler).
unsigned host_setup_threads();
void set_host_setup_threads(unsigned threads);

// Symmetric eigensystem of the periodic dDNKG operator diag(mp2) - shift(+-1) (eigensystem.cpp:
// 15-18): ascending eigenvalues, omegas = sqrt(eigenvalues), eigenvectors column-major
// (eigvec[k*n + s] = component s of eigenvector k), as Armadillo's eig_sym would return them.
// nlc_eig_host.cpp: divide and conquer from 64 sites, else (and as the checked fallback)
// Householder tridiagonalisation followed by the implicit symmetric QR iteration.
bool eigensystem_periodic(const std::vector<double> &mp2, std::vector<double> &omegas,
                          std::vector<double> &eigvec);

// What the request server needs to know about a plan (nlc_plan.cpp).
struct PlanInfo {
	int model = 0, variant = 0;
	RealShape shape;
	RealArgs args;          // integrator constants (device pointers included)
	size_t device_bytes = 0;  // device memory held by the plan
	int sms = 0;
	// cost model of the move kernel: FP64 work of one block's step over the sustained fraction of
	// peak, resident blocks per SM, warps per block, and the plan's own grid
	double block_ops = 0;
	int per_sm = 1, block_warps = 1, grid = 0;
	bool windowed = false;   // windowed tier: its own launches only, never in a batched launch
};
bool plan_info(const nlc_plan *plan, PlanInfo *info);
// free a plan's device memory in the order of `stream` (after the work already queued there),
// without the device-wide wait of nlc_plan_destroy
void plan_destroy_ordered(nlc_plan *plan, cudaStream_t stream);
// nlc_move of one segment of a round (seg: NLC_SEG_* flags)
int move_segment(nlc_plan *plan, void *state, uint32_t steps, uint32_t seg, cudaStream_t stream);
// `rounds` consecutive nlc_move launches of round_steps steps each (no sample in between), with up
// to rounds_per_launch of them fused into one launch: bit-identical to one launch per round
int move_rounds(nlc_plan *plan, void *state, uint64_t rounds, uint32_t round_steps, cudaStream_t stream);
uint32_t rounds_per_launch(const nlc_plan *plan, uint32_t round_steps);
// NLC_ETIMEDOUT (and the flag cleared) when a bounded wait of the plan's tensor-core projection ran
// out since the last call, else NLC_OK; synchronous.  Asked only when a sample is not finite.
int plan_device_status(nlc_plan *plan);
// a batched launch of the resident integrator (args.batch / nbatch / batch_units set)
cudaError_t launch_real_move_batch(int model, int variant, const RealShape &shape, const RealArgs &args,
                                   cudaStream_t stream);

}  // namespace nlc
