// nlc_linenergies_noalloc: the linear-mode energy diagnostics without any device allocation.
//
// Who needs it: code that may not allocate device memory at the moment it wants the diagnostics.
// Typical cases are an application whose device memory belongs to its own pool or framework
// allocator and must not be fragmented by a library, and long-running services that reserve all
// their memory at start-up and treat any later allocation as a failure.  The regular
// nlc_linenergies needs a plan, and creating a plan allocates tables and reduction rows.
//
// Limits: chains of at most 4096 sites, and only lengths whose prime factors are all at most 61.
// The static array has no room for the padded-length (Bluestein) tables that nlc_linenergies uses
// for a large prime factor, and without them a prime p is one direct p-point DFT per chain done by
// a single thread (p^2 complex products), which for p near 4096 would take seconds per call.
//
// How: every temporary (twiddles, per-mode coefficients, the per-team partial rows of the copy sum)
// lives in one file-scope device array of kNoAllocScratchBytes (4 MiB), which every GPU that loads
// the library keeps until the process exits.  The tables are recomputed on the device at each call
// and every partial row is zeroed by the kernel that fills it, so nothing left by an earlier call
// leaks into the result.  Because all calls share that one array, calls whose work overlaps on the
// GPU (different streams, or different host threads, without ordering between them) race and give
// wrong results: order them on one stream or with events.
#include <cmath>
#include <mutex>

#include "nlc_fft.cuh"
#include "nlc_host.h"

namespace nlc {

const void *lin_kernel_ptr(int model, int team_block);   // nlc_diag.cu

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr size_t kNoAllocScratchDoubles = kNoAllocScratchBytes / sizeof(double);
constexpr uint32_t kNoAllocMaxChain = 4096;
constexpr int kNoAllocMaxPrime = 61;   // largest prime factor a chain length may have
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

struct DeviceSetup {
	double *scratch = nullptr;   // device address of g_noalloc_scratch on that device
	int sms = 0;
	bool done = false;
};
std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

// twiddles exp(-2 pi i e/n), the FMA-form twiddle entries of the radix-2/3/4 passes (entry e of
// every pass after more than e points) and the per-mode coefficients: (omega+1)/2, (omega-1)/2 for
// the real models, omega for DNLS (omega as in DNKG_FPUT_Toda/dispersion.cpp:9-16,
// DNLS/dispersion.cpp:10-17)
__global__ void noalloc_tables_kernel(uint32_t n, int model, double m, const FftPlanDev f, double2 *tw, double2 *gw,
                                      double *ca, double *cb) {
	const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n) return;
	double s, c;
	sincospi(2. * e / n, &s, &c);
	tw[e] = make_double2(c, -s);
	unsigned long long ns = 1;
	for (int r = 0; r < f.nradix; r++) {
		const int p = f.radix[r];
		const int per = fma_twiddle_double2s(p);
		if (ns > 1 && per && e < ns) {
			const unsigned long long span = ns * (unsigned long long) p;
			double cu[4] = {1., 1., 1., 1.}, su[4] = {0., 0., 0., 0.}, v[6];
			for (int u = 1; u < p; u++) sincospi(2. * double((u * (unsigned long long) e) % span) / double(span), &su[u], &cu[u]);
			fma_twiddle_entry(p, cu, su, v);
			double2 *o = gw + f.gw_off[r] + (size_t) per * e;
			for (int i = 0; i < per; i++) o[i] = make_double2(v[2 * i], v[2 * i + 1]);
		}
		ns *= (unsigned long long) p;
	}
	const double s2 = 2. * sinpi(double(e) / n);
	if (model == NLC_DNLS) {
		ca[e] = s2 * s2;
		cb[e] = 0.;
	} else {
		const double omega = sqrt(m + s2 * s2);
		ca[e] = (omega + 1.) / 2.;
		cb[e] = (omega - 1.) / 2.;
	}
}

int fill_radices(uint32_t n, FftPlanDev &f) {
	int cnt = 0;
	auto push = [&](int r) {
		if (cnt >= kMaxRadices) return false;
		f.radix[cnt++] = r;
		return true;
	};
	while (n % 4 == 0) if (!push(4)) return -1; else n /= 4;
	while (n % 2 == 0) if (!push(2)) return -1; else n /= 2;
	for (uint32_t p = 3; p * p <= n; p += 2)
		while (n % p == 0) if (!push(int(p))) return -1; else n /= p;
	if (n > 1 && !push(int(n))) return -1;
	f.nradix = cnt;
	return 0;
}

// Once per device, with that device current: the device address of the scratch array (the host
// name of a __device__ variable is only a host-side stand-in) and the kernels' shared-memory limit.
int setup_device(int dev, DeviceSetup **out) {
	if (dev < 0 || dev >= kMaxDevices) return set_error(NLC_EUNSUPPORTED, "device index beyond the no-alloc table");
	std::lock_guard<std::mutex> lk(g_setup_mutex);
	DeviceSetup &S = g_setup[dev];
	if (!S.done) {
		void *p = nullptr;
		int rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
		if (rc) return rc;
		int sms = 0, optin = 0;
		if ((rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute")))
			return rc;
		if ((rc = cuda_status(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
		                      "cudaDeviceGetAttribute")))
			return rc;
		for (int team_block = 0; team_block < 2; team_block++) {
			const void *k = lin_kernel_ptr(NLC_DNKG, team_block);
			cudaFuncAttributes attr{};
			if ((rc = cuda_status(cudaFuncGetAttributes(&attr, k), "cudaFuncGetAttributes"))) return rc;
			if ((rc = cuda_status(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                                           int(optin - attr.sharedSizeBytes)),
			                      "cudaFuncSetAttribute")))
				return rc;
		}
		S.scratch = static_cast<double *>(p);
		S.sms = sms;
		S.done = true;
	}
	*out = &S;
	return NLC_OK;
}

}  // namespace
}  // namespace nlc

using namespace nlc;

extern "C" int nlc_linenergies_noalloc(int32_t model, uint32_t chain_length, uint32_t copies, double m,
                                       const void *state_dev, const uint8_t *entropy_mask_dev, double *lin_dev,
                                       double *entropies_dev, void *stream) {
	if (model != NLC_DNKG && model != NLC_FPUT && model != NLC_TODA && model != NLC_DNLS)
		return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: model must be DNKG, FPUT, Toda or DNLS");
	if (!state_dev || !lin_dev) return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: NULL state or output");
	if (chain_length < 2 || !copies) return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: chain_length >= 2 and copies > 0");
	if (chain_length > kNoAllocMaxChain)
		return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: chain_length above 4096 does not fit the 4 MiB "
		                             "static scratch; use nlc_plan_create + nlc_linenergies");
	const uint32_t n = chain_length;
	DiagArgs g{};
	g.n = n, g.copies = copies, g.model = model;
	g.fft.n = int(n);
	g.fft.len = int(n);   // direct passes only: the static scratch holds no Bluestein tables
	if (fill_radices(n, g.fft)) return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: too many prime factors");
	for (int r = 0; r < g.fft.nradix; r++)
		if (g.fft.radix[r] > kNoAllocMaxPrime)
			return set_error(NLC_EUNSUPPORTED, "nlc_linenergies_noalloc: chain_length has a prime factor above 61 "
			                                   "(a direct transform of that length is too slow without the padded-"
			                                   "length tables); use nlc_plan_create + nlc_linenergies");
	int dev = 0;
	int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
	if (rc) return rc;
	DeviceSetup *S = nullptr;
	if ((rc = setup_device(dev, &S))) return rc;

	// offsets of the FMA-form twiddle entries: Ns entries for each radix-2/3/4 pass after Ns > 1
	// points, at most 3 n double2s in all (the Ns of the passes sum to less than n)
	{
		int off = 0;
		unsigned long long ns = 1;
		for (int r = 0; r < g.fft.nradix; r++) {
			g.fft.gw_off[r] = off;
			if (ns > 1) off += fma_twiddle_double2s(g.fft.radix[r]) * int(ns);
			ns *= (unsigned long long) g.fft.radix[r];
		}
	}
	// scratch layout: [twiddles 2n][FMA-form twiddles 6n][coef a n][coef b n][partial rows rows x n]
	double *base = S->scratch;
	double2 *tw = reinterpret_cast<double2 *>(base);
	double2 *gw = tw + n;
	double *ca = base + 8 * size_t(n), *cb = ca + n;
	double *rows_base = cb + n;
	const size_t rows_cap = (kNoAllocScratchDoubles - 10 * size_t(n)) / n;
	const int team_block = n > 1024;
	const int teams = team_block ? 1 : 4;
	const int threads = team_block ? 256 : 128;
	const size_t smem = size_t(teams) * 2 * n * sizeof(double2);
	unsigned long long blocks = (copies + teams - 1) / teams;
	blocks = std::min<unsigned long long>(blocks, 4ull * S->sms);
	blocks = std::min<unsigned long long>(blocks, rows_cap / teams);
	if (!blocks) return set_error(NLC_EINVAL, "nlc_linenergies_noalloc: scratch too small for this chain_length");
	g.fft.tw = tw;
	g.fft.gw = gw;
	if (model == NLC_DNLS) g.omega = ca;
	else g.coef_a = ca, g.coef_b = cb;
	g.partials = rows_base;

	cudaStream_t st = static_cast<cudaStream_t>(stream);
	count_launch();
	noalloc_tables_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, model, model == NLC_DNKG ? m : 0., g.fft, tw, gw, ca, cb);
	if ((rc = cuda_status(cudaGetLastError(), "nlc_linenergies_noalloc tables launch"))) return rc;
	if ((rc = cuda_status(launch_linenergies_partials(g, state_dev, int(blocks), threads, smem, team_block, st),
	                      "nlc_linenergies_noalloc launch")))
		return rc;
	FinishArgs f{};
	f.partials = rows_base;
	f.nblocks = int(blocks) * teams;
	f.n = n;
	// normalisations of results::calc_linenergies (DNKG_FPUT_Toda.cpp:129, DNLS.cpp:150) and a0is0
	f.norm = model == NLC_DNLS ? 1. / (double(copies) * n) : (0.5 / copies) / n;
	f.a0is0 = model == NLC_DNKG ? m == 0. : 1;
	f.model = model;
	f.omega = ca;
	f.mask = entropy_mask_dev;
	f.lin = lin_dev;
	f.entropies = entropies_dev;
	return cuda_status(launch_linenergies_finish(f, st), "nlc_linenergies_noalloc finish launch");
}
