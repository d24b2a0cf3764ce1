// Per-chain energies (Hamiltonians) of an ensemble, for energy-drift checks of the integrators.
//
// The reference C++ has no energy routine; its post-processing defines them
// (supporting-material/post-processing/nlchains.m:40-48), with periodic differences
// d_s = q_{s+1} - q_s:
//   DNKG    sum p^2/2 + d^2/2 + m q^2/2 + beta q^4/4      (dDNKG: per-site m_s)
//   FPUT    sum p^2/2 + d^2/2 + alpha d^3/3 + beta d^4/4
//   Toda    sum p^2/2 + (e^{2 alpha d} - 2 alpha d - 1)/(4 alpha^2)   (written with expm1)
//   DNLS    sum |psi_{s+1} - psi_s|^2 + beta/2 |psi_s|^4
// One warp per chain: lane l sums sites l, l + 32, ..., then a fixed butterfly reduction, so the
// result does not depend on the launch.  Diagnostics, not a hot path: plain FP64 arithmetic.
#include "nlc_device.cuh"

namespace nlc {

__global__ void energies_kernel(const double2 *__restrict__ state, EnergyArgs a, double *__restrict__ out) {
	const unsigned long long chain = (unsigned long long) blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
	const int lane = threadIdx.x & 31;
	if (chain >= a.copies) return;   // whole warps leave together
	const uint32_t n = a.n;
	const double2 *c = state + chain * n;
	double h = 0.;
	for (uint32_t s = lane; s < n; s += 32) {
		const double2 v = c[s], w = c[s + 1 < n ? s + 1 : 0];
		if (a.model == NLC_DNLS) {
			const double dr = w.x - v.x, di = w.y - v.y, a2 = v.x * v.x + v.y * v.y;
			h += dr * dr + di * di + a.beta / 2 * a2 * a2;
			continue;
		}
		const double q = v.x, p = v.y, d = w.x - q;
		double e = p * p / 2;
		switch (a.model) {
			case NLC_DNKG: e += d * d / 2 + a.m * q * q / 2 + a.beta * q * q * q * q / 4; break;
			case NLC_DDNKG: e += d * d / 2 + (a.mp2_site[s] - 2) * q * q / 2 + a.beta * q * q * q * q / 4; break;
			case NLC_FPUT: e += d * d / 2 + a.alpha * d * d * d / 3 + a.beta * d * d * d * d / 4; break;
			default: {   // Toda
				const double x = 2 * a.alpha * d;
				e += (expm1(x) - x) / (4 * a.alpha * a.alpha);
			}
		}
		h += e;
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
	if (lane == 0) out[chain] = h;
}

cudaError_t launch_energies(const EnergyArgs &a, const double2 *state, double *out, cudaStream_t stream) {
	count_launch();
	const unsigned long long blocks = (a.copies + 7) / 8;
	energies_kernel<<<(unsigned) blocks, 256, 0, stream>>>(state, a, out);
	return cudaGetLastError();
}

}  // namespace nlc
