// Instantiations of the resident integrator for one model (one translation unit per model so the
// build compiles the models in parallel).
#include "nlc_real.cuh"

namespace nlc {
const void *real_kernel_ddnkg(int variant, int sites, bool win) {
	return (const void *) RealKernels<NLC_DDNKG>::lookup(variant, sites, win);
}
}  // namespace nlc
