// Instantiations of the resident integrator for one model (one translation unit per model so the
// build compiles the models in parallel).  Toda's kernels (the table exp in every bond) take the
// longest to compile, so half of them are in nlc_real_toda_short.cu.
#include "nlc_real.cuh"

namespace nlc {
const void *real_kernel_toda_short(int variant, int sites, bool win);
const void *real_kernel_toda(int variant, int sites, bool win) {
	if (RealKernels<NLC_TODA>::is_short(sites, win)) return real_kernel_toda_short(variant, sites, win);
	return (const void *) RealKernels<NLC_TODA>::lookup_long(variant, sites, win);
}
}  // namespace nlc
