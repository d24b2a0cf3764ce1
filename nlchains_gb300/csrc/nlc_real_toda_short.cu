// Toda's resident-integrator instantiations for lanes of 2..13 sites and 4-site windows (the rest in
// nlc_real_toda.cu).
#include "nlc_real.cuh"

namespace nlc {
const void *real_kernel_toda_short(int variant, int sites, bool win) {
	return (const void *) RealKernels<NLC_TODA>::lookup_short(variant, sites, win);
}
}  // namespace nlc
