// Test infrastructure only: exposes the reference's own Yoshida coefficient tables
// (common/symplectic.hpp:5-8, compiled where they lie in the reference sources) so that the tests
// can pin the oracle's tables to them.  That header is the one file of the reference's integration
// path that compiles on its own; the rest needs Boost, MPI, FFTW3 and Armadillo.
#include "symplectic.hpp"

extern "C" void ref_symplectic(double *c, double *d) {
	for (int i = 0; i < 8; i++) c[i] = symplectic_c[i], d[i] = symplectic_d[i];
}
