/*
 * TEST INFRASTRUCTURE ONLY -- one translation unit over the reference's own GPU sources, compiled
 * in place by oracle/build.py into a device-code-only fatbin per optimised chain length
 * (-Doptimized_chain_length=N, as the reference's CMakeLists.txt:73-78 does).  The kernels keep
 * the reference's names; the host side that launches them is this repository's
 * oracle/ref_shim/ref_gpu_host.cpp, which loads the fatbin through the CUDA driver API.
 */
#include <common/utilities_cuda.cu>
#include <DNKG_FPUT_Toda/DNKG_FPUT_Toda.cu>
#include <dDNKG/dDNKG.cu>
#include <DNLS/DNLS.cu>
