/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for the FFTW3 calls of the reference's CPU path
 * (DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp:76-94, DNLS/cpu-implementation/
 * DNLS.cpp:56-69,116-122, common/wisdom_sync.hpp).  FFTW 3 computes the unnormalised discrete
 * Fourier transform X_k = sum_j x_j exp(sign 2 pi i j k / n) (sign -1 forward); the stand-in
 * computes that definition directly in long double (ref_shim_impl.cpp), which rounds to the
 * double result within an ulp or two of the exact transform.  Wisdom is accepted and ignored.
 */
#pragma once

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;
typedef struct {
	int n, is, os;
} fftw_iodim;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

fftw_complex *fftw_alloc_complex(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim *dims, int howmany_rank,
                                   const fftw_iodim *howmany_dims, double *ri, double *ii, double *ro,
                                   double *io, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);
void fftw_forget_wisdom(void);
int fftw_import_wisdom_from_string(const char *s);
int fftw_import_wisdom_from_filename(const char *name);
char *fftw_export_wisdom_to_string(void);

#ifdef __cplusplus
}
#endif
