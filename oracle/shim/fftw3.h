/*
 * Minimal FFTW3-compatible interface used ONLY to compile the reference
 * Kirchhoff.c as a CPU oracle (test infrastructure).  FFTW3 itself is not
 * installed and the reference pins no version of it; its call sites are
 * Kirchhoff.c:11 (include), 1426-1433 (plans), 1465/1474 (execute),
 * 1603-1607 (destroy/free).  Only the complex 1-D double-precision API the
 * reference calls is provided.  Semantics follow FFTW's published
 * definition: unnormalised DFT, sign -1 for FFTW_FORWARD and +1 for
 * FFTW_BACKWARD, out-of-place allowed.
 */
#ifndef KPSTM_ORACLE_FFTW3_SHIM_H
#define KPSTM_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct kref_fft_plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

/* Direct use by the oracle restatement: out = DFT_sign(in), length n. */
void kref_dft(int n, int sign, const double *in_re_im, double *out_re_im);

#ifdef __cplusplus
}
#endif

#endif
