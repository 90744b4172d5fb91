/*
 * Own double-precision mixed-radix DFT behind the FFTW3 calls that the
 * reference makes (Kirchhoff.c:1426-1433, 1465, 1474, 1603-1607).  Test
 * infrastructure only: it lets the reference compile as the CPU oracle and
 * gives the C restatement the same transform.  FFTW3 is absent here and
 * unpinned by the reference, so this follows FFTW's published definition
 *     out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / n)
 * (no normalisation).  Algorithm: recursive decimation in time on the
 * smallest prime factor (Cooley-Tukey for any n; a prime n degenerates to
 * the direct O(n^2) sum).  Twiddles are tabulated once per plan with libm
 * cos/sin in double.
 */
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct kref_fft_plan {
    int n, sign;
    fftw_complex *in, *out;
    double *tw;      /* 2*n: exp(sign*2*pi*i*k/n) */
    double *work;    /* 2*n scratch */
};

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

static int smallest_factor(int n)
{
    if (n % 2 == 0) return 2;
    for (int p = 3; (long)p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* DFT of the length-n sequence in[0], in[s], in[2s], ... into out[0..n-1].
 * tw holds exp(sign*2*pi*i*k/N) for the top-level N; this level uses
 * tw[(j * (N/n)) % N]. */
static void fft_rec(int n, int s, const double *in, double *out, const double *tw, int N)
{
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; ++r)
        fft_rec(m, s * p, in + 2 * (size_t)r * s, out + 2 * (size_t)r * m, tw, N);
    int step = N / n;
    double tmp_re[64], tmp_im[64];
    double *yr = tmp_re, *yi = tmp_im;
    double *heap = NULL;
    if (p > 64) {
        heap = (double *)malloc(sizeof(double) * 2 * (size_t)p);
        yr = heap;
        yi = heap + p;
    }
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            yr[r] = out[2 * ((size_t)r * m + k)];
            yi[r] = out[2 * ((size_t)r * m + k) + 1];
        }
        for (int q = 0; q < p; ++q) {
            long kk = k + (long)q * m;
            double sr = 0.0, si = 0.0;
            for (int r = 0; r < p; ++r) {
                long e = ((long)r * kk) % n;
                double wr = tw[2 * (e * step)], wi = tw[2 * (e * step) + 1];
                sr += yr[r] * wr - yi[r] * wi;
                si += yr[r] * wi + yi[r] * wr;
            }
            out[2 * kk] = sr;
            out[2 * kk + 1] = si;
        }
    }
    free(heap);
}

void kref_dft(int n, int sign, const double *in, double *out)
{
    double *tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n; ++k) {
        double a = two_pi * (double)k / (double)n;
        tw[2 * k] = cos(a);
        tw[2 * k + 1] = sign * sin(a);
    }
    fft_rec(n, 1, in, out, tw, n);
    free(tw);
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
    (void)flags;
    struct kref_fft_plan *p = (struct kref_fft_plan *)calloc(1, sizeof(*p));
    p->n = n;
    p->sign = sign;
    p->in = in;
    p->out = out;
    p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    p->work = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n; ++k) {
        double a = two_pi * (double)k / (double)n;
        p->tw[2 * k] = cos(a);
        p->tw[2 * k + 1] = sign * sin(a);
    }
    return p;
}

void fftw_execute(const fftw_plan p)
{
    /* Copy the input first so that in-place plans work as in FFTW. */
    memcpy(p->work, p->in, sizeof(double) * 2 * (size_t)p->n);
    fft_rec(p->n, 1, p->work, (double *)p->out, p->tw, p->n);
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    free(p->tw);
    free(p->work);
    free(p);
}
