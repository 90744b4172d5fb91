/*
 * Internal definitions shared by the host C code (kpstm_host.c) and the
 * CUDA code (kpstm_cuda.cu) of libkpstm.  Not part of the ABI.
 */
#ifndef KPSTM_INTERNAL_H
#define KPSTM_INTERNAL_H

#include <stdint.h>

#include "../../include/kpstm.h"

#ifdef __cplusplus
extern "C" {
#endif

#define KPSTM_PI 3.14159265359 /* the reference's PI literal, Kirchhoff.c:96 */

/* Columns per imaging CTA (one warp per image column). */
#define KPSTM_COLS_PER_CTA 8
/* Largest number of offset classes the device bucketing supports. */
#define KPSTM_MAX_CLASSES 1024

/* Per-trace geometry in the rotated survey frame (Kirchhoff.c:1297-1309),
   plus the trace's offset class and its index in the caller's block. */
typedef struct {
    float sxt, syt, gxt, gyt, cmpx, cmpy;
    int32_t cls;     /* offset class; -1: no class or outside the slab cull */
    int32_t src;     /* index of the trace in the block */
} kpstm_geom;

/* Set-up values derived once per context (main(), Kirchhoff.c:266-313 and
   create_aliasfilter :380-441). */
typedef struct {
    kpstm_dims dims;
    int32_t xslice, yslice;
    int32_t ncol;            /* nx * ny */
    int32_t nclass;          /* classes imaged: nh, or 1 for a stack */
    float sinA, cosA;
    float IXc, IYc;          /* slab centre, Kirchhoff.c:1332-1333 */
    double cull_radius;      /* aperture + add_on, Kirchhoff.c:1335-1338 */
    int32_t lmax;            /* full mode: largest triangle half-width */
} kpstm_setup;

/* Host helpers (kpstm_host.c). */
int kpstm_setup_of(const kpstm_params *p, kpstm_setup *s);
int kpstm_velocity_check(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s);
/* Column coordinates IX/IY (Kirchhoff.c:1346-1347) and velocity row of each
   column (Kirchhoff.c:1357-1365): colxy[2*ncol], colrow[ncol]. */
int kpstm_interp_rows(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s, const int32_t *colrow,
                      float *rows2);
int kpstm_columns(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s,
                  float *colxy, int32_t *colrow);
/* t2[t] (Kirchhoff.c:1247) and the velocity time index t1[t] (:1376-1378). */
void kpstm_time_tables(const kpstm_params *p, const kpstm_velocity *v, float *t2, int32_t *t1);
/* Real even impulse response h[ns] of the finishing low-pass: the
   reference's forward FFT, spectrum x anti_alias, inverse FFT / ns
   (Kirchhoff.c:1465-1479) is the circular convolution with h. */
int kpstm_lowpass_kernel(const kpstm_params *p, double *h);
int kpstm_su_headers(const kpstm_params *p, const kpstm_setup *s, int32_t col, int32_t cls,
                     int64_t tracl, uint8_t *hdr240);

#ifdef __cplusplus
}
#endif

#endif
