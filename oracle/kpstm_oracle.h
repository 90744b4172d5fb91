/*
 * CPU oracle for the Kirchhoff PSTM path - TEST INFRASTRUCTURE ONLY.
 *
 * A C restatement of the reference's kirchhoff() job (Kirchhoff.c:1104-1616)
 * and its set-up (:266-313, 380-441, 447-626), used by tests/, the smoke
 * check and bench.py's CPU-baseline leg as the checker.  The product library
 * (random_gb300/csrc) never links or calls it.
 *
 * Parity pin: the reference is compiled from its own source by
 * oracle/refbuild.py with the documented flags (-w -ffast-math, no -O,
 * Kirchhoff.c:3); tests/test_oracle_vs_reference.py requires this
 * restatement to reproduce that binary's SU output bit for bit.  The
 * arithmetic below therefore follows what gcc makes of each expression under
 * -ffast-math at -O0 (measured expression by expression): divisions chained
 * as (a/b)/c are evaluated as a/(b*c) (Kirchhoff.c:1320, 403, 416), every
 * other expression keeps C's evaluation order and float/double types.
 */
#ifndef KPSTM_ORACLE_H
#define KPSTM_ORACLE_H

#include <stdint.h>

#include "../include/kpstm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Derived job geometry, main() of Kirchhoff.c:266-313. */
typedef struct {
    int Nx, Ny, nx, ny, xslice, yslice, trange_max, ns, nh;
    float sinA, cosA, dt, fs;
} ko_dims;

int ko_dims_of(const kpstm_params *p, ko_dims *d);

/* create_aliasfilter, Kirchhoff.c:380-441 (fast-math evaluation). */
int ko_aliasfilter(int ns, float dt, double il_dist, double xl_dist, double cutoff,
                   int *trange_max, float *anti_alias);

/* Per-trace double running integral, Kirchhoff.c:1312-1328: dataP has
   ns + 2*trange_max entries, dataP[trange_max + t] corresponds to sample t. */
void ko_prep_trace(int ns, int trange_max, float dt, const float *t2, const float *trace,
                   float *dataP);

/* Whole job: imaging of all ntr traces (in order) into km/fold
   ([nx][ny][nh][ns], fold starting at 1.0), then the finishing filter into
   image (same layout).  Any output pointer may be NULL.  nthreads <= 0 uses
   all online CPUs.  mode must be KPSTM_MODE_REFERENCE. */
int ko_kirchhoff(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be,
                 const float *samples, int64_t ntr, float *km, float *fold, float *image,
                 int nthreads, int64_t *pairs);

/* The same job with every quantity in double precision (geometry, running
   integrals, taps, traveltimes, accumulation, finishing): the FP64 oracle
   against which the GPU's fp32/bf16 results are measured.  Reference and
   full modes; outputs [nx][ny][nh][ns] (any may be NULL). */
int ko_kirchhoff64(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be,
                   const float *samples, int64_t ntr, double *km, double *fold, double *image);

/* Least-squares operator pair of the full-physics mode, in double:
   direction 0: model = L^T data (migration, [nx][ny][nh][ns], no fold);
   direction 1: data = L model (demigration, [ntr][ns]), its exact transpose. */
int ko_lsm_apply(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be, int64_t ntr,
                 int direction, const double *in, double *out);

/* Finishing only (Kirchhoff.c:1440-1479) of given accumulators. */
int ko_finish(const kpstm_params *p, const float *km, const float *fold, float *image);

#ifdef __cplusplus
}
#endif

#endif
