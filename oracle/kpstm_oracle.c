/*
 * CPU oracle for the Kirchhoff PSTM path - TEST INFRASTRUCTURE ONLY.
 * See kpstm_oracle.h for the role of this file and how it is pinned to the
 * compiled reference.  Every function cites the reference lines it restates.
 *
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction, which aarch64 gcc
 * would otherwise apply to float expressions such as cosA*i + sinA*j).
 */
#include "kpstm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "shim/fftw3.h"

#define KO_PI 3.14159265359 /* Kirchhoff.c:96 */

static uint32_t be32(int32_t w)
{
    uint32_t u = (uint32_t)w;
    return (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
}

/* main(), Kirchhoff.c:266-313. */
int ko_dims_of(const kpstm_params *p, ko_dims *d)
{
    if (!p || !d || p->ns <= 0 || !(p->dt > 0) || p->jobs_x <= 0 || p->jobs_y <= 0 || p->nh <= 0)
        return KPSTM_ERR_INVALID_ARG;
    if (p->velocity_interp != 0 && p->velocity_interp != 1) return KPSTM_ERR_INVALID_ARG;
    if (p->velocity_interp && p->mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED;
    memset(d, 0, sizeof(*d));
    int Nx = p->inc_iline == 0 ? 1 : (int)ceil((p->end_iline - p->start_iline) / p->inc_iline);
    int Ny = p->inc_xline == 0 ? 1 : (int)ceil((p->end_xline - p->start_xline) / p->inc_xline);
    if (Nx == 0) Nx = 1;
    if (Ny == 0) Ny = 1;
    int nx = (int)ceil(1.0 * Nx / p->jobs_x);
    int ny = (int)ceil(1.0 * Ny / p->jobs_y);
    if (nx == 0) nx = 1;
    if (ny == 0) ny = 1;
    if (Nx < 0 || Ny < 0 || p->job_id < 0 || p->job_id >= p->jobs_x * p->jobs_y)
        return KPSTM_ERR_INVALID_ARG;
    d->Nx = Nx;
    d->Ny = Ny;
    d->nx = nx;
    d->ny = ny;
    d->xslice = p->job_id / p->jobs_y; /* Kirchhoff.c:286-294 */
    d->yslice = p->job_id % p->jobs_y;
    d->sinA = (float)sin(p->angle_e_to_n_deg * KO_PI / 180.0); /* :312-313 */
    d->cosA = (float)cos(p->angle_e_to_n_deg * KO_PI / 180.0);
    d->ns = p->ns;
    d->nh = p->output == KPSTM_OUT_STACK ? 1 : p->nh;
    d->dt = p->dt;
    d->fs = (float)(2.0 / ((double)p->dt * (double)p->ns)); /* :403 (a/b)/c -> a/(b*c) */
    return KPSTM_OK;
}

/* create_aliasfilter, Kirchhoff.c:380-441. */
int ko_aliasfilter(int ns, float dt, double il_dist, double xl_dist, double cutoff,
                   int *trange_max, float *anti_alias)
{
    if (ns <= 0 || !(dt > 0)) return KPSTM_ERR_INVALID_ARG;
    float DIP = 45.0f, V_max = 1500.0f;
    float tanA = (float)tan(DIP * KO_PI / 180.0);
    float mm = (float)(il_dist <= xl_dist ? il_dist : xl_dist);
    float fmax = (float)((double)V_max / ((4.0 * (double)mm) * (double)tanA));
    if (trange_max) *trange_max = (int)floor(0.5 / ((double)fmax * (double)dt));
    if (!anti_alias) return KPSTM_OK;
    float fs = (float)(2.0 / ((double)dt * (double)ns));
    float fm = (float)cutoff;
    fm = (float)((double)fm * 3.0);
    float den = ((fm * fm) * fm) * fm;
    for (int i = 0; i < ns; ++i) anti_alias[i] = 0.0f; /* calloc, Kirchhoff.c:1053 */
    for (int i = 0; i <= ns / 2; ++i) {
        float x = (float)i * fs;
        float num = ((x * x) * x) * x;
        anti_alias[i] = (float)(1.0 / sqrt(1.0 + (double)(num / den)));
    }
    for (int i = ns / 2; i < ns; ++i) anti_alias[i] = anti_alias[ns - i]; /* :419-423 */
    return KPSTM_OK;
}

/* Kirchhoff.c:1312-1328. */
void ko_prep_trace(int ns, int tm, float dt, const float *t2, const float *f, float *P)
{
    P[tm] = f[0];
    for (int t = 1; t < ns; ++t)
        P[t + tm] = (float)((double)P[t - 1 + tm] + (double)f[t] / (4.0 * (double)t2[t]));
    for (int t = ns; t < ns + tm; ++t)
        P[t + tm] = P[t - 1 + tm] + f[ns - 1] / (((dt * dt) * (float)t) * (float)t);
    for (int t = 1; t < ns + tm; ++t) P[t + tm] = P[t - 1 + tm] + P[t + tm];
    for (int t = 0; t < tm; ++t) P[t] = P[2 * tm - t];
}

typedef struct {
    float sxt, syt, gxt, gyt, cmpx, cmpy;
    int off, live;
} ko_geom;

/* v_rms of image column (xg, yg) (global column indices) at every output
   sample t, in double.  Nearest (velocity_interp = 0): the grid node and the
   velocity sample the reference rounds to (Kirchhoff.c:1357-1378).
   Trilinear (velocity_interp = 1, full mode): the same continuous grid
   position (integer division of the origin difference plus the column's
   fractional step) and continuous sample t * (dt / dtm), clamped to the
   grid.  Returns 0, or -1 where the rounded position is below the grid. */
static int ko_col_vrms(const kpstm_params *p, const kpstm_velocity *v, int xg, int yg, int ns, double *out)
{
    const double gx = (p->start_iline - v->o_iline) / v->d_iline + xg * (p->inc_iline / v->d_iline);
    const double gy = (p->start_xline - v->o_xline) / v->d_xline + yg * (p->inc_xline / v->d_xline);
    int xc1 = (int)round(gx), yc1 = (int)round(gy);
    if (xc1 > v->n_iline - 1) xc1 = v->n_iline - 1;
    if (yc1 > v->n_xline - 1) yc1 = v->n_xline - 1;
    if (xc1 < 0 || yc1 < 0) return -1;
    const float step = p->dt / v->dtm;
    if (!p->velocity_interp) {
        const float *vr = v->vrms + ((size_t)xc1 * v->n_xline + yc1) * v->nsm;
        for (int t = 0; t < ns; ++t) {
            int q = (int)round((double)((float)t * step));
            out[t] = vr[q > v->nsm - 1 ? v->nsm - 1 : q];
        }
        return 0;
    }
    const double cx = gx < 0 ? 0 : (gx > v->n_iline - 1 ? v->n_iline - 1 : gx);
    const double cy = gy < 0 ? 0 : (gy > v->n_xline - 1 ? v->n_xline - 1 : gy);
    const int i0 = (int)floor(cx), j0 = (int)floor(cy);
    const int i1 = i0 + 1 < v->n_iline ? i0 + 1 : i0, j1 = j0 + 1 < v->n_xline ? j0 + 1 : j0;
    const double wx = cx - i0, wy = cy - j0;
    for (int t = 0; t < ns; ++t) {
        double gt = (double)((float)t * step);
        if (gt > v->nsm - 1) gt = v->nsm - 1;
        const int k0 = (int)floor(gt), k1 = k0 + 1 < v->nsm ? k0 + 1 : k0;
        const double wt = gt - k0;
        double c[2];
        for (int e = 0; e < 2; ++e) {
            const int k = e ? k1 : k0;
            const double a = v->vrms[((size_t)i0 * v->n_xline + j0) * v->nsm + k];
            const double b = v->vrms[((size_t)i0 * v->n_xline + j1) * v->nsm + k];
            const double cc = v->vrms[((size_t)i1 * v->n_xline + j0) * v->nsm + k];
            const double dd = v->vrms[((size_t)i1 * v->n_xline + j1) * v->nsm + k];
            c[e] = (1.0 - wx) * ((1.0 - wy) * a + wy * b) + wx * ((1.0 - wy) * cc + wy * dd);
        }
        out[t] = (1.0 - wt) * c[0] + wt * c[1];
    }
    return 0;
}

typedef struct {
    const kpstm_params *p;
    const kpstm_velocity *v;
    const ko_dims *d;
    const float *vel2;     /* [n_iline][n_xline][nsm] v^2 */
    const float *t2;
    const int *t1;         /* [ns] velocity time index */
    const ko_geom *geom;
    const float *D;        /* [ntr][ns] triangle taps per output index T */
    const float *P;        /* full mode: [ntr][ns] the traces' samples */
    int tm, lmax;
    int64_t ntr;
    float *km, *fold;
    int next_col;
    pthread_mutex_t mu;
    int64_t pairs;
    int err;
} ko_job;

/* Full-physics operator (no counterpart in the reference; the GPU's
   KPSTM_MODE_FULL), in double.  For image sample t of a column and a trace
   with source S and receiver R:
     ts = sqrt((t0/2)^2 + |I-S|^2/v^2), tr likewise, T = (ts + tr)/dt
     (a pair counts when T < ns - 1),
     Lf = clamp(1 + |dT/dx| dx + |dT/dy| dy, 1, lmax), the operator's lateral
     slope in samples per trace spacing,
     tri = sum_k f[k] max(0, Lf - |T - k|)   (a triangle of real half-width
     Lf centred on T: what the GPU reads from the double running integral
     of the trace as [P(T-1+Lf) - 2P(T-1) + P(T-1-Lf)] with linear
     interpolation and P = 0 before the trace),
     contribution t0 (1/ts + 1/tr)^2 / 8 * tri / Lf^2.
   The reference's 1/(t dt)^2 data scaling (Kirchhoff.c:1316) is not used:
   it puts a factor dt^-2 on the second sample and ruins float running
   integrals of noisy traces. */
static double full_tri(const float *f, int ns, double T, double Lf)
{
    int k0 = (int)ceil(T - Lf), k1 = (int)floor(T + Lf);
    if (k0 < 0) k0 = 0;
    if (k1 > ns - 1) k1 = ns - 1;
    double tri = 0.0;
    for (int k = k0; k <= k1; ++k) {
        double w = Lf - fabs(T - k);
        if (w > 0) tri += (double)f[k] * w;
    }
    return tri;
}

static void full_pairs(const ko_job *J, const ko_geom *g, float IX, float IY, const float *vv_t,
                       const float *f, float *k, float *fo)
{
    const kpstm_params *p = J->p;
    const int ns = J->d->ns;
    const double dt = (double)J->d->dt;
    const double sx = (double)IX - g->sxt, sy = (double)IY - g->syt;
    const double gx = (double)IX - g->gxt, gy = (double)IY - g->gyt;
    const double dS2 = sx * sx + sy * sy, dR2 = gx * gx + gy * gy;
    const double ax = p->iline_distance / dt, ay = p->xline_distance / dt;
    for (int t = 0; t < ns; ++t) {
        double rv2 = 1.0 / (double)vv_t[t];
        double t0 = (double)t * dt;
        double th2 = 0.25 * t0 * t0;
        double as = th2 + dS2 * rv2, ar = th2 + dR2 * rv2;
        if (as < 1e-30) as = 1e-30;
        if (ar < 1e-30) ar = 1e-30;
        double ts = sqrt(as), tr = sqrt(ar);
        double Tf = (ts + tr) / dt;
        if (!(Tf < ns - 1)) continue;
        double slx = (sx / ts + gx / tr) * rv2 * ax, sly = (sy / ts + gy / tr) * rv2 * ay;
        double Lf = 1.0 + fabs(slx) + fabs(sly);
        if (Lf > J->lmax) Lf = J->lmax;
        double u = 1.0 / ts + 1.0 / tr;
        double w = t0 / 8.0 * u * u / (Lf * Lf);
        k[t] = (float)((double)k[t] + w * full_tri(f, ns, Tf, Lf));
        fo[t] = fo[t] + 1.0f;
    }
}

/* Image loop of Kirchhoff.c:1341-1403 for the columns a worker claims. */
static void *column_worker(void *arg)
{
    ko_job *J = (ko_job *)arg;
    const kpstm_params *p = J->p;
    const ko_dims *d = J->d;
    const int ns = d->ns, nh = d->nh;
    int64_t pairs = 0;
    double *vtmp = (double *)malloc(sizeof(double) * ns);
    float *vvt = (float *)malloc(sizeof(float) * ns);
    if (!vtmp || !vvt) {
        free(vtmp);
        free(vvt);
        pthread_mutex_lock(&J->mu);
        J->err = KPSTM_ERR_OUT_OF_MEMORY;
        pthread_mutex_unlock(&J->mu);
        return NULL;
    }
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int col = J->next_col++;
        pthread_mutex_unlock(&J->mu);
        if (col >= d->nx * d->ny) break;
        int xc = col / d->ny, yc = col % d->ny;
        float IX = (float)((p->start_iline + ((xc + d->xslice * d->nx) * p->inc_iline)) * p->iline_distance);
        float IY = (float)((p->start_xline + ((yc + d->yslice * d->ny) * p->inc_xline)) * p->xline_distance);
        int xc1 = (int)round((p->start_iline - J->v->o_iline) / J->v->d_iline +
                             (xc + d->xslice * d->nx) * (p->inc_iline / J->v->d_iline));
        int yc1 = (int)round((p->start_xline - J->v->o_xline) / J->v->d_xline +
                             (yc + d->yslice * d->ny) * (p->inc_xline / J->v->d_xline));
        if (xc1 > J->v->n_iline - 1) xc1 = J->v->n_iline - 1;
        if (yc1 > J->v->n_xline - 1) yc1 = J->v->n_xline - 1;
        const float *v2 = J->vel2 + ((size_t)(xc1 < 0 ? 0 : xc1) * J->v->n_xline + (yc1 < 0 ? 0 : yc1)) * J->v->nsm;
        int bad_vel = (xc1 < 0 || yc1 < 0);
        if (p->mode == KPSTM_MODE_FULL && !bad_vel) {
            /* v^2 per output sample as the product builds its rows: the nearest
               node's float v^2, or the interpolated v_rms squared in double */
            if (ko_col_vrms(p, J->v, xc + d->xslice * d->nx, yc + d->yslice * d->ny, ns, vtmp)) bad_vel = 1;
            for (int t = 0; t < ns && !bad_vel; ++t)
                vvt[t] = p->velocity_interp ? (float)(vtmp[t] * vtmp[t]) : v2[J->t1[t]];
        }
        float *km = J->km + (size_t)col * nh * ns;
        float *fold = J->fold + (size_t)col * nh * ns;
        for (int64_t it = 0; it < J->ntr; ++it) {
            const ko_geom *g = &J->geom[it];
            if (!g->live) continue;
            float dIS2 = (IX - g->sxt) * (IX - g->sxt) + (IY - g->syt) * (IY - g->syt);
            float dIR2 = (IX - g->gxt) * (IX - g->gxt) + (IY - g->gyt) * (IY - g->gyt);
            float dIC = sqrtf((IX - g->cmpx) * (IX - g->cmpx) + (IY - g->cmpy) * (IY - g->cmpy));
            if (!((double)dIC < p->aperture)) continue;
            if (bad_vel) {
                pthread_mutex_lock(&J->mu);
                J->err = KPSTM_ERR_VELOCITY_RANGE;
                pthread_mutex_unlock(&J->mu);
                break;
            }
            float *k = km + (size_t)g->off * ns;
            float *f = fold + (size_t)g->off * ns;
            if (p->mode == KPSTM_MODE_FULL) {
                full_pairs(J, g, IX, IY, vvt, J->P + (size_t)it * ns, k, f);
                pairs += ns;
                continue;
            }
            const float *Dt = J->D + (size_t)it * ns;
            for (int t = 0; t < ns; ++t) {
                float vv = v2[J->t1[t]];
                float s1 = J->t2[t] + dIS2 / vv;
                float s2 = J->t2[t] + dIR2 / vv;
                float dsr = (float)(sqrt((double)s1) + sqrt((double)s2));
                int T = (int)floor(dsr / d->dt);
                if (T < ns) {
                    k[t] = k[t] + Dt[T];
                    f[t] = f[t] + 1.0f;
                }
            }
            pairs += ns;
        }
    }
    free(vtmp);
    free(vvt);
    pthread_mutex_lock(&J->mu);
    J->pairs += pairs;
    pthread_mutex_unlock(&J->mu);
    return NULL;
}

int ko_finish(const kpstm_params *p, const float *km, const float *fold, float *image)
{
    ko_dims d;
    int st = ko_dims_of(p, &d);
    if (st) return st;
    int ns = d.ns;
    float *aa = (float *)malloc(sizeof(float) * ns);
    double *x = (double *)malloc(sizeof(double) * 2 * ns);
    double *X = (double *)malloc(sizeof(double) * 2 * ns);
    double *y = (double *)malloc(sizeof(double) * 2 * ns);
    if (!aa || !x || !X || !y) {
        free(aa); free(x); free(X); free(y);
        return KPSTM_ERR_OUT_OF_MEMORY;
    }
    ko_aliasfilter(ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, NULL, aa);
    float dt = p->dt;
    size_t ntrace = (size_t)d.nx * d.ny * d.nh;
    for (size_t tr = 0; tr < ntrace; ++tr) {
        const float *k = km + tr * ns;
        const float *f = fold + tr * ns;
        x[0] = 0.0;
        x[1] = 0.0;
        for (int t = 1; t < ns; ++t) { /* Kirchhoff.c:1457-1462 */
            float v = ((((-dt) * (float)t) * (k[t] - k[t - 1])) * dt) / f[t];
            x[2 * t] = v;
            x[2 * t + 1] = 0.0;
        }
        kref_dft(ns, FFTW_FORWARD, x, X); /* :1465 */
        for (int t = 0; t < ns; ++t) {    /* :1467-1473; a,b,c,d are float (:1419) */
            float a = aa[t], b = 0.0f, c = (float)X[2 * t], e = (float)X[2 * t + 1];
            X[2 * t] = (double)(a * c - b * e);
            X[2 * t + 1] = (double)(a * e + b * c);
        }
        kref_dft(ns, FFTW_BACKWARD, X, y); /* :1474 */
        float *o = image + tr * ns;
        o[0] = 0.0f;
        for (int t = 1; t < ns; ++t) o[t] = (float)(y[2 * t] / ns); /* :1475-1479 */
    }
    free(aa); free(x); free(X); free(y);
    return KPSTM_OK;
}

int ko_kirchhoff(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be,
                 const float *samples, int64_t ntr, float *km_out, float *fold_out, float *image,
                 int nthreads, int64_t *pairs_out)
{
    if (!p || !v || !v->vrms || (ntr > 0 && (!hdr_be || !samples)) || ntr < 0)
        return KPSTM_ERR_INVALID_ARG;
    if (p->mode != KPSTM_MODE_REFERENCE && p->mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED;
    const int full = p->mode == KPSTM_MODE_FULL;
    ko_dims d;
    int st = ko_dims_of(p, &d);
    if (st) return st;
    const int ns = d.ns, nh = d.nh;
    int tm;
    ko_aliasfilter(ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, &tm, NULL);
    if (tm < 2) return KPSTM_ERR_TRANGE;
    d.trange_max = tm;

    size_t nvel = (size_t)v->n_iline * v->n_xline * v->nsm;
    size_t nimg = (size_t)d.nx * d.ny * nh * ns;
    float *vel2 = (float *)malloc(sizeof(float) * nvel);
    float *t2 = (float *)malloc(sizeof(float) * ns);
    int *t1 = (int *)malloc(sizeof(int) * ns);
    ko_geom *geom = (ko_geom *)calloc((size_t)(ntr > 0 ? ntr : 1), sizeof(ko_geom));
    const size_t prow = (size_t)ns + 2 * tm;
    float *D = (float *)malloc(sizeof(float) * (size_t)(ntr > 0 ? ntr : 1) * (full ? prow : (size_t)ns));
    float *P = (float *)malloc(sizeof(float) * prow);
    float *km = (float *)calloc(nimg, sizeof(float));
    float *fold = (float *)malloc(sizeof(float) * nimg);
    if (!vel2 || !t2 || !t1 || !geom || !D || !P || !km || !fold) {
        st = KPSTM_ERR_OUT_OF_MEMORY;
        goto done;
    }
    for (size_t i = 0; i < nvel; ++i) { /* Kirchhoff.c:612-618 */
        if (v->vrms[i] == 0.0f) { st = KPSTM_ERR_VELOCITY_ZERO; goto done; }
        vel2[i] = v->vrms[i] * v->vrms[i];
    }
    for (size_t i = 0; i < nimg; ++i) fold[i] = 1.0f; /* :1270 */
    for (int t = 0; t < ns; ++t) { /* :1246-1247, 1376-1378 */
        t2[t] = (float)(0.25 * t * t * (double)p->dt * (double)p->dt);
        int q = (int)round((double)((float)t * (p->dt / v->dtm)));
        t1[t] = q > v->nsm - 1 ? v->nsm - 1 : q;
    }
    /* slab centre and half-diagonal, Kirchhoff.c:1332-1335 */
    float IXc = (float)((p->start_iline + ((d.nx / 2.0 + d.xslice * d.nx) * p->inc_iline)) * p->iline_distance);
    float IYc = (float)((p->start_xline + ((d.ny / 2.0 + d.yslice * d.ny) * p->inc_xline)) * p->xline_distance);
    float add_on = (float)(0.5 * sqrt(d.nx * p->inc_iline * p->iline_distance * d.nx * p->inc_iline * p->iline_distance +
                                      d.ny * p->inc_xline * p->xline_distance * d.ny * p->inc_xline * p->xline_distance));
    for (int64_t it = 0; it < ntr; ++it) {
        const int32_t *h = hdr_be + (size_t)it * 60;
        double w[4];
        for (int k = 0; k < 4; ++k) w[k] = (double)be32(h[18 + k]) - (k % 2 == 0 ? p->ox : p->oy);
        for (int k = 0; k < 4; ++k)
            if (!(w[k] > -2147483649.0 && w[k] < 2147483648.0)) { st = KPSTM_ERR_GEOMETRY; goto done; }
        int i = (int)w[0], j = (int)w[1];
        ko_geom *g = &geom[it];
        g->sxt = d.cosA * (float)i + d.sinA * (float)j; /* :1297-1299 */
        g->syt = -d.sinA * (float)i + d.cosA * (float)j;
        i = (int)w[2];
        j = (int)w[3];
        g->gxt = d.cosA * (float)i + d.sinA * (float)j; /* :1302-1304 */
        g->gyt = -d.sinA * (float)i + d.cosA * (float)j;
        float h2 = (float)(0.25 * (double)((g->sxt - g->gxt) * (g->sxt - g->gxt) +
                                           (g->syt - g->gyt) * (g->syt - g->gyt)));
        g->cmpx = (float)(0.5 * (double)(g->sxt + g->gxt));
        g->cmpy = (float)(0.5 * (double)(g->syt + g->gyt));
        int off = (int)floor((2.0 * sqrt((double)h2) - p->oh) / p->dh); /* :1310 */
        if (p->output == KPSTM_OUT_STACK) off = (off >= 0 && off < p->nh) ? 0 : -1;
        g->off = off;
        float dIC = sqrtf((IXc - g->cmpx) * (IXc - g->cmpx) + (IYc - g->cmpy) * (IYc - g->cmpy));
        g->live = (off >= 0 && off < nh) && ((double)dIC < p->aperture + (double)add_on);
        if (g->live && full) {
            memcpy(D + (size_t)it * ns, samples + (size_t)it * ns, sizeof(float) * ns);
        } else if (g->live) {
            ko_prep_trace(ns, tm, p->dt, t2, samples + (size_t)it * ns, P);
            float *Dt = D + (size_t)it * ns;
            for (int T = 0; T < ns; ++T) /* :1391-1392, taps at T and T +- 2 */
                Dt[T] = (float)(-2.0 * (double)P[T + tm] + (double)P[T + tm - 2] + (double)P[T + tm + 2]);
        }
    }
    {
        ko_job J;
        memset(&J, 0, sizeof(J));
        J.p = p; J.v = v; J.d = &d; J.vel2 = vel2; J.t2 = t2; J.t1 = t1; J.geom = geom; J.D = D;
        J.P = D;
        J.tm = tm;
        {
            int lmax = p->aa_max_halfwidth > 0 ? p->aa_max_halfwidth : tm - 1;
            if (lmax > tm - 1) lmax = tm - 1;
            if (lmax > 63) lmax = 63;
            if (lmax < 1) lmax = 1;
            J.lmax = lmax;
        }
        J.ntr = ntr; J.km = km; J.fold = fold;
        pthread_mutex_init(&J.mu, NULL);
        if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
        if (nthreads < 1) nthreads = 1;
        if (nthreads > 256) nthreads = 256;
        pthread_t th[256];
        int started = 0;
        for (int k = 0; k < nthreads; ++k)
            if (pthread_create(&th[k], NULL, column_worker, &J) == 0) started++;
        if (started == 0) column_worker(&J);
        for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
        pthread_mutex_destroy(&J.mu);
        if (J.err) { st = J.err; goto done; }
        if (pairs_out) *pairs_out = J.pairs;
    }
    if (km_out) memcpy(km_out, km, sizeof(float) * nimg);
    if (fold_out) memcpy(fold_out, fold, sizeof(float) * nimg);
    if (image) st = ko_finish(p, km, fold, image);
done:
    free(vel2); free(t2); free(t1); free(geom); free(D); free(P); free(km); free(fold);
    return st;
}

/* Least-squares operator pair (full physics, see full_pairs), in double.
   The pair set and the geometry follow ko_kirchhoff exactly; every pair
   couples data sample k of the trace with model sample t of the column by
   t0 (1/ts + 1/tr)^2 / (8 Lf^2) * max(0, Lf - |T - k|).
   Threads: L^T (direction 0) splits the image columns, L (direction 1) the
   traces, so every output element is summed by one thread in the order of
   the single-threaded loop (traces in order for a model sample, columns in
   (xc, yc) order for a data sample) and the result does not depend on the
   thread count. */
typedef struct {
    float sxt, syt, gxt, gyt, cmpx, cmpy;
    int off, live;
} ko_lgeom;

typedef struct {
    const kpstm_params *p;
    const ko_dims *d;
    const ko_lgeom *geom;
    const double *vcol;    /* [ncol][ns] v_rms per column and sample, or NaN row: below the grid */
    int64_t ntr;
    int direction, lmax;
    const double *in;
    double *out;
    int64_t next;
    int err;
    pthread_mutex_t mu;
} ko_ljob;

/* the pairs of (trace g, column col): d = L m adds to out_d, m = L^T d adds to out_m */
static int ko_lsm_pairs(const ko_ljob *J, const ko_lgeom *g, int64_t it, int col)
{
    const kpstm_params *p = J->p;
    const ko_dims *d = J->d;
    const int ns = d->ns, nh = d->nh;
    const int xc = col / d->ny, yc = col % d->ny;
    float IX = (float)((p->start_iline + ((xc + d->xslice * d->nx) * p->inc_iline)) * p->iline_distance);
    float IY = (float)((p->start_xline + ((yc + d->yslice * d->ny) * p->inc_xline)) * p->xline_distance);
    float cdx = IX - g->cmpx, cdy = IY - g->cmpy;
    float dC = sqrtf(cdx * cdx + cdy * cdy);
    if (!((double)dC < p->aperture)) return 0;
    const double *vcol = J->vcol + (size_t)col * ns;
    if (vcol[0] != vcol[0]) return KPSTM_ERR_VELOCITY_RANGE;
    const double dt = (double)p->dt;
    const double ax = p->iline_distance / dt, ay = p->xline_distance / dt;
    const double sx = (double)IX - g->sxt, sy = (double)IY - g->syt;
    const double gx = (double)IX - g->gxt, gy = (double)IY - g->gyt;
    const double dS2 = sx * sx + sy * sy, dR2 = gx * gx + gy * gy;
    const size_t mbase = ((size_t)col * nh + g->off) * ns;
    const size_t dbase = (size_t)it * ns;
    for (int t = 1; t < ns; ++t) {
        /* v^2 as the product stores it: the node's float square, or the
           interpolated v_rms squared in double, rounded to float */
        const float vvf = p->velocity_interp ? (float)(vcol[t] * vcol[t]) : (float)vcol[t] * (float)vcol[t];
        double rv2 = 1.0 / (double)vvf;
        double t0 = (double)t * dt;
        double th2 = 0.25 * t0 * t0;
        double ts = sqrt(th2 + dS2 * rv2), tr = sqrt(th2 + dR2 * rv2);
        double T = (ts + tr) / dt;
        if (!(T < ns - 1)) continue;
        double Lf = 1.0 + fabs((sx / ts + gx / tr) * rv2 * ax) + fabs((sy / ts + gy / tr) * rv2 * ay);
        if (Lf > J->lmax) Lf = J->lmax;
        double u = 1.0 / ts + 1.0 / tr;
        double W = t0 / 8.0 * u * u / (Lf * Lf);
        int k0 = (int)ceil(T - Lf), k1 = (int)floor(T + Lf);
        if (k0 < 0) k0 = 0;
        if (k1 > ns - 1) k1 = ns - 1;
        if (J->direction == 0) {
            double tri = 0.0;
            for (int k = k0; k <= k1; ++k) {
                double wk = Lf - fabs(T - k);
                if (wk > 0) tri += J->in[dbase + k] * wk;
            }
            J->out[mbase + t] += W * tri;
        } else {
            double mv = W * J->in[mbase + t];
            for (int k = k0; k <= k1; ++k) {
                double wk = Lf - fabs(T - k);
                if (wk > 0) J->out[dbase + k] += mv * wk;
            }
        }
    }
    return 0;
}

static void *ko_lsm_worker(void *arg)
{
    ko_ljob *J = (ko_ljob *)arg;
    const int ncol = J->d->nx * J->d->ny;
    const int64_t nunit = J->direction == 0 ? ncol : J->ntr;
    int st = 0;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int64_t u = J->next++;
        const int stop = J->err != 0;
        pthread_mutex_unlock(&J->mu);
        if (u >= nunit || stop) break;
        if (J->direction == 0) { /* one column, every trace in order */
            for (int64_t it = 0; it < J->ntr && !st; ++it)
                if (J->geom[it].live) st = ko_lsm_pairs(J, &J->geom[it], it, (int)u);
        } else { /* one trace, every column in order */
            if (J->geom[u].live)
                for (int col = 0; col < ncol && !st; ++col) st = ko_lsm_pairs(J, &J->geom[u], u, col);
        }
        if (st) {
            pthread_mutex_lock(&J->mu);
            J->err = st;
            pthread_mutex_unlock(&J->mu);
            break;
        }
    }
    return NULL;
}

int ko_lsm_apply(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be, int64_t ntr,
                 int direction, const double *in, double *out)
{
    if (!p || !v || !hdr_be || !in || !out || ntr <= 0) return KPSTM_ERR_INVALID_ARG;
    if (p->mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED;
    ko_dims d;
    int st = ko_dims_of(p, &d);
    if (st) return st;
    const int ns = d.ns, nh = d.nh, ncol = d.nx * d.ny;
    int tm;
    ko_aliasfilter(ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, &tm, NULL);
    if (tm < 2) return KPSTM_ERR_TRANGE;
    int lmax = p->aa_max_halfwidth > 0 ? p->aa_max_halfwidth : tm - 1;
    if (lmax > tm - 1) lmax = tm - 1;
    if (lmax > 63) lmax = 63;
    if (lmax < 1) lmax = 1;
    const size_t nmod = (size_t)ncol * nh * ns;
    if (direction == 0) memset(out, 0, sizeof(double) * nmod);
    else memset(out, 0, sizeof(double) * (size_t)ntr * ns);
    ko_lgeom *geom = (ko_lgeom *)malloc(sizeof(ko_lgeom) * (size_t)ntr);
    double *vcol = (double *)malloc(sizeof(double) * (size_t)ncol * ns);
    if (!geom || !vcol) {
        free(geom);
        free(vcol);
        return KPSTM_ERR_OUT_OF_MEMORY;
    }
    for (int col = 0; col < ncol; ++col) { /* v_rms of every column once (NaN row: below the grid) */
        double *vc = vcol + (size_t)col * ns;
        if (ko_col_vrms(p, v, col / d.ny + d.xslice * d.nx, col % d.ny + d.yslice * d.ny, ns, vc))
            for (int t = 0; t < ns; ++t) vc[t] = NAN;
    }
    float IXc = (float)((p->start_iline + ((d.nx / 2.0 + d.xslice * d.nx) * p->inc_iline)) * p->iline_distance);
    float IYc = (float)((p->start_xline + ((d.ny / 2.0 + d.yslice * d.ny) * p->inc_xline)) * p->xline_distance);
    float add_on = (float)(0.5 * sqrt(d.nx * p->inc_iline * p->iline_distance * d.nx * p->inc_iline * p->iline_distance +
                                      d.ny * p->inc_xline * p->xline_distance * d.ny * p->inc_xline * p->xline_distance));
    for (int64_t it = 0; it < ntr; ++it) { /* geometry, class and slab cull as ko_kirchhoff */
        const int32_t *h = hdr_be + (size_t)it * 60;
        double w4[4];
        for (int k = 0; k < 4; ++k) w4[k] = (double)be32(h[18 + k]) - (k % 2 == 0 ? p->ox : p->oy);
        ko_lgeom *g = &geom[it];
        int i = (int)w4[0], j = (int)w4[1];
        g->sxt = d.cosA * (float)i + d.sinA * (float)j;
        g->syt = -d.sinA * (float)i + d.cosA * (float)j;
        i = (int)w4[2];
        j = (int)w4[3];
        g->gxt = d.cosA * (float)i + d.sinA * (float)j;
        g->gyt = -d.sinA * (float)i + d.cosA * (float)j;
        float h2 = (float)(0.25 * (double)((g->sxt - g->gxt) * (g->sxt - g->gxt) + (g->syt - g->gyt) * (g->syt - g->gyt)));
        g->cmpx = (float)(0.5 * (double)(g->sxt + g->gxt));
        g->cmpy = (float)(0.5 * (double)(g->syt + g->gyt));
        int off = (int)floor((2.0 * sqrt((double)h2) - p->oh) / p->dh);
        g->live = off >= 0 && off < p->nh;
        g->off = p->output == KPSTM_OUT_STACK ? 0 : off;
        float dIC = sqrtf((IXc - g->cmpx) * (IXc - g->cmpx) + (IYc - g->cmpy) * (IYc - g->cmpy));
        if (!((double)dIC < p->aperture + (double)add_on)) g->live = 0;
    }
    ko_ljob J;
    memset(&J, 0, sizeof(J));
    J.p = p;
    J.d = &d;
    J.geom = geom;
    J.vcol = vcol;
    J.ntr = ntr;
    J.direction = direction;
    J.lmax = lmax;
    J.in = in;
    J.out = out;
    pthread_mutex_init(&J.mu, NULL);
    long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
    int nth = ncpu > 0 ? (int)ncpu : 1;
    if (nth > 256) nth = 256;
    pthread_t th[256];
    int started = 0;
    for (int k = 1; k < nth; ++k)
        if (pthread_create(&th[started], NULL, ko_lsm_worker, &J) == 0) ++started;
    ko_lsm_worker(&J);
    for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
    pthread_mutex_destroy(&J.mu);
    st = J.err;
    free(geom);
    free(vcol);
    return st;
}

/* ------------------------------------------------------------------------ */
/* FP64 oracle. */
typedef struct {
    double sxt, syt, gxt, gyt, cx, cy;
    int off, live;
} ko_geom64;

typedef struct {
    const kpstm_params *p;
    const kpstm_velocity *v;
    const ko_dims *d;
    const ko_geom64 *geom;
    const double *D;       /* reference mode: [ntr][ns] taps */
    const float *samples;  /* full mode */
    const double *t2;
    const int *t1;
    int64_t ntr;
    int full, lmax;
    double *km, *fold;
    int next_col, err;
    pthread_mutex_t mu;
} ko_job64;

static void *column_worker64(void *arg)
{
    ko_job64 *J = (ko_job64 *)arg;
    const kpstm_params *p = J->p;
    const kpstm_velocity *v = J->v;
    const ko_dims *d = J->d;
    const int ns = d->ns, nh = d->nh;
    const double dt = (double)p->dt;
    double *vcol = (double *)malloc(sizeof(double) * ns);
    if (!vcol) {
        pthread_mutex_lock(&J->mu);
        J->err = KPSTM_ERR_OUT_OF_MEMORY;
        pthread_mutex_unlock(&J->mu);
        return NULL;
    }
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int col = J->next_col++;
        pthread_mutex_unlock(&J->mu);
        if (col >= d->nx * d->ny) break;
        const int xc = col / d->ny, yc = col % d->ny;
        const double IX = (p->start_iline + ((xc + d->xslice * d->nx) * p->inc_iline)) * p->iline_distance;
        const double IY = (p->start_xline + ((yc + d->yslice * d->ny) * p->inc_xline)) * p->xline_distance;
        /* v_rms per output sample (nearest node and sample, or trilinear) */
        const int bad = ko_col_vrms(p, v, xc + d->xslice * d->nx, yc + d->yslice * d->ny, ns, vcol) != 0;
        for (int64_t it = 0; it < J->ntr; ++it) {
            const ko_geom64 *g = &J->geom[it];
            if (!g->live) continue;
            if (!(sqrt((IX - g->cx) * (IX - g->cx) + (IY - g->cy) * (IY - g->cy)) < p->aperture)) continue;
            if (bad) {
                pthread_mutex_lock(&J->mu);
                J->err = KPSTM_ERR_VELOCITY_RANGE;
                pthread_mutex_unlock(&J->mu);
                break;
            }
            const double sx = IX - g->sxt, sy = IY - g->syt, gx = IX - g->gxt, gy = IY - g->gyt;
            const double dS2 = sx * sx + sy * sy, dR2 = gx * gx + gy * gy;
            double *k = J->km + ((size_t)col * nh + g->off) * ns;
            double *fo = J->fold + ((size_t)col * nh + g->off) * ns;
            const double *D = J->D ? J->D + (size_t)it * ns : NULL;
            const float *f = J->samples + (size_t)it * ns;
            for (int t = 0; t < ns; ++t) {
                const double vv = vcol[t] * vcol[t];
                if (!J->full) {
                    const double dsr = sqrt(J->t2[t] + dS2 / vv) + sqrt(J->t2[t] + dR2 / vv);
                    const double Tq = floor(dsr / dt);
                    if (Tq < ns) {
                        k[t] += D[(int)Tq];
                        fo[t] += 1.0;
                    }
                } else {
                    const double rv2 = 1.0 / vv, t0 = t * dt;
                    double as = 0.25 * t0 * t0 + dS2 * rv2, ar = 0.25 * t0 * t0 + dR2 * rv2;
                    if (as < 1e-30) as = 1e-30;
                    if (ar < 1e-30) ar = 1e-30;
                    const double ts = sqrt(as), tr = sqrt(ar), T = (ts + tr) / dt;
                    if (!(T < ns - 1)) continue;
                    double Lf = 1.0 + fabs((sx / ts + gx / tr) * rv2 * p->iline_distance / dt) +
                                fabs((sy / ts + gy / tr) * rv2 * p->xline_distance / dt);
                    if (Lf > J->lmax) Lf = J->lmax;
                    const double u = 1.0 / ts + 1.0 / tr;
                    k[t] += t0 / 8.0 * u * u / (Lf * Lf) * full_tri(f, ns, T, Lf);
                    fo[t] += 1.0;
                }
            }
        }
    }
    free(vcol);
    return NULL;
}

int ko_kirchhoff64(const kpstm_params *p, const kpstm_velocity *v, const int32_t *hdr_be,
                   const float *samples, int64_t ntr, double *km_out, double *fold_out, double *image)
{
    if (!p || !v || (ntr > 0 && (!hdr_be || !samples))) return KPSTM_ERR_INVALID_ARG;
    ko_dims d;
    int st = ko_dims_of(p, &d);
    if (st) return st;
    const int ns = d.ns, nh = d.nh, full = p->mode == KPSTM_MODE_FULL;
    int tm;
    ko_aliasfilter(ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, &tm, NULL);
    if (tm < 2) return KPSTM_ERR_TRANGE;
    int lmax = p->aa_max_halfwidth > 0 ? p->aa_max_halfwidth : tm - 1;
    if (lmax > tm - 1) lmax = tm - 1;
    if (lmax > 63) lmax = 63;
    if (lmax < 1) lmax = 1;
    const double dt = (double)p->dt;
    const double cosA = cos(p->angle_e_to_n_deg * KO_PI / 180.0), sinA = sin(p->angle_e_to_n_deg * KO_PI / 180.0);
    const size_t nimg = (size_t)d.nx * d.ny * nh * ns;
    double *km = (double *)calloc(nimg, sizeof(double));
    double *fold = (double *)malloc(sizeof(double) * nimg);
    double *P = (double *)malloc(sizeof(double) * (ns + 2 * tm));
    double *D = full ? NULL : (double *)malloc(sizeof(double) * (size_t)(ntr > 0 ? ntr : 1) * ns);
    double *t2 = (double *)malloc(sizeof(double) * ns);
    int *t1 = (int *)malloc(sizeof(int) * ns);
    ko_geom64 *geom = (ko_geom64 *)calloc((size_t)(ntr > 0 ? ntr : 1), sizeof(ko_geom64));
    if (!km || !fold || !P || (!full && !D) || !t2 || !t1 || !geom) {
        st = KPSTM_ERR_OUT_OF_MEMORY;
        goto done64;
    }
    for (size_t i = 0; i < nimg; ++i) fold[i] = 1.0;
    for (int t = 0; t < ns; ++t) {
        t2[t] = 0.25 * t * t * dt * dt;
        int q = (int)round((double)t * dt / (double)v->dtm);
        t1[t] = q > v->nsm - 1 ? v->nsm - 1 : q;
    }
    {
        const double IXc = (p->start_iline + ((d.nx / 2.0 + d.xslice * d.nx) * p->inc_iline)) * p->iline_distance;
        const double IYc = (p->start_xline + ((d.ny / 2.0 + d.yslice * d.ny) * p->inc_xline)) * p->xline_distance;
        const double add_on = 0.5 * sqrt(d.nx * p->inc_iline * p->iline_distance * d.nx * p->inc_iline * p->iline_distance +
                                         d.ny * p->inc_xline * p->xline_distance * d.ny * p->inc_xline * p->xline_distance);
        for (int64_t it = 0; it < ntr; ++it) {
            const int32_t *h = hdr_be + (size_t)it * 60;
            double w4[4];
            for (int k = 0; k < 4; ++k) w4[k] = (double)be32(h[18 + k]) - (k % 2 == 0 ? p->ox : p->oy);
            const double si = (double)(int)w4[0], sj = (double)(int)w4[1];
            const double gi = (double)(int)w4[2], gj = (double)(int)w4[3];
            ko_geom64 *g = &geom[it];
            g->sxt = cosA * si + sinA * sj;
            g->syt = -sinA * si + cosA * sj;
            g->gxt = cosA * gi + sinA * gj;
            g->gyt = -sinA * gi + cosA * gj;
            const double h2 = 0.25 * ((g->sxt - g->gxt) * (g->sxt - g->gxt) + (g->syt - g->gyt) * (g->syt - g->gyt));
            g->cx = 0.5 * (g->sxt + g->gxt);
            g->cy = 0.5 * (g->syt + g->gyt);
            int off = (int)floor((2.0 * sqrt(h2) - p->oh) / p->dh);
            if (!(off >= 0 && off < p->nh)) continue;
            g->off = p->output == KPSTM_OUT_STACK ? 0 : off;
            g->live = sqrt((IXc - g->cx) * (IXc - g->cx) + (IYc - g->cy) * (IYc - g->cy)) < p->aperture + add_on;
            if (g->live && !full) { /* reference operator in double (Kirchhoff.c:1312-1328, 1391-1392) */
                const float *f = samples + (size_t)it * ns;
                P[tm] = f[0];
                for (int t = 1; t < ns; ++t) P[t + tm] = P[t - 1 + tm] + (double)f[t] / (4.0 * t2[t]);
                for (int t = ns; t < ns + tm; ++t) P[t + tm] = P[t - 1 + tm] + (double)f[ns - 1] / (dt * dt * t * t);
                for (int t = 1; t < ns + tm; ++t) P[t + tm] = P[t - 1 + tm] + P[t + tm];
                for (int t = 0; t < tm; ++t) P[t] = P[2 * tm - t];
                double *Dt = D + (size_t)it * ns;
                for (int T = 0; T < ns; ++T) Dt[T] = -2.0 * P[T + tm] + P[T + tm - 2] + P[T + tm + 2];
            }
        }
    }
    {
        ko_job64 J;
        memset(&J, 0, sizeof(J));
        J.p = p; J.v = v; J.d = &d; J.geom = geom; J.D = D; J.samples = samples; J.t2 = t2; J.t1 = t1;
        J.ntr = ntr; J.full = full; J.lmax = lmax; J.km = km; J.fold = fold;
        pthread_mutex_init(&J.mu, NULL);
        int nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
        if (nthreads < 1) nthreads = 1;
        if (nthreads > 256) nthreads = 256;
        pthread_t th[256];
        int started = 0;
        for (int k = 0; k < nthreads; ++k)
            if (pthread_create(&th[k], NULL, column_worker64, &J) == 0) started++;
        if (started == 0) column_worker64(&J);
        for (int k = 0; k < started; ++k) pthread_join(th[k], NULL);
        pthread_mutex_destroy(&J.mu);
        st = J.err;
    }
    if (!st && image) { /* finishing in double (Kirchhoff.c:1457-1479) */
        double *x = (double *)malloc(sizeof(double) * 2 * ns), *X = (double *)malloc(sizeof(double) * 2 * ns);
        double *y = (double *)malloc(sizeof(double) * 2 * ns), *aa = (double *)malloc(sizeof(double) * ns);
        if (!x || !X || !y || !aa) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
        } else {
            const double fs = 2.0 / dt / ns, fm = 3.0 * p->anti_alias_cutoff;
            for (int i = 0; i < ns; ++i) aa[i] = 0.0;
            for (int i = 0; i <= ns / 2; ++i) {
                const double q = i * fs;
                aa[i] = 1.0 / sqrt(1.0 + q * q * q * q / (fm * fm * fm * fm));
            }
            for (int i = ns / 2; i < ns; ++i) aa[i] = aa[ns - i];
            for (size_t tr = 0; tr < nimg / ns; ++tr) {
                const double *kk = km + tr * ns, *ff = fold + tr * ns;
                x[0] = x[1] = 0.0;
                for (int t = 1; t < ns; ++t) {
                    x[2 * t] = -dt * t * (kk[t] - kk[t - 1]) * dt / ff[t];
                    x[2 * t + 1] = 0.0;
                }
                kref_dft(ns, FFTW_FORWARD, x, X);
                for (int t = 0; t < ns; ++t) {
                    X[2 * t] *= aa[t];
                    X[2 * t + 1] *= aa[t];
                }
                kref_dft(ns, FFTW_BACKWARD, X, y);
                double *o = image + tr * ns;
                o[0] = 0.0;
                for (int t = 1; t < ns; ++t) o[t] = y[2 * t] / ns;
            }
        }
        free(x); free(X); free(y); free(aa);
    }
    if (!st && km_out) memcpy(km_out, km, sizeof(double) * nimg);
    if (!st && fold_out) memcpy(fold_out, fold, sizeof(double) * nimg);
done64:
    free(km); free(fold); free(P); free(D); free(t2); free(t1); free(geom);
    return st;
}
