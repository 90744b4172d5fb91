/*
 * Host-side set-up of libkpstm: the parts of the reference's main(),
 * create_aliasfilter(), build_vel_model() and SEG-Y/SU handling that run
 * once per job or per file, restated in C.
 *
 * Compiled with -ffp-contract=off: every float expression here is rounded
 * operation by operation as the reference's own build rounds it (gcc, no
 * FMA contraction), on x86-64 and aarch64 alike.  Where the reference is
 * built with -ffast-math (Kirchhoff.c:3) and gcc rewrites a chain of
 * divisions (a/b)/c into a/(b*c), the rewritten form is used and marked.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "kpstm_internal.h"

static uint32_t be32(uint32_t u)
{
    return (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
}

static void put_be32(uint8_t *p, int32_t v)
{
    uint32_t u = (uint32_t)v;
    p[0] = (uint8_t)(u >> 24);
    p[1] = (uint8_t)(u >> 16);
    p[2] = (uint8_t)(u >> 8);
    p[3] = (uint8_t)u;
}

static void put_be16(uint8_t *p, uint16_t v)
{
    p[0] = (uint8_t)(v >> 8);
    p[1] = (uint8_t)v;
}

int kpstm_abi_version(void) { return KPSTM_ABI_VERSION; }

const char *kpstm_strerror(int st)
{
    switch (st) {
    case KPSTM_OK: return "ok";
    case KPSTM_ERR_INVALID_ARG: return "invalid argument";
    case KPSTM_ERR_CUDA: return "CUDA runtime error";
    case KPSTM_ERR_OUT_OF_MEMORY: return "out of memory";
    case KPSTM_ERR_VELOCITY_ZERO: return "zero v_rms sample in the velocity model";
    case KPSTM_ERR_VELOCITY_RANGE: return "image column below the velocity grid origin";
    case KPSTM_ERR_GEOMETRY: return "trace coordinate outside the int range after the origin shift";
    case KPSTM_ERR_STATE: return "call out of order";
    case KPSTM_ERR_TIMEOUT: return "device wait timed out";
    case KPSTM_ERR_NO_DEVICE: return "no CUDA device";
    case KPSTM_ERR_SEGY: return "malformed SEG-Y data";
    case KPSTM_ERR_UNSUPPORTED: return "not supported by this build";
    case KPSTM_ERR_TRANGE: return "trangeMax < 2: triangle taps would leave the trace";
    case KPSTM_ERR_TOO_LARGE: return "image or trace length beyond the fixed scratch of kpstm_finish_noalloc";
    default: return "unknown status";
    }
}

/* create_aliasfilter, Kirchhoff.c:380-441.  tanA, mm, fmax are floats; the
   chains V_max/4.0/mm/tanA, 1.0/2.0/fmax/dt, 2.0/dt/ns and
   x/fmax/fmax/fmax/fmax are the fast-math a/(b*c) forms. */
int kpstm_aliasfilter(int32_t ns, float dt, double il_dist, double xl_dist, double cutoff,
                      int32_t *trange_max, float *anti_alias)
{
    if (ns <= 0 || !(dt > 0.0f) || !(il_dist > 0.0) || !(xl_dist > 0.0)) return KPSTM_ERR_INVALID_ARG;
    const float DIP = 45.0f, V_max = 1500.0f;
    float tanA = (float)tan(DIP * KPSTM_PI / 180.0);
    float mm = (float)(il_dist <= xl_dist ? il_dist : xl_dist);
    float fmax = (float)((double)V_max / ((4.0 * (double)mm) * (double)tanA));
    if (trange_max) *trange_max = (int32_t)floor(0.5 / ((double)fmax * (double)dt));
    if (!anti_alias) return KPSTM_OK;
    float fs = (float)(2.0 / ((double)dt * (double)ns));
    float fm = (float)cutoff;
    fm = (float)((double)fm * 3.0);
    float den = ((fm * fm) * fm) * fm;
    for (int i = 0; i < ns; ++i) anti_alias[i] = 0.0f; /* calloc'd array, Kirchhoff.c:1053 */
    for (int i = 0; i <= ns / 2; ++i) {
        float x = (float)i * fs;
        float num = ((x * x) * x) * x;
        anti_alias[i] = (float)(1.0 / sqrt(1.0 + (double)(num / den)));
    }
    /* Kirchhoff.c:419-423: for odd ns this copies the still-zero bin ns/2+1
       into ns/2 and back, leaving both zero. */
    for (int i = ns / 2; i < ns; ++i) anti_alias[i] = anti_alias[ns - i];
    return KPSTM_OK;
}

/* Kirchhoff.c:1284-1290 (also 524-530). */
int kpstm_ibm_to_ieee(const uint32_t *ibm_be, float *out, int64_t n)
{
    if ((n > 0 && (!ibm_be || !out)) || n < 0) return KPSTM_ERR_INVALID_ARG;
    for (int64_t i = 0; i < n; ++i) {
        int32_t w = (int32_t)be32(ibm_be[i]);
        int s = (((w >> 31) & 0x01) * (-2)) + 1;
        float frac = (float)(w & 0x00ffffff) / (float)0x1000000;
        float scale = (float)ldexp(1.0, 4 * (((w >> 24) & 0x7f) - 64)); /* 16^(e-64) */
        out[i] = ((float)s * frac) * scale;
    }
    return KPSTM_OK;
}

/* count_size_file, Kirchhoff.c:650-661. */
int kpstm_segy_info(const void *file_bytes, int64_t nbytes, int32_t *ns, float *dt, int64_t *ntraces)
{
    if (!file_bytes || nbytes < 3600 + 240) return KPSTM_ERR_SEGY;
    const uint8_t *b = (const uint8_t *)file_bytes;
    uint16_t ns1 = (uint16_t)((b[3600 + 114] << 8) | b[3600 + 115]);
    uint16_t dt1 = (uint16_t)((b[3600 + 116] << 8) | b[3600 + 117]);
    if (ns1 == 0 || dt1 == 0) return KPSTM_ERR_SEGY;
    if (ns) *ns = ns1;
    if (dt) *dt = (float)(dt1 / 1000000.0);
    if (ntraces) *ntraces = (nbytes - 3600) / (240 + (int64_t)ns1 * 4);
    return KPSTM_OK;
}

/* main(), Kirchhoff.c:266-313, plus the derived constants kirchhoff() uses. */
int kpstm_setup_of(const kpstm_params *p, kpstm_setup *s)
{
    if (!p || !s) return KPSTM_ERR_INVALID_ARG;
    if (p->velocity_interp != 0 && p->velocity_interp != 1) return KPSTM_ERR_INVALID_ARG;
    if (p->velocity_interp && p->mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED; /* reference mode is exact */
    if (p->ns < 8 || p->ns > 32768 || !(p->dt > 0.0f) || p->nh <= 0 || p->nh > KPSTM_MAX_CLASSES ||
        p->jobs_x <= 0 || p->jobs_y <= 0 || p->job_id < 0 || p->job_id >= p->jobs_x * p->jobs_y ||
        !(p->iline_distance > 0) || !(p->xline_distance > 0) || !(p->dh != 0) ||
        !(p->aperture > 0) || !(p->anti_alias_cutoff > 0) || !(p->xy_scale > 0) ||
        (p->mode != KPSTM_MODE_REFERENCE && p->mode != KPSTM_MODE_FULL) ||
        (p->precision != KPSTM_PREC_FP32 && p->precision != KPSTM_PREC_BF16_KAHAN) ||
        (p->output != KPSTM_OUT_OFFSET_GATHERS && p->output != KPSTM_OUT_STACK))
        return KPSTM_ERR_INVALID_ARG;
    memset(s, 0, sizeof(*s));
    kpstm_dims *d = &s->dims;
    int Nx = p->inc_iline == 0 ? 1 : (int)ceil((p->end_iline - p->start_iline) / p->inc_iline);
    int Ny = p->inc_xline == 0 ? 1 : (int)ceil((p->end_xline - p->start_xline) / p->inc_xline);
    if (Nx == 0) Nx = 1;
    if (Ny == 0) Ny = 1;
    if (Nx < 0 || Ny < 0) return KPSTM_ERR_INVALID_ARG;
    int nx = (int)ceil(1.0 * Nx / p->jobs_x);
    int ny = (int)ceil(1.0 * Ny / p->jobs_y);
    if (nx == 0) nx = 1;
    if (ny == 0) ny = 1;
    d->Nx = Nx;
    d->Ny = Ny;
    d->nx = nx;
    d->ny = ny;
    d->ns = p->ns;
    s->nclass = p->output == KPSTM_OUT_STACK ? 1 : p->nh;
    d->nh = s->nclass;
    s->xslice = p->job_id / p->jobs_y; /* Kirchhoff.c:286-294 */
    s->yslice = p->job_id % p->jobs_y;
    d->x0 = s->xslice * nx;
    d->y0 = s->yslice * ny;
    s->ncol = nx * ny;
    d->out_elems = (int64_t)nx * ny * s->nclass * p->ns;
    int32_t tm;
    kpstm_aliasfilter(p->ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, &tm, NULL);
    d->trange_max = tm;
    if (tm < 2) return KPSTM_ERR_TRANGE;
    s->sinA = (float)sin(p->angle_e_to_n_deg * KPSTM_PI / 180.0); /* :312-313 */
    s->cosA = (float)cos(p->angle_e_to_n_deg * KPSTM_PI / 180.0);
    /* slab centre and half diagonal, Kirchhoff.c:1332-1335 */
    s->IXc = (float)((p->start_iline + ((nx / 2.0 + s->xslice * nx) * p->inc_iline)) * p->iline_distance);
    s->IYc = (float)((p->start_xline + ((ny / 2.0 + s->yslice * ny) * p->inc_xline)) * p->xline_distance);
    float add_on = (float)(0.5 * sqrt(nx * p->inc_iline * p->iline_distance * nx * p->inc_iline * p->iline_distance +
                                      ny * p->inc_xline * p->xline_distance * ny * p->inc_xline * p->xline_distance));
    s->cull_radius = p->aperture + (double)add_on;
    int lmax = p->aa_max_halfwidth > 0 ? p->aa_max_halfwidth : tm - 1;
    if (lmax > tm - 1) lmax = tm - 1;
    if (lmax > 63) lmax = 63; /* size of the device 1/L^2 table */
    if (lmax < 1) lmax = 1;
    s->lmax = lmax;
    return KPSTM_OK;
}

int kpstm_velocity_check(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s)
{
    (void)p;
    (void)s;
    if (!v || !v->vrms || v->n_iline <= 0 || v->n_xline <= 0 || v->nsm <= 0 || v->d_iline == 0 ||
        v->d_xline == 0 || !(v->dtm > 0.0f))
        return KPSTM_ERR_INVALID_ARG;
    size_t n = (size_t)v->n_iline * v->n_xline * v->nsm;
    for (size_t i = 0; i < n; ++i) /* Kirchhoff.c:612-615 reports zero samples */
        if (v->vrms[i] == 0.0f || !isfinite(v->vrms[i])) return KPSTM_ERR_VELOCITY_ZERO;
    return KPSTM_OK;
}

/* Kirchhoff.c:1346-1347 (IX, IY) and 1357-1365 (velocity grid indices:
   integer division of the origin difference, round(), upper clamp only). */
int kpstm_columns(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s,
                  float *colxy, int32_t *colrow)
{
    const int nx = s->dims.nx, ny = s->dims.ny;
    for (int xc = 0; xc < nx; ++xc) {
        for (int yc = 0; yc < ny; ++yc) {
            int c = xc * ny + yc;
            colxy[2 * c] = (float)((p->start_iline + ((xc + s->xslice * nx) * p->inc_iline)) * p->iline_distance);
            colxy[2 * c + 1] = (float)((p->start_xline + ((yc + s->yslice * ny) * p->inc_xline)) * p->xline_distance);
            int xc1 = (int)round((p->start_iline - v->o_iline) / v->d_iline +
                                 (xc + s->xslice * nx) * (p->inc_iline / v->d_iline));
            int yc1 = (int)round((p->start_xline - v->o_xline) / v->d_xline +
                                 (yc + s->yslice * ny) * (p->inc_xline / v->d_xline));
            if (xc1 > v->n_iline - 1) xc1 = v->n_iline - 1;
            if (yc1 > v->n_xline - 1) yc1 = v->n_xline - 1;
            /* The reference has no lower clamp (Kirchhoff.c:1367-1371 is
               commented out) and would read outside the model; such a column
               is marked and reported if a trace reaches it. */
            colrow[c] = (xc1 < 0 || yc1 < 0) ? -1 : xc1 * v->n_xline + yc1;
        }
    }
    return KPSTM_OK;
}

/* Velocity rows of every column by trilinear interpolation of v_rms
   (kpstm_params.velocity_interp = 1): at the continuous grid position the
   reference rounds (Kirchhoff.c:1357-1365: integer division of the origin
   difference plus the column's fractional step) and the continuous sample
   t * (dt / dtm) it rounds (:1376-1378), each clamped to the grid; the
   interpolated v_rms is squared in double and stored as float, with
   RN(1/v^2) beside it.  rows: [ncol][ns] {v^2, 1/v^2}; columns whose rounded
   position is below the grid keep colrow = -1 (refused when reached). */
int kpstm_interp_rows(const kpstm_params *p, const kpstm_velocity *v, const kpstm_setup *s, const int32_t *colrow,
                      float *rows2)
{
    const int nx = s->dims.nx, ny = s->dims.ny, ns = p->ns, nsm = v->nsm;
    const float step = p->dt / v->dtm;
    double *acc = (double *)malloc(sizeof(double) * (size_t)nsm);
    if (!acc) return KPSTM_ERR_OUT_OF_MEMORY;
    for (int xc = 0; xc < nx; ++xc)
        for (int yc = 0; yc < ny; ++yc) {
            const int c = xc * ny + yc;
            float *row = rows2 + (size_t)c * 2 * ns;
            if (colrow[c] < 0) {
                for (int t = 0; t < ns; ++t) {
                    row[2 * t] = 1.0f;
                    row[2 * t + 1] = 1.0f;
                }
                continue;
            }
            double gx = (p->start_iline - v->o_iline) / v->d_iline + (xc + s->xslice * nx) * (p->inc_iline / v->d_iline);
            double gy = (p->start_xline - v->o_xline) / v->d_xline + (yc + s->yslice * ny) * (p->inc_xline / v->d_xline);
            gx = gx < 0.0 ? 0.0 : (gx > v->n_iline - 1 ? v->n_iline - 1 : gx);
            gy = gy < 0.0 ? 0.0 : (gy > v->n_xline - 1 ? v->n_xline - 1 : gy);
            const int i0 = (int)floor(gx), j0 = (int)floor(gy);
            const int i1 = i0 + 1 < v->n_iline ? i0 + 1 : i0, j1 = j0 + 1 < v->n_xline ? j0 + 1 : j0;
            const double wx = gx - i0, wy = gy - j0;
            const float *v00 = v->vrms + ((size_t)i0 * v->n_xline + j0) * nsm;
            const float *v01 = v->vrms + ((size_t)i0 * v->n_xline + j1) * nsm;
            const float *v10 = v->vrms + ((size_t)i1 * v->n_xline + j0) * nsm;
            const float *v11 = v->vrms + ((size_t)i1 * v->n_xline + j1) * nsm;
            for (int k = 0; k < nsm; ++k)
                acc[k] = (1.0 - wx) * ((1.0 - wy) * v00[k] + wy * v01[k]) + wx * ((1.0 - wy) * v10[k] + wy * v11[k]);
            for (int t = 0; t < ns; ++t) {
                double gt = (double)((float)t * step);
                gt = gt > nsm - 1 ? nsm - 1 : gt;
                const int k0 = (int)floor(gt), k1 = k0 + 1 < nsm ? k0 + 1 : k0;
                const double wt = gt - k0;
                const double vr = (1.0 - wt) * acc[k0] + wt * acc[k1];
                const float vv = (float)(vr * vr);
                if (!(vv > 0.0f)) {
                    free(acc);
                    return KPSTM_ERR_VELOCITY_ZERO;
                }
                row[2 * t] = vv;
                row[2 * t + 1] = 1.0f / vv;
            }
        }
    free(acc);
    return KPSTM_OK;
}

/* Kirchhoff.c:1246-1247 and 1376-1378. */
void kpstm_time_tables(const kpstm_params *p, const kpstm_velocity *v, float *t2, int32_t *t1)
{
    for (int t = 0; t < p->ns; ++t) {
        t2[t] = (float)(0.25 * t * t * (double)p->dt * (double)p->dt);
        int q = (int)round((double)((float)t * (p->dt / v->dtm)));
        t1[t] = q > v->nsm - 1 ? v->nsm - 1 : q;
    }
}

int kpstm_lowpass_kernel(const kpstm_params *p, double *h)
{
    const int ns = p->ns;
    float *aa = (float *)malloc(sizeof(float) * (size_t)ns);
    if (!aa) return KPSTM_ERR_OUT_OF_MEMORY;
    kpstm_aliasfilter(ns, p->dt, p->iline_distance, p->xline_distance, p->anti_alias_cutoff, NULL, aa);
    const double w = 6.283185307179586476925286766559 / ns;
    for (int m = 0; m < ns; ++m) {
        double acc = 0.0;
        for (int k = 0; k < ns; ++k) acc += (double)aa[k] * cos(w * (double)(((int64_t)k * m) % ns));
        h[m] = acc / ns;
    }
    free(aa);
    return KPSTM_OK;
}

/* The 240-byte header the reference writes per output trace,
   Kirchhoff.c:1482-1584.  tracl counts from nx*ny*nh*job_id + 1; the
   scratch words at bytes 204, 220, 224 and 232 hold 0 for the first trace
   of a job and 9999 afterwards, because the reference reuses its `mess`
   variable after writing 9999 into bytes 236-239 (:1581-1582). */
int kpstm_su_headers(const kpstm_params *p, const kpstm_setup *s, int32_t col, int32_t cls,
                     int64_t tracl, uint8_t *h)
{
    const int nx = s->dims.nx, ny = s->dims.ny;
    int xc = col / ny, yc = col % ny;
    memset(h, 0, 240);
    int first = tracl == (int64_t)nx * ny * s->nclass * p->job_id + 1;
    int cdp = (xc + s->xslice * nx) + s->dims.Nx * (yc + s->yslice * ny) + 1;
    int iline = (int)(p->start_iline + ((xc + s->xslice * nx) * p->inc_iline));
    int cline = (int)(p->start_xline + ((yc + s->yslice * ny) * p->inc_xline));
    int offset = (int)ceil(p->oh + cls * p->dh);
    int xc1 = (int)((p->start_iline + ((xc + s->xslice * nx) * p->inc_iline)) * p->iline_distance);
    int yc1 = (int)((p->start_xline + ((yc + s->yslice * ny) * p->inc_xline)) * p->xline_distance);
    int cdpx = (int)(((float)(int)p->ox + s->cosA * (float)xc1) - s->sinA * (float)yc1);
    int cdpy = (int)(((float)(int)p->oy + s->sinA * (float)xc1) + s->cosA * (float)yc1);
    put_be32(h + 0, (int32_t)tracl);
    put_be32(h + 20, cdp);
    put_be32(h + 36, offset);
    put_be32(h + 72, 1); /* sx, sy, gx, gy = 1 (Kirchhoff.c:1179-1182) */
    put_be32(h + 76, 1);
    put_be32(h + 80, 1);
    put_be32(h + 84, 1);
    put_be16(h + 114, (uint16_t)p->ns);
    put_be16(h + 116, (uint16_t)(p->dt * 1000000));
    put_be32(h + 180, cdpx);
    put_be32(h + 184, cdpy);
    put_be32(h + 188, iline);
    put_be32(h + 192, cline);
    if (!first) {
        put_be32(h + 204, 9999);
        put_be32(h + 220, 9999);
        put_be32(h + 224, 9999);
        put_be32(h + 232, 9999);
    }
    put_be32(h + 236, 9999);
    return KPSTM_OK;
}

/* Front headers of the output SEG-Y file, write_segy_ebdic_header
   (Kirchhoff.c:729-814): a 3200-byte text header and a 400-byte binary header
   that the combine script (:821-874) places before the slabs' SU records.
   Text: the reference formats two lines into the same buffer, so the second
   overwrites the start of the first ("written by G. O'Brien\n", NUL, then
   the tail "from prototype code\n" and its NUL: bytes 0-43); it leaves the
   rest of the 3200 bytes uninitialised, written as zeros here.  Binary header (16-bit
   big-endian words): 3213 traces per ensemble (the reference computes
   Nx*Ny*nh but writes an uninitialised short; the value is written here,
   truncated to 16 bits), 3217 sample interval in us, 3221 and 3223 samples
   per trace, 3225 format 5 (IEEE float), 3227, 3229, 3231 = 1; the rest
   zero. */
int kpstm_segy_front_headers(const kpstm_params *p, void *dst, int64_t dst_bytes)
{
    if (!p || !dst) return KPSTM_ERR_INVALID_ARG;
    if (dst_bytes < 3600) return KPSTM_ERR_INVALID_ARG;
    kpstm_setup s;
    int st = kpstm_setup_of(p, &s);
    if (st) return st;
    uint8_t *o = (uint8_t *)dst;
    memset(o, 0, 3600);
    static const char first[] = "outputting cdp gathers from prototype code\n";
    static const char second[] = "written by G. O'Brien\n";
    memcpy(o, first, sizeof(first));   /* with its NUL */
    memcpy(o, second, sizeof(second)); /* over the start, with its NUL */
    uint8_t *b = o + 3200;
    const int64_t ntr = (int64_t)s.dims.Nx * s.dims.Ny * s.dims.nh;
    put_be16(b + 12, (uint16_t)ntr);
    put_be16(b + 16, (uint16_t)(p->dt * 1000000));
    put_be16(b + 20, (uint16_t)p->ns);
    put_be16(b + 22, (uint16_t)p->ns);
    put_be16(b + 24, 5);
    put_be16(b + 26, 1);
    put_be16(b + 28, 1);
    put_be16(b + 30, 1);
    return KPSTM_OK;
}

/* build_vel_model (Kirchhoff.c:447-626): the gridded v_rms model from the
   velocity SEG-Y file image.  Sampling from the first trace header (:482-489,
   as kpstm_segy_info); for every trace in file order, header words 47 and 48
   (iline, xline, :537-538) give the cell (iline - o_iline) / d_iline,
   (xline - o_xline) / d_xline with C's truncating division (:539), and a cell
   inside the grid takes the trace's IBM-decoded samples (:524-530, 544) - a
   later trace overwrites an earlier one; cells no trace reaches stay 0 (the
   reference's calloc), which kpstm_create then reports as a zero velocity
   where a column needs it.  vrms: [n_iline][n_xline][nsm] floats, nsm from
   kpstm_segy_info. */
int kpstm_velocity_from_segy(const void *file_bytes, int64_t nbytes, int32_t n_iline, int32_t n_xline,
                             int32_t o_iline, int32_t o_xline, int32_t d_iline, int32_t d_xline, float *vrms,
                             int64_t vrms_elems)
{
    int32_t nsm = 0;
    float dtm = 0.0f;
    int64_t ntm = 0;
    int st = kpstm_segy_info(file_bytes, nbytes, &nsm, &dtm, &ntm);
    if (st) return st;
    if (!vrms || n_iline <= 0 || n_xline <= 0 || d_iline == 0 || d_xline == 0) return KPSTM_ERR_INVALID_ARG;
    if (vrms_elems < (int64_t)n_iline * n_xline * nsm) return KPSTM_ERR_INVALID_ARG;
    memset(vrms, 0, sizeof(float) * (size_t)n_iline * n_xline * nsm);
    const uint8_t *b = (const uint8_t *)file_bytes + 3600;
    const int64_t rec = 240 + 4 * (int64_t)nsm;
    for (int64_t k = 0; k < ntm; ++k) {
        const uint8_t *r = b + k * rec;
        const int32_t iline = (int32_t)(((uint32_t)r[188] << 24) | ((uint32_t)r[189] << 16) | ((uint32_t)r[190] << 8) | r[191]);
        const int32_t xline = (int32_t)(((uint32_t)r[192] << 24) | ((uint32_t)r[193] << 16) | ((uint32_t)r[194] << 8) | r[195]);
        const int32_t i = (iline - o_iline) / d_iline, j = (xline - o_xline) / d_xline;
        if (i < 0 || i >= n_iline || j < 0 || j >= n_xline) continue;
        st = kpstm_ibm_to_ieee((const uint32_t *)(const void *)(r + 240), vrms + ((int64_t)i * n_xline + j) * nsm, nsm);
        if (st) return st;
    }
    return KPSTM_OK;
}
