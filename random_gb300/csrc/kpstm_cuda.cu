/*
 * libkpstm: context, device memory, streams and the C ABI of include/kpstm.h.
 *
 * One context images one slab (job) of the reference's image box.  It owns
 * a compute stream and a copy stream: kpstm_add_traces copies block b+1 to
 * the device (copy stream) while block b is imaged (compute stream), using
 * two staging slots; the call returns once its own host buffers have been
 * read.  Per block the compute stream runs
 *     k_geometry -> k_bucket -> k_prep -> k_image
 * with no host synchronisation; kpstm_finish runs k_deriv -> k_lowpass.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "kpstm_kernels.cuh"

#define KP_CUDA(call)                                                                                        \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) {                                                                             \
            return e_ == cudaErrorMemoryAllocation ? KPSTM_ERR_OUT_OF_MEMORY : KPSTM_ERR_CUDA;               \
        }                                                                                                    \
    } while (0)

struct kpstm_ctx {
    kpstm_params p;
    kpstm_setup s;
    int device;
    int finished_state; /* reserved */
    cudaStream_t cs, xs;         /* compute, copy */
    cudaEvent_t copy_done[2], comp_done[2];
    int slot;
    int K, nwin, ntile;
    int64_t row;                 /* floats per tap-table row */
    /* constant tables */
    float2 *d_colxy;
    int32_t *d_colrow;
    float4 *d_tilebox;
    float2 *d_vrows;
    float *d_t2;
    float2 *d_t2c;
    float *d_tscale;             /* full mode: per-sample read-out factor t dt/8 */
    double *d_c4, *d_c4r;
    float *d_h;
    float *d_invl2;
    /* image */
    float *d_km, *d_kc;
    int32_t *d_cnt;
    /* per-block work buffers (compute stream) */
    int64_t cap;                 /* traces */
    kpstm_geom *d_graw, *d_geom;
    int32_t *d_cls, *d_order, *d_cstart, *d_nlive;
    float *d_table;
    /* staging (two slots) */
    int64_t scap;
    int32_t *d_hdr[2];
    float *d_smp[2];
    uint32_t *d_raw;
    int64_t rawcap;
    /* status */
    int *d_status;
    unsigned long long *d_hits;
    /* finishing scratch */
    float *d_x, *d_y;
    /* least-squares migration state */
    int64_t lsm_ntr, lsm_nlive, lrow;
    kpstm_geom *d_lgraw, *d_lgeom;
    int32_t *d_lcls, *d_lorder, *d_lcstart, *d_lnlive, *d_lcnt;
    float *d_ltable, *d_lkm;
    unsigned long long *d_lhits;
    double *d_dotpart, *d_dot;
    /* stream handling / profiling */
    cudaStream_t own_cs;
    int prof;
    int nev, capev;
    cudaEvent_t *ev;             /* pairs: start, stop */
    int *evstage;                /* 0 image, 1 prep, 2 finish */
    int *evlaunches;
};

/* Stage bracketing for kpstm_profile_*; no-ops when profiling is off. */
static int prof_begin(kpstm_ctx *c)
{
    if (!c->prof) return -1;
    if (c->nev + 2 > c->capev) {
        int cap = c->capev ? 2 * c->capev : 256;
        cudaEvent_t *ev = (cudaEvent_t *)realloc(c->ev, sizeof(cudaEvent_t) * cap);
        if (!ev) return -1;
        c->ev = ev;
        int *st = (int *)realloc(c->evstage, sizeof(int) * cap);
        if (!st) return -1;
        c->evstage = st;
        int *nl = (int *)realloc(c->evlaunches, sizeof(int) * cap);
        if (!nl) return -1;
        c->evlaunches = nl;
        c->capev = cap;
    }
    int i = c->nev;
    if (cudaEventCreate(&c->ev[i]) != cudaSuccess) return -1;
    if (cudaEventCreate(&c->ev[i + 1]) != cudaSuccess) {
        cudaEventDestroy(c->ev[i]);
        return -1;
    }
    cudaEventRecord(c->ev[i], c->cs);
    c->nev += 2;
    return i;
}

static void prof_end(kpstm_ctx *c, int i, int stage, int launches)
{
    if (i < 0) return;
    cudaEventRecord(c->ev[i + 1], c->cs);
    c->evstage[i] = stage;
    c->evlaunches[i] = launches;
}

static int kp_free_all(kpstm_ctx *c);

static size_t image_smem(const kpstm_ctx *c)
{
    const int W = 32 * c->K;
    const int TB = c->p.mode == KPSTM_MODE_FULL ? KP_TB_FULL : KP_TB_REF;
    size_t b = sizeof(float2) * KPSTM_COLS_PER_CTA * W + sizeof(float2) * W + sizeof(float) * 2 * TB * c->row +
               sizeof(int32_t) * (KP_LCH + 8 + 2);
    b = (b + 7) & ~size_t(7);
    return b + 2 * sizeof(uint64_t);
}

template <int K>
static cudaError_t launch_image_k(const kpstm_ctx *c, const KpImageArgs &a, dim3 grid, size_t smem)
{
    const bool full = c->p.mode == KPSTM_MODE_FULL;
    const bool kahan = c->p.precision == KPSTM_PREC_BF16_KAHAN;
    void (*fn)(KpImageArgs);
    if (full)
        fn = kahan ? k_image<K, true, true> : k_image<K, true, false>;
    else
        fn = kahan ? k_image<K, false, true> : k_image<K, false, false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, KP_THREADS, smem, c->cs>>>(a);
    return cudaGetLastError();
}

static cudaError_t launch_image(const kpstm_ctx *c, const KpImageArgs &a)
{
    dim3 grid(c->ntile, c->s.nclass, c->nwin);
    size_t smem = image_smem(c);
    switch (c->K) {
    case 8: return launch_image_k<8>(c, a, grid, smem);
    case 16: return launch_image_k<16>(c, a, grid, smem);
    case 24: return launch_image_k<24>(c, a, grid, smem);
    default: return launch_image_k<32>(c, a, grid, smem);
    }
}

static int grow_work(kpstm_ctx *c, int64_t ntr)
{
    if (ntr <= c->cap) return KPSTM_OK;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    cudaFree(c->d_graw);
    cudaFree(c->d_geom);
    cudaFree(c->d_cls);
    cudaFree(c->d_order);
    cudaFree(c->d_table);
    c->d_graw = c->d_geom = nullptr;
    c->d_cls = c->d_order = nullptr;
    c->d_table = nullptr;
    c->cap = 0;
    int64_t n = ntr + ntr / 8 + 64;
    KP_CUDA(cudaMalloc(&c->d_graw, sizeof(kpstm_geom) * n));
    KP_CUDA(cudaMalloc(&c->d_geom, sizeof(kpstm_geom) * n));
    KP_CUDA(cudaMalloc(&c->d_cls, sizeof(int32_t) * n));
    KP_CUDA(cudaMalloc(&c->d_order, sizeof(int32_t) * n));
    KP_CUDA(cudaMalloc(&c->d_table, sizeof(float) * c->row * n));
    c->cap = n;
    return KPSTM_OK;
}

static int grow_stage(kpstm_ctx *c, int64_t ntr)
{
    if (ntr <= c->scap) return KPSTM_OK;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    KP_CUDA(cudaStreamSynchronize(c->xs));
    for (int s = 0; s < 2; ++s) {
        cudaFree(c->d_hdr[s]);
        cudaFree(c->d_smp[s]);
        c->d_hdr[s] = nullptr;
        c->d_smp[s] = nullptr;
    }
    c->scap = 0;
    int64_t n = ntr + ntr / 8 + 64;
    for (int s = 0; s < 2; ++s) {
        KP_CUDA(cudaMalloc(&c->d_hdr[s], sizeof(int32_t) * 60 * n));
        KP_CUDA(cudaMalloc(&c->d_smp[s], sizeof(float) * c->p.ns * n));
    }
    c->scap = n;
    return KPSTM_OK;
}

/* The per-block device pipeline on the compute stream. */
static int run_block(kpstm_ctx *c, const int32_t *d_hdr, const float *d_smp, int64_t ntr)
{
    if (ntr == 0) return KPSTM_OK;
    int st = grow_work(c, ntr);
    if (st) return st;
    const kpstm_params *p = &c->p;
    const kpstm_setup *s = &c->s;

    KpGeomArgs g;
    g.hdr_be = d_hdr;
    g.ntr = ntr;
    g.geom = c->d_graw;
    g.cls = c->d_cls;
    g.status = c->d_status;
    g.ox = p->ox;
    g.oy = p->oy;
    g.xy_scale = p->xy_scale;
    g.oh = p->oh;
    g.dh = p->dh;
    g.cull_radius = s->cull_radius;
    g.sinA = s->sinA;
    g.cosA = s->cosA;
    g.IXc = s->IXc;
    g.IYc = s->IYc;
    g.nh = p->nh;
    g.stack = p->output == KPSTM_OUT_STACK;
    int pe = prof_begin(c);
    k_geometry<<<(unsigned)((ntr + 255) / 256), 256, 0, c->cs>>>(g);
    KP_CUDA(cudaGetLastError());

    k_bucket<<<1, 1024, sizeof(int32_t) * (s->nclass + 1), c->cs>>>(c->d_cls, ntr, s->nclass, c->d_cstart,
                                                                     c->d_order, c->d_nlive);
    KP_CUDA(cudaGetLastError());

    KpPrepArgs pa;
    memset(&pa, 0, sizeof(pa));
    pa.samples = d_smp;
    pa.geom_raw = c->d_graw;
    pa.order = c->d_order;
    pa.nlive = c->d_nlive;
    pa.geom = c->d_geom;
    pa.table = c->d_table;
    pa.c4 = c->d_c4;
    pa.c4r = c->d_c4r;
    pa.row = c->row;
    pa.ns = p->ns;
    pa.tm = s->dims.trange_max;
    pa.full = p->mode == KPSTM_MODE_FULL;
    pa.dt = p->dt;
    k_prep<<<(unsigned)((ntr + 127) / 128), 128, 0, c->cs>>>(pa);
    KP_CUDA(cudaGetLastError());
    prof_end(c, pe, 1, 3);

    KpImageArgs a;
    memset(&a, 0, sizeof(a));
    a.geom = c->d_geom;
    a.class_start = c->d_cstart;
    a.table = c->d_table;
    a.row = c->row;
    a.colxy = c->d_colxy;
    a.colrow = c->d_colrow;
    a.tilebox = c->d_tilebox;
    a.vrows = c->d_vrows;
    a.t2 = c->d_t2;
    a.t2c = c->d_t2c;
    a.inv_l2 = c->d_invl2;
    a.km = c->d_km;
    a.kc = c->d_kc;
    a.cnt = c->d_cnt;
    a.hits = c->d_hits;
    a.status = c->d_status;
    a.ncol = s->ncol;
    a.ns = p->ns;
    a.tm = s->dims.trange_max;
    a.lmax = s->lmax;
    a.lmaxf = (float)s->lmax;
    a.dt = p->dt;
    a.rdt = 1.0f / p->dt;
    a.nsf = (float)p->ns;
    a.aperture = p->aperture;
    float r = (float)(p->aperture * (1.0 + 1e-5) + 1e-3);
    a.tile_r2 = r * r;
    a.aax = (float)p->iline_distance; /* slopes in samples per trace spacing (sample units) */
    a.aay = (float)p->xline_distance;
    int pi = prof_begin(c);
    KP_CUDA(launch_image(c, a));
    prof_end(c, pi, 0, 1);
    return KPSTM_OK;
}

/* ------------------------------------------------------------------------ */

extern "C" int kpstm_create(const kpstm_params *params, const kpstm_velocity *vel, kpstm_ctx **out)
{
    if (!params || !vel || !out) return KPSTM_ERR_INVALID_ARG;
    *out = nullptr;
    kpstm_setup s;
    int st = kpstm_setup_of(params, &s);
    if (st) return st;
    st = kpstm_velocity_check(params, vel, &s);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return KPSTM_ERR_NO_DEVICE;

    kpstm_ctx *c = (kpstm_ctx *)calloc(1, sizeof(kpstm_ctx));
    if (!c) return KPSTM_ERR_OUT_OF_MEMORY;
    c->p = *params;
    c->s = s;
    cudaGetDevice(&c->device);
    const int ns = params->ns, tm = s.dims.trange_max;
    const int ncol = s.ncol;
    /* samples per lane: as many as fit the 128-register budget of 2 CTAs/SM
       without spilling (reference 32, full 24, Kahan variants 8 fewer) */
    const bool fullm = params->mode == KPSTM_MODE_FULL, kah = params->precision == KPSTM_PREC_BF16_KAHAN;
    const int kmax = (fullm ? 24 : 32) - (kah ? 8 : 0);
    c->nwin = (ns + 32 * kmax - 1) / (32 * kmax);
    int per = (ns + c->nwin - 1) / c->nwin;
    c->K = per <= 256 ? 8 : per <= 512 ? 16 : per <= 768 ? 24 : 32;
    c->ntile = (ncol + KPSTM_COLS_PER_CTA - 1) / KPSTM_COLS_PER_CTA;
    if (params->mode == KPSTM_MODE_FULL)
        c->row = ((2 * (int64_t)(ns + 2 * tm - 3)) + 3) & ~int64_t(3);
    else
        c->row = (ns + 1 + 3) & ~3; /* D[0..ns-1] plus a zero sentinel D[ns] */

    /* host tables */
    float *colxy = (float *)malloc(sizeof(float) * 2 * ncol);
    int32_t *colrow = (int32_t *)malloc(sizeof(int32_t) * ncol);
    float *t2 = (float *)malloc(sizeof(float) * ns);
    int32_t *t1 = (int32_t *)malloc(sizeof(int32_t) * ns);
    double *c4 = (double *)malloc(sizeof(double) * ns);
    double *c4r = (double *)malloc(sizeof(double) * ns);
    float2 *t2c = (float2 *)malloc(sizeof(float2) * ns);
    float *tsc = (float *)malloc(sizeof(float) * ns);
    double *hd = (double *)malloc(sizeof(double) * ns);
    float *hf = (float *)malloc(sizeof(float) * ns);
    float4 *box = (float4 *)malloc(sizeof(float4) * c->ntile);
    int32_t *rowmap = nullptr;
    float2 *vrows = nullptr;
    float invl2[64];
    int nrow = 0;
    do {
        if (!colxy || !colrow || !t2 || !t1 || !c4 || !c4r || !t2c || !tsc || !hd || !hf || !box) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        kpstm_columns(params, vel, &s, colxy, colrow);
        kpstm_time_tables(params, vel, t2, t1);
        for (int t = 0; t < ns; ++t) {
            c4[t] = 4.0 * (double)t2[t];
            c4r[t] = t > 0 ? 1.0 / c4[t] : 0.0;
            double t0 = (double)t * (double)params->dt;
            (void)t0;
            /* full mode works in sample units: (t/2)^2 and t0/(8 dt^2) = t/(8 dt);
               t = 0 gets a tiny positive time so that rsqrt never sees 0 */
            t2c[t] = make_float2(t > 0 ? (float)(0.25 * (double)t * (double)t) : 1e-12f,
                                 (float)((double)t / (8.0 * (double)params->dt)));
            tsc[t] = (float)((double)t / (8.0 * (double)params->dt)); /* t0/(8 dt^2), sample units */
        }
        st = kpstm_lowpass_kernel(params, hd);
        if (st) break;
        for (int t = 0; t < ns; ++t) hf[t] = (float)hd[t];
        for (int b = 0; b < c->ntile; ++b) {
            float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
            for (int k = 0; k < KPSTM_COLS_PER_CTA; ++k) {
                int cc = b * KPSTM_COLS_PER_CTA + k;
                if (cc >= ncol) break;
                x0 = fminf(x0, colxy[2 * cc]);
                x1 = fmaxf(x1, colxy[2 * cc]);
                y0 = fminf(y0, colxy[2 * cc + 1]);
                y1 = fmaxf(y1, colxy[2 * cc + 1]);
            }
            box[b] = make_float4(x0, x1, y0, y1);
        }
        /* compact the velocity rows the slab uses; v^2 in float as
           Kirchhoff.c:617, RN(1/v^2) for the exact division */
        int64_t ngrid = (int64_t)vel->n_iline * vel->n_xline;
        rowmap = (int32_t *)malloc(sizeof(int32_t) * ngrid);
        if (!rowmap) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        for (int64_t i = 0; i < ngrid; ++i) rowmap[i] = -1;
        for (int cc = 0; cc < ncol; ++cc) {
            int r = colrow[cc];
            if (r < 0) continue;
            if (rowmap[r] < 0) rowmap[r] = nrow++;
            colrow[cc] = rowmap[r];
        }
        vrows = (float2 *)malloc(sizeof(float2) * (size_t)(nrow > 0 ? nrow : 1) * ns);
        if (!vrows) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        for (int64_t i = 0; i < ngrid; ++i) {
            int r = rowmap[i];
            if (r < 0) continue;
            const float *v = vel->vrms + i * vel->nsm;
            for (int t = 0; t < ns; ++t) {
                float vv = v[t1[t]] * v[t1[t]];
                vrows[(size_t)r * ns + t] = make_float2(vv, 1.0f / vv);
            }
        }
        for (int L = 0; L < 64; ++L) invl2[L] = L > 0 ? 1.0f / (float)(L * L) : 0.0f;
    } while (0);

    if (!st) {
        do {
            cudaError_t e = cudaStreamCreateWithFlags(&c->cs, cudaStreamNonBlocking);
            c->own_cs = c->cs;
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->xs, cudaStreamNonBlocking);
            for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
                e = cudaEventCreateWithFlags(&c->copy_done[k], cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->comp_done[k], cudaEventDisableTiming);
            }
            if (e != cudaSuccess) {
                st = KPSTM_ERR_CUDA;
                break;
            }
            size_t nimg = (size_t)s.nclass * ncol * ns;
#define KP_ALLOC(ptr, bytes)                                                                                 \
    if (cudaMalloc(&(ptr), (bytes)) != cudaSuccess) {                                                        \
        st = KPSTM_ERR_OUT_OF_MEMORY;                                                                        \
        break;                                                                                               \
    }
            KP_ALLOC(c->d_colxy, sizeof(float2) * ncol);
            KP_ALLOC(c->d_colrow, sizeof(int32_t) * ncol);
            KP_ALLOC(c->d_tilebox, sizeof(float4) * c->ntile);
            KP_ALLOC(c->d_vrows, sizeof(float2) * (size_t)(nrow > 0 ? nrow : 1) * ns);
            KP_ALLOC(c->d_t2, sizeof(float) * ns);
            KP_ALLOC(c->d_t2c, sizeof(float2) * ns);
            if (params->mode == KPSTM_MODE_FULL) KP_ALLOC(c->d_tscale, sizeof(float) * ns);
            KP_ALLOC(c->d_c4, sizeof(double) * ns);
            KP_ALLOC(c->d_c4r, sizeof(double) * ns);
            KP_ALLOC(c->d_h, sizeof(float) * ns);
            KP_ALLOC(c->d_invl2, sizeof(float) * 64);
            KP_ALLOC(c->d_km, sizeof(float) * nimg);
            KP_ALLOC(c->d_cnt, sizeof(int32_t) * nimg);
            if (params->precision == KPSTM_PREC_BF16_KAHAN) KP_ALLOC(c->d_kc, sizeof(float) * nimg);
            KP_ALLOC(c->d_cstart, sizeof(int32_t) * (s.nclass + 1));
            KP_ALLOC(c->d_nlive, sizeof(int32_t));
            KP_ALLOC(c->d_status, sizeof(int));
            KP_ALLOC(c->d_hits, sizeof(unsigned long long));
#undef KP_ALLOC
            cudaMemcpyAsync(c->d_colxy, colxy, sizeof(float2) * ncol, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_colrow, colrow, sizeof(int32_t) * ncol, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_tilebox, box, sizeof(float4) * c->ntile, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_vrows, vrows, sizeof(float2) * (size_t)(nrow > 0 ? nrow : 1) * ns,
                            cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_t2, t2, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_t2c, t2c, sizeof(float2) * ns, cudaMemcpyHostToDevice, c->cs);
            if (c->d_tscale) cudaMemcpyAsync(c->d_tscale, tsc, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_c4, c4, sizeof(double) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_c4r, c4r, sizeof(double) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_h, hf, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_invl2, invl2, sizeof(float) * 64, cudaMemcpyHostToDevice, c->cs);
            cudaMemsetAsync(c->d_km, 0, sizeof(float) * nimg, c->cs);
            cudaMemsetAsync(c->d_cnt, 0, sizeof(int32_t) * nimg, c->cs);
            if (c->d_kc) cudaMemsetAsync(c->d_kc, 0, sizeof(float) * nimg, c->cs);
            cudaMemsetAsync(c->d_status, 0, sizeof(int), c->cs);
            cudaMemsetAsync(c->d_hits, 0, sizeof(unsigned long long), c->cs);
            if (cudaStreamSynchronize(c->cs) != cudaSuccess) st = KPSTM_ERR_CUDA;
        } while (0);
    }
    free(colxy);
    free(colrow);
    free(t2);
    free(t1);
    free(c4);
    free(c4r);
    free(t2c);
    free(tsc);
    free(hd);
    free(hf);
    free(box);
    free(rowmap);
    free(vrows);
    if (st) {
        kp_free_all(c);
        return st;
    }
    *out = c;
    return KPSTM_OK;
}

static int kp_free_all(kpstm_ctx *c)
{
    if (!c) return KPSTM_OK;
    if (c->cs) cudaStreamSynchronize(c->cs);
    if (c->own_cs && c->own_cs != c->cs) cudaStreamSynchronize(c->own_cs);
    if (c->xs) cudaStreamSynchronize(c->xs);
    void *ptrs[] = {c->d_colxy, c->d_colrow, c->d_tilebox, c->d_vrows, c->d_t2, c->d_t2c, c->d_tscale, c->d_c4, c->d_c4r,
                    c->d_h, c->d_invl2, c->d_km, c->d_kc, c->d_cnt, c->d_graw, c->d_geom, c->d_cls,
                    c->d_order, c->d_cstart, c->d_nlive, c->d_table, c->d_hdr[0], c->d_hdr[1], c->d_smp[0],
                    c->d_smp[1], c->d_raw, c->d_status, c->d_hits, c->d_x, c->d_y, c->d_lgraw, c->d_lgeom,
                    c->d_lcls, c->d_lorder, c->d_lcstart, c->d_lnlive, c->d_lcnt, c->d_ltable, c->d_lkm,
                    c->d_lhits, c->d_dotpart, c->d_dot};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i)
        if (ptrs[i]) cudaFree(ptrs[i]);
    for (int k = 0; k < 2; ++k) {
        if (c->copy_done[k]) cudaEventDestroy(c->copy_done[k]);
        if (c->comp_done[k]) cudaEventDestroy(c->comp_done[k]);
    }
    for (int i = 0; i < c->nev; ++i) cudaEventDestroy(c->ev[i]);
    free(c->ev);
    free(c->evstage);
    free(c->evlaunches);
    if (c->own_cs) cudaStreamDestroy(c->own_cs);
    if (c->xs) cudaStreamDestroy(c->xs);
    free(c);
    return KPSTM_OK;
}

extern "C" void kpstm_destroy(kpstm_ctx *c) { kp_free_all(c); }

extern "C" int kpstm_get_dims(const kpstm_ctx *c, kpstm_dims *d)
{
    if (!c || !d) return KPSTM_ERR_INVALID_ARG;
    *d = c->s.dims;
    return KPSTM_OK;
}

static int check_status(kpstm_ctx *c)
{
    int h = 0;
    KP_CUDA(cudaMemcpyAsync(&h, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->cs));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    return h;
}

extern "C" int kpstm_synchronize(kpstm_ctx *c)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->xs));
    return check_status(c);
}

extern "C" int kpstm_reset(kpstm_ctx *c)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    size_t nimg = (size_t)c->s.nclass * c->s.ncol * c->p.ns;
    KP_CUDA(cudaStreamSynchronize(c->xs));
    KP_CUDA(cudaMemsetAsync(c->d_km, 0, sizeof(float) * nimg, c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_cnt, 0, sizeof(int32_t) * nimg, c->cs));
    if (c->d_kc) KP_CUDA(cudaMemsetAsync(c->d_kc, 0, sizeof(float) * nimg, c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_hits, 0, sizeof(unsigned long long), c->cs));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    return KPSTM_OK;
}

extern "C" int kpstm_add_traces(kpstm_ctx *c, const int32_t *hdr_be, const float *samples, int64_t ntr)
{
    if (!c || ntr < 0 || (ntr > 0 && (!hdr_be || !samples))) return KPSTM_ERR_INVALID_ARG;
    if (ntr == 0) return KPSTM_OK;
    if (ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    int st = grow_stage(c, ntr);
    if (st) return st;
    const int s = c->slot;
    /* the copy into slot s may start once the block that last used it is imaged */
    KP_CUDA(cudaStreamWaitEvent(c->xs, c->comp_done[s], 0));
    KP_CUDA(cudaMemcpyAsync(c->d_hdr[s], hdr_be, sizeof(int32_t) * 60 * ntr, cudaMemcpyHostToDevice, c->xs));
    KP_CUDA(cudaMemcpyAsync(c->d_smp[s], samples, sizeof(float) * c->p.ns * ntr, cudaMemcpyHostToDevice, c->xs));
    KP_CUDA(cudaEventRecord(c->copy_done[s], c->xs));
    KP_CUDA(cudaStreamWaitEvent(c->cs, c->copy_done[s], 0));
    st = run_block(c, c->d_hdr[s], c->d_smp[s], ntr);
    if (st) return st;
    KP_CUDA(cudaEventRecord(c->comp_done[s], c->cs));
    c->slot ^= 1;
    /* the caller may reuse its buffers once they have been read */
    KP_CUDA(cudaEventSynchronize(c->copy_done[s]));
    return KPSTM_OK;
}

extern "C" int kpstm_add_traces_device(kpstm_ctx *c, const int32_t *d_hdr_be, const float *d_samples, int64_t ntr)
{
    if (!c || ntr < 0 || (ntr > 0 && (!d_hdr_be || !d_samples))) return KPSTM_ERR_INVALID_ARG;
    if (ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    return run_block(c, d_hdr_be, d_samples, ntr);
}

extern "C" int kpstm_add_segy_block(kpstm_ctx *c, const void *rec, int64_t ntr)
{
    if (!c || ntr < 0 || (ntr > 0 && !rec)) return KPSTM_ERR_INVALID_ARG;
    if (ntr == 0) return KPSTM_OK;
    if (ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    int st = grow_stage(c, ntr);
    if (st) return st;
    const int64_t words = (60 + (int64_t)c->p.ns) * ntr;
    if (words > c->rawcap) {
        KP_CUDA(cudaStreamSynchronize(c->cs));
        KP_CUDA(cudaStreamSynchronize(c->xs));
        cudaFree(c->d_raw);
        c->d_raw = nullptr;
        c->rawcap = 0;
        KP_CUDA(cudaMalloc(&c->d_raw, sizeof(uint32_t) * words));
        c->rawcap = words;
    }
    const int s = c->slot;
    KP_CUDA(cudaStreamWaitEvent(c->xs, c->comp_done[s], 0));
    KP_CUDA(cudaStreamWaitEvent(c->xs, c->comp_done[s ^ 1], 0)); /* single raw buffer */
    KP_CUDA(cudaMemcpyAsync(c->d_raw, rec, sizeof(uint32_t) * words, cudaMemcpyHostToDevice, c->xs));
    KP_CUDA(cudaEventRecord(c->copy_done[s], c->xs));
    KP_CUDA(cudaStreamWaitEvent(c->cs, c->copy_done[s], 0));
    k_segy_decode<<<1024, 256, 0, c->cs>>>(c->d_raw, ntr, c->p.ns, c->d_hdr[s], c->d_smp[s]);
    KP_CUDA(cudaGetLastError());
    st = run_block(c, c->d_hdr[s], c->d_smp[s], ntr);
    if (st) return st;
    KP_CUDA(cudaEventRecord(c->comp_done[s], c->cs));
    c->slot ^= 1;
    KP_CUDA(cudaEventSynchronize(c->copy_done[s]));
    return KPSTM_OK;
}

static int ensure_finish_scratch(kpstm_ctx *c)
{
    if (c->d_x) return KPSTM_OK;
    size_t nimg = (size_t)c->s.nclass * c->s.ncol * c->p.ns;
    KP_CUDA(cudaMalloc(&c->d_x, sizeof(float) * nimg));
    KP_CUDA(cudaMalloc(&c->d_y, sizeof(float) * nimg));
    return KPSTM_OK;
}

/* Finishing into device buffers out/fold ([col][cls][ns] order); either may be null. */
static int finish_dev(kpstm_ctx *c, float *out, float *fold)
{
    const int ns = c->p.ns, ncol = c->s.ncol, ncls = c->s.nclass;
    const int64_t nrows = (int64_t)ncol * ncls;
    if (out) {
        int st = ensure_finish_scratch(c);
        if (st) return st;
        int pf = prof_begin(c);
        k_deriv<<<1024, 256, 0, c->cs>>>(c->d_km, c->d_cnt, c->d_tscale, ncol, ncls, ns, c->p.dt, c->d_x);
        KP_CUDA(cudaGetLastError());
        size_t smem = sizeof(float) * (((2 * (size_t)ns + 3) & ~size_t(3)) + (size_t)ns * KP_LP_ROWS);
        if (smem > 220 * 1024) return KPSTM_ERR_UNSUPPORTED;
        KP_CUDA(cudaFuncSetAttribute(k_lowpass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_lowpass<<<(unsigned)((nrows + KP_LP_ROWS - 1) / KP_LP_ROWS), 256, smem, c->cs>>>(c->d_x, c->d_h, nrows,
                                                                                          ns, out);
        KP_CUDA(cudaGetLastError());
        prof_end(c, pf, 2, 2);
    }
    if (fold) {
        k_relayout<<<1024, 256, 0, c->cs>>>(nullptr, c->d_cnt, nullptr, ncol, ncls, ns, fold);
        KP_CUDA(cudaGetLastError());
    }
    return KPSTM_OK;
}

extern "C" int kpstm_finish_device(kpstm_ctx *c, float *d_out, float *d_fold)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->xs));
    int st = finish_dev(c, d_out, d_fold);
    if (st) return st;
    return check_status(c);
}

extern "C" int kpstm_finish(kpstm_ctx *c, float *out, float *fold)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->xs));
    int st = ensure_finish_scratch(c);
    if (st) return st;
    const size_t bytes = sizeof(float) * (size_t)c->s.dims.out_elems;
    if (out) {
        st = finish_dev(c, c->d_y, nullptr);
        if (st) return st;
        KP_CUDA(cudaMemcpyAsync(out, c->d_y, bytes, cudaMemcpyDeviceToHost, c->cs));
    }
    if (fold) {
        /* d_x is free again once the low-pass has read it (stream order) */
        st = finish_dev(c, nullptr, c->d_x);
        if (st) return st;
        KP_CUDA(cudaMemcpyAsync(fold, c->d_x, bytes, cudaMemcpyDeviceToHost, c->cs));
    }
    return check_status(c);
}

extern "C" int kpstm_get_accumulators(kpstm_ctx *c, float *km, float *fold)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->xs));
    int st = ensure_finish_scratch(c);
    if (st) return st;
    const int ns = c->p.ns, ncol = c->s.ncol, ncls = c->s.nclass;
    const size_t bytes = sizeof(float) * (size_t)c->s.dims.out_elems;
    if (km) {
        k_relayout<<<1024, 256, 0, c->cs>>>(c->d_km, nullptr, c->d_tscale, ncol, ncls, ns, c->d_x);
        KP_CUDA(cudaGetLastError());
        KP_CUDA(cudaMemcpyAsync(km, c->d_x, bytes, cudaMemcpyDeviceToHost, c->cs));
    }
    if (fold) {
        k_relayout<<<1024, 256, 0, c->cs>>>(nullptr, c->d_cnt, nullptr, ncol, ncls, ns, c->d_y);
        KP_CUDA(cudaGetLastError());
        KP_CUDA(cudaMemcpyAsync(fold, c->d_y, bytes, cudaMemcpyDeviceToHost, c->cs));
    }
    return check_status(c);
}

extern "C" int kpstm_pair_count(const kpstm_ctx *c, int64_t *pairs)
{
    if (!c || !pairs) return KPSTM_ERR_INVALID_ARG;
    unsigned long long h = 0;
    KP_CUDA(cudaMemcpyAsync(&h, c->d_hits, sizeof(h), cudaMemcpyDeviceToHost, c->cs));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    *pairs = (int64_t)h * c->p.ns;
    return KPSTM_OK;
}

extern "C" int kpstm_write_su(const kpstm_ctx *c, const float *image, void *dst, int64_t dst_bytes)
{
    if (!c || !image || !dst) return KPSTM_ERR_INVALID_ARG;
    const int ns = c->p.ns, ncls = c->s.nclass, ncol = c->s.ncol;
    const int64_t rec = 240 + 4 * (int64_t)ns;
    const int64_t ntrace = (int64_t)ncol * ncls;
    if (dst_bytes < ntrace * rec) return KPSTM_ERR_INVALID_ARG;
    uint8_t *o = (uint8_t *)dst;
    int64_t tracl = (int64_t)ncol * ncls * c->p.job_id + 1;
    for (int col = 0; col < ncol; ++col) {
        for (int cls = 0; cls < ncls; ++cls) {
            uint8_t *r = o + ((int64_t)col * ncls + cls) * rec;
            kpstm_su_headers(&c->p, &c->s, col, cls, tracl++, r);
            const float *d = image + ((int64_t)col * ncls + cls) * ns;
            for (int t = 0; t < ns; ++t) {
                uint32_t u;
                memcpy(&u, &d[t], 4);
                r[240 + 4 * t + 0] = (uint8_t)(u >> 24);
                r[240 + 4 * t + 1] = (uint8_t)(u >> 16);
                r[240 + 4 * t + 2] = (uint8_t)(u >> 8);
                r[240 + 4 * t + 3] = (uint8_t)u;
            }
        }
    }
    return KPSTM_OK;
}

extern "C" int kpstm_set_stream(kpstm_ctx *c, void *stream)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    cudaStream_t next = stream ? (cudaStream_t)stream : c->own_cs;
    if (next == c->cs) return KPSTM_OK;
    /* order the new stream after everything queued so far */
    cudaEvent_t e;
    KP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    KP_CUDA(cudaEventRecord(e, c->cs));
    KP_CUDA(cudaStreamWaitEvent(next, e, 0));
    cudaEventDestroy(e);
    c->cs = next;
    return KPSTM_OK;
}

extern "C" int kpstm_profile_enable(kpstm_ctx *c, int enable)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    c->prof = enable ? 1 : 0;
    return KPSTM_OK;
}

extern "C" int kpstm_profile_read(kpstm_ctx *c, kpstm_profile *out)
{
    if (!c || !out) return KPSTM_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    for (int i = 0; i + 1 < c->nev; i += 2) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, c->ev[i], c->ev[i + 1]) != cudaSuccess) ms = 0.0f;
        if (c->evstage[i] == 0) {
            out->image_ms += ms;
            out->image_launches += c->evlaunches[i];
        } else {
            if (c->evstage[i] == 1) out->prep_ms += ms;
            else out->finish_ms += ms;
            out->other_launches += c->evlaunches[i];
        }
        cudaEventDestroy(c->ev[i]);
        cudaEventDestroy(c->ev[i + 1]);
    }
    c->nev = 0;
    return KPSTM_OK;
}

/* ------------------------------------------------------------------------ */
/* Finishing without device allocation (kpstm_finish_noalloc).
   The scratch a finishing pass needs - the derivative traces between
   k_deriv and k_lowpass, and the low-pass impulse response - is this one
   file-scope array instead of context buffers.  Nothing in it has to start
   at zero: every call rewrites the parts it reads. */
#define KP_NOALLOC_MAX_NS 32768
static __device__ __align__(256) float g_noalloc_scratch[KPSTM_NOALLOC_MAX_SAMPLES + KP_NOALLOC_MAX_NS];

/* Device address of g_noalloc_scratch per device, looked up once per device
   with that device current (the array's name is only a host-side handle in
   host code). */
#define KP_NOALLOC_MAX_DEVICES 64
static float *g_noalloc_ptr[KP_NOALLOC_MAX_DEVICES];
static pthread_mutex_t g_noalloc_mu = PTHREAD_MUTEX_INITIALIZER;

static int noalloc_scratch(float **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return KPSTM_ERR_NO_DEVICE;
    if (dev < 0 || dev >= KP_NOALLOC_MAX_DEVICES) return KPSTM_ERR_UNSUPPORTED;
    pthread_mutex_lock(&g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            pthread_mutex_unlock(&g_noalloc_mu);
            return KPSTM_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (float *)p;
    }
    *out = g_noalloc_ptr[dev];
    pthread_mutex_unlock(&g_noalloc_mu);
    return KPSTM_OK;
}

/* Low-pass impulse response h[m] = (1/ns) sum_k A[k] cos(2 pi k m / ns), with
   the anti-alias spectrum A of Kirchhoff.c:380-441 evaluated per bin in the
   same float/double steps as kpstm_aliasfilter (fs, den from the host). */
__global__ void k_noalloc_impulse(int ns, float fs, float den, float *h)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ns) return;
    const int half = ns / 2;
    double acc = 0.0;
    for (int k = 0; k < ns; ++k) {
        int j = k;
        bool zero = (ns & 1) && (k == half || k == half + 1);
        if (k > half) j = ns - k;
        float a = 0.0f;
        if (!zero) {
            float x = __fmul_rn(__int2float_rn(j), fs);
            float num = __fmul_rn(__fmul_rn(__fmul_rn(x, x), x), x);
            a = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, (double)__fdiv_rn(num, den)))));
        }
        long long km = ((long long)k * m) % ns;
        acc += (double)a * cos(6.283185307179586476925286766559 * (double)km / (double)ns);
    }
    h[m] = (float)(acc / ns);
}

/* k_deriv for accumulators in the caller's layout [col][cls][ns] with the
   fold given as floats: x[t] = -dt*t*(km[t]-km[t-1])*dt/fold[t], x[0] = 0. */
__global__ void k_deriv_caller(const float *km, const float *fold, int64_t n, int ns, float dt, float *x)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int t = (int)(i % ns);
        float v = 0.0f;
        if (t > 0)
            v = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(-dt, __int2float_rn(t)), __fsub_rn(km[i], km[i - 1])), dt),
                          fold[i]);
        x[i] = v;
    }
}

extern "C" int kpstm_finish_noalloc(const kpstm_params *params, const float *d_km, const float *d_fold,
                                    float *d_out, void *cuda_stream)
{
    if (!params || !d_km || !d_fold || !d_out) return KPSTM_ERR_INVALID_ARG;
    kpstm_setup s;
    int st = kpstm_setup_of(params, &s);
    if (st) return st;
    const int ns = params->ns;
    const int64_t n = s.dims.out_elems;
    if (n > KPSTM_NOALLOC_MAX_SAMPLES || ns > KP_NOALLOC_MAX_NS) return KPSTM_ERR_TOO_LARGE;
    const size_t smem = sizeof(float) * (((2 * (size_t)ns + 3) & ~size_t(3)) + (size_t)ns * KP_LP_ROWS);
    if (smem > 220 * 1024) return KPSTM_ERR_TOO_LARGE;
    float *scratch = nullptr;
    st = noalloc_scratch(&scratch);
    if (st) return st;
    float *x = scratch, *h = scratch + KPSTM_NOALLOC_MAX_SAMPLES;
    /* scalars of create_aliasfilter (Kirchhoff.c:403-412), as kpstm_aliasfilter */
    const float fs = (float)(2.0 / ((double)params->dt * (double)ns));
    float fm = (float)params->anti_alias_cutoff;
    fm = (float)((double)fm * 3.0);
    const float den = ((fm * fm) * fm) * fm;
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    k_noalloc_impulse<<<(ns + 127) / 128, 128, 0, stream>>>(ns, fs, den, h);
    KP_CUDA(cudaGetLastError());
    k_deriv_caller<<<1024, 256, 0, stream>>>(d_km, d_fold, n, ns, params->dt, x);
    KP_CUDA(cudaGetLastError());
    KP_CUDA(cudaFuncSetAttribute(k_lowpass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t nrows = n / ns;
    k_lowpass<<<(unsigned)((nrows + KP_LP_ROWS - 1) / KP_LP_ROWS), 256, smem, stream>>>(x, h, nrows, ns, d_out);
    KP_CUDA(cudaGetLastError());
    return KPSTM_OK;
}

/* ------------------------------------------------------------------------ */
/* Least-squares migration (kpstm_lsm_*). */

static KpImageArgs image_args(const kpstm_ctx *c)
{
    const kpstm_params *p = &c->p;
    const kpstm_setup *s = &c->s;
    KpImageArgs a;
    memset(&a, 0, sizeof(a));
    a.colxy = c->d_colxy;
    a.colrow = c->d_colrow;
    a.tilebox = c->d_tilebox;
    a.vrows = c->d_vrows;
    a.t2 = c->d_t2;
    a.t2c = c->d_t2c;
    a.inv_l2 = c->d_invl2;
    a.status = c->d_status;
    a.ncol = s->ncol;
    a.ns = p->ns;
    a.tm = s->dims.trange_max;
    a.lmax = s->lmax;
    a.lmaxf = (float)s->lmax;
    a.dt = p->dt;
    a.rdt = 1.0f / p->dt;
    a.nsf = (float)p->ns;
    a.aperture = p->aperture;
    float r = (float)(p->aperture * (1.0 + 1e-5) + 1e-3);
    a.tile_r2 = r * r;
    a.aax = (float)p->iline_distance;
    a.aay = (float)p->xline_distance;
    return a;
}

template <int K>
static cudaError_t launch_image_hilo_k(const kpstm_ctx *c, const KpImageArgs &a, dim3 grid, size_t smem)
{
    void (*fn)(KpImageArgs) = k_image<K, true, false, true>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, KP_THREADS, smem, c->cs>>>(a);
    return cudaGetLastError();
}

static int lsm_adjoint_impl(kpstm_ctx *c, const float *d_data, const uint16_t *d_data16, const float *d_scale,
                            float *d_model)
{
    const int ns = c->p.ns, ncol = c->s.ncol, ncls = c->s.nclass;
    const size_t nimg = (size_t)ncls * ncol * ns;
    KP_CUDA(cudaMemsetAsync(c->d_lkm, 0, sizeof(float) * nimg, c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_lcnt, 0, sizeof(int32_t) * nimg, c->cs));
    if (c->lsm_nlive > 0) {
        KpPrepArgs pa;
        memset(&pa, 0, sizeof(pa));
        pa.samples = d_data;
        pa.samples_bf16 = d_data16;
        pa.scale = d_scale;
        pa.geom_raw = c->d_lgraw;
        pa.order = c->d_lorder;
        pa.nlive = c->d_lnlive;
        pa.geom = c->d_lgeom;
        pa.table = c->d_ltable;
        pa.c4 = c->d_c4;
        pa.c4r = c->d_c4r;
        pa.row = c->lrow;
        pa.ns = ns;
        pa.tm = c->s.dims.trange_max;
        pa.full = 1;
        pa.hilo = 1;
        pa.dt = c->p.dt;
        k_prep<<<(unsigned)((c->lsm_nlive + 127) / 128), 128, 0, c->cs>>>(pa);
        KP_CUDA(cudaGetLastError());
        KpImageArgs a = image_args(c);
        a.geom = c->d_lgeom;
        a.class_start = c->d_lcstart;
        a.table = c->d_ltable;
        a.row = c->lrow;
        a.km = c->d_lkm;
        a.cnt = c->d_lcnt;
        a.hits = c->d_lhits;
        const int W = 32 * c->K;
        size_t smem = sizeof(float2) * KPSTM_COLS_PER_CTA * W + sizeof(float2) * W +
                      sizeof(float) * 2 * KP_TB_FULL * c->lrow + sizeof(int32_t) * (KP_LCH + 8 + 2);
        smem = ((smem + 7) & ~size_t(7)) + 2 * sizeof(uint64_t);
        dim3 grid(c->ntile, ncls, c->nwin);
        cudaError_t e;
        switch (c->K) {
        case 8: e = launch_image_hilo_k<8>(c, a, grid, smem); break;
        case 16: e = launch_image_hilo_k<16>(c, a, grid, smem); break;
        default: e = launch_image_hilo_k<24>(c, a, grid, smem); break;
        }
        KP_CUDA(e);
    }
    k_relayout<<<1024, 256, 0, c->cs>>>(c->d_lkm, nullptr, c->d_tscale, ncol, ncls, ns, d_model);
    KP_CUDA(cudaGetLastError());
    return KPSTM_OK;
}

static int lsm_forward_impl(kpstm_ctx *c, const float *d_model, float *d_data)
{
    const int ns = c->p.ns;
    KP_CUDA(cudaMemsetAsync(d_data, 0, sizeof(float) * (size_t)c->lsm_ntr * ns, c->cs));
    if (c->lsm_nlive == 0) return KPSTM_OK;
    const kpstm_params *p = &c->p;
    const kpstm_setup *s = &c->s;
    KpDemigArgs a;
    memset(&a, 0, sizeof(a));
    a.geom = c->d_lgeom;
    a.nlive = c->d_lnlive;
    a.model = d_model;
    a.tscale = c->d_tscale;
    a.colxy = c->d_colxy;
    a.colrow = c->d_colrow;
    a.vrows = c->d_vrows;
    a.t2c = c->d_t2c;
    a.out = d_data;
    a.status = c->d_status;
    a.nx = s->dims.nx;
    a.ny = s->dims.ny;
    a.ncls = s->nclass;
    a.ns = ns;
    a.ax0 = (float)((p->start_iline + (s->xslice * s->dims.nx) * p->inc_iline) * p->iline_distance);
    a.adx = (float)(p->inc_iline * p->iline_distance);
    a.ay0 = (float)((p->start_xline + (s->yslice * s->dims.ny) * p->inc_xline) * p->xline_distance);
    a.ady = (float)(p->inc_xline * p->xline_distance);
    if (a.adx == 0.0f) a.adx = 1.0f;
    if (a.ady == 0.0f) a.ady = 1.0f;
    a.aperture = p->aperture;
    a.tmax = (float)ns - 1.0f;
    a.lmaxf = (float)s->lmax;
    const float rdt = 1.0f / p->dt;
    a.rdt2 = rdt * rdt;
    a.aax = (float)p->iline_distance;
    a.aay = (float)p->xline_distance;
    const size_t smem = sizeof(float) * 8 * (size_t)((ns + 3) & ~3);
    if (smem > 200 * 1024) return KPSTM_ERR_UNSUPPORTED;
    KP_CUDA(cudaFuncSetAttribute(k_demig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_demig<<<(unsigned)((c->lsm_nlive + 7) / 8), 256, smem, c->cs>>>(a);
    KP_CUDA(cudaGetLastError());
    return KPSTM_OK;
}

extern "C" int kpstm_lsm_geometry(kpstm_ctx *c, const int32_t *hdr_be, int64_t ntr)
{
    if (!c || !hdr_be || ntr <= 0 || ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    if (c->p.mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    void *old[] = {c->d_lgraw, c->d_lgeom, c->d_lcls, c->d_lorder, c->d_lcstart, c->d_lnlive,
                   c->d_lcnt, c->d_ltable, c->d_lkm, c->d_lhits, c->d_dotpart, c->d_dot};
    for (size_t i = 0; i < sizeof(old) / sizeof(old[0]); ++i)
        if (old[i]) cudaFree(old[i]);
    c->d_lgraw = c->d_lgeom = nullptr;
    c->d_lcls = c->d_lorder = c->d_lcstart = c->d_lnlive = c->d_lcnt = nullptr;
    c->d_ltable = c->d_lkm = nullptr;
    c->d_lhits = nullptr;
    c->d_dotpart = c->d_dot = nullptr;
    c->lsm_ntr = c->lsm_nlive = 0;
    const int ns = c->p.ns, ncls = c->s.nclass, tm = c->s.dims.trange_max;
    const size_t nimg = (size_t)ncls * c->s.ncol * ns;
    int32_t *d_hdr = nullptr;
    KP_CUDA(cudaMalloc(&d_hdr, sizeof(int32_t) * 60 * ntr));
    int st = KPSTM_OK;
    do {
#define KP_LALLOC(ptr, bytes)                                                                                \
    if (cudaMalloc(&(ptr), (bytes)) != cudaSuccess) {                                                        \
        st = KPSTM_ERR_OUT_OF_MEMORY;                                                                        \
        break;                                                                                               \
    }
        KP_LALLOC(c->d_lgraw, sizeof(kpstm_geom) * ntr);
        KP_LALLOC(c->d_lgeom, sizeof(kpstm_geom) * ntr);
        KP_LALLOC(c->d_lcls, sizeof(int32_t) * ntr);
        KP_LALLOC(c->d_lorder, sizeof(int32_t) * ntr);
        KP_LALLOC(c->d_lcstart, sizeof(int32_t) * (ncls + 1));
        KP_LALLOC(c->d_lnlive, sizeof(int32_t));
        KP_LALLOC(c->d_lkm, sizeof(float) * nimg);
        KP_LALLOC(c->d_lcnt, sizeof(int32_t) * nimg);
        KP_LALLOC(c->d_lhits, sizeof(unsigned long long));
        KP_LALLOC(c->d_dotpart, sizeof(double) * KP_DOT_BLOCKS);
        KP_LALLOC(c->d_dot, sizeof(double) * 4);
#undef KP_LALLOC
        if (cudaMemcpyAsync(d_hdr, hdr_be, sizeof(int32_t) * 60 * ntr, cudaMemcpyHostToDevice, c->cs) !=
            cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        KpGeomArgs g;
        memset(&g, 0, sizeof(g));
        g.hdr_be = d_hdr;
        g.ntr = ntr;
        g.geom = c->d_lgraw;
        g.cls = c->d_lcls;
        g.status = c->d_status;
        g.ox = c->p.ox;
        g.oy = c->p.oy;
        g.xy_scale = c->p.xy_scale;
        g.oh = c->p.oh;
        g.dh = c->p.dh;
        g.cull_radius = c->s.cull_radius;
        g.sinA = c->s.sinA;
        g.cosA = c->s.cosA;
        g.IXc = c->s.IXc;
        g.IYc = c->s.IYc;
        g.nh = c->p.nh;
        g.stack = c->p.output == KPSTM_OUT_STACK;
        k_geometry<<<(unsigned)((ntr + 255) / 256), 256, 0, c->cs>>>(g);
        k_bucket<<<1, 1024, sizeof(int32_t) * (ncls + 1), c->cs>>>(c->d_lcls, ntr, ncls, c->d_lcstart,
                                                                      c->d_lorder, c->d_lnlive);
        k_gather_geom<<<(unsigned)((ntr + 255) / 256), 256, 0, c->cs>>>(c->d_lgraw, c->d_lorder, c->d_lnlive,
                                                                        c->d_lgeom);
        int32_t nl = 0;
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&nl, c->d_lnlive, sizeof(int32_t), cudaMemcpyDeviceToHost, c->cs) != cudaSuccess ||
            cudaStreamSynchronize(c->cs) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        c->lsm_ntr = ntr;
        c->lsm_nlive = nl;
        c->lrow = ((4 * (int64_t)(ns + 2 * tm - 3)) + 3) & ~int64_t(3);
        if (cudaMalloc(&c->d_ltable, sizeof(float) * c->lrow * (size_t)(nl > 0 ? nl : 1)) != cudaSuccess) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
    } while (0);
    cudaFree(d_hdr);
    if (st) return st;
    return check_status(c);
}

extern "C" int kpstm_lsm_adjoint(kpstm_ctx *c, const float *d_data, float *d_model)
{
    if (!c || !d_data || !d_model) return KPSTM_ERR_INVALID_ARG;
    if (!c->d_lgeom) return KPSTM_ERR_STATE;
    int st = lsm_adjoint_impl(c, d_data, nullptr, nullptr, d_model);
    if (st) return st;
    return check_status(c);
}

extern "C" int kpstm_lsm_forward(kpstm_ctx *c, const float *d_model, float *d_data)
{
    if (!c || !d_data || !d_model) return KPSTM_ERR_INVALID_ARG;
    if (!c->d_lgeom) return KPSTM_ERR_STATE;
    int st = lsm_forward_impl(c, d_model, d_data);
    if (st) return st;
    return check_status(c);
}

static int dot(kpstm_ctx *c, const float *x, const float *y, int64_t n, double *out)
{
    k_dot_partial<<<KP_DOT_BLOCKS, 256, 0, c->cs>>>(x, y, n, c->d_dotpart);
    k_dot_final<<<1, 256, 0, c->cs>>>(c->d_dotpart, KP_DOT_BLOCKS, c->d_dot);
    KP_CUDA(cudaGetLastError());
    KP_CUDA(cudaMemcpyAsync(out, c->d_dot, sizeof(double), cudaMemcpyDeviceToHost, c->cs));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    return KPSTM_OK;
}

/* CGLS: r = d - L x, s = L^T r, p = s; q = L p, alpha = |s|^2/|q|^2,
   x += alpha p, r -= alpha q, s = L^T r, beta = |s_new|^2/|s|^2, p = s + beta p. */
extern "C" int kpstm_lsm_cg(kpstm_ctx *c, const float *d_data, int32_t niter, float *d_model, double *resid)
{
    if (!c || !d_data || !d_model || niter < 0) return KPSTM_ERR_INVALID_ARG;
    if (!c->d_lgeom) return KPSTM_ERR_STATE;
    const int ns = c->p.ns;
    const int64_t nd = c->lsm_ntr * (int64_t)ns, nm = c->s.dims.out_elems;
    const bool bf16 = c->p.precision == KPSTM_PREC_BF16_KAHAN;
    float *r = nullptr, *q = nullptr, *sv = nullptr, *pv = nullptr, *scale = nullptr;
    uint16_t *r16 = nullptr;
    int st = KPSTM_OK;
    do {
        if (cudaMalloc(&r, sizeof(float) * nd) != cudaSuccess || cudaMalloc(&q, sizeof(float) * nd) != cudaSuccess ||
            cudaMalloc(&sv, sizeof(float) * nm) != cudaSuccess || cudaMalloc(&pv, sizeof(float) * nm) != cudaSuccess) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        if (bf16 && (cudaMalloc(&r16, sizeof(uint16_t) * nd) != cudaSuccess ||
                     cudaMalloc(&scale, sizeof(float) * c->lsm_ntr) != cudaSuccess)) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        const unsigned tb = (unsigned)((c->lsm_ntr * 32 + 255) / 256);
        /* x = 0, r = d (stored bf16 when asked) */
        if (cudaMemsetAsync(d_model, 0, sizeof(float) * nm, c->cs) != cudaSuccess ||
            cudaMemcpyAsync(r, d_data, sizeof(float) * nd, cudaMemcpyDeviceToDevice, c->cs) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        auto store_r = [&]() -> int {
            if (!bf16) return KPSTM_OK;
            k_to_bf16<<<tb, 256, 0, c->cs>>>(r, c->lsm_ntr, ns, r16, scale);
            k_from_bf16<<<1024, 256, 0, c->cs>>>(r16, scale, c->lsm_ntr, ns, r);
            KP_CUDA(cudaGetLastError());
            return KPSTM_OK;
        };
        auto adjoint_r = [&](float *out) -> int {
            return bf16 ? lsm_adjoint_impl(c, nullptr, r16, scale, out) : lsm_adjoint_impl(c, r, nullptr, nullptr, out);
        };
        if ((st = store_r())) break;
        double rr = 0.0;
        if ((st = dot(c, r, r, nd, &rr))) break;
        if (resid) resid[0] = sqrt(rr);
        if ((st = adjoint_r(sv))) break;
        if (cudaMemcpyAsync(pv, sv, sizeof(float) * nm, cudaMemcpyDeviceToDevice, c->cs) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        double gamma = 0.0;
        if ((st = dot(c, sv, sv, nm, &gamma))) break;
        for (int it = 0; it < niter; ++it) {
            if ((st = lsm_forward_impl(c, pv, q))) break;
            double qq = 0.0;
            if ((st = dot(c, q, q, nd, &qq))) break;
            const double alpha = qq > 0.0 ? gamma / qq : 0.0;
            k_axpby<<<1024, 256, 0, c->cs>>>(d_model, pv, (float)alpha, 1.0f, nm);
            k_axpby<<<1024, 256, 0, c->cs>>>(r, q, (float)(-alpha), 1.0f, nd);
            if ((st = store_r())) break;
            if (resid) {
                if ((st = dot(c, r, r, nd, &rr))) break;
                resid[it + 1] = sqrt(rr);
            }
            if ((st = adjoint_r(sv))) break;
            double gnew = 0.0;
            if ((st = dot(c, sv, sv, nm, &gnew))) break;
            const double beta = gamma > 0.0 ? gnew / gamma : 0.0;
            gamma = gnew;
            k_axpby<<<1024, 256, 0, c->cs>>>(pv, sv, 1.0f, (float)beta, nm);
            if (cudaGetLastError() != cudaSuccess) {
                st = KPSTM_ERR_CUDA;
                break;
            }
        }
    } while (0);
    cudaStreamSynchronize(c->cs);
    cudaFree(r);
    cudaFree(q);
    cudaFree(sv);
    cudaFree(pv);
    cudaFree(r16);
    cudaFree(scale);
    if (st) return st;
    return check_status(c);
}
