/*
 * libkpstm: context, device memory, streams and the C ABI of include/kpstm.h.
 *
 * One context images one slab (job) of the reference's image box.  It owns
 * a compute stream and a copy stream: kpstm_add_traces copies block b+1 to
 * the device (copy stream) while block b is imaged (compute stream), using
 * two staging slots; the call returns once its own host buffers have been
 * read.  Per block the compute stream runs
 *     k_geometry -> k_bucket -> k_prep (k_prep_ref in reference mode) -> k_image
 * with no host synchronisation; kpstm_finish runs k_deriv -> k_lowpass.
 */
#include <cuda_runtime.h>

#include <atomic>

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

#define KP_GRAPHS 4 /* cached block graphs (two staging slots x full / last block) */
struct kp_graph {
    cudaGraphExec_t exec;
    int64_t ntr;
    const void *hdr, *smp;
    uint64_t used;
};

struct kpstm_ctx {
    kpstm_params p;
    kpstm_setup s;
    int device;
    int finished_state; /* reserved */
    cudaStream_t cs, xs;         /* compute, copy */
    cudaEvent_t copy_done[2], comp_done[2], decoded[2];
    int slot;
    int K, nwin;                 /* samples per lane, time windows */
    int64_t ntile;               /* image tiles of 8 columns */
    int tile_px;                 /* tile patch: tile_px x (8 / tile_px) columns */
    int persistent, use_graph;   /* launch configuration (kpstm_launch) */
    int minb;                    /* imaging CTAs per SM the kernel variant is built for: 2, 3 or 4 */
    int dirty;                   /* traces imaged since create / reset */
    int nsm;                     /* multiprocessors of the device */
    int64_t row;                 /* floats per tap-table row */
    int32_t *d_tilecols;         /* [ntile][8] column of each warp, -1: none */
    int *d_queue;                /* persistent launch: work-item counter */
    int32_t *d_clsorder;         /* persistent launch: classes by size */
    float *h_colxy;              /* [ncol][2] column coordinates (tile boxes) */
    kp_graph graphs[KP_GRAPHS];
    uint64_t graph_clock;
    /* constant tables */
    float2 *d_colxy;
    int32_t *d_colrow;
    float4 *d_tilebox;
    float2 *d_vrows;
    float *d_t2;
    float2 *d_t2c;
    float *d_tscale;             /* full mode: per-sample read-out factor t dt/8 */
    double *d_c4, *d_c4r;
    float2 *d_c4rw;              /* [ns + 2] the reciprocals of the precision-mode integral as double-word floats */
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
    uint16_t *d_smp16;           /* precision mode: the block's traces as bf16 */
    float *d_scl16;              /* and their per-trace scales */
    /* staging (two slots) */
    int64_t scap;
    int32_t *d_hdr[2];
    float *d_smp[2];
    uint32_t *d_raw[2];          /* raw SEG-Y records, one per staging slot */
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
    float *d_ltable, *d_lkm, *d_lkc;
    unsigned long long *d_lhits;
    double *d_dotpart, *d_dot;
    unsigned int *d_absmax;      /* demigration: bits of max |model|, then the 64-bit nonzero count */
    float *d_dbound;             /* demigration: per live trace max_k (L 1)[k] */
    float *d_wbound;             /* demigration: per live trace largest pair weight x t/(8 dt) */
    unsigned long long *d_dacc;  /* demigration: [nlive][ng] fixed-point trace accumulators */
    int32_t *d_dorder;           /* demigration: live slots in Morton order of their midpoints */
    float *d_rvdt;               /* demigration: [nrow][ns] 1/(v dt)^2 */
    int nrow;                    /* velocity rows of the slab */
    int dbound_ok;
    uint32_t wait_polls;         /* imaging stage waits give up after this many polls */
    int32_t cull;                /* the imaging kernel's dead-window trace cull */
    /* stream handling / profiling */
    cudaStream_t own_cs;
    int prof;
    int nev, capev;
    cudaEvent_t *ev;             /* pairs: start, stop */
    int *evstage;                /* 0 image, 1 prep, 2 finish */
    int *evlaunches;
    int64_t prof_extra;          /* launches inside image stages besides k_image (class ranking) */
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

/* Device allocations of the set-up and of the staging buffers go through
   kp_dmalloc, so that kpstm_debug_fail_alloc can make one of them fail. */
static std::atomic<int> g_fail_alloc(-1);

template <class T>
static cudaError_t kp_dmalloc(T **p, size_t bytes)
{
    int n = g_fail_alloc.load();
    while (n >= 0 && !g_fail_alloc.compare_exchange_weak(n, n - 1)) {
    }
    if (n == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc((void **)p, bytes);
}

extern "C" int kpstm_debug_fail_alloc(int32_t nth)
{
    if (nth < -1) return KPSTM_ERR_INVALID_ARG;
    g_fail_alloc.store(nth);
    return KPSTM_OK;
}

static int kp_free_all(kpstm_ctx *c);

/* The float T with (x < T) == ((double)x < A) for every float x: the
   reference compares a float distance with the double aperture
   (Kirchhoff.c:1352-1354); the kernels make the same decision in fp32. */
static float strict_bound_f(double A)
{
    const float f = (float)A;
    if (A != A || (double)f >= A) return f; /* exact, or f is the next float above A */
    return nextafterf(f, INFINITY);
}

/* The float X with (RN(sqrt(x)) < a) == (x < X) for every float x >= 0, so
   that the kernels test the squared distance instead of rounding its square
   root (RN(sqrt(.)) is monotone, so the passing x form a down-set; the float
   square root is correctly rounded through double). */
static float sq_bound_f(float a)
{
    if (!(a > 0.0f)) return 0.0f;
    if (isinf(a)) return INFINITY;
    float x = (float)((double)a * (double)a);
    while (x > 0.0f && (float)sqrt((double)nextafterf(x, 0.0f)) >= a) x = nextafterf(x, 0.0f);
    while (!isinf(x) && (float)sqrt((double)x) < a) x = nextafterf(x, INFINITY);
    return x;
}

/* ---- imaging launch ------------------------------------------------------- */

static size_t image_smem_row(const kpstm_ctx *c, int64_t row, bool hilo, uint32_t *bar_offset)
{
    return kp_image_smem(c->K, kp_stages(c->p.mode == KPSTM_MODE_FULL, hilo ? 2 : c->minb), row, bar_offset);
}

typedef void (*kp_image_fn)(KpImageArgs);

template <int K>
static kp_image_fn image_fn_k(bool full, bool kahan, bool hilo, int minb)
{
    if (hilo) {
        if constexpr (K <= 16) {
            if (kahan) return k_image<K, true, true, true>;
        }
        if constexpr (K <= 24) {
            if (!kahan) return k_image<K, true, false, true>;
        }
        return nullptr;
    }
    if (!full && minb == 3) {
        if constexpr (K <= 8) return kahan ? k_image<K, false, true, false, 3> : k_image<K, false, false, false, 3>;
        return nullptr;
    }
    if (kahan) {
        if (full && minb == 3) {
            if constexpr (K <= 8) return k_image<K, true, true, false, 3>;
            return nullptr;
        }
        if constexpr (K <= 16) return full ? k_image<K, true, true> : k_image<K, false, true>;
        return nullptr;
    }
    if (full && minb == 3) {
        if constexpr (K <= 16) return k_image<K, true, false, false, 3>;
        return nullptr;
    }
    if (full && minb == 4) {
        if constexpr (K <= 8) return k_image<K, true, false, false, 4>;
        return nullptr;
    }
    if (full) {
        if constexpr (K <= 24) return k_image<K, true, false>;
        return nullptr;
    }
    return k_image<K, false, false>;
}

static kp_image_fn image_fn(const kpstm_ctx *c, bool hilo)
{
    const bool full = c->p.mode == KPSTM_MODE_FULL;
    const bool kahan = c->p.precision == KPSTM_PREC_BF16_KAHAN;
    const int minb = hilo ? 2 : c->minb;
    switch (c->K) {
    case 8: return image_fn_k<8>(full, kahan, hilo, minb);
    case 16: return image_fn_k<16>(full, kahan, hilo, minb);
    case 24: return image_fn_k<24>(full, kahan, hilo, minb);
    default: return image_fn_k<32>(full, kahan, hilo, minb);
    }
}

/* Launches the imaging kernel over nclass classes of the args' table.
   Grid mode: one CTA per (tile, class, window).  Persistent mode: the
   classes are ranked by size on the device, the work counter is cleared and
   a grid of the resident CTAs drains the items. */
static cudaError_t launch_image(kpstm_ctx *c, KpImageArgs a, int nclass, bool hilo)
{
    kp_image_fn fn = image_fn(c, hilo);
    if (!fn) return cudaErrorInvalidValue;
    size_t smem = image_smem_row(c, a.row, hilo, &a.bar_offset);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    a.ntile = c->ntile;
    a.nwin = c->nwin;
    a.tilecols = c->d_tilecols;
    a.tilebox = c->d_tilebox;
    const int64_t nitems = (int64_t)nclass * c->ntile * c->nwin;
    if (nitems == 0) return cudaSuccess;
    if (c->persistent && nitems < INT32_MAX) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, KP_THREADS, smem);
        if (e != cudaSuccess) return e;
        if (occ < 1) occ = 1;
        int64_t grid = (int64_t)occ * c->nsm;
        if (grid > nitems) grid = nitems;
        k_class_order<<<1, 1024, 0, c->cs>>>(a.class_start, nclass, c->d_clsorder);
        if (c->prof) ++c->prof_extra;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemsetAsync(c->d_queue, 0, sizeof(int), c->cs);
        if (e != cudaSuccess) return e;
        a.queue = c->d_queue;
        a.nitems = (int)nitems;
        a.cls_order = c->d_clsorder;
        fn<<<(unsigned)grid, KP_THREADS, smem, c->cs>>>(a);
    } else {
        if (c->ntile > INT32_MAX || nclass > 65535 || c->nwin > 65535) return cudaErrorInvalidValue;
        fn<<<dim3(c->ntile, nclass, c->nwin), KP_THREADS, smem, c->cs>>>(a);
    }
    return cudaGetLastError();
}

/* Largest samples-per-lane the mode's register budget allows (2 CTAs/SM,
   128 registers, no spills): reference 32, full 24, Kahan variants 16. */
static int kmax_of(const kpstm_params *p)
{
    if (p->precision == KPSTM_PREC_BF16_KAHAN) return 16;
    return p->mode == KPSTM_MODE_FULL ? 24 : 32;
}

/* Largest samples-per-lane of the 3-CTAs-per-SM variant (80 registers, no
   spills): full mode 16, full mode with Kahan sums and the reference mode 8. */
static int occ3_kmax(const kpstm_params *p)
{
    if (p->mode != KPSTM_MODE_FULL) return 8;
    return p->precision == KPSTM_PREC_BF16_KAHAN ? 8 : 16;
}

static int default_K(const kpstm_params *p)
{
    const int kmax = kmax_of(p);
    const int nwin = (p->ns + 32 * kmax - 1) / (32 * kmax);
    const int per = (p->ns + nwin - 1) / nwin;
    return per <= 256 ? 8 : per <= 512 ? 16 : per <= 768 ? 24 : 32;
}

/* k_prep runs one thread per trace, a sequential integral each: CTAs of 32
   to 128 threads, so that a small block still spreads over every SM (two
   CTAs per SM before any SM gets a third). */
static unsigned prep_threads(const kpstm_ctx *c, int64_t ntr)
{
    const int64_t per = 64 * (int64_t)c->nsm;
    int64_t w = (ntr + per - 1) / per;
    if (w < 1) w = 1;
    if (w > 4) w = 4;
    return (unsigned)(32 * w);
}

/* The tap tables of up to ntr traces: k_prep_ref (32 traces per CTA) in
   reference mode, k_prep (a thread per trace) in the full and precision
   modes. */
static void launch_prep(const kpstm_ctx *c, const KpPrepArgs &pa, int64_t ntr)
{
    if (!pa.full && !pa.exact) {
        k_prep_ref<<<(unsigned)((ntr + KP_PR_TR - 1) / KP_PR_TR), 32 * KP_PR_WARPS, 0, c->cs>>>(pa);
    } else {
        const unsigned ptb = prep_threads(c, ntr);
        k_prep<<<(unsigned)((ntr + ptb - 1) / ptb), ptb, 0, c->cs>>>(pa);
    }
}

/* default patch: the fewest tiles (fewest idle warps), ties to the 4 x 2
   patch, then 2 x 4, 8 x 1, 1 x 8 (4 x 2 measured fastest on the 3-D survey) */
static int default_px(const kpstm_setup *s)
{
    static const int order[4] = {4, 2, 8, 1};
    int best = 4;
    int64_t bn = -1;
    for (int o = 0; o < 4; ++o) {
        const int px = order[o], py = 8 / px;
        const int64_t n = (int64_t)((s->dims.nx + px - 1) / px) * ((s->dims.ny + py - 1) / py);
        if (bn < 0 || n < bn) {
            bn = n;
            best = px;
        }
    }
    return best;
}

/* (Re)builds the tile -> column map and the tiles' bounding boxes for
   tile_px x (8 / tile_px) patches. */
static int set_tiles(kpstm_ctx *c, int px)
{
    const int nx = c->s.dims.nx, ny = c->s.dims.ny, py = 8 / px;
    const int ntx = (nx + px - 1) / px, nty = (ny + py - 1) / py;
    const int64_t ntile = (int64_t)ntx * nty;
    int32_t *cols = (int32_t *)malloc(sizeof(int32_t) * KPSTM_COLS_PER_CTA * ntile);
    float4 *box = (float4 *)malloc(sizeof(float4) * ntile);
    if (!cols || !box) {
        free(cols);
        free(box);
        return KPSTM_ERR_OUT_OF_MEMORY;
    }
    for (int tx = 0; tx < ntx; ++tx)
        for (int ty = 0; ty < nty; ++ty) {
            const int64_t t = (int64_t)tx * nty + ty;
            float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
            for (int w = 0; w < KPSTM_COLS_PER_CTA; ++w) {
                const int xc = tx * px + w / py, yc = ty * py + w % py;
                int32_t col = -1;
                if (xc < nx && yc < ny) {
                    col = xc * ny + yc;
                    const float X = c->h_colxy[2 * col], Y = c->h_colxy[2 * col + 1];
                    x0 = fminf(x0, X);
                    x1 = fmaxf(x1, X);
                    y0 = fminf(y0, Y);
                    y1 = fmaxf(y1, Y);
                }
                cols[t * KPSTM_COLS_PER_CTA + w] = col;
            }
            box[t] = make_float4(x0, x1, y0, y1);
        }
    int st = KPSTM_OK;
    do {
        if (cudaStreamSynchronize(c->cs) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        if (ntile != c->ntile || !c->d_tilecols) {
            cudaFree(c->d_tilecols);
            cudaFree(c->d_tilebox);
            c->d_tilecols = nullptr;
            c->d_tilebox = nullptr;
            c->ntile = 0;
            if (cudaMalloc(&c->d_tilecols, sizeof(int32_t) * KPSTM_COLS_PER_CTA * ntile) != cudaSuccess ||
                cudaMalloc(&c->d_tilebox, sizeof(float4) * ntile) != cudaSuccess) {
                st = KPSTM_ERR_OUT_OF_MEMORY;
                break;
            }
        }
        if (cudaMemcpy(c->d_tilecols, cols, sizeof(int32_t) * KPSTM_COLS_PER_CTA * ntile, cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(c->d_tilebox, box, sizeof(float4) * ntile, cudaMemcpyHostToDevice) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        c->ntile = ntile;
        c->tile_px = px;
    } while (0);
    free(cols);
    free(box);
    return st;
}

static void set_K(kpstm_ctx *c, int K)
{
    c->K = K;
    c->nwin = (c->p.ns + 32 * K - 1) / (32 * K);
}

static void drop_graphs(kpstm_ctx *c)
{
    for (int i = 0; i < KP_GRAPHS; ++i) {
        if (c->graphs[i].exec) cudaGraphExecDestroy(c->graphs[i].exec);
        c->graphs[i].exec = nullptr;
    }
}

static int grow_work(kpstm_ctx *c, int64_t ntr)
{
    if (ntr <= c->cap) return KPSTM_OK;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    drop_graphs(c); /* they hold the old buffers */
    cudaFree(c->d_graw);
    cudaFree(c->d_geom);
    cudaFree(c->d_cls);
    cudaFree(c->d_order);
    cudaFree(c->d_table);
    cudaFree(c->d_smp16);
    cudaFree(c->d_scl16);
    c->d_graw = c->d_geom = nullptr;
    c->d_cls = c->d_order = nullptr;
    c->d_table = nullptr;
    c->d_smp16 = nullptr;
    c->d_scl16 = nullptr;
    c->cap = 0;
    int64_t n = ntr + ntr / 8 + 64;
    if (kp_dmalloc(&c->d_graw, sizeof(kpstm_geom) * n) != cudaSuccess ||
        kp_dmalloc(&c->d_geom, sizeof(kpstm_geom) * n) != cudaSuccess ||
        kp_dmalloc(&c->d_cls, sizeof(int32_t) * n) != cudaSuccess ||
        kp_dmalloc(&c->d_order, sizeof(int32_t) * n) != cudaSuccess ||
        kp_dmalloc(&c->d_table, sizeof(float) * c->row * n) != cudaSuccess)
        return KPSTM_ERR_OUT_OF_MEMORY;
    if (c->p.precision == KPSTM_PREC_BF16_KAHAN &&
        (kp_dmalloc(&c->d_smp16, sizeof(uint16_t) * c->p.ns * n) != cudaSuccess ||
         kp_dmalloc(&c->d_scl16, sizeof(float) * n) != cudaSuccess))
        return KPSTM_ERR_OUT_OF_MEMORY;
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
    for (int s = 0; s < 2; ++s)
        if (kp_dmalloc(&c->d_hdr[s], sizeof(int32_t) * 60 * n) != cudaSuccess ||
            kp_dmalloc(&c->d_smp[s], sizeof(float) * c->p.ns * n) != cudaSuccess)
            return KPSTM_ERR_OUT_OF_MEMORY;
    c->scap = n;
    return KPSTM_OK;
}

static KpImageArgs image_args(const kpstm_ctx *c);

/* The per-block device pipeline, enqueued on the compute stream (the work
   buffers must already hold ntr traces). */
static int enqueue_block(kpstm_ctx *c, const int32_t *d_hdr, const float *d_smp, int64_t ntr)
{
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
    if (p->precision == KPSTM_PREC_BF16_KAHAN) {
        /* precision mode: the block is kept as bf16 with a per-trace scale and
           the taps are built from it with double integrals */
        k_to_bf16<<<(unsigned)((ntr * 32 + 255) / 256), 256, 0, c->cs>>>(d_smp, ntr, p->ns, c->d_smp16, c->d_scl16);
        KP_CUDA(cudaGetLastError());
        pa.samples = nullptr;
        pa.samples_bf16 = c->d_smp16;
        pa.scale = c->d_scl16;
        pa.exact = 1;
    }
    pa.geom_raw = c->d_graw;
    pa.order = c->d_order;
    pa.nlive = c->d_nlive;
    pa.geom = c->d_geom;
    pa.table = c->d_table;
    pa.c4 = c->d_c4;
    pa.c4r = c->d_c4r;
    pa.c4rw = c->d_c4rw;
    pa.row = c->row;
    pa.ns = p->ns;
    pa.tm = s->dims.trange_max;
    pa.full = p->mode == KPSTM_MODE_FULL;
    pa.dt = p->dt;
    launch_prep(c, pa, ntr);
    KP_CUDA(cudaGetLastError());
    prof_end(c, pe, 1, 3);

    KpImageArgs a = image_args(c);
    a.geom = c->d_geom;
    a.class_start = c->d_cstart;
    a.table = c->d_table;
    a.row = c->row;
    a.km = c->d_km;
    a.kc = c->d_kc;
    a.cnt = c->d_cnt;
    a.hits = c->d_hits;
    int pi = prof_begin(c);
    KP_CUDA(launch_image(c, a, s->nclass, false));
    prof_end(c, pi, 0, 1);
    return KPSTM_OK;
}

/* One block: directly, or (graph flag, profiling off) by replaying the
   block's pipeline from a CUDA graph captured on first use of this
   (ntr, buffers) shape; a few shapes are cached, least recently used out. */
static int run_block(kpstm_ctx *c, const int32_t *d_hdr, const float *d_smp, int64_t ntr)
{
    if (ntr == 0) return KPSTM_OK;
    int st = grow_work(c, ntr);
    if (st) return st;
    c->dirty = 1;
    if (!c->use_graph || c->prof) return enqueue_block(c, d_hdr, d_smp, ntr);
    kp_graph *g = nullptr, *victim = &c->graphs[0];
    for (int i = 0; i < KP_GRAPHS; ++i) {
        kp_graph *q = &c->graphs[i];
        if (q->exec && q->ntr == ntr && q->hdr == d_hdr && q->smp == d_smp) g = q;
        if (!q->exec || (victim->exec && q->used < victim->used)) victim = q;
    }
    if (!g) {
        if (victim->exec) cudaGraphExecDestroy(victim->exec);
        victim->exec = nullptr;
        cudaGraph_t graph = nullptr;
        KP_CUDA(cudaStreamBeginCapture(c->cs, cudaStreamCaptureModeThreadLocal));
        st = enqueue_block(c, d_hdr, d_smp, ntr);
        cudaError_t e = cudaStreamEndCapture(c->cs, &graph);
        if (st || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return st ? st : KPSTM_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&victim->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            victim->exec = nullptr;
            return KPSTM_ERR_CUDA;
        }
        victim->ntr = ntr;
        victim->hdr = d_hdr;
        victim->smp = d_smp;
        g = victim;
    }
    g->used = ++c->graph_clock;
    KP_CUDA(cudaGraphLaunch(g->exec, c->cs));
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
    c->wait_polls = KP_WAIT_POLLS;
    c->cull = 1;
    c->p = *params;
    c->s = s;
    cudaGetDevice(&c->device);
    const int ns = params->ns, tm = s.dims.trange_max;
    const int ncol = s.ncol;
    /* full mode with fp32 storage: the 3-CTAs-per-SM variant (K <= 16) in a
       persistent launch, measured faster than 2 CTAs with K = 24 and than the
       grid launch on the 3-D survey */
    c->minb = (params->mode == KPSTM_MODE_FULL && params->precision == KPSTM_PREC_FP32) ? 3 : 2;
    c->persistent = c->minb == 3;
    set_K(c, c->minb == 3 && default_K(params) > 16 ? 16 : default_K(params));
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c->nsm < 1)
            c->nsm = 1;
    }
    if (params->mode == KPSTM_MODE_FULL)
        c->row = KP_ROW_HDR + (((2 * (int64_t)(ns + 2 * tm - 2)) + 3) & ~int64_t(3)); /* entries 0 .. ns + 2tm - 3 */
    else
        c->row = KP_ROW_HDR + ((ns + 1 + 3) & ~3); /* D[0..ns-1] plus a zero sentinel D[ns] */

    /* host tables */
    float *colxy = (float *)malloc(sizeof(float) * 2 * ncol);
    int32_t *colrow = (int32_t *)malloc(sizeof(int32_t) * ncol);
    float *t2 = (float *)malloc(sizeof(float) * ns);
    int32_t *t1 = (int32_t *)malloc(sizeof(int32_t) * ns);
    double *c4 = (double *)malloc(sizeof(double) * ns);
    double *c4r = (double *)malloc(sizeof(double) * ns);
    float2 *c4rw = (float2 *)malloc(sizeof(float2) * (ns + 2));
    float2 *t2c = (float2 *)malloc(sizeof(float2) * ns);
    float *tsc = (float *)malloc(sizeof(float) * ns);
    double *hd = (double *)malloc(sizeof(double) * ns);
    float *hf = (float *)malloc(sizeof(float) * ns);
    int32_t *rowmap = nullptr;
    float2 *vrows = nullptr;
    float invl2[64];
    int nrow = 0;
    do {
        if (!colxy || !colrow || !t2 || !t1 || !c4 || !c4r || !c4rw || !t2c || !tsc || !hd || !hf) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        kpstm_columns(params, vel, &s, colxy, colrow);
        kpstm_time_tables(params, vel, t2, t1);
        for (int t = 0; t < ns; ++t) {
            c4[t] = 4.0 * (double)t2[t];
            c4r[t] = t > 0 ? 1.0 / c4[t] : 0.0;
            /* full mode works in sample units: (t/2)^2 and t0/(8 dt^2) = t/(8 dt);
               t = 0 gets a tiny positive time so that rsqrt never sees 0 */
            t2c[t] = make_float2(t > 0 ? (float)(0.25 * (double)t * (double)t) : 1e-12f,
                                 (float)((double)t / (8.0 * (double)params->dt)));
            tsc[t] = (float)((double)t / (8.0 * (double)params->dt)); /* t0/(8 dt^2), sample units */
        }
        /* 1/(4 t2[t]) for 0 < t < ns and 1/(dt t)^2 for the tail steps t = ns,
           ns + 1 (Kirchhoff.c:1316-1320), as a float plus its remainder */
        for (int t = 0; t < ns + 2; ++t) {
            const double dtd = (double)params->dt;
            const double r = t == 0 ? 0.0 : (t < ns ? 1.0 / c4[t] : 1.0 / (dtd * dtd * (double)t * (double)t));
            const float rh = (float)r;
            c4rw[t] = make_float2(rh, (float)(r - (double)rh));
        }
        st = kpstm_lowpass_kernel(params, hd);
        if (st) break;
        for (int t = 0; t < ns; ++t) hf[t] = (float)hd[t];
        if (params->velocity_interp) {
            /* one interpolated row per column */
            vrows = (float2 *)malloc(sizeof(float2) * (size_t)ncol * ns);
            if (!vrows) {
                st = KPSTM_ERR_OUT_OF_MEMORY;
                break;
            }
            st = kpstm_interp_rows(params, vel, &s, colrow, reinterpret_cast<float *>(vrows));
            if (st) break;
            for (int cc = 0; cc < ncol; ++cc)
                if (colrow[cc] >= 0) colrow[cc] = cc;
            nrow = ncol;
            for (int L = 0; L < 64; ++L) invl2[L] = L > 0 ? 1.0f / (float)(L * L) : 0.0f;
            break;
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
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->decoded[k], cudaEventDisableTiming);
            }
            if (e != cudaSuccess) {
                st = KPSTM_ERR_CUDA;
                break;
            }
            size_t nimg = (size_t)s.nclass * ncol * ns;
#define KP_ALLOC(ptr, bytes)                                                                                 \
    if (kp_dmalloc(&(ptr), (bytes)) != cudaSuccess) {                                                        \
        st = KPSTM_ERR_OUT_OF_MEMORY;                                                                        \
        break;                                                                                               \
    }
            KP_ALLOC(c->d_colxy, sizeof(float2) * ncol);
            KP_ALLOC(c->d_colrow, sizeof(int32_t) * ncol);
            KP_ALLOC(c->d_queue, sizeof(int));
            KP_ALLOC(c->d_clsorder, sizeof(int32_t) * s.nclass);
            KP_ALLOC(c->d_vrows, sizeof(float2) * (size_t)(nrow > 0 ? nrow : 1) * ns);
            c->nrow = nrow;
            KP_ALLOC(c->d_t2, sizeof(float) * ns);
            KP_ALLOC(c->d_t2c, sizeof(float2) * ns);
            if (params->mode == KPSTM_MODE_FULL) KP_ALLOC(c->d_tscale, sizeof(float) * ns);
            KP_ALLOC(c->d_c4, sizeof(double) * ns);
            KP_ALLOC(c->d_c4r, sizeof(double) * ns);
            KP_ALLOC(c->d_c4rw, sizeof(float2) * (ns + 2));
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
            cudaMemcpyAsync(c->d_vrows, vrows, sizeof(float2) * (size_t)(nrow > 0 ? nrow : 1) * ns,
                            cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_t2, t2, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_t2c, t2c, sizeof(float2) * ns, cudaMemcpyHostToDevice, c->cs);
            if (c->d_tscale) cudaMemcpyAsync(c->d_tscale, tsc, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_c4, c4, sizeof(double) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_c4r, c4r, sizeof(double) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_c4rw, c4rw, sizeof(float2) * (ns + 2), cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_h, hf, sizeof(float) * ns, cudaMemcpyHostToDevice, c->cs);
            cudaMemcpyAsync(c->d_invl2, invl2, sizeof(float) * 64, cudaMemcpyHostToDevice, c->cs);
            cudaMemsetAsync(c->d_km, 0, sizeof(float) * nimg, c->cs);
            cudaMemsetAsync(c->d_cnt, 0, sizeof(int32_t) * nimg, c->cs);
            if (c->d_kc) cudaMemsetAsync(c->d_kc, 0, sizeof(float) * nimg, c->cs);
            cudaMemsetAsync(c->d_status, 0, sizeof(int), c->cs);
            cudaMemsetAsync(c->d_hits, 0, sizeof(unsigned long long), c->cs);
            if (cudaStreamSynchronize(c->cs) != cudaSuccess) {
                st = KPSTM_ERR_CUDA;
                break;
            }
            c->h_colxy = colxy;
            colxy = nullptr;
            st = set_tiles(c, default_px(&s));
        } while (0);
    }
    free(colxy);
    free(colrow);
    free(t2);
    free(t1);
    free(c4);
    free(c4r);
    free(c4rw);
    free(t2c);
    free(tsc);
    free(hd);
    free(hf);
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
    void *ptrs[] = {c->d_colxy, c->d_colrow, c->d_tilebox, c->d_vrows, c->d_t2, c->d_t2c, c->d_tscale, c->d_c4, c->d_c4r, c->d_c4rw,
                    c->d_h, c->d_invl2, c->d_km, c->d_kc, c->d_cnt, c->d_graw, c->d_geom, c->d_cls,
                    c->d_order, c->d_cstart, c->d_nlive, c->d_table, c->d_hdr[0], c->d_hdr[1], c->d_smp[0],
                    c->d_smp[1], c->d_raw[0], c->d_raw[1], c->d_status, c->d_hits, c->d_x, c->d_y, c->d_lgraw, c->d_lgeom,
                    c->d_lcls, c->d_lorder, c->d_lcstart, c->d_lnlive, c->d_lcnt, c->d_ltable, c->d_lkm,
                    c->d_lhits, c->d_dotpart, c->d_dot, c->d_smp16, c->d_scl16, c->d_tilecols, c->d_queue,
                    c->d_clsorder, c->d_absmax, c->d_dbound, c->d_wbound, c->d_lkc, c->d_dacc, c->d_dorder, c->d_rvdt};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i)
        if (ptrs[i]) cudaFree(ptrs[i]);
    for (int k = 0; k < 2; ++k) {
        if (c->copy_done[k]) cudaEventDestroy(c->copy_done[k]);
        if (c->decoded[k]) cudaEventDestroy(c->decoded[k]);
        if (c->comp_done[k]) cudaEventDestroy(c->comp_done[k]);
    }
    drop_graphs(c);
    free(c->h_colxy);
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
    c->dirty = 0;
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
    if (st) {
        cudaEventSynchronize(c->copy_done[s]); /* the caller's buffers are read before it hears back */
        return st;
    }
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
        for (int k = 0; k < 2; ++k) {
            cudaFree(c->d_raw[k]);
            c->d_raw[k] = nullptr;
        }
        c->rawcap = 0;
        const int64_t cap = words + words / 8;
        KP_CUDA(cudaMalloc(&c->d_raw[0], sizeof(uint32_t) * cap));
        KP_CUDA(cudaMalloc(&c->d_raw[1], sizeof(uint32_t) * cap));
        c->rawcap = cap;
    }
    const int s = c->slot;
    /* raw slot s is free once the block that last used it is decoded; the
       header/sample slot s once that block is imaged, so the copy of this
       block overlaps the imaging of the previous one */
    KP_CUDA(cudaStreamWaitEvent(c->xs, c->decoded[s], 0));
    KP_CUDA(cudaMemcpyAsync(c->d_raw[s], rec, sizeof(uint32_t) * words, cudaMemcpyHostToDevice, c->xs));
    KP_CUDA(cudaEventRecord(c->copy_done[s], c->xs));
    KP_CUDA(cudaStreamWaitEvent(c->cs, c->copy_done[s], 0));
    k_segy_decode<<<1024, 256, 0, c->cs>>>(c->d_raw[s], ntr, c->p.ns, c->d_hdr[s], c->d_smp[s]);
    KP_CUDA(cudaGetLastError());
    KP_CUDA(cudaEventRecord(c->decoded[s], c->cs));
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
    out->other_launches += c->prof_extra;
    c->prof_extra = 0;
    c->nev = 0;
    return KPSTM_OK;
}

/* ------------------------------------------------------------------------ */
/* Launch configuration and autotuner (kpstm_launch). */

extern "C" int kpstm_debug_wait_limit(kpstm_ctx *c, uint32_t polls)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    drop_graphs(c); /* captured launches hold the old limit */
    c->wait_polls = polls;
    return KPSTM_OK;
}

extern "C" int kpstm_debug_trace_cull(kpstm_ctx *c, int32_t enable)
{
    if (!c) return KPSTM_ERR_INVALID_ARG;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    drop_graphs(c); /* captured launches hold the old setting */
    c->cull = enable ? 1 : 0;
    return KPSTM_OK;
}

extern "C" int kpstm_get_launch(const kpstm_ctx *c, kpstm_launch *cfg)
{
    if (!c || !cfg) return KPSTM_ERR_INVALID_ARG;
    memset(cfg, 0, sizeof(*cfg));
    cfg->tile_px = c->tile_px;
    cfg->samples_per_lane = c->K;
    cfg->persistent = c->persistent;
    cfg->graph = c->use_graph;
    cfg->ctas_per_sm = c->minb;
    return KPSTM_OK;
}

static bool valid_K(const kpstm_ctx *c, int K)
{
    return (K == 8 || K == 16 || K == 24 || K == 32) && K <= kmax_of(&c->p);
}

extern "C" int kpstm_set_launch(kpstm_ctx *c, const kpstm_launch *cfg)
{
    if (!c || !cfg) return KPSTM_ERR_INVALID_ARG;
    const int px = cfg->tile_px ? cfg->tile_px : default_px(&c->s);
    const bool occ3 = c->p.mode == KPSTM_MODE_FULL && c->p.precision == KPSTM_PREC_FP32;
    const int minb = cfg->ctas_per_sm ? cfg->ctas_per_sm : (occ3 ? 3 : 2);
    const int kmax3 = occ3_kmax(&c->p);
    int K = cfg->samples_per_lane ? cfg->samples_per_lane : default_K(&c->p);
    if (minb == 3 && !cfg->samples_per_lane && K > kmax3) K = kmax3;
    if ((px != 1 && px != 2 && px != 4 && px != 8) || !valid_K(c, K)) return KPSTM_ERR_INVALID_ARG;
    if ((cfg->persistent != 0 && cfg->persistent != 1) || (cfg->graph != 0 && cfg->graph != 1))
        return KPSTM_ERR_INVALID_ARG;
    if (minb == 4 && !cfg->samples_per_lane) K = 8;
    if (minb != 2 && minb != 3 && minb != 4) return KPSTM_ERR_INVALID_ARG;
    if (minb == 3 && K > kmax3) return KPSTM_ERR_INVALID_ARG;
    if (minb == 4 && (!occ3 || K > 8)) return KPSTM_ERR_INVALID_ARG; /* full mode, fp32, K = 8 only */
    drop_graphs(c);
    if (px != c->tile_px) {
        int st = set_tiles(c, px);
        if (st) return st;
    }
    set_K(c, K);
    c->minb = minb;
    c->persistent = cfg->persistent;
    c->use_graph = cfg->graph;
    return KPSTM_OK;
}

extern "C" int kpstm_autotune(kpstm_ctx *c, const int32_t *d_hdr_be, const float *d_samples, int64_t ntr,
                              kpstm_launch *best, float *best_ms)
{
    if (!c || ntr <= 0 || !d_hdr_be || !d_samples || ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    if (c->dirty) return KPSTM_ERR_STATE;
    int st = grow_work(c, ntr);
    if (st) return st;
    const int prof = c->prof, graph = c->use_graph;
    c->prof = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) st = KPSTM_ERR_CUDA;
    /* patches with at most twice the fewest tiles (others leave most warps idle) */
    int64_t nmin = -1;
    for (int px = 1; px <= 8; px *= 2) {
        const int py = 8 / px;
        const int64_t n = (int64_t)((c->s.dims.nx + px - 1) / px) * ((c->s.dims.ny + py - 1) / py);
        if (nmin < 0 || n < nmin) nmin = n;
    }
    kpstm_launch win;
    memset(&win, 0, sizeof(win));
    float win_ms = -1.0f;
    for (int px = 1; px <= 8 && !st; px *= 2) {
        const int py = 8 / px;
        const int64_t n = (int64_t)((c->s.dims.nx + px - 1) / px) * ((c->s.dims.ny + py - 1) / py);
        if (n > 2 * nmin) continue;
        for (int K = 8; K <= 32 && !st; K += 8) {
            if (!valid_K(c, K)) continue;
            for (int v = 0; v < 6 && !st; ++v) {
                const int pers = v & 1, minb = 2 + (v >> 1);
                if (minb == 3 && K > occ3_kmax(&c->p)) continue;
                if (minb == 4 && (K > 8 || c->p.mode != KPSTM_MODE_FULL || c->p.precision != KPSTM_PREC_FP32))
                    continue;
                kpstm_launch cfg;
                memset(&cfg, 0, sizeof(cfg));
                cfg.tile_px = px;
                cfg.samples_per_lane = K;
                cfg.persistent = pers;
                cfg.ctas_per_sm = minb;
                st = kpstm_set_launch(c, &cfg);
                if (st) break;
                float ms = 0.0f;
                for (int rep = 0; rep < 2 && !st; ++rep) { /* the first run warms caches and attributes */
                    if (cudaEventRecord(e0, c->cs) != cudaSuccess) st = KPSTM_ERR_CUDA;
                    if (!st) st = enqueue_block(c, d_hdr_be, d_samples, ntr);
                    if (!st && (cudaEventRecord(e1, c->cs) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                        st = KPSTM_ERR_CUDA;
                }
                if (!st) st = check_status(c);
                if (!st && (win_ms < 0.0f || ms < win_ms)) {
                    win_ms = ms;
                    win = cfg;
                }
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    c->prof = prof;
    if (!st) {
        win.graph = graph;
        st = kpstm_set_launch(c, &win);
    }
    int st2 = kpstm_reset(c);
    if (!st) st = st2;
    if (st) return st;
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return KPSTM_OK;
}

/* ------------------------------------------------------------------------ */
/* Finishing without device allocation (kpstm_finish_noalloc).
   The scratch a finishing pass needs - the derivative traces between
   k_deriv and k_lowpass, and the low-pass impulse response - is this one
   file-scope array instead of context buffers.  Nothing in it has to start
   at zero: every call rewrites the parts it reads. */
/* ns is bounded by k_lowpass's shared memory (2 ns + 8 ns floats <= 220 KB) */
static_assert(sizeof(float) * (((2 * KPSTM_NOALLOC_MAX_NS + 3) & ~3) + KPSTM_NOALLOC_MAX_NS * KP_LP_ROWS) <= 220 * 1024,
              "KPSTM_NOALLOC_MAX_NS exceeds the low-pass kernel's shared memory");
static __device__ __align__(256) float g_noalloc_scratch[KPSTM_NOALLOC_MAX_SAMPLES + KPSTM_NOALLOC_MAX_NS];

/* Device address of g_noalloc_scratch per device, looked up once per device
   with that device current (the array's name is only a host-side handle in
   host code), and the low-pass response last uploaded there: (ns, dt,
   cutoff) of the last upload, so that calls with the same sampling and
   filter skip it.  The cache does not survive cudaDeviceReset. */
#define KP_NOALLOC_MAX_DEVICES 64
static float *g_noalloc_ptr[KP_NOALLOC_MAX_DEVICES];
struct kp_noalloc_key {
    int ns;
    float dt;
    double cutoff;
};
static kp_noalloc_key g_noalloc_key[KP_NOALLOC_MAX_DEVICES];
static double g_noalloc_hd[KPSTM_NOALLOC_MAX_NS]; /* host staging of the response (no allocation) */
static float g_noalloc_hf[KPSTM_NOALLOC_MAX_NS];
static pthread_mutex_t g_noalloc_mu = PTHREAD_MUTEX_INITIALIZER;

/* The scratch of this device, with the low-pass impulse response of params
   (kpstm_lowpass_kernel, the host computation kpstm_finish uses) in its last
   KPSTM_NOALLOC_MAX_NS floats. */
static int noalloc_scratch(const kpstm_params *params, cudaStream_t stream, float **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return KPSTM_ERR_NO_DEVICE;
    if (dev < 0 || dev >= KP_NOALLOC_MAX_DEVICES) return KPSTM_ERR_UNSUPPORTED;
    int st = KPSTM_OK;
    pthread_mutex_lock(&g_noalloc_mu);
    do {
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                st = KPSTM_ERR_CUDA;
                break;
            }
            g_noalloc_ptr[dev] = (float *)p;
        }
        kp_noalloc_key &k = g_noalloc_key[dev];
        if (k.ns != params->ns || k.dt != params->dt || k.cutoff != params->anti_alias_cutoff) {
            const int ns = params->ns;
            if ((st = kpstm_lowpass_kernel(params, g_noalloc_hd))) break;
            for (int i = 0; i < ns; ++i) g_noalloc_hf[i] = (float)g_noalloc_hd[i];
            /* from pageable memory: returns once the bytes are staged, so the
               host buffer may be reused */
            if (cudaMemcpyAsync(g_noalloc_ptr[dev] + KPSTM_NOALLOC_MAX_SAMPLES, g_noalloc_hf, sizeof(float) * ns,
                                cudaMemcpyHostToDevice, stream) != cudaSuccess) {
                k.ns = 0;
                st = KPSTM_ERR_CUDA;
                break;
            }
            k.ns = ns;
            k.dt = params->dt;
            k.cutoff = params->anti_alias_cutoff;
        }
        *out = g_noalloc_ptr[dev];
    } while (0);
    pthread_mutex_unlock(&g_noalloc_mu);
    return st;
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
    if (n > KPSTM_NOALLOC_MAX_SAMPLES || ns > KPSTM_NOALLOC_MAX_NS) return KPSTM_ERR_TOO_LARGE;
    const size_t smem = sizeof(float) * (((2 * (size_t)ns + 3) & ~size_t(3)) + (size_t)ns * KP_LP_ROWS);
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    float *scratch = nullptr;
    st = noalloc_scratch(params, stream, &scratch);
    if (st) return st;
    float *x = scratch, *h = scratch + KPSTM_NOALLOC_MAX_SAMPLES;
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
    a.aperture_f = strict_bound_f(p->aperture);
    a.aperture_x2 = sq_bound_f(a.aperture_f);
    float r = (float)(p->aperture * (1.0 + 1e-5) + 1e-3);
    a.tile_r2 = r * r;
    a.aax = (float)p->iline_distance;
    a.aay = (float)p->xline_distance;
    a.wait_polls = c->wait_polls;
    a.cull = c->cull;
    return a;
}

static int lsm_adjoint_impl(kpstm_ctx *c, const float *d_data, const uint16_t *d_data16, const float *d_scale,
                            float *d_model)
{
    const int ns = c->p.ns, ncol = c->s.ncol, ncls = c->s.nclass;
    const size_t nimg = (size_t)ncls * ncol * ns;
    KP_CUDA(cudaMemsetAsync(c->d_lkm, 0, sizeof(float) * nimg, c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_lcnt, 0, sizeof(int32_t) * nimg, c->cs));
    if (c->d_lkc) KP_CUDA(cudaMemsetAsync(c->d_lkc, 0, sizeof(float) * nimg, c->cs));
    KP_CUDA(cudaMemsetAsync(c->d_lhits, 0, sizeof(unsigned long long), c->cs));
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
        launch_prep(c, pa, c->lsm_nlive);
        KP_CUDA(cudaGetLastError());
        KpImageArgs a = image_args(c);
        a.geom = c->d_lgeom;
        a.class_start = c->d_lcstart;
        a.table = c->d_ltable;
        a.row = c->lrow;
        a.km = c->d_lkm;
        a.kc = c->d_lkc;
        a.cnt = c->d_lcnt;
        a.hits = c->d_lhits;
        /* the adjoint's own split: 2 CTAs/SM and the largest K of the hi/lo
           tables (the imaging launch may use the 3-CTA variant's K <= 16) */
        const int K0 = c->K;
        set_K(c, default_K(&c->p));
        cudaError_t e = launch_image(c, a, ncls, true);
        set_K(c, K0);
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
    a.rvdt = c->d_rvdt;
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
    a.aperture_f = strict_bound_f(p->aperture);
    a.aperture_x2 = sq_bound_f(a.aperture_f);
    a.tmax = (float)ns - 1.0f;
    a.lmaxf = (float)s->lmax;
    const float rdt = 1.0f / p->dt;
    a.rdt2 = rdt * rdt;
    a.aax = (float)p->iline_distance;
    a.aay = (float)p->xline_distance;
    a.dt = p->dt;
    a.ng = ns + s->dims.trange_max - 1; /* G index <= ns - 1 + lmax, lmax <= tm - 1 */
    /* Worst case of one trace: every (column, sample) pair of the slab covering
       one sample with the largest weight and width lmax + 1 (the triangle plus
       the float rounding of its tap positions). */
    const double cover = (double)s->ncol * ns * (s->lmax + 1);
    /* Below its support a pair leaves gs (ya + yb - 2 y0) in every sample, |.|
       <= one spacing u of floats below 2^ceil(log2 ng) (the roundings of
       y0 +- Lf).  Summed over a trace's pairs that is at most u max|m| sum(w ts),
       and sum(w ts) <= 2 sum_k (L 1)[k] <= 2 ng (L 1)max (a triangle of
       half-width Lf >= 1 sums to at least Lf^2 / 2 over the samples), so the
       tails add at most 2 ng u = tailf times (L 1)max; twice that is used. */
    {
        const int eg = (int)ceil(log2((double)a.ng + 1.0));
        a.tailf = (float)(4.0 * a.ng * ldexp(1.0, eg - 24));
    }
    /* shared-memory rows: an entry gets at most 4 units of 2^(R-1) per sample
       of a column; norm_cols columns between normalisations must keep the low
       limb within 2^31: (4 ns norm_cols + 2) 2^(R-1) <= 2^31 */
    a.norm_cols = 2;
    a.limb_r = 32 - (int)ceil(log2(4.0 * ns * a.norm_cols + 2.0));
    while (a.limb_r < 12 && a.norm_cols > 1) {
        a.norm_cols /= 2;
        a.limb_r = 32 - (int)ceil(log2(4.0 * ns * a.norm_cols + 2.0));
    }
    if (a.limb_r > 21) a.limb_r = 21;
    a.absmax = c->d_absmax;
    a.nmodel = (int64_t)s->nclass * s->ncol * ns;
    a.order = c->d_dorder;
    /* accumulator rows in shared memory when four of them fit with room for
       several CTAs per SM (and the radix leaves the limbs room), else in L2 */
    const bool use_sh = kp_demig_smem(ns, a.ng, true) <= 48 * 1024 && a.limb_r >= 12;
    /* bound pass (all-ones model, |gs| < 2^bound_g): shared rows need
       4 cover 2^g + 2^31 < 2^(31+R) and |2 gs| < 2^(22+R); the L2 rows need
       cover 2^g < 2^62 and |2 gs| <= 2^45 */
    const int lc = (int)ceil(log2(cover));
    a.bound_g = use_sh ? (21 < 28 - lc ? 21 : 28 - lc) + a.limb_r : (30 < 61 - lc ? 30 : 61 - lc);
    const size_t smem = kp_demig_smem(ns, a.ng, use_sh);
    if (smem > 200 * 1024) return KPSTM_ERR_UNSUPPORTED;
    const size_t accb = sizeof(unsigned long long) * (size_t)a.ng * (size_t)c->lsm_nlive;
    if (!c->d_dacc && !use_sh) {
        if (cudaMalloc(&c->d_dacc, accb) != cudaSuccess) return KPSTM_ERR_OUT_OF_MEMORY;
    }
    if (!c->d_rvdt) {
        const int64_t nv = (int64_t)(c->nrow > 0 ? c->nrow : 1) * ns;
        if (cudaMalloc(&c->d_rvdt, sizeof(float) * nv) != cudaSuccess) return KPSTM_ERR_OUT_OF_MEMORY;
        const float rdt = 1.0f / p->dt;
        k_rvdt<<<2 * c->nsm, 256, 0, c->cs>>>(c->d_vrows, nv, rdt * rdt, c->d_rvdt);
        KP_CUDA(cudaGetLastError());
    }
    a.rvdt = c->d_rvdt;
    a.acc = use_sh ? nullptr : c->d_dacc;
    void (*dm)(KpDemigArgs) = use_sh ? k_demig<true, false> : k_demig<false, false>;
    void (*dmb)(KpDemigArgs) = use_sh ? k_demig<true, true> : k_demig<false, true>;
    KP_CUDA(cudaFuncSetAttribute(dm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    KP_CUDA(cudaFuncSetAttribute(dmb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned nblk = (unsigned)((c->lsm_nlive + KP_DM_WARPS - 1) / KP_DM_WARPS);
    if (!c->dbound_ok) {
        /* once per geometry: max_k (L 1)[trace, k], the fixed-point range of each trace */
        KpDemigArgs b = a;
        b.model = nullptr;
        b.dbound_out = c->d_dbound;
        b.wbound_out = c->d_wbound;
        if (!use_sh) KP_CUDA(cudaMemsetAsync(c->d_dacc, 0, accb, c->cs));
        dmb<<<nblk, 32 * KP_DM_WARPS, smem, c->cs>>>(b);
        KP_CUDA(cudaGetLastError());
        c->dbound_ok = 1;
    }
    if (!use_sh) KP_CUDA(cudaMemsetAsync(c->d_dacc, 0, accb, c->cs));
    a.dbound = c->d_dbound;
    a.wbound = c->d_wbound;
    const int64_t nmodel = (int64_t)s->nclass * s->ncol * ns;
    KP_CUDA(cudaMemsetAsync(c->d_absmax, 0, 2 * sizeof(unsigned long long), c->cs));
    k_absmax<<<4 * c->nsm, 256, 0, c->cs>>>(d_model, nmodel, c->d_absmax);
    KP_CUDA(cudaGetLastError());
    dm<<<nblk, 32 * KP_DM_WARPS, smem, c->cs>>>(a);
    KP_CUDA(cudaGetLastError());
    return KPSTM_OK;
}

/* The demigration's trace order: live slots sorted by a Morton (Z-order)
   key of their midpoints on a grid of a quarter aperture, so that the warps
   of a CTA, and CTAs running side by side, walk nearly the same image columns
   and share their model and velocity rows in the caches.  (The migration
   keeps class order; the result does not depend on this order.) */
struct kp_zkey {
    uint32_t key;
    int32_t slot;
};

static int kp_zcmp(const void *a, const void *b)
{
    const kp_zkey *x = (const kp_zkey *)a, *y = (const kp_zkey *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->slot - y->slot;
}

static uint32_t kp_spread16(uint32_t v)
{
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

static int spatial_order(kpstm_ctx *c, int32_t nl)
{
    cudaFree(c->d_dorder);
    c->d_dorder = nullptr;
    if (nl <= 0) return KPSTM_OK;
    kpstm_geom *g = (kpstm_geom *)malloc(sizeof(kpstm_geom) * (size_t)nl);
    kp_zkey *k = (kp_zkey *)malloc(sizeof(kp_zkey) * (size_t)nl);
    int32_t *o = (int32_t *)malloc(sizeof(int32_t) * (size_t)nl);
    int st = KPSTM_OK;
    do {
        if (!g || !k || !o) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        if (cudaMemcpy(g, c->d_lgeom, sizeof(kpstm_geom) * (size_t)nl, cudaMemcpyDeviceToHost) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        float x0 = g[0].cmpx, y0 = g[0].cmpy;
        for (int32_t i = 1; i < nl; ++i) {
            x0 = fminf(x0, g[i].cmpx);
            y0 = fminf(y0, g[i].cmpy);
        }
        const double cell = c->p.aperture > 0.0 ? 0.25 * c->p.aperture : 1.0;
        for (int32_t i = 0; i < nl; ++i) {
            double qx = floor((g[i].cmpx - x0) / cell), qy = floor((g[i].cmpy - y0) / cell);
            qx = qx < 0.0 ? 0.0 : (qx > 65535.0 ? 65535.0 : qx);
            qy = qy < 0.0 ? 0.0 : (qy > 65535.0 ? 65535.0 : qy);
            k[i].key = kp_spread16((uint32_t)qx) | (kp_spread16((uint32_t)qy) << 1);
            k[i].slot = i;
        }
        qsort(k, (size_t)nl, sizeof(kp_zkey), kp_zcmp);
        for (int32_t i = 0; i < nl; ++i) o[i] = k[i].slot;
        if (cudaMalloc(&c->d_dorder, sizeof(int32_t) * (size_t)nl) != cudaSuccess) {
            st = KPSTM_ERR_OUT_OF_MEMORY;
            break;
        }
        if (cudaMemcpy(c->d_dorder, o, sizeof(int32_t) * (size_t)nl, cudaMemcpyHostToDevice) != cudaSuccess)
            st = KPSTM_ERR_CUDA;
    } while (0);
    free(g);
    free(k);
    free(o);
    return st;
}

extern "C" int kpstm_lsm_pair_count(kpstm_ctx *c, int64_t *pairs)
{
    if (!c || !pairs) return KPSTM_ERR_INVALID_ARG;
    if (!c->d_lhits) return KPSTM_ERR_STATE;
    unsigned long long h = 0;
    KP_CUDA(cudaMemcpyAsync(&h, c->d_lhits, sizeof(h), cudaMemcpyDeviceToHost, c->cs));
    KP_CUDA(cudaStreamSynchronize(c->cs));
    *pairs = (int64_t)h * c->p.ns;
    return KPSTM_OK;
}

extern "C" int kpstm_lsm_geometry(kpstm_ctx *c, const int32_t *hdr_be, int64_t ntr)
{
    if (!c || !hdr_be || ntr <= 0 || ntr > INT32_MAX / 2) return KPSTM_ERR_INVALID_ARG;
    if (c->p.mode != KPSTM_MODE_FULL) return KPSTM_ERR_UNSUPPORTED;
    KP_CUDA(cudaStreamSynchronize(c->cs));
    void *old[] = {c->d_lgraw, c->d_lgeom, c->d_lcls, c->d_lorder, c->d_lcstart, c->d_lnlive,
                   c->d_lcnt, c->d_ltable, c->d_lkm, c->d_lhits, c->d_dotpart, c->d_dot, c->d_absmax,
                   c->d_dbound, c->d_wbound, c->d_lkc, c->d_dacc, c->d_dorder};
    for (size_t i = 0; i < sizeof(old) / sizeof(old[0]); ++i)
        if (old[i]) cudaFree(old[i]);
    c->d_lkc = nullptr;
    c->d_dacc = nullptr;
    c->d_dorder = nullptr;
    c->d_absmax = nullptr;
    c->d_dbound = nullptr;
    c->d_wbound = nullptr;
    c->dbound_ok = 0;
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
        if (cudaMemsetAsync(c->d_lhits, 0, sizeof(unsigned long long), c->cs) != cudaSuccess) {
            st = KPSTM_ERR_CUDA;
            break;
        }
        KP_LALLOC(c->d_dotpart, sizeof(double) * KP_DOT_BLOCKS);
        KP_LALLOC(c->d_dot, sizeof(double) * 4);
        KP_LALLOC(c->d_absmax, 2 * sizeof(unsigned long long));
        KP_LALLOC(c->d_dbound, sizeof(float) * (size_t)ntr);
        KP_LALLOC(c->d_wbound, sizeof(float) * (size_t)ntr);
        if (c->p.precision == KPSTM_PREC_BF16_KAHAN) KP_LALLOC(c->d_lkc, sizeof(float) * nimg);
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
        st = spatial_order(c, nl);
        if (st) break;
        c->lrow = KP_ROW_HDR + 4 * (int64_t)(ns + 2 * tm - 2);
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
    return kpstm_lsm_cg_ex(c, d_data, niter, d_model, resid, nullptr, nullptr);
}

extern "C" int kpstm_lsm_cg_ex(kpstm_ctx *c, const float *d_data, int32_t niter, float *d_model, double *resid,
                               kpstm_cg_monitor monitor, void *user)
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
        if (niter == 0) break; /* m = 0 is the answer; no search direction is needed */
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
            if (resid || monitor) {
                if ((st = dot(c, r, r, nd, &rr))) break;
                if (resid) resid[it + 1] = sqrt(rr);
            }
            if (monitor) {
                if (cudaGetLastError() != cudaSuccess) {
                    st = KPSTM_ERR_CUDA;
                    break;
                }
                if (monitor(it + 1, d_model, sqrt(rr), user)) break; /* the caller's stop */
            }
            if (it + 1 == niter) { /* x and r are final; the next direction (one L^T) is never used */
                if (cudaGetLastError() != cudaSuccess) st = KPSTM_ERR_CUDA;
                break;
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
