/*
 * Kernels of libkpstm (sm_103a).
 *
 *  k_segy_decode   raw SEG-Y records -> header words + IEEE samples
 *                  (Kirchhoff.c:1280-1290)
 *  k_geometry      trace geometry, offset class, slab cull (:1297-1338)
 *  k_bucket        stable partition of the block's traces by class
 *  k_prep          per-trace double running integral (:1312-1328) and the
 *                  tap table the imaging kernel gathers from
 *  k_image         imaging (:1341-1403) as a gather: a CTA owns 8 image
 *                  columns x a time window of one offset class in registers
 *                  and streams that class's traces through shared memory
 *                  with TMA bulk copies, in trace order
 *  k_deriv / k_lowpass / k_relayout   finishing (:1440-1479)
 */
#ifndef KPSTM_KERNELS_CUH
#define KPSTM_KERNELS_CUH

#include <type_traits>

#include "kpstm_device.cuh"

#define KP_TB_REF 4     /* traces per staged batch, reference mode */
#define KP_TB_FULL 2    /* traces per staged batch, full mode */
#define KP_LCH 1024     /* traces examined per compaction chunk */
#define KP_THREADS 256  /* 8 warps = KPSTM_COLS_PER_CTA columns */
#define KP_ROW_HDR 8    /* floats of trace geometry at the start of every tap-table row */

struct KpGeomArgs {
    const int32_t *hdr_be; /* [ntr][60] */
    int64_t ntr;
    kpstm_geom *geom;      /* [ntr], block order */
    int32_t *cls;          /* [ntr] */
    int *status;
    double ox, oy, xy_scale, oh, dh, cull_radius;
    float sinA, cosA, IXc, IYc;
    int nh, stack;
};

struct KpPrepArgs {
    const float *samples;          /* [ntr][ns], fp32 */
    const uint16_t *samples_bf16;  /* [ntr][ns], bf16 (precision mode) or null */
    const float *scale;            /* [ntr] per-trace scale for bf16 */
    const kpstm_geom *geom_raw;    /* [ntr] block order */
    const int32_t *order;          /* [nslot] slot -> trace */
    const int32_t *nlive;          /* device scalar */
    kpstm_geom *geom;              /* [nslot] slot order */
    float *table;                  /* [nslot][row] */
    const double *c4;              /* [ns] 4*t2[t] */
    const double *c4r;             /* [ns] RN(1/(4*t2[t])) */
    const float2 *c4rw;            /* [ns + 2] 1/(4 t2[t]) (t < ns), 1/(dt t)^2 (tail) as double-word floats */
    int64_t row;                   /* floats per table row */
    int ns, tm, full, hilo;        /* hilo: full-mode rows of float4 {hi, lo, dP, 0} */
    int exact;                     /* reference-mode taps from double integrals (precision mode) */
    float dt;
};

struct KpImageArgs {
    const kpstm_geom *geom;        /* slot order */
    const int32_t *class_start;    /* [ncls+1] */
    const float *table;            /* [nslot][row] */
    int64_t row;
    const float2 *colxy;           /* [ncol] */
    const int32_t *colrow;         /* [ncol] compact velocity row, -1 = below grid */
    const float4 *tilebox;         /* [ntile] xmin, xmax, ymin, ymax */
    const float2 *vrows;           /* [nrow][ns] {v^2, RN(1/v^2)} */
    const float *t2;               /* [ns] reference t2 */
    const float2 *t2c;             /* [ns] full mode {(t dt/2)^2, t dt/8} */
    const float *inv_l2;           /* [lmax+1] 1/L^2 */
    float *km;                     /* [ncls][ncol][ns] */
    float *kc;                     /* Kahan compensation, negated (-c), same layout, or null */
    int32_t *cnt;                  /* [ncls][ncol][ns] fold - 1 */
    unsigned long long *hits;      /* (trace, column) pairs in aperture */
    int *status;
    int ncol, ns, tm, lmax;
    float dt, rdt, nsf, lmaxf;
    double aperture;
    float aperture_f;              /* float x: x < aperture_f exactly when (double)x < aperture */
    float aperture_x2;             /* float X: RN(sqrt(x)) < aperture_f exactly when x < X (x >= 0) */
    float tile_r2;                 /* squared tile-test radius (aperture + margin) */
    float aax, aay;                /* full mode: line spacings */
    const int32_t *tilecols;       /* [ntile][8] column of each warp, -1 = none */
    int ntile, nwin;
    uint32_t bar_offset;           /* byte offset of the two mbarriers in shared memory */
    int *queue;                    /* persistent mode: work-item counter (zeroed per launch) */
    int nitems;                    /* persistent mode: ntile * nwin * classes */
    const int32_t *cls_order;      /* persistent mode: classes, largest first */
    uint32_t wait_polls;           /* polls before a stage wait gives up (KP_WAIT_POLLS) */
    int32_t cull;                  /* leave out traces dead over a tile's whole window */
};

/* ------------------------------------------------------------------------ */

__global__ void k_segy_decode(const uint32_t *rec, int64_t ntr, int ns, int32_t *hdr, float *samples)
{
    const int64_t words = 60 + (int64_t)ns;
    const int64_t n = ntr * words;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t tr = i / words, k = i - tr * words;
        uint32_t u = rec[i];
        if (k < 60) {
            hdr[tr * 60 + k] = (int32_t)u; /* kept big-endian, as read */
        } else {
            int32_t w = (int32_t)__byte_perm(u, 0, 0x0123);
            int s = (((w >> 31) & 0x01) * (-2)) + 1;
            float frac = __fdiv_rn(__int2float_rn(w & 0x00ffffff), 16777216.0f);
            float scale = ldexpf(1.0f, 4 * (((w >> 24) & 0x7f) - 64));
            samples[tr * ns + (k - 60)] = __fmul_rn(__fmul_rn(__int2float_rn(s), frac), scale);
        }
    }
}

__device__ __forceinline__ int kp_coord(const KpGeomArgs &a, uint32_t w_be, double o, bool *ok)
{
    uint32_t u = __byte_perm(w_be, 0, 0x0123);
    double v = (double)u - (a.xy_scale == 1.0 ? o : o / a.xy_scale);
    if (!(v > -2147483649.0 && v < 2147483648.0)) {
        *ok = false;
        return 0;
    }
    return (int)v; /* truncation, as the assignment to int i at Kirchhoff.c:1297 */
}

/* Kirchhoff.c:1297-1310 and the slab cull of :1332-1338. */
__global__ void k_geometry(KpGeomArgs a)
{
    int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (it >= a.ntr) return;
    const uint32_t *h = (const uint32_t *)a.hdr_be + it * 60;
    bool ok = true;
    int si = kp_coord(a, h[18], a.ox, &ok), sj = kp_coord(a, h[19], a.oy, &ok);
    int gi = kp_coord(a, h[20], a.ox, &ok), gj = kp_coord(a, h[21], a.oy, &ok);
    kpstm_geom g;
    if (a.xy_scale == 1.0) {
        g.sxt = __fadd_rn(__fmul_rn(a.cosA, __int2float_rn(si)), __fmul_rn(a.sinA, __int2float_rn(sj)));
        g.syt = __fadd_rn(__fmul_rn(-a.sinA, __int2float_rn(si)), __fmul_rn(a.cosA, __int2float_rn(sj)));
        g.gxt = __fadd_rn(__fmul_rn(a.cosA, __int2float_rn(gi)), __fmul_rn(a.sinA, __int2float_rn(gj)));
        g.gyt = __fadd_rn(__fmul_rn(-a.sinA, __int2float_rn(gi)), __fmul_rn(a.cosA, __int2float_rn(gj)));
    } else { /* Kirchhoff_GHTest1.c:1302-1312: float products scaled in double */
        const double s = a.xy_scale;
        g.sxt = (float)((double)__fmul_rn(a.cosA, __int2float_rn(si)) * s + (double)__fmul_rn(a.sinA, __int2float_rn(sj)) * s);
        g.syt = (float)((double)__fmul_rn(-a.sinA, __int2float_rn(si)) * s + (double)__fmul_rn(a.cosA, __int2float_rn(sj)) * s);
        g.gxt = (float)((double)__fmul_rn(a.cosA, __int2float_rn(gi)) * s + (double)__fmul_rn(a.sinA, __int2float_rn(gj)) * s);
        g.gyt = (float)((double)__fmul_rn(-a.sinA, __int2float_rn(gi)) * s + (double)__fmul_rn(a.cosA, __int2float_rn(gj)) * s);
    }
    float dx = __fsub_rn(g.sxt, g.gxt), dy = __fsub_rn(g.syt, g.gyt);
    float h2 = (float)(0.25 * (double)__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    g.cmpx = (float)(0.5 * (double)__fadd_rn(g.sxt, g.gxt));
    g.cmpy = (float)(0.5 * (double)__fadd_rn(g.syt, g.gyt));
    double offd = floor(__ddiv_rn(__dsub_rn(__dmul_rn(2.0, __dsqrt_rn((double)h2)), a.oh), a.dh));
    int off = (offd > -2147483648.0 && offd < 2147483647.0) ? (int)offd : -1;
    bool valid = off >= 0 && off < a.nh;
    float cx = __fsub_rn(a.IXc, g.cmpx), cy = __fsub_rn(a.IYc, g.cmpy);
    float dIC = __fsqrt_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)));
    bool live = valid && ((double)dIC < a.cull_radius);
    g.cls = live ? (a.stack ? 0 : off) : -1;
    g.src = (int32_t)it;
    if (!ok) {
        g.cls = -1;
        kp_fail(a.status, KPSTM_ERR_GEOMETRY);
    }
    a.geom[it] = g;
    a.cls[it] = g.cls;
}

/* Stable partition of the block by class (single CTA): class_start[c] is
   the first slot of class c, order[slot] the trace, in block order within a
   class - so the gather visits a class's traces in the reference's order. */
__global__ void __launch_bounds__(1024) k_bucket(const int32_t *cls, int64_t ntr, int ncls,
                                                 int32_t *class_start, int32_t *order, int32_t *nlive)
{
    extern __shared__ int32_t hist[]; /* [ncls + 1] */
    for (int c = threadIdx.x; c <= ncls; c += blockDim.x) hist[c] = 0;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < ntr; i += blockDim.x) {
        int c = cls[i];
        if (c >= 0) atomicAdd(&hist[c], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int c = 0; c < ncls; ++c) {
            int n = hist[c];
            hist[c] = run;
            class_start[c] = run;
            run += n;
        }
        class_start[ncls] = run;
        *nlive = run;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    for (int64_t base = 0; base < ntr; base += 32) {
        int64_t i = base + lane;
        int c = i < ntr ? cls[i] : -1;
        unsigned peers = __match_any_sync(0xffffffffu, c);
        int rank = __popc(peers & ((1u << lane) - 1u));
        int pos = 0;
        if (c >= 0) pos = hist[c] + rank;
        __syncwarp();
        if (c >= 0) {
            order[pos] = (int32_t)i;
            if (rank == 0) hist[c] += __popc(peers);
        }
        __syncwarp();
    }
}

/* Classes by decreasing trace count (ties: lower class first), for the
   persistent imaging launch: cls_order[r] is the class of rank r.  One CTA,
   ncls <= KPSTM_MAX_CLASSES. */
__global__ void __launch_bounds__(1024) k_class_order(const int32_t *class_start, int ncls, int32_t *cls_order)
{
    __shared__ int32_t sz[KPSTM_MAX_CLASSES];
    for (int c = threadIdx.x; c < ncls; c += blockDim.x) sz[c] = class_start[c + 1] - class_start[c];
    __syncthreads();
    for (int c = threadIdx.x; c < ncls; c += blockDim.x) {
        const int mine = sz[c];
        int r = 0;
        for (int j = 0; j < ncls; ++j) {
            const int o = sz[j];
            r += (o > mine) || (o == mine && j < c);
        }
        cls_order[r] = c;
    }
}

/* Per-trace tap tables of the full and precision modes, one thread per
   trace (reference mode: k_prep_ref below).
   Full mode: the double running integral P of the unscaled trace (P = 0
   before the trace, f = 0 after it), accumulated in double-word floats and
   stored over [-tm, ns+tm-4] as pairs {P[i], P[i+1]-P[i]} for linear
   interpolation (ns + 2tm - 3 entries per row).
   Precision mode: the reference-mode taps from the same integrals in
   double-word floats, rounded once.  No FP64. */
__global__ void k_prep(KpPrepArgs a)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= *a.nlive) return;
    const int32_t src = a.order[i];
    kpstm_geom g = a.geom_raw[src];
    a.geom[i] = g;
    const int ns = a.ns, tm = a.tm;
    /* the row starts with the trace's geometry (staged with the taps) */
    *reinterpret_cast<float4 *>(a.table + i * a.row) = make_float4(g.sxt, g.syt, g.gxt, g.gyt);
    *reinterpret_cast<float4 *>(a.table + i * a.row + 4) =
        make_float4(g.cmpx, g.cmpy, __int_as_float(g.cls), __int_as_float(g.src));
    float *row = a.table + i * a.row + KP_ROW_HDR;
    const float *f32 = a.samples ? a.samples + (int64_t)src * ns : nullptr;
    const uint16_t *f16 = a.samples_bf16 ? a.samples_bf16 + (int64_t)src * ns : nullptr;
    const float sc = f16 ? a.scale[src] : 1.0f;
#define KP_SAMPLE(t) (f32 ? f32[(t)] : __fmul_rn(__uint_as_float(((uint32_t)f16[(t)]) << 16), sc))
    if (a.full) {
        float2 *q = reinterpret_cast<float2 *>(row); /* q[i + tm] for P index i */
        float4 *q4 = reinterpret_cast<float4 *>(row);
        for (int j = tm; j > 1; --j) {
            if (a.hilo) q4[tm - j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            else q[tm - j] = make_float2(0.0f, 0.0f);
        }
        /* P1 (running sum of the samples) and P2 (running sum of P1) as
           double-word floats: no FP64 on the device, ~48 bits */
        kp_dw p1 = {0.0f, 0.0f}, p2 = {0.0f, 0.0f};
        /* last P index stored: the imaging kernel reads entry floor(x) + tm with
           x = RN(x0 + Lf) <= ns - 2 + lmax (x0 < ns - 2, Lf <= lmax; the sum can
           round up onto the bound) and lmax <= tm - 1, i.e. entries
           0 .. ns + 2tm - 3 */
        const int iend = ns + tm - 3;
        for (int t = 0; t <= iend + 1; ++t) {
            if (t < ns) p1 = kp_dw_add1(p1, KP_SAMPLE(t));
            const kp_dw prev = p2;
            p2 = kp_dw_add(p2, p1); /* P[t] */
            if (a.hilo) {
                /* {hi, lo} of P[t-1]: the normalised pair is its float rounding
                   and the remainder */
                q4[t - 1 + tm] = make_float4(prev.h, prev.l, p1.h, 0.0f);
            } else {
                q[t - 1 + tm] = make_float2(prev.h, p1.h); /* entry of P index t-1 */
            }
        }
        return;
    }
    if (a.exact) {
        /* the same integrals and taps in double-word floats (no FP64 on the
           device), rounded once when the tap is stored (no float running
           sums); c4rw[t] = 1/(4 t2[t]) for t < ns, 1/(dt t)^2 for the two
           tail steps, as double-word floats */
        const float fl = KP_SAMPLE(ns - 1);
        kp_dw q1 = {KP_SAMPLE(0), 0.0f}, q2 = q1;
        kp_dw s0 = {0.0f, 0.0f}, s1 = s0, s2 = s0, s3 = s0, s4 = q2, n1 = s0, n2 = s0;
        for (int t = 1; t < ns + 2; ++t) {
            const float2 r = a.c4rw[t];
            q1 = kp_dw_add(q1, kp_dw_mul1(kp_dw{r.x, r.y}, t < ns ? KP_SAMPLE(t) : fl));
            q2 = kp_dw_add(q2, q1);
            if (t == 1) n1 = q2;
            if (t == 2) n2 = q2;
            s0 = s1; s1 = s2; s2 = s3; s3 = s4; s4 = q2;
            if (t >= 2) {
                const int T = t - 2;
                const kp_dw pm = T >= 2 ? s0 : (T == 1 ? n1 : n2);
                /* -2 s2 + pm + s4: the doubling is exact */
                const kp_dw d = kp_dw_add(kp_dw_add(kp_dw{-2.0f * s2.h, -2.0f * s2.l}, pm), s4);
                if (T < ns) row[T] = __fadd_rn(d.h, d.l);
            }
        }
        row[ns] = 0.0f;
    }
#undef KP_SAMPLE
}

/* Reference-mode tap tables: the running integrals of Kirchhoff.c:1312-1328
   in the reference's order and precision - the first integral P1 adds
   f[t]/(4 t2[t]) in double and stores float, the tail adds
   f[ns-1]/(dt dt t t) in float (the fast-math a/(b c) form of :1320), the
   second integral P2 is a float running sum, the front is mirrored - and
   the taps D[T] = -2 P2[T] + P2[T-2] + P2[T+2] summed in double
   (:1391-1392), plus a zero sentinel D[ns].  FP64 because the reference
   defines these steps in double and parity needs them.
   GB300 runs one FP64 warp instruction per ~64 cycles per sub-partition
   whatever the active lanes, so a CTA takes 32 traces and the work is
   split by what is sequential: per chunk of KP_PR_CH steps, all warps form
   the 32 x CH double quotients (coalesced sample reads), warp 0 runs the 32
   traces' running sums in lockstep (lane j = trace j: the only sequential
   part, the same operations in the same order as a thread per trace), and
   all warps form the taps from P2 in shared memory and store them
   coalesced.  -2 P2[T] + P2[T-2] is one fma: the product is exact. */
#define KP_PR_TR 32     /* traces per CTA */
#define KP_PR_WARPS 8
#define KP_PR_CH 64     /* steps per chunk */
__global__ void __launch_bounds__(32 * KP_PR_WARPS) k_prep_ref(KpPrepArgs a)
{
    __shared__ double s_q[KP_PR_TR][KP_PR_CH + 1]; /* f[t] / (4 t2[t]), t = c0 + k */
    __shared__ double s_p[KP_PR_TR][KP_PR_CH + 5]; /* P2[c0 - 4 + k] (widened, exact) */
    __shared__ int32_t s_src[KP_PR_TR];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int ns = a.ns;
    const int64_t base = blockIdx.x * (int64_t)KP_PR_TR;
    const int64_t nl = *a.nlive;
    if (base >= nl) return; /* block-uniform */
    const int nh = (int)min((int64_t)KP_PR_TR, nl - base);
    if (tid < KP_PR_TR) {
        s_src[tid] = tid < nh ? a.order[base + tid] : 0;
        if (tid < nh) {
            const int64_t i = base + tid;
            const kpstm_geom g = a.geom_raw[s_src[tid]];
            a.geom[i] = g;
            /* the row starts with the trace's geometry (staged with the taps) */
            *reinterpret_cast<float4 *>(a.table + i * a.row) = make_float4(g.sxt, g.syt, g.gxt, g.gyt);
            *reinterpret_cast<float4 *>(a.table + i * a.row + 4) =
                make_float4(g.cmpx, g.cmpy, __int_as_float(g.cls), __int_as_float(g.src));
            a.table[i * a.row + KP_ROW_HDR + ns] = 0.0f; /* sentinel read for samples whose T >= ns */
        }
    }
    __syncthreads();
    auto sample = [&](int j, int t) -> float {
        const int64_t o = (int64_t)s_src[j] * ns + t;
        return a.samples ? a.samples[o] : __fmul_rn(__uint_as_float(((uint32_t)a.samples_bf16[o]) << 16), a.scale[s_src[j]]);
    };
    float p1 = 0.0f, p2 = 0.0f; /* warp 0, lane j: trace j's running sums */
    const float flast = (w == 0 && lane < nh) ? sample(lane, ns - 1) : 0.0f;
    const float dt2 = __fmul_rn(a.dt, a.dt);
    for (int c0 = 0; c0 < ns + 2; c0 += KP_PR_CH) {
        const int cend = min(c0 + KP_PR_CH, ns + 2);
        for (int idx = tid; idx < KP_PR_TR * KP_PR_CH; idx += 32 * KP_PR_WARPS) {
            const int j = idx / KP_PR_CH, k = idx % KP_PR_CH, t = c0 + k;
            if (j < nh && t >= 1 && t < ns) s_q[j][k] = kp_ddiv_rn((double)sample(j, t), a.c4[t], a.c4r[t]);
        }
        __syncthreads();
        if (w == 0 && lane < nh) {
            double *sp = s_p[lane];
            const double *sq = s_q[lane];
            int t = c0;
            if (t == 0) {
                p1 = sample(lane, 0);
                p2 = p1;
                sp[4] = (double)p2;
                t = 1;
            }
            const int tq = min(cend, ns);
            for (; t < tq; ++t) {
                p1 = __double2float_rn(__dadd_rn((double)p1, sq[t - c0]));
                p2 = __fadd_rn(p2, p1);
                sp[4 + t - c0] = (double)p2;
            }
            for (; t < cend; ++t) { /* the two tail steps t = ns, ns + 1 */
                const float tf = __int2float_rn(t);
                p1 = __fadd_rn(p1, __fdiv_rn(flast, __fmul_rn(__fmul_rn(dt2, tf), tf)));
                p2 = __fadd_rn(p2, p1);
                sp[4 + t - c0] = (double)p2;
            }
        }
        __syncthreads();
        /* taps T whose last term P2[T + 2] is in this chunk: P2[x] sits at
           s_p[j][4 + x - c0]; T = 0, 1 mirror the front (P2[2], P2[1]) */
        for (int idx = tid; idx < KP_PR_TR * KP_PR_CH; idx += 32 * KP_PR_WARPS) {
            const int j = idx / KP_PR_CH, T = c0 - 2 + idx % KP_PR_CH;
            if (j >= nh || T < 0 || T >= ns || T >= cend - 2) continue;
            const double *sp = s_p[j];
            const double pm = T >= 2 ? sp[2 + T - c0] : sp[6 - T - c0];
            const double d = __dadd_rn(__fma_rn(-2.0, sp[4 + T - c0], pm), sp[6 + T - c0]);
            a.table[(base + j) * a.row + KP_ROW_HDR + T] = __double2float_rn(d);
        }
        __syncthreads();
        if (cend == c0 + KP_PR_CH && tid < KP_PR_TR * 4) /* halo: P2[c0 + CH - 4 ..] */
            s_p[tid >> 2][tid & 3] = s_p[tid >> 2][KP_PR_CH + (tid & 3)];
        __syncthreads();
    }
}

/* ------------------------------------------------------------------------ */
/* Full-mode pair arithmetic shared by the migration (k_image) and its
   adjoint (k_demig), so that both see bit-identical pair sets, traveltimes,
   triangle widths and weights.  Sample units: tv = {(t/2)^2, 1/(v dt)^2},
   dIS2/dIR2 the squared image-source/receiver distances, a* the distance
   components times the line spacings. */
struct KpPair {
    float Tf;  /* traveltime in samples */
    float Lf;  /* triangle half-width in samples, 1..lmax */
    float w;   /* (1/ts' + 1/tr')^2 / Lf^2; the factor t/(8 dt) is applied outside */
};

__device__ __forceinline__ float kp_pair_time(float dIS2, float dIR2, float2 tv, float &rs, float &rr)
{
    const float as = __fmaf_rn(dIS2, tv.y, tv.x), ar = __fmaf_rn(dIR2, tv.y, tv.x);
    rs = kp_rsqrt_approx(as);
    rr = kp_rsqrt_approx(ar);
    return __fmaf_rn(as, rs, __fmul_rn(ar, rr));
}

__device__ __forceinline__ void kp_pair_width(float rs, float rr, float axs, float axr, float ays, float ayr,
                                              float rv2, float lmaxf, float &Lf, float &w)
{
    const float gxx = __fmaf_rn(axs, rs, __fmul_rn(axr, rr)), gyy = __fmaf_rn(ays, rs, __fmul_rn(ayr, rr));
    Lf = fminf(__fmaf_rn(__fadd_rn(fabsf(gxx), fabsf(gyy)), rv2, 1.0f), lmaxf);
    const float ui = __fmul_rn(__fadd_rn(rs, rr), kp_rcp_approx(Lf));
    w = __fmul_rn(ui, ui);
}

/* ------------------------------------------------------------------------ */
/* Imaging.  Grid (ntile, ncls, nwin); block 256 = 8 warps; warp w owns image
   column blockIdx.x*8 + w, lane l owns samples tw0 + l + 32k, k < K. */

__device__ __forceinline__ bool kp_tile_test(const float4 &box, float cx, float cy, float r2)
{
    float dx = fmaxf(fmaxf(box.x - cx, cx - box.y), 0.0f);
    float dy = fmaxf(fmaxf(box.z - cy, cy - box.w), 0.0f);
    return dx * dx + dy * dy < r2;
}

/* distance from (x, y) to the tile's box of column positions: at most the
   distance to any of its columns */
__device__ __forceinline__ float kp_box_dist(const float4 &box, float x, float y)
{
    const float dx = fmaxf(fmaxf(box.x - x, x - box.y), 0.0f);
    const float dy = fmaxf(fmaxf(box.z - y, y - box.w), 0.0f);
    return sqrtf(dx * dx + dy * dy);
}

/* Shared-memory layout of k_image: s_v (8 warps x W float2), s_t (W
   float2), S one-trace TMA stages (kp_stages), the compaction list, then 50
   words (8 column positions, 8 critical distances, 8 warp counts, 8 stage
   counters, 8 last-issued sequence numbers, 2 flags) ending right before the
   S mbarriers.  Returns the total bytes;
   *bar_offset receives the barriers' offset (8-byte aligned). */
#define KP_IMG_INTS 50
/* TMA stages of the imaging kernel: 2 x the batch of the mode, or 2 for the
   three-CTAs-per-SM variant (MINB 3), whose shared memory must fit 3 times */
__host__ __device__ constexpr int kp_stages(bool full, int minb)
{
    return minb >= 3 ? 2 : 2 * (full ? KP_TB_FULL : KP_TB_REF);
}
__host__ __device__ inline size_t kp_image_smem(int K, int S, int64_t row, uint32_t *bar_offset)
{
    const size_t W = 32 * (size_t)K;
    size_t b = sizeof(float2) * KPSTM_COLS_PER_CTA * W + sizeof(float2) * W + sizeof(float) * S * (size_t)row +
               sizeof(int32_t) * KP_LCH;
    b = (b + sizeof(int32_t) * KP_IMG_INTS + 7) & ~size_t(7); /* end of the ints, 8-byte aligned */
    if (bar_offset) *bar_offset = (uint32_t)b;
    return b + S * sizeof(uint64_t);
}

/* One work item of the imaging kernel: image tile `tile` (8 columns, one per
   warp), offset class `cls`, time window `win`.  nb counts the TMA batches
   this CTA has issued (it selects the buffer and the mbarrier phase and
   carries over between items).  Returns false if a bounded wait gave up. */
template <int K, bool FULL, bool KAHAN, bool HILO, int MINB>
__device__ __forceinline__ bool k_image_item(const KpImageArgs &a, uint8_t *smem, int tile, int cls, int win,
                                             uint32_t &nb)
{
    constexpr int W = 32 * K;
    constexpr int S = kp_stages(FULL, MINB); /* one-trace pipeline stages */
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int tw0 = win * W;
    const int col = a.tilecols[tile * KPSTM_COLS_PER_CTA + w]; /* -1: no column */
    const bool colok = col >= 0;
    const int ns = a.ns;
    const int64_t row = a.row;

    /* shared layout (lane l owns samples tw0 + l + 32k; both modes take two
       samples per packed-fp32 instruction, k = 2q and 2q + 1, i.e. t and t + 32):
       reference:
         s_v float4 [8][K/2][32] {v2(t), v2(t+32), -RN(1/v2(t)), -RN(1/v2(t+32))}
         s_t float2 [K/2][32]    {t2(t), t2(t+32)}            (t2: Kirchhoff.c:1247)
       full:
         s_v float4 [8][K/2][32] {(t/2)^2, (t'/2)^2, 1/(v(t) dt)^2, 1/(v(t') dt)^2},
                                 t' = t + 32 (sample units: the square roots of
                                 the DSR terms come out in samples) */
    uint8_t *p = smem;
    float2 *s_v = reinterpret_cast<float2 *>(p);
    p += sizeof(float2) * KPSTM_COLS_PER_CTA * W;
    float *s_t = reinterpret_cast<float *>(p);
    p += sizeof(float2) * W;
    float *s_buf = reinterpret_cast<float *>(p);                 /* [S][row] */
    int32_t *s_list = reinterpret_cast<int32_t *>(p + sizeof(float) * S * row); /* [KP_LCH] */
    /* the ints end right before the barriers (kp_image_smem computes the same layout) */
    uint64_t *s_bar = reinterpret_cast<uint64_t *>(smem + a.bar_offset);     /* [S] stage full */
    int32_t *s_flag = reinterpret_cast<int32_t *>(smem + a.bar_offset) - 2;  /* [2]: abort, work item */
    int32_t *s_last = s_flag - 8;                                            /* [S] last q issued per stage */
    int32_t *s_cnt = s_last - 8;                                             /* [S] warps done with a stage */
    int32_t *s_wsum = s_cnt - 8;                                             /* [8] */
    volatile int32_t *vflag = s_flag;

    float *s_crit = reinterpret_cast<float *>(s_wsum) - 8;                   /* [8] */
    float2 *s_col = reinterpret_cast<float2 *>(s_crit - 16);                 /* [8] column x, y (NaN: none) */

    __syncthreads(); /* the previous item of this CTA is done with shared memory */
    const int vrow = colok ? a.colrow[col] : -1;
    const float rdt2 = a.rdt * a.rdt;
    /* the window's critical squared distance crit: every pair of this
       column and window lies past the trace end for a trace whose source
       and receiver distances dS, dR satisfy (dS + dR)^2 >= crit, because
       sqrt(x + dS^2 y) + sqrt(x + dR^2 y) >= sqrt(4 x + (dS + dR)^2 y)
       (Minkowski).  Full mode, in samples: x = tx, y = ty, crit = max of
       (T^2 - 4 tx) / ty with T = (ns - 1)(1 + 2^-12) (Tf >= ns - 1 skips);
       reference mode, in seconds: x = t2, y = 1 / v2, crit = max of
       (T^2 - 4 t2) v2 with T = ns dt (1 + 2^-12) (RN(S/dt) >= ns skips).
       The margin covers every rounding and the SFU square roots.  +inf
       (no culling) where the column has no velocity row, so that the
       velocity-range error is still raised; fmaxf drops NaN (a NaN y makes
       every pair of its sample dead) */
    float crit = colok ? (vrow < 0 ? INFINITY : -INFINITY) : -INFINITY;
    if (FULL) {
        const float T = (a.nsf - 1.0f) * (1.0f + 1.0f / 4096.0f);
        const float T2 = T * T;
        for (int i = lane; i < (K / 2) * 32; i += 32) {
            const int q = i >> 5, l = i & 31;
            const int ta = tw0 + l + 64 * q, tb = ta + 32;
            float2 va = make_float2(1.0f, 1.0f), vb = make_float2(1.0f, 1.0f);
            if (vrow >= 0 && ta < ns) va = a.vrows[(int64_t)vrow * ns + ta];
            if (vrow >= 0 && tb < ns) vb = a.vrows[(int64_t)vrow * ns + tb];
            const float4 e =
                make_float4(ta < ns ? a.t2c[ta].x : 1.0f, tb < ns ? a.t2c[tb].x : 1.0f, va.y * rdt2, vb.y * rdt2);
            reinterpret_cast<float4 *>(s_v)[(w * (K / 2) + q) * 32 + l] = e;
            if (vrow >= 0) {
                if (ta < ns) crit = fmaxf(crit, __fdiv_rn(__fsub_rn(T2, 4.0f * e.x), e.z));
                if (tb < ns) crit = fmaxf(crit, __fdiv_rn(__fsub_rn(T2, 4.0f * e.y), e.w));
            }
        }
    } else {
        const float T = a.nsf * a.dt * (1.0f + 1.0f / 4096.0f);
        const float T2 = T * T;
        for (int i = lane; i < (K / 2) * 32; i += 32) {
            const int q = i >> 5, l = i & 31;
            const int ta = tw0 + l + 64 * q, tb = ta + 32;
            float2 va = make_float2(1.0f, 1.0f), vb = make_float2(1.0f, 1.0f);
            if (vrow >= 0 && ta < ns) va = a.vrows[(int64_t)vrow * ns + ta];
            if (vrow >= 0 && tb < ns) vb = a.vrows[(int64_t)vrow * ns + tb];
            reinterpret_cast<float4 *>(s_v)[(w * (K / 2) + q) * 32 + l] = make_float4(va.x, vb.x, -va.y, -vb.y);
            if (vrow >= 0) {
                if (ta < ns) crit = fmaxf(crit, __fmul_rn(__fsub_rn(T2, 4.0f * a.t2[ta]), va.x));
                if (tb < ns) crit = fmaxf(crit, __fmul_rn(__fsub_rn(T2, 4.0f * a.t2[tb]), vb.x));
            }
        }
        for (int i = tid; i < (K / 2) * 32; i += KP_THREADS) {
            const int ta = tw0 + (i & 31) + 64 * (i >> 5), tb = ta + 32;
            reinterpret_cast<float2 *>(s_t)[i] = make_float2(ta < ns ? a.t2[ta] : 0.0f, tb < ns ? a.t2[tb] : 0.0f);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) crit = fmaxf(crit, __shfl_xor_sync(0xffffffffu, crit, o));
    if (lane == 0) s_crit[w] = crit;
    const float2 cxy = colok ? a.colxy[col] : make_float2(0.f, 0.f);
    const float IX = cxy.x, IY = cxy.y;
    if (lane == 0) s_col[w] = colok ? cxy : make_float2(NAN, NAN);
    const float4 box = a.tilebox[tile];
    const int64_t obase = ((int64_t)cls * a.ncol + (colok ? col : 0)) * ns + tw0 + lane;

    /* accumulators as sample pairs: acc[q] = samples 2q (x) and 2q + 1 (y), i.e.
       tw0 + lane + 64q and + 32; comp[q] the negated Kahan compensations (so
       that no update needs a negation); cnt2[q] the pair's fold increments as
       two 16-bit halves (x low, y high), added to the global counts before
       they can overflow */
    float2 acc[K / 2], comp[KAHAN ? K / 2 : 1];
    uint32_t cnt2[K / 2];
#pragma unroll
    for (int q = 0; q < K / 2; ++q) {
        const int ta = tw0 + lane + 64 * q, tb = ta + 32;
        acc[q].x = (colok && ta < ns) ? a.km[obase + 64 * q] : 0.0f;
        acc[q].y = (colok && tb < ns) ? a.km[obase + 64 * q + 32] : 0.0f;
        if (KAHAN) {
            comp[q].x = (colok && ta < ns) ? a.kc[obase + 64 * q] : 0.0f;
            comp[q].y = (colok && tb < ns) ? a.kc[obase + 64 * q + 32] : 0.0f;
        }
        cnt2[q] = 0u;
    }
    auto flush_counts = [&]() {
        if (!colok) return;
#pragma unroll
        for (int q = 0; q < K / 2; ++q) {
            const int ta = tw0 + lane + 64 * q, tb = ta + 32;
            if (ta < ns) a.cnt[obase + 64 * q] += (int32_t)(cnt2[q] & 0xffffu);
            if (tb < ns) a.cnt[obase + 64 * q + 32] += (int32_t)(cnt2[q] >> 16);
            cnt2[q] = 0u;
        }
    };
    __syncthreads();

    const int cb = a.class_start[cls], ce = a.class_start[cls + 1];
    const uint32_t row_bytes = (uint32_t)(row * sizeof(float));
    int my_hits = 0, cull_hits = 0;
    bool abort = false;
    const float tmax = a.nsf - 1.0f;

    for (int c0 = cb; c0 < ce && !abort; c0 += KP_LCH) {
        /* order-preserving compaction of the chunk's traces that can reach
           any column of this tile and whose traveltimes can fall inside the
           trace somewhere in the window */
        int n = 0;
        float crit2 = -INFINITY; /* the tile's critical squared distance */
#pragma unroll
        for (int v = 0; v < 8; ++v) crit2 = fmaxf(crit2, s_crit[v]);
        for (int r = 0; r < KP_LCH / KP_THREADS; ++r) {
            int i = c0 + r * KP_THREADS + tid;
            bool pass = false;
            if (i < ce) {
                const kpstm_geom &g = a.geom[i];
                pass = kp_tile_test(box, g.cmpx, g.cmpy, a.tile_r2);
                if (pass && a.cull) {
                    const float D = kp_box_dist(box, g.sxt, g.syt) + kp_box_dist(box, g.gxt, g.gyt);
                    if (D * D >= crit2) {
                        pass = false;
                        /* the pair count takes every (trace, column) in aperture
                           (Kirchhoff.c:1352-1354): window 0 counts the culled
                           trace's columns with the warps' own test */
                        if (win == 0)
#pragma unroll
                            for (int v = 0; v < 8; ++v) {
                                const float2 c = s_col[v];
                                const float ex = __fsub_rn(c.x, g.cmpx), ey = __fsub_rn(c.y, g.cmpy);
                                cull_hits += __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)) < a.aperture_x2;
                            }
                    }
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, pass);
            if (lane == 0) s_wsum[w] = __popc(m);
            __syncthreads();
            int before = 0, total = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                int v = s_wsum[q];
                before += q < w ? v : 0;
                total += v;
            }
            if (pass) s_list[n + before + __popc(m & ((1u << lane) - 1u))] = i;
            n += total;
            __syncthreads();
        }
        /* per-warp pipeline of S one-trace stages: the prologue stages the
           first S traces; the last warp to finish with a stage refills it with
           the trace S positions later, so warps drift apart by up to S - 1
           traces instead of meeting at a barrier after every batch */
        auto issue = [&](int j, uint32_t q) {
            const int slot = (int)(q % S);
            uint64_t *bar = &s_bar[slot];
            kp_fence_proxy_async();
            kp_mbar_expect_tx(bar, row_bytes);
            kp_bulk_g2s(s_buf + slot * row, a.table + (int64_t)s_list[j] * row, row_bytes, bar);
            s_last[slot] = (int32_t)q;
        };
        if (tid == 0)
            for (int j = 0; j < min(n, S); ++j) issue(j, nb + (uint32_t)j);
        for (int j = 0; j < n; ++j) {
            const uint32_t q = nb + (uint32_t)j;
            const int slot = (int)(q % S);
            if (vflag[0]) break;
            if (!kp_mbar_wait(&s_bar[slot], (q / S) & 1, a.wait_polls)) {
                vflag[0] = 1;
                kp_fail(a.status, KPSTM_ERR_TIMEOUT);
                break;
            }
            if (colok) {
                do {
                    const float *hdr = s_buf + slot * row; /* geometry, then taps */
                    const float4 g0 = *reinterpret_cast<const float4 *>(hdr);
                    const float2 g1 = *reinterpret_cast<const float2 *>(hdr + 4);
                    kpstm_geom g;
                    g.sxt = g0.x;
                    g.syt = g0.y;
                    g.gxt = g0.z;
                    g.gyt = g0.w;
                    g.cmpx = g1.x;
                    g.cmpy = g1.y;
                    float cx = __fsub_rn(IX, g.cmpx), cy = __fsub_rn(IY, g.cmpy);
                    /* RN(sqrt(dIC2)) < aperture_f, decided on the square (Kirchhoff.c:1352-1354),
                       warp-uniform */
                    const float dIC2 = __fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy));
                    if (!(dIC2 < a.aperture_x2)) break;
                    if (vrow < 0) {
                        kp_fail(a.status, KPSTM_ERR_VELOCITY_RANGE);
                        break;
                    }
                    /* every 32,768 hits the 16-bit counts go to the global ones
                       (warp-uniform: the aperture test is) */
                    if ((++my_hits & 0x7fff) == 0) flush_counts();
                    float sx = __fsub_rn(IX, g.sxt), sy = __fsub_rn(IY, g.syt);
                    float gx = __fsub_rn(IX, g.gxt), gy = __fsub_rn(IY, g.gyt);
                    const float dIS2 = __fadd_rn(__fmul_rn(sx, sx), __fmul_rn(sy, sy));
                    const float dIR2 = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
                    const float *tab = hdr + KP_ROW_HDR;
                    if (!FULL) {
                        const float4 *sv4 = reinterpret_cast<const float4 *>(s_v) + w * (K / 2) * 32 + lane;
                        const float2 *st2 = reinterpret_cast<const float2 *>(s_t) + lane;
                        const float2 nS = kp_bc2(-dIS2), nR = kp_bc2(-dIR2);
                        const float2 dt2 = kp_bc2(a.dt), nrdt2 = kp_bc2(-a.rdt);
                        const float nnsf = -a.nsf;
#pragma unroll
                        for (int q = 0; q < K / 2; ++q) {
                            const float4 vv = sv4[32 * q];
                            const float2 t2 = st2[32 * q];
                            const float2 v2 = make_float2(vv.x, vv.y), nr = make_float2(vv.z, vv.w);
                            /* RN(d/v^2): q = (-d)(-1/v^2); e' = q v^2 - d; q + e'(-1/v^2) */
                            float2 q1 = __fmul2_rn(nS, nr);
                            q1 = __ffma2_rn(__ffma2_rn(q1, v2, nS), nr, q1);
                            float2 q2 = __fmul2_rn(nR, nr);
                            q2 = __ffma2_rn(__ffma2_rn(q2, v2, nR), nr, q2);
                            const float2 S = kp_dsqrt_sum2(__fadd2_rn(t2, q1), __fadd2_rn(t2, q2));
                            /* -RN(S/dt) (Kirchhoff.c:1384): nq = S(-1/dt); e = S + nq dt; nq + e(-1/dt) */
                            float2 nq = __fmul2_rn(S, nrdt2);
                            nq = __ffma2_rn(__ffma2_rn(nq, dt2, S), nrdt2, nq);
                            /* floor(RN(S/dt)): -(q + 1.5*2^23) toward zero; its bits minus
                               0xCB400000 (sign + magic) are T; T >= ns reads the zero D[ns] */
                            const float2 fb = __fadd2_rz(nq, kp_bc2(-KP_MAGIC));
                            const bool va = nq.x > nnsf, vb = nq.y > nnsf; /* T < ns, :1387 */
                            const int ia = va ? (int)((uint32_t)__float_as_int(fb.x) - 0xCB400000u) : ns;
                            const int ib = vb ? (int)((uint32_t)__float_as_int(fb.y) - 0xCB400000u) : ns;
                            const float2 d = make_float2(tab[ia], tab[ib]);
                            if (KAHAN) { /* comp = -c: y = d - c, -c' = y - (s - acc) */
                                const float2 y = __fadd2_rn(d, comp[q]);
                                const float2 s = __fadd2_rn(acc[q], y);
                                comp[q] = kp_sub2(y, kp_sub2(s, acc[q]));
                                acc[q] = s;
                            } else {
                                acc[q] = __fadd2_rn(acc[q], d); /* + 0 where T >= ns: exact no-op */
                            }
                            cnt2[q] += (uint32_t)va | ((uint32_t)vb << 16);
                        }
                    } else {
                        /* full physics in sample units: a = (t/2)^2 + |I-S|^2/(v dt)^2,
                           Tf = sqrt(a_s) + sqrt(a_r); a triangle of real half-width Lf
                           (1 + the operator's lateral slope in samples per trace
                           spacing, <= lmax) read from the double running integral at
                           three fractional positions; weight t0 (1/ts + 1/tr)^2 / 8
                           divided by Lf^2, of which (1/ts' + 1/tr')^2 / Lf^2 is applied
                           here and the per-sample factor t0 / (8 dt^2) when the
                           accumulators are read (ts' = ts/dt) */
                        const float axs = __fmul_rn(sx, a.aax), axr = __fmul_rn(gx, a.aax);
                        const float ays = __fmul_rn(sy, a.aay), ayr = __fmul_rn(gy, a.aay);
                        /* the entry of P index floor(y) - 1 (x = y - 1 in the P index):
                           q2[i] holds {P(i), P(i+1) - P(i)} for P index i >= -tm;
                           the hi/lo table {hi(P(i)), lo(P(i)), P(i+1)-P(i), 0} keeps P to
                           ~1e-14 for noisy traces (least-squares operators) */
                        const float2 *q2 = reinterpret_cast<const float2 *>(tab) + (a.tm - 1);
                        const float4 *q4 = reinterpret_cast<const float4 *>(tab) + (a.tm - 1);
                        const float4 *sv4 = reinterpret_cast<const float4 *>(s_v) + w * (K / 2) * 32 + lane;
                        /* the triangle-filtered tap of one sample from the floors' bits
                           b* and the fractions f* of y = Tf, Tf + Lf, Tf - Lf; second
                           difference without cancellation: table differences (exact for
                           neighbouring values) plus the interpolation terms; equals
                           sum_k f[k] max(0, Lf - |Tf - k|) */
                        auto tri_of = [&](int b0, int ba, int bb, float m2f0, float fa, float fb) -> float {
                            /* m2f0 = -2 f0 */
                            if (HILO) {
                                const float4 Q0 = q4[b0 - KP_MAGIC_BITS], Qa = q4[ba - KP_MAGIC_BITS];
                                const float4 Qb = q4[bb - KP_MAGIC_BITS];
                                const float big = ((Qa.x - Q0.x) + (Qb.x - Q0.x)) + ((Qa.y - Q0.y) + (Qb.y - Q0.y));
                                return fmaf(m2f0, Q0.z, fmaf(fa, Qa.z, fmaf(fb, Qb.z, big)));
                            } else {
                                const float2 Q0 = q2[b0 - KP_MAGIC_BITS], Qa = q2[ba - KP_MAGIC_BITS];
                                const float2 Qb = q2[bb - KP_MAGIC_BITS];
                                /* each interpolation term joins the table difference of its
                                   own tap (values of like size), the centre term last */
                                const float ua = fmaf(fa, Qa.y, Qa.x - Q0.x), ub = fmaf(fb, Qb.y, Qb.x - Q0.x);
                                return fmaf(m2f0, Q0.y, ua + ub);
                            }
                        };
#pragma unroll
                        for (int q = 0; q < K / 2; ++q) {
                            /* samples t = tw0 + lane + 64q and t + 32 as one pair: the
                               packed operations round each half exactly as the scalar
                               kp_pair_time / kp_pair_width do, so that the demigration,
                               which uses those, sees identical pairs */
                            const float4 vv = sv4[32 * q];
                            const float2 tx = make_float2(vv.x, vv.y), ty = make_float2(vv.z, vv.w);
                            const float2 as2 = __ffma2_rn(kp_bc2(dIS2), ty, tx), ar2 = __ffma2_rn(kp_bc2(dIR2), ty, tx);
                            const float2 rs2 = make_float2(kp_rsqrt_approx(as2.x), kp_rsqrt_approx(as2.y));
                            const float2 rr2 = make_float2(kp_rsqrt_approx(ar2.x), kp_rsqrt_approx(ar2.y));
                            const float2 Tf2 = __ffma2_rn(as2, rs2, __fmul2_rn(ar2, rr2));
                            const bool va = Tf2.x < tmax, vb = Tf2.y < tmax; /* late samples of far traces skip */
                            /* both halves through the packed arithmetic.  MASKED: a half
                               past the trace end reads the table at Tf = 0 (inside it:
                               floor(-Lf) >= -lmax >= 1 - tm) and leaves its sums as they
                               were (plain sums add exactly 0: weight and tap both set to 0,
                               so that no NaN of the table reaches them; Kahan sums keep
                               their old value and compensation) */
                            auto packed = [&](auto masked_t) {
                                constexpr bool MASKED = decltype(masked_t)::value;
                                const float2 Tp = MASKED ? make_float2(va ? Tf2.x : 0.0f, vb ? Tf2.y : 0.0f) : Tf2;
                                const float2 gxx = __ffma2_rn(kp_bc2(axs), rs2, __fmul2_rn(kp_bc2(axr), rr2));
                                const float2 gyy = __ffma2_rn(kp_bc2(ays), rs2, __fmul2_rn(kp_bc2(ayr), rr2));
                                const float2 sg = make_float2(__fadd_rn(fabsf(gxx.x), fabsf(gyy.x)),
                                                              __fadd_rn(fabsf(gxx.y), fabsf(gyy.y)));
                                float2 Lf2 = __ffma2_rn(sg, ty, kp_bc2(1.0f));
                                Lf2 = make_float2(fminf(Lf2.x, a.lmaxf), fminf(Lf2.y, a.lmaxf));
                                const float2 ui = __fmul2_rn(__fadd2_rn(rs2, rr2),
                                                             make_float2(kp_rcp_approx(Lf2.x), kp_rcp_approx(Lf2.y)));
                                float2 w2 = __fmul2_rn(ui, ui);
                                const float2 ya2 = __fadd2_rn(Tp, Lf2), yb2 = kp_sub2(Tp, Lf2);
                                const float2 mg = kp_bc2(KP_MAGIC);
                                const float2 B0 = __fadd2_rz(Tp, mg), Ba = __fadd2_rz(ya2, mg), Bb = __fadd2_rz(yb2, mg);
                                /* fractions y - floor(y), with M - B = -floor(y) exactly */
                                const float2 fa = __fadd2_rn(ya2, kp_sub2(mg, Ba));
                                const float2 fb = __fadd2_rn(yb2, kp_sub2(mg, Bb));
                                /* -2 f0 = 2 floor(Tf) - 2 Tf: 2 B0 - 2M is exact, and so is
                                   -2 (Tf - floor(Tf)) for Tf >= 0 (one rounding of an exact value) */
                                const float2 m2f0 = __ffma2_rn(Tp, kp_bc2(-2.0f),
                                                               __ffma2_rn(B0, kp_bc2(2.0f), kp_bc2(-2.0f * KP_MAGIC)));
                                float2 tri2 = make_float2(
                                    tri_of(__float_as_int(B0.x), __float_as_int(Ba.x), __float_as_int(Bb.x), m2f0.x, fa.x, fb.x),
                                    tri_of(__float_as_int(B0.y), __float_as_int(Ba.y), __float_as_int(Bb.y), m2f0.y, fa.y, fb.y));
                                if (MASKED) {
                                    w2 = make_float2(va ? w2.x : 0.0f, vb ? w2.y : 0.0f);
                                    tri2 = make_float2(va ? tri2.x : 0.0f, vb ? tri2.y : 0.0f);
                                }
                                if (KAHAN) { /* comp = -c: y = w tri - c, -c' = y - (s - acc) */
                                    const float2 y = __ffma2_rn(w2, tri2, comp[q]);
                                    const float2 s2 = __fadd2_rn(acc[q], y);
                                    const float2 c2 = kp_sub2(y, kp_sub2(s2, acc[q]));
                                    if (MASKED) {
                                        comp[q] = make_float2(va ? c2.x : comp[q].x, vb ? c2.y : comp[q].y);
                                        acc[q] = make_float2(va ? s2.x : acc[q].x, vb ? s2.y : acc[q].y);
                                    } else {
                                        comp[q] = c2;
                                        acc[q] = s2;
                                    }
                                } else {
                                    acc[q] = __ffma2_rn(w2, tri2, acc[q]); /* + 0 for a masked half: exact */
                                }
                                cnt2[q] += MASKED ? ((uint32_t)va | ((uint32_t)vb << 16)) : 0x00010001u;
                            };
                            /* warp-uniform choice: a warp with a half past the trace end
                               takes the masked body once, not the packed and a scalar one
                               in turn */
                            if (__all_sync(0xffffffffu, va && vb)) packed(std::false_type{});
                            else if (__any_sync(0xffffffffu, va || vb)) packed(std::true_type{});
                        }
                    }
                } while (0);
            }
            __syncwarp();
            if (lane == 0) {
                __threadfence_block(); /* this warp's reads of the stage come first */
                if (atomicAdd(&s_cnt[slot], 1) == KPSTM_COLS_PER_CTA - 1) {
                    s_cnt[slot] = 0;
                    __threadfence_block();
                    if (j + S < n) issue(j + S, q + S);
                }
            }
        }
        nb += (uint32_t)n;
        __syncthreads();
        if (vflag[0]) abort = true; /* the same for every thread after the barrier */
    }
    if (abort) {
        /* leave no copy landing in shared memory: at most one phase per stage
           is outstanding, the last one issued; these waits keep the full
           bound whatever a.wait_polls is */
        if (tid == 0)
            for (int sl = 0; sl < S; ++sl)
                if (s_last[sl] >= 0) kp_mbar_wait(&s_bar[sl], ((uint32_t)s_last[sl] / S) & 1);
        return false;
    }
    if (colok) {
#pragma unroll
        for (int q = 0; q < K / 2; ++q) {
            const int ta = tw0 + lane + 64 * q, tb = ta + 32;
            if (ta < ns) {
                a.km[obase + 64 * q] = acc[q].x;
                if (KAHAN) a.kc[obase + 64 * q] = comp[q].x;
            }
            if (tb < ns) {
                a.km[obase + 64 * q + 32] = acc[q].y;
                if (KAHAN) a.kc[obase + 64 * q + 32] = comp[q].y;
            }
        }
    }
    flush_counts();
    if (win == 0) {
        const int h = __reduce_add_sync(0xffffffffu, cull_hits) + (lane == 0 ? my_hits : 0);
        if (lane == 0 && h) atomicAdd(a.hits, (unsigned long long)h);
    }
    return true;
}

/* Imaging kernel.  Grid mode (a.queue == null): one work item per CTA,
   blockIdx = (tile, class, window).  Persistent mode: a grid sized to the
   resident CTAs pulls items from a device counter; items are numbered class
   by class in the order a.cls_order gives (largest classes first), so the
   uneven class volumes of a batched launch finish together. */
template <int K, bool FULL, bool KAHAN, bool HILO = false, int MINB = 2>
__global__ void __launch_bounds__(KP_THREADS, MINB) k_image(KpImageArgs a)
{
    extern __shared__ __align__(128) uint8_t smem[];
    /* barriers live at the end of the layout (see k_image_item) */
    constexpr int S = kp_stages(FULL, MINB);
    uint64_t *s_bar = reinterpret_cast<uint64_t *>(smem + a.bar_offset);
    int32_t *s_flag = reinterpret_cast<int32_t *>(smem + a.bar_offset) - 2;
    if (threadIdx.x == 0) {
        for (int sl = 0; sl < S; ++sl) {
            kp_mbar_init(&s_bar[sl], 1);
            s_flag[-16 + sl] = 0;  /* stage counters */
            s_flag[-8 + sl] = -1;  /* nothing issued yet */
        }
        s_flag[0] = 0;
        s_flag[1] = 0;
        kp_fence_mbar_init();
    }
    uint32_t nb = 0;
    if (!a.queue) {
        k_image_item<K, FULL, KAHAN, HILO, MINB>(a, smem, blockIdx.x, blockIdx.y, blockIdx.z, nb);
        return;
    }
    const int per_class = a.ntile * a.nwin;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_flag[1] = atomicAdd(a.queue, 1);
        __syncthreads();
        const int item = s_flag[1];
        if (item >= a.nitems) break;
        const int r = item / per_class, rem = item - r * per_class;
        if (!k_image_item<K, FULL, KAHAN, HILO, MINB>(a, smem, rem / a.nwin, a.cls_order[r], rem % a.nwin, nb)) break;
    }
}

/* ------------------------------------------------------------------------ */
/* Least-squares migration: the adjoint of the full-mode migration
   (demigration, data = L model) and vector kernels for conjugate gradients. */

struct KpDemigArgs {
    const kpstm_geom *geom;        /* live traces, slot order; geom.cls = class */
    const int32_t *nlive;
    const float *model;            /* [ncol][ncls][ns]; null: the all-ones model (bound pass) */
    const float *tscale;           /* [ns] t / (8 dt) */
    const float2 *colxy;
    const int32_t *colrow;
    const float *rvdt;             /* [nrow][ns] RN(RN(1/v^2) / dt^2): k_image's 1/(v dt)^2 */
    const float2 *t2c;             /* [ns] {(t/2)^2, .} */
    const unsigned int *absmax;    /* bits of max |model|, then (at +8 bytes) the nonzero count (k_absmax) */
    int64_t nmodel;                /* model samples */
    const float *dbound;           /* [nlive] max_k (L 1)[trace, k] (bound pass), or null */
    const int32_t *order;          /* [nlive] visiting order of the live slots, or null */
    float *dbound_out;             /* bound pass: receives dbound */
    float *out;                    /* [ntr][ns] in block order */
    unsigned long long *acc;       /* [nlive][ng] zeroed fixed-point rows in L2 (k_demig<false>); null when the rows are in shared memory */
    int *status;
    int nx, ny, ncls, ns, ng;      /* ng: accumulator entries per trace, ns + tm - 1 */
    int bound_g;                   /* bound pass: |gs| < 2^bound_g */
    int limb_r;                    /* SH rows: G = hi 2^limb_r + lo */
    int norm_cols;                 /* SH rows: columns between limb normalisations */
    float tailf;                   /* the pairs' float-position tails, as a fraction of (L 1) */
    const float *wbound;           /* [nlive] largest weight x t/(8 dt) of the trace's pairs (bound pass) */
    float *wbound_out;             /* bound pass: receives wbound */
    float ax0, adx, ay0, ady;      /* column coordinates: IX(xc) ~ ax0 + xc adx */
    double aperture;
    float aperture_f;              /* as KpImageArgs */
    float aperture_x2;             /* as KpImageArgs */
    float tmax, lmaxf, rdt2, aax, aay, dt;
};

#define KP_DM_WARPS 4  /* traces (warps) per demigration CTA */
#define KP_DM_UNROLL 3 /* samples per lane per load batch; the lane stride of dense models (odd) */

/* 1/(v dt)^2 per velocity-row sample, computed as k_image does it. */
__global__ void k_rvdt(const float2 *vrows, int64_t n, float rdt2, float *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __fmul_rn(vrows[i].y, rdt2);
}

/* Largest |x| as float bits (the order of non-negative floats is that of
   their bits; NaN counts as infinity) into out[0], and the count of nonzero
   samples into the 64-bit word at out + 2. */
__global__ void __launch_bounds__(256) k_absmax(const float *x, int64_t n, unsigned int *out)
{
    unsigned int m = 0, nz = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = fabsf(x[i]);
        m = max(m, v == v ? __float_as_uint(v) : 0x7f800000u);
        nz += v != 0.0f;
    }
    m = __reduce_max_sync(0xffffffffu, m);
    nz = __reduce_add_sync(0xffffffffu, nz);
    if ((threadIdx.x & 31) == 0) {
        if (m) atomicMax(out, m);
        if (nz) atomicAdd(reinterpret_cast<unsigned long long *>(out + 2), (unsigned long long)nz);
    }
}

/* Fire-and-forget 64-bit add in global memory (RED: no value comes back, so
   the warp does not wait for L2). */
__device__ __forceinline__ void kp_red_add_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

#define KP_DM_NONE (-(1 << 29)) /* entry index of a lane without a pair */

/* RN(x) as an int64 for |x| <= 2^45 with fp32 and integer operations only
   (__float2ll_rn runs on the FP64 pipe, slow on this GPU): x = qh 2^23 + r
   exactly with qh = RN(x 2^-23) and |r| <= 2^22; both roundings are the
   1.5 * 2^23 shift (a float add whose spacing there is 1, ties to even), and
   qh 2^23 is even, so the sum rounds x exactly as __float2ll_rn does. */
__device__ __forceinline__ long long kp_f2ll_rn45(float x)
{
    const float sh = __fadd_rn(__fmul_rn(x, 0x1p-23f), KP_MAGIC);
    const int qh = __float_as_int(sh) - KP_MAGIC_BITS;
    const float r = __fmaf_rn(__fadd_rn(sh, -KP_MAGIC), -0x1p23f, x); /* x - qh 2^23, exact */
    const int ql = __float_as_int(__fadd_rn(r, KP_MAGIC)) - KP_MAGIC_BITS;
    return (long long)qh * 8388608LL + (long long)ql;
}

/* RN(x) as the limb pair h 2^R + l of the shared-memory rows:
   h = RN(x 2^-R) and l = RN(x - h 2^R), |l| <= 2^(R-1), for |x| < 2^(22+R)
   and R <= 21.  x 2^-R is exact and the 1.5 * 2^23 shift rounds it to an
   integer; x - h 2^R is exact in one fma (it is a multiple of x's spacing
   and at most 2^(R-1) in size); the second shift rounds that to an integer,
   and h 2^R + l = RN(x) because h 2^R is an integer.  Six FMA-pipe/ALU
   operations, no conversion instruction. */
__device__ __forceinline__ void kp_split(float x, float sR, float nR, int &h, int &l)
{
    const float sh = __fmaf_rn(x, sR, KP_MAGIC);
    h = __float_as_int(sh) - KP_MAGIC_BITS;
    const float lf = __fmaf_rn(__fadd_rn(sh, -KP_MAGIC), nR, x);
    l = __float_as_int(__fadd_rn(lf, KP_MAGIC)) - KP_MAGIC_BITS;
}

/* Dynamic shared memory of k_demig: t2[ns] and ts[ns], then (SH) one
   accumulator row per warp: ngp int32 low limbs followed by ngp int32 high
   limbs (ngp = ng rounded up to a multiple of 4). */
__host__ __device__ inline int kp_demig_ngp(int ng) { return (ng + 3) & ~3; }
__host__ __device__ inline size_t kp_demig_smem(int ns, int ng, bool sh)
{
    const size_t head = sizeof(float) * 2 * (size_t)((ns + 3) & ~3);
    return head + (sh ? (size_t)KP_DM_WARPS * 2 * (size_t)kp_demig_ngp(ng) * sizeof(int) : 0);
}

/* Demigration d = L m, the exact transpose of the full-mode migration of
   k_image (HILO).  One warp per live trace visits the image columns within
   the aperture of the trace's midpoint (the same exact float test as
   k_image) and computes every pair with the same routines.  The migration
   reads V(x) = (1 - f) P[n] + f P[n + 1] (n = floor(x), P the double running
   integral, P[i] = sum_{k <= i} f[k] (i - k + 1)) at x0 = Tf - 1 (coefficient
   -2) and x0 +- Lf (coefficient 1); the transpose adds c g (1 - f) at n and
   c g f at n + 1, g = weight x t/(8 dt) x m - six entries per pair instead
   of the 2 Lf + 1 of an explicit triangle - and the trace is
   d[k] = sum_{i >= k} G[i] (i - k + 1), two reverse prefix sums.
   Exactness: G is integer fixed point, e1 = RN(c gs f), e0 = c Q - e1 with
   Q = RN(gs), so each pair's entries sum to exactly zero and integer sums
   carry no rounding into the prefix sums.  The per-trace scale 2^E follows
   from |L m| <= max|m| (L 1) (L has non-negative coefficients), (L 1) per
   trace from a bound pass of this kernel on the all-ones model, which also
   records the trace's largest pair weight.  The result is deterministic.
   SH (the rows fit in shared memory): each entry is two int32 limbs, G[n] =
   hi[n] 2^R + lo[n], in two planar rows of the warp (consecutive entries in
   consecutive banks); an entry is added as two returnless 32-bit shared
   atomics with no carry between them.  Every a.norm_cols columns the warp
   moves each lo limb's multiple of 2^R into hi.  Bounds (the host picks R
   and the bound pass's scale): an entry receives at most 4 units of 2^(R-1)
   per sample of a column (coefficients 1, -2, 1; coinciding neighbour
   entries), so lo stays within 2^31 for 4 ns norm_cols + 1 units; every
   partial sum of an entry is a second difference of a partial trace,
   |G| <= 4 max|d|, and the scale keeps 4 max|d| 2^E + 2^31 below 2^(31+R).
   At the end the two prefix sums run in int64 in place (each lane's chunk
   of entries, the low and high words of each value stored back in the two
   limbs).
   Else (long rows) the entries are added with fire-and-forget 64-bit RED
   into the trace's row in global memory, which stays in L2.
   BOUND: the bound pass (compiled apart, so that the main pass carries none
   of its per-sample work). */
template <bool SH, bool BOUND>
__global__ void __launch_bounds__(32 * KP_DM_WARPS, SH ? 7 : 8) k_demig(KpDemigArgs a)
{
    extern __shared__ __align__(16) float dm_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ns = a.ns, ng = a.ng, ngp = kp_demig_ngp(ng);
    const int nsp = (ns + 3) & ~3;
    float *s_t2 = dm_smem;       /* [ns] (t/2)^2 */
    float *s_ts = dm_smem + nsp; /* [ns] t/(8 dt) */
    int *s_lo = reinterpret_cast<int *>(dm_smem + 2 * nsp) + (size_t)w * 2 * ngp;
    int *s_hi = s_lo + ngp;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) {
        s_t2[k] = a.t2c[k].x;
        s_ts[k] = a.tscale[k];
    }
    if (SH)
        for (int i = lane; i < 2 * ngp; i += 32) s_lo[i] = 0;
    __syncthreads();
    constexpr bool bound = BOUND; /* the bound pass: the all-ones model (a.model unused) */
    const unsigned int mb = bound ? __float_as_uint(1.0f) : *a.absmax;
    if (mb == 0u) return; /* zero model: the data stay zero */
    if (mb >= 0x7f800000u) {
        if (threadIdx.x == 0) kp_fail(a.status, KPSTM_ERR_INVALID_ARG); /* non-finite model */
        return;
    }
    const int wi = blockIdx.x * KP_DM_WARPS + w;
    if (wi >= *a.nlive) return; /* no block barrier below */
    const int slot = a.order ? a.order[wi] : wi;
    const float bw = 2.002f / a.dt; /* >= weight x t/(8 dt) over all pairs */
    const int R = a.limb_r;
    int E;
    if (bound) {
        E = a.bound_g - (ilogbf(bw) + 1); /* |gs| < 2^bound_g */
    } else if (SH) {
        /* Limb rows.  max|d| 2^E <= 2^E max|m| ((L 1) + tails) with (L 1) from the
           bound pass (its own fixed point costs < 1%: a factor 2 covers it) and
           the tails at most tailf (L 1): 2^E max|m| (1 + tailf) (L 1) < 2^(27+R)
           keeps 4 max|d| 2^E + 2^31 < 2^(31+R).  The split needs |x| <= 2 |gs|
           < 2^(22+R), |gs| <= 2^E max|m| wmax (1 + 2^-20), wmax the trace's
           largest weight x t/(8 dt) from the bound pass. */
        const float mm = __uint_as_float(mb);
        const float v = mm * a.dbound[slot] * (1.0f + a.tailf);
        const float wv = mm * fminf(a.wbound[slot] * 1.001f, bw);
        E = min(v > 0.0f ? 27 + R - (ilogbf(fminf(v, 3.0e38f)) + 1) : 127,
                wv > 0.0f ? 21 + R - (ilogbf(fminf(wv, 3.0e38f)) + 1) : 127);
    } else {
        /* 2^E max|m| max(2 (1 + tailf) (L 1), 2 bw) < 2^61, and |2 gs| < 2^45 for kp_f2ll_rn45 */
        const float v = __uint_as_float(mb) * fmaxf(2.0f * (1.0f + a.tailf) * a.dbound[slot], 2.0f * bw);
        E = min(61 - (ilogbf(fminf(v, 3.0e38f)) + 1),
                43 - ilogbf(fminf(__uint_as_float(mb) * bw, 3.0e38f)));
    }
    E = max(-126, min(127, E));
    const float scale = __int_as_float((E + 127) << 23);
    const float inv = ldexpf(1.0f, -E);
    const float sR = ldexpf(1.0f, -R), nR = -ldexpf(1.0f, R);

    const kpstm_geom g = a.geom[slot];
    const int cls = g.cls;
    /* lane mapping: strided for models at least half nonzero (and the all-ones bound pass) */
    const bool dense = bound || 2ull * reinterpret_cast<const unsigned long long *>(a.absmax)[1] >=
                                    (unsigned long long)a.nmodel;
    const int l0 = dense ? KP_DM_UNROLL * lane : lane, ls = dense ? 1 : 32;
    unsigned long long *Gg = SH ? nullptr : a.acc + (int64_t)slot * ng;
    const float apm = (float)a.aperture * 1.00001f + 1.0f; /* range margin; exact test below */
    const int x_lo = max(0, (int)floorf((g.cmpx - apm - a.ax0) / a.adx) - 1);
    const int x_hi = min(a.nx - 1, (int)ceilf((g.cmpx + apm - a.ax0) / a.adx) + 1);
    int since_norm = 0;
    float wmax = 0.0f; /* bound pass: largest weight x t/(8 dt) */
    for (int xc = x_lo; xc <= x_hi; ++xc) {
        const float dxc = fmaf((float)xc, a.adx, a.ax0) - g.cmpx;
        const float rem = apm * apm - dxc * dxc;
        if (rem < 0.0f) continue;
        const float dyr = sqrtf(rem) + 1.0f;
        const int y_lo = max(0, (int)floorf((g.cmpy - dyr - a.ay0) / a.ady) - 1);
        const int y_hi = min(a.ny - 1, (int)ceilf((g.cmpy + dyr - a.ay0) / a.ady) + 1);
        for (int yc = y_lo; yc <= y_hi; ++yc) {
            const int col = xc * a.ny + yc;
            const float2 cxy = a.colxy[col];
            const float IX = cxy.x, IY = cxy.y;
            float cx = __fsub_rn(IX, g.cmpx), cy = __fsub_rn(IY, g.cmpy);
            const float dIC2 = __fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy));
            if (!(dIC2 < a.aperture_x2)) continue; /* RN(sqrt(dIC2)) < aperture_f, as k_image */
            const int vrow = a.colrow[col];
            if (vrow < 0) {
                kp_fail(a.status, KPSTM_ERR_VELOCITY_RANGE);
                continue;
            }
            if (SH && since_norm == a.norm_cols) {
                /* each lo limb keeps its centred remainder mod 2^R, hi takes the rest */
                __syncwarp();
                for (int i = lane; i < ng; i += 32) {
                    const int lo = s_lo[i];
                    const int q = (lo + (1 << (R - 1))) >> R;
                    s_lo[i] = lo - (q << R);
                    s_hi[i] += q;
                }
                __syncwarp();
                since_norm = 0;
            }
            ++since_norm;
            float sx = __fsub_rn(IX, g.sxt), sy = __fsub_rn(IY, g.syt);
            float gx = __fsub_rn(IX, g.gxt), gy = __fsub_rn(IY, g.gyt);
            const float dIS2 = __fadd_rn(__fmul_rn(sx, sx), __fmul_rn(sy, sy));
            const float dIR2 = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
            const float axs = __fmul_rn(sx, a.aax), axr = __fmul_rn(gx, a.aax);
            const float ays = __fmul_rn(sy, a.aay), ayr = __fmul_rn(gy, a.aay);
            const float *m = bound ? nullptr : a.model + ((int64_t)col * a.ncls + cls) * ns;
            const float *vr = a.rvdt + (int64_t)vrow * ns;
            /* 3 x 32 samples per step.  Dense models: lane l takes t0 + 3 l + u,
               so that one warp instruction's entries span three times as many
               rows where the traveltime is flat in t (same-address atomics
               serialise) while an odd stride keeps steep runs on distinct
               banks.  Sparse models: lane l takes t0 + 32 u + l, so that the
               clustered nonzero samples leave more warp instructions with
               nothing to do (they skip).  The integer sums do not depend on
               the order.  The model and velocity loads (non-coherent, so they
               can move ahead of the atomics) are all issued first. */
            for (int t0 = 0; t0 < ns; t0 += 32 * KP_DM_UNROLL) {
                float mv[KP_DM_UNROLL], rv[KP_DM_UNROLL];
#pragma unroll
                for (int u = 0; u < KP_DM_UNROLL; ++u) {
                    const int t = t0 + l0 + ls * u;
                    mv[u] = t < ns ? (bound ? 1.0f : __ldg(m + t)) : 0.0f;
                    rv[u] = t < ns ? __ldg(vr + t) : 1.0f;
                }
#pragma unroll
                for (int u = 0; u < KP_DM_UNROLL; ++u) {
                    const int t = t0 + l0 + ls * u, tt = min(t, ns - 1);
                    const float2 tv = make_float2(s_t2[tt], rv[u]); /* as k_image's s_v */
                    float rs, rr;
                    const float Tf = kp_pair_time(dIS2, dIR2, tv, rs, rr);
                    const bool ok = mv[u] != 0.0f && Tf < a.tmax;
                    if (!__any_sync(0xffffffffu, ok)) continue; /* warp-uniform */
                    float Lf, wgt;
                    kp_pair_width(rs, rr, axs, axr, ays, ayr, tv.y, a.lmaxf, Lf, wgt);
                    const float wts = __fmul_rn(wgt, __fmul_rn(s_ts[tt], mv[u]));
                    if (bound && ok) wmax = fmaxf(wmax, wts);
                    const float gs = ok ? __fmul_rn(wts, scale) : 0.0f;
                    /* the positions exactly as k_image computes them: y = Tf, Tf +- Lf,
                       P index n = floor(y) - 1, fraction y - floor(y) */
                    const float y0 = ok ? Tf : 1.0f, ya = y0 + Lf, yb = y0 - Lf;
                    const int ba = kp_floor_bits(ya), bb = kp_floor_bits(yb), b00 = kp_floor_bits(y0);
                    const float fa = ya - (__int_as_float(ba) - KP_MAGIC);
                    const float fb = yb - (__int_as_float(bb) - KP_MAGIC);
                    const float f0 = y0 - (__int_as_float(b00) - KP_MAGIC);
                    const int na = ba - KP_MAGIC_BITS - 1, nb = bb - KP_MAGIC_BITS - 1;
                    const int n0 = b00 - KP_MAGIC_BITS - 1;
                    if (SH) {
                        int qh, ql, h1, l1;
                        kp_split(gs, sR, nR, qh, ql);
                        /* tap at ya (c = 1): e1 = RN(gs fa) at na + 1, e0 = Q - e1 at na */
                        kp_split(__fmul_rn(gs, fa), sR, nR, h1, l1);
                        if (ok && na >= 0) {
                            atomicAdd(s_lo + na, ql - l1);
                            atomicAdd(s_hi + na, qh - h1);
                        }
                        if (ok && na >= -1) {
                            atomicAdd(s_lo + na + 1, l1);
                            atomicAdd(s_hi + na + 1, h1);
                        }
                        kp_split(__fmul_rn(gs, fb), sR, nR, h1, l1); /* tap at yb (c = 1) */
                        if (ok && nb >= 0) {
                            atomicAdd(s_lo + nb, ql - l1);
                            atomicAdd(s_hi + nb, qh - h1);
                        }
                        if (ok && nb >= -1) {
                            atomicAdd(s_lo + nb + 1, l1);
                            atomicAdd(s_hi + nb + 1, h1);
                        }
                        kp_split(__fmul_rn(-2.0f * gs, f0), sR, nR, h1, l1); /* tap at y0 (c = -2) */
                        if (ok && n0 >= 0) {
                            atomicAdd(s_lo + n0, -2 * ql - l1);
                            atomicAdd(s_hi + n0, -2 * qh - h1);
                        }
                        if (ok && n0 >= -1) {
                            atomicAdd(s_lo + n0 + 1, l1);
                            atomicAdd(s_hi + n0 + 1, h1);
                        }
                    } else {
                        const long long Q = kp_f2ll_rn45(gs);
                        const long long a1 = kp_f2ll_rn45(__fmul_rn(gs, fa));
                        const long long b1 = kp_f2ll_rn45(__fmul_rn(gs, fb));
                        const long long c1 = kp_f2ll_rn45(__fmul_rn(-2.0f * gs, f0));
                        if (ok && na >= 0) kp_red_add_u64(&Gg[na], (unsigned long long)(Q - a1));
                        if (ok && na >= -1) kp_red_add_u64(&Gg[na + 1], (unsigned long long)a1);
                        if (ok && nb >= 0) kp_red_add_u64(&Gg[nb], (unsigned long long)(Q - b1));
                        if (ok && nb >= -1) kp_red_add_u64(&Gg[nb + 1], (unsigned long long)b1);
                        if (ok && n0 >= 0) kp_red_add_u64(&Gg[n0], (unsigned long long)(-2 * Q - c1));
                        if (ok && n0 >= -1) kp_red_add_u64(&Gg[n0 + 1], (unsigned long long)c1);
                    }
                }
            }
        }
    }
    /* order the row's atomics before the warp reads it back (past L1) */
    if (!SH) __threadfence();
    __syncwarp();
    /* d = two reverse prefix sums of G in int64, lane l owning entries
       [l C, l C + C).  SH: pass 1 reads the limb form hi 2^R + lo and both
       passes store each int64 as its low word (lo row) and high word (hi
       row); else the row is int64 in L2. */
    auto ldA = [&](int i) -> unsigned long long {
        if constexpr (SH) return ((unsigned long long)(long long)s_hi[i] << R) + (unsigned long long)(long long)s_lo[i];
        else return __ldcg(&Gg[i]);
    };
    auto ldB = [&](int i) -> unsigned long long {
        if constexpr (SH) return ((unsigned long long)(unsigned int)s_hi[i] << 32) | (unsigned int)s_lo[i];
        else return __ldcg(&Gg[i]);
    };
    auto stB = [&](int i, unsigned long long v) {
        if constexpr (SH) {
            s_lo[i] = (int)(unsigned int)v;
            s_hi[i] = (int)(unsigned int)(v >> 32);
        } else {
            __stcg(&Gg[i], v);
        }
    };
    const int C = (ng + 31) >> 5;
    const int lo = min(ng, lane * C), hi = min(ng, lo + C);
    for (int pass = 0; pass < 2; ++pass) {
        unsigned long long tot = 0ull;
        for (int i = lo; i < hi; ++i) tot += pass ? ldB(i) : ldA(i);
        unsigned long long incl = tot; /* sum over lanes >= lane */
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long v = __shfl_down_sync(0xffffffffu, incl, d);
            if (lane + d < 32) incl += v;
        }
        unsigned long long run = incl - tot;
        for (int i = hi - 1; i >= lo; --i) {
            run += pass ? ldB(i) : ldA(i);
            stB(i, run);
        }
    }
    __syncwarp(); /* the lanes' rows are visible to the whole warp */
    if (bound) {
        /* the bound covers every entry of the row (the partial sums of all of
           them must fit), not only the samples that are output */
        float dmax = 0.0f;
        for (int k = lane; k < ng; k += 32) dmax = fmaxf(dmax, fabsf(__ll2float_rn((long long)ldB(k)) * inv));
        dmax = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(dmax)));
        wmax = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(wmax)));
        if (lane == 0) {
            a.dbound_out[slot] = dmax;
            a.wbound_out[slot] = wmax;
        }
    } else {
        float *o = a.out + (int64_t)g.src * ns;
        for (int k = lane; k < ns; k += 32) o[k] = __fmul_rn(__ll2float_rn((long long)ldB(k)), inv);
    }
}

/* live slot -> geometry in slot order */
__global__ void k_gather_geom(const kpstm_geom *graw, const int32_t *order, const int32_t *nlive, kpstm_geom *geom)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *nlive) geom[i] = graw[order[i]];
}

/* Deterministic FP64 dot product: per-block partial sums, then one block. */
#define KP_DOT_BLOCKS 1024
__global__ void __launch_bounds__(256) k_dot_partial(const float *x, const float *y, int64_t n, double *part)
{
    __shared__ double red[256];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) k_dot_final(const double *part, int nparts, double *out)
{
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

/* y = a*x + b*y (a, b from the host, FP64 scalars rounded once to float) */
__global__ void k_axpby(float *y, const float *x, float av, float bv, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fmaf(av, x[i], bv * y[i]);
}

/* fp32 traces -> bf16 with a per-trace scale (max |x| / 256, a power of two
   so that decode is exact); one warp per trace. */
__global__ void k_to_bf16(const float *x, int64_t ntr, int ns, uint16_t *out, float *scale)
{
    const int64_t tr = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (tr >= ntr) return;
    const float *xr = x + tr * ns;
    float mx = 0.0f;
    for (int k = lane; k < ns; k += 32) mx = fmaxf(mx, fabsf(xr[k]));
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    /* scale = 2^e with max|x|/scale in [128, 256): bf16 keeps 8 significant bits */
    float sc = 1.0f;
    if (mx > 1e-30f) sc = exp2f(floorf(log2f(mx)) - 7.0f); /* zero or denormal traces keep scale 1 */
    const float inv = 1.0f / sc;
    uint16_t *o = out + tr * ns;
    for (int k = lane; k < ns; k += 32) {
        const float v = xr[k] * inv;
        const uint32_t u = __float_as_uint(v);
        o[k] = (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16); /* round to nearest even */
    }
    if (lane == 0) scale[tr] = sc;
}

/* bf16 traces (with per-trace scale) -> fp32 */
__global__ void k_from_bf16(const uint16_t *in, const float *scale, int64_t ntr, int ns, float *x)
{
    const int64_t n = ntr * ns;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = __uint_as_float(((uint32_t)in[i]) << 16) * scale[i / ns];
}

/* ------------------------------------------------------------------------ */
/* Finishing, Kirchhoff.c:1457-1462: x[t] = -dt*t*(km[t]-km[t-1])*dt/fold[t]
   in float, x[0] = 0; rows written in output order [col][cls]. */
__global__ void k_deriv(const float *km, const int32_t *cnt, const float *tscale, int ncol, int ncls, int ns,
                        float dt, float *x)
{
    const int64_t n = (int64_t)ncls * ncol * ns;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i / ns;
        int t = (int)(i - r * ns);
        int cls = (int)(r / ncol), col = (int)(r - (int64_t)cls * ncol);
        float v = 0.0f;
        if (t > 0) {
            float fold = __int2float_rn(cnt[i] + 1);
            float k1 = km[i], k0 = km[i - 1];
            if (tscale) { /* full mode: the factor t dt/8 kept out of the accumulation */
                k1 = __fmul_rn(k1, tscale[t]);
                k0 = __fmul_rn(k0, tscale[t - 1]);
            }
            v = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(-dt, __int2float_rn(t)), __fsub_rn(k1, k0)), dt), fold);
        }
        x[((int64_t)col * ncls + cls) * ns + t] = v;
    }
}

/* Low-pass of Kirchhoff.c:1465-1479 as the equivalent circular convolution
   y = x (*) h (h real and even, from the anti-alias spectrum); y[0] = 0.
   A CTA convolves 8 rows; h is held twice in shared memory so that
   h[(t - j) mod ns] = hh[t - j + ns]. */
#define KP_LP_ROWS 8
__global__ void __launch_bounds__(256) k_lowpass(const float *x, const float *h, int64_t nrows, int ns, float *y)
{
    extern __shared__ __align__(16) float lp[];
    const int hn = (2 * ns + 3) & ~3; /* keeps xs 16-byte aligned for the float4 reads */
    float *hh = lp;                   /* [2*ns] */
    float *xs = lp + hn;              /* [ns][KP_LP_ROWS], row-interleaved */
    const int64_t r0 = (int64_t)blockIdx.x * KP_LP_ROWS;
    for (int i = threadIdx.x; i < 2 * ns; i += blockDim.x) hh[i] = h[i < ns ? i : i - ns];
    for (int i = threadIdx.x; i < ns * KP_LP_ROWS; i += blockDim.x) {
        int r = i / ns, j = i - r * ns;
        xs[j * KP_LP_ROWS + r] = (r0 + r < nrows) ? x[(r0 + r) * ns + j] : 0.0f;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ns; t += blockDim.x) {
        float acc[KP_LP_ROWS];
#pragma unroll
        for (int r = 0; r < KP_LP_ROWS; ++r) acc[r] = 0.0f;
        const float *hp = hh + t + ns;
        for (int j = 0; j < ns; ++j) {
            float hv = hp[-j];
            float4 xa = *reinterpret_cast<const float4 *>(xs + j * KP_LP_ROWS);
            float4 xb = *reinterpret_cast<const float4 *>(xs + j * KP_LP_ROWS + 4);
            acc[0] = fmaf(xa.x, hv, acc[0]);
            acc[1] = fmaf(xa.y, hv, acc[1]);
            acc[2] = fmaf(xa.z, hv, acc[2]);
            acc[3] = fmaf(xa.w, hv, acc[3]);
            acc[4] = fmaf(xb.x, hv, acc[4]);
            acc[5] = fmaf(xb.y, hv, acc[5]);
            acc[6] = fmaf(xb.z, hv, acc[6]);
            acc[7] = fmaf(xb.w, hv, acc[7]);
        }
#pragma unroll
        for (int r = 0; r < KP_LP_ROWS; ++r)
            if (r0 + r < nrows) y[(r0 + r) * ns + t] = t == 0 ? 0.0f : acc[r];
    }
}

/* [cls][col][ns] -> [col][cls][ns]; fold = 1 + count when cnt is given;
   src scaled per sample by tscale when given (full mode). */
__global__ void k_relayout(const float *src, const int32_t *cnt, const float *tscale, int ncol, int ncls, int ns,
                           float *dst)
{
    const int64_t n = (int64_t)ncls * ncol * ns;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i / ns;
        int t = (int)(i - r * ns);
        int cls = (int)(r / ncol), col = (int)(r - (int64_t)cls * ncol);
        float v = cnt ? __int2float_rn(cnt[i] + 1) : (tscale ? __fmul_rn(src[i], tscale[t]) : src[i]);
        dst[((int64_t)col * ncls + cls) * ns + t] = v;
    }
}

#endif
