/*
 * kpstm.h - C ABI of the GB300 Kirchhoff prestack time migration.
 *
 * Drop-in boundary for the reference's imaging job
 *     void kirchhoff(int job_id)                       Kirchhoff.c:92, 1104-1616
 * and the set-up it depends on (count_size_file Kirchhoff.c:633-722,
 * create_aliasfilter :380-441, build_vel_model :447-626, the image/slab
 * arithmetic of main :266-313).  The reference passes everything through
 * globals and compile-time #defines (Kirchhoff.c:17-65); here the same
 * quantities travel in kpstm_params / kpstm_velocity, and the file reads and
 * writes of kirchhoff() become buffer arguments:
 *
 *   reference (Kirchhoff.c)                      this ABI
 *   -------------------------------------------  ------------------------------
 *   main: sinA/cosA, Nx/Ny, nx/ny, slabs :266-313  kpstm_create
 *   create_aliasfilter :380-441                    kpstm_create (and
 *                                                  kpstm_aliasfilter, stand-alone)
 *   build_vel_model :447-626 (v_rms grid, v^2)     kpstm_velocity + kpstm_create
 *   kirchhoff: one ntblock iteration :1276-1408    kpstm_add_traces /
 *     (fread + IBM decode :1280-1290,              kpstm_add_segy_block /
 *      geometry :1297-1310, imaging :1312-1403)    kpstm_add_traces_device
 *   kirchhoff: finishing :1426-1479                kpstm_finish
 *   kirchhoff: SU writer :1482-1593                kpstm_write_su
 *
 * Conventions (the reference prints and calls exit(1) on every error; this
 * ABI never exits and never prints):
 *   - every call returns a kpstm_status; kpstm_strerror() names it;
 *   - the caller owns every host buffer it passes; a context owns its device
 *     buffers and its CUDA stream; all device work of a context is ordered on
 *     that stream;
 *   - one context per host thread; contexts are independent.
 */
#ifndef KPSTM_H
#define KPSTM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KPSTM_ABI_VERSION 1

typedef enum {
    KPSTM_OK = 0,
    KPSTM_ERR_INVALID_ARG = 1,     /* NULL pointer, size <= 0, inconsistent parameters */
    KPSTM_ERR_CUDA = 2,            /* a CUDA runtime call failed */
    KPSTM_ERR_OUT_OF_MEMORY = 3,   /* host or device allocation failed */
    KPSTM_ERR_VELOCITY_ZERO = 4,   /* a v_rms sample is 0 (Kirchhoff.c:614-615 reports it) */
    KPSTM_ERR_VELOCITY_RANGE = 5,  /* an image column maps below the velocity grid origin:
                                      Kirchhoff.c:1357-1365 clamps only the upper end */
    KPSTM_ERR_GEOMETRY = 6,        /* header coordinate minus origin does not fit an int */
    KPSTM_ERR_STATE = 7,           /* call out of order (e.g. traces after finish) */
    KPSTM_ERR_TIMEOUT = 8,         /* a bounded device-side wait gave up */
    KPSTM_ERR_NO_DEVICE = 9,       /* no CUDA device visible */
    KPSTM_ERR_SEGY = 10,           /* malformed SEG-Y buffer */
    KPSTM_ERR_UNSUPPORTED = 11,    /* valid request this build does not implement */
    KPSTM_ERR_TRANGE = 12,         /* trangeMax < 2: the reference's triangle taps
                                      (Kirchhoff.c:1391-1392) would read before the trace */
    KPSTM_ERR_TOO_LARGE = 13       /* request exceeds the fixed scratch of kpstm_finish_noalloc */
} kpstm_status;

/* Imaging operator. */
typedef enum {
    KPSTM_MODE_REFERENCE = 0,  /* Kirchhoff.c:1341-1403 bit for bit: nearest-sample
                                  T, fixed [P(T+2) - 2P(T) + P(T-2)] triangle, unit weight */
    KPSTM_MODE_FULL = 1        /* linear trace interpolation, obliquity and spreading
                                  weight, variable-width triangle anti-alias */
} kpstm_mode;

/* Trace storage / image accumulation. */
typedef enum {
    KPSTM_PREC_FP32 = 0,       /* fp32 traces, fp32 image accumulators */
    KPSTM_PREC_BF16_KAHAN = 1  /* bf16 traces with a per-trace fp32 scale, fp32
                                  Kahan-compensated image accumulators */
} kpstm_precision;

/* Output layout. */
typedef enum {
    KPSTM_OUT_OFFSET_GATHERS = 0, /* [nx][ny][nh][ns], as Kirchhoff.c:1438-1445 writes */
    KPSTM_OUT_STACK = 1           /* [nx][ny][ns]: all offset classes in one image */
} kpstm_output;

/* Everything kirchhoff() reads from globals and #defines. */
typedef struct {
    /* trace sampling, count_size_file (Kirchhoff.c:655-661) */
    int32_t ns;
    float dt;                       /* seconds (header microseconds / 1e6) */
    /* image box in line numbers (Kirchhoff.c:34-37) and increments (:40-41) */
    int32_t start_iline, end_iline, start_xline, end_xline;
    double inc_iline, inc_xline;
    /* physical line spacing (Kirchhoff.c:54-55) */
    double iline_distance, xline_distance;
    /* offset classes (Kirchhoff.c:44-46): class = floor((2*sqrt(h^2) - oh)/dh) */
    int32_t nh;
    double oh, dh;
    /* survey origin and rotation (Kirchhoff.c:49-51) */
    double ox, oy, angle_e_to_n_deg;
    /* 1.0: coordinates used as in Kirchhoff.c:1297-1304.  Any other value:
       coordinates scaled as in Kirchhoff_GHTest1.c:56, 1302-1312. */
    double xy_scale;
    /* aperture (Kirchhoff.c:58) in coordinate units; low-pass cutoff in Hz (:59) */
    double aperture, anti_alias_cutoff;
    /* image slab grid and the slab this context images (Kirchhoff.c:64-65,
       280-300, 1104): jobs_x * jobs_y slabs, job_id in [0, jobs_x*jobs_y) */
    int32_t jobs_x, jobs_y, job_id;
    int32_t mode;       /* kpstm_mode */
    int32_t precision;  /* kpstm_precision */
    int32_t output;     /* kpstm_output */
    /* KPSTM_MODE_FULL only: largest triangle half-width in samples (0 = trangeMax) */
    int32_t aa_max_halfwidth;
    /* KPSTM_MODE_FULL only: 0 = the reference's nearest grid node and nearest
       velocity sample (Kirchhoff.c:1357-1378); 1 = trilinear interpolation of
       v_rms at the same continuous grid position and time that the reference
       rounds (clamped to the grid; below-grid columns are still refused) */
    int32_t velocity_interp;
    int32_t reserved[6];
} kpstm_params;

/* Gridded v_rms model, build_vel_model (Kirchhoff.c:22-27, 447-626).  Values
   are v_rms (not squared; the library squares them as Kirchhoff.c:617 does),
   laid out [n_iline][n_xline][nsm].  Grid line (i, j) holds the trace whose
   headers carry iline = o_iline + i*d_iline, xline = o_xline + j*d_xline. */
typedef struct {
    int32_t n_iline, n_xline, nsm;
    int32_t o_iline, o_xline, d_iline, d_xline;
    float dtm;                      /* seconds */
    const float *vrms;              /* host pointer, read during kpstm_create only */
} kpstm_velocity;

/* Sizes of the image slab a context produces. */
typedef struct {
    int32_t Nx, Ny;          /* whole image, Kirchhoff.c:266-277 */
    int32_t nx, ny;          /* this slab, Kirchhoff.c:280-281, 295-298 */
    int32_t nh, ns;          /* classes (1 for a stack), samples */
    int32_t trange_max;      /* Kirchhoff.c:394 */
    int32_t x0, y0;          /* first column of the slab: xslice*nx, yslice*ny */
    int64_t out_elems;       /* floats kpstm_finish writes */
} kpstm_dims;

typedef struct kpstm_ctx kpstm_ctx;

/* Set-up (= main :263-331 for one job).  Uploads the velocity model and the
   per-column tables; allocates the slab's image accumulators. */
int kpstm_create(const kpstm_params *params, const kpstm_velocity *vel, kpstm_ctx **out);
void kpstm_destroy(kpstm_ctx *ctx);
int kpstm_get_dims(const kpstm_ctx *ctx, kpstm_dims *dims);
/* Zero the image accumulators (start a new job with the same set-up). */
int kpstm_reset(kpstm_ctx *ctx);

/* One ntblock iteration of Kirchhoff.c:1276-1408 from host buffers.
   hdr_be:  [ntr][60] SEG-Y trace-header words exactly as read from the file
            (big-endian); words 18-21 (sx, sy, gx, gy) are used.
   samples: [ntr][ns] IEEE float samples in host byte order (already decoded).
   Traces are imaged in the order given, as the reference does. */
int kpstm_add_traces(kpstm_ctx *ctx, const int32_t *hdr_be, const float *samples, int64_t ntr);

/* Same, from a raw SEG-Y trace block: ntr records of 240 header bytes plus
   ns big-endian IBM floats (the buffer Kirchhoff.c:1280-1281 freads).  The
   IBM decode of Kirchhoff.c:1284-1290 runs on the device. */
int kpstm_add_segy_block(kpstm_ctx *ctx, const void *segy_records, int64_t ntr);

/* Same, with headers and samples already in device memory (no host copies).
   d_hdr_be: [ntr][60] big-endian words; d_samples: [ntr][ns] floats. */
int kpstm_add_traces_device(kpstm_ctx *ctx, const int32_t *d_hdr_be, const float *d_samples,
                            int64_t ntr);

/* Finishing, Kirchhoff.c:1426-1479: derivative with -t*dt^2/fold scaling,
   low-pass by the anti-alias spectrum, first sample zeroed.  out receives
   dims.out_elems floats in [nx][ny][nh][ns] order (stack: [nx][ny][ns]);
   fold (nullable) receives the fold counts (1 + contributing traces) in the
   same layout.  Host pointers.  The accumulators are left untouched, so more
   traces may follow. */
int kpstm_finish(kpstm_ctx *ctx, float *out, float *fold);
/* Same, into device memory. */
int kpstm_finish_device(kpstm_ctx *ctx, float *d_out, float *d_fold);

/* Raw accumulators before finishing (km_data and fold of Kirchhoff.c:1263-1274),
   [nx][ny][nh][ns] (stack: [nx][ny][ns]); host pointers, either nullable. */
int kpstm_get_accumulators(kpstm_ctx *ctx, float *km, float *fold);

/* Number of (trace, in-aperture column, sample) pairs imaged so far. */
int kpstm_pair_count(const kpstm_ctx *ctx, int64_t *pairs);

/* Device synchronisation of the context's stream. */
int kpstm_synchronize(kpstm_ctx *ctx);

/* Run the context's device work on the caller's CUDA stream (a
   cudaStream_t; NULL restores the context's own stream), so that a host
   framework can order its own work and timers with it.  No counterpart in
   the reference, which has no device. */
int kpstm_set_stream(kpstm_ctx *ctx, void *cuda_stream);

/* Per-stage device timing with CUDA events on the compute stream (no
   counterpart in the reference, which only prints wall clocks,
   Kirchhoff.c:243, 338, 362).  While enabled every stage launch is
   bracketed by events; kpstm_profile_read synchronises, sums and resets. */
typedef struct {
    int64_t image_launches;   /* imaging kernel launches */
    double image_ms;          /* summed imaging kernel time */
    double prep_ms;           /* geometry + bucketing + integral prep */
    double finish_ms;         /* finishing kernels */
    int64_t other_launches;   /* all other kernel launches */
} kpstm_profile;
int kpstm_profile_enable(kpstm_ctx *ctx, int enable);
int kpstm_profile_read(kpstm_ctx *ctx, kpstm_profile *out);

/* ---- launch configuration of the imaging kernel ----------------------------- */
/* No counterpart in the reference (its loop order is fixed: trace, column,
   sample, Kirchhoff.c:1292-1403).  A work item of the imaging kernel is one
   image tile (8 columns: a tile_px x tile_py patch, one column per warp) x one
   offset class x one time window of 32*samples_per_lane samples.  None of the
   choices changes a result: every column still sums its traces in block
   order, so all configurations give bit-identical images. */
typedef struct {
    int tile_px;          /* patch columns along the inline axis: 1, 2, 4 or 8
                             (tile_py = 8 / tile_px); 0 = default (the fewest
                             tiles, ties to 4 x 2) */
    int samples_per_lane; /* 8, 16, 24 or 32 (full mode <= 24, BF16/Kahan <= 16);
                             0 = default (the fewest windows, then the smallest K,
                             at most 16 with 3 CTAs per SM) */
    int persistent;       /* 1: one resident grid takes (class, tile, window) items
                             from a device counter, largest classes first;
                             0: one CTA per item.  Default: 1 for full mode
                             with fp32 storage, else 0 */
    int graph;            /* 1: each block's device pipeline (geometry, bucketing,
                             tap tables, imaging) is captured once per block shape
                             into a CUDA graph and replayed; ignored while
                             profiling is enabled */
    int ctas_per_sm;      /* imaging kernel variant: 2, 3 or 4 resident CTAs per SM -
                             3 trades register space (80 per thread, so
                             samples_per_lane <= 16 in full mode, <= 8 with
                             Kahan sums or in reference mode) and pipeline
                             depth for 24 resident warps; 4 (64 registers,
                             32 warps) exists for full mode with fp32 storage
                             and samples_per_lane = 8 only; 0 = default (3 for
                             full mode with fp32 storage, else 2) */
    int reserved[3];
} kpstm_launch;
int kpstm_get_launch(const kpstm_ctx *ctx, kpstm_launch *cfg);
/* KPSTM_ERR_INVALID_ARG for a value outside the lists above. */
int kpstm_set_launch(kpstm_ctx *ctx, const kpstm_launch *cfg);
/* Autotuner: images the given device block (the layout of
   kpstm_add_traces_device) once per candidate configuration (tile_px x
   samples_per_lane x persistent x ctas_per_sm; the caller's graph flag is
   kept), times the
   imaging kernel with CUDA events, selects the fastest, clears the image
   accumulators again and returns the choice in *best (nullable) and its time
   in *best_ms (nullable).  Only on a context without traces since
   kpstm_create / kpstm_reset (else KPSTM_ERR_STATE).  A few thousand traces
   of the job's own data are a representative sample. */
int kpstm_autotune(kpstm_ctx *ctx, const int32_t *d_hdr_be, const float *d_samples, int64_t ntr,
                   kpstm_launch *best, float *best_ms);

/* ---- least-squares migration ------------------------------------------------ */
/* No counterpart in the reference.  The operator pair is the full-physics
   migration without its finishing: L^T (migration) maps data d[ntr][ns] to
   the image accumulators m[nx][ny][nh][ns] (the values
   kpstm_get_accumulators would return), L (demigration) is its exact
   transpose.  The context must be created with KPSTM_MODE_FULL.  Data and
   model vectors are device pointers; data traces follow the order of the
   headers given to kpstm_lsm_geometry. */

/* Fix the acquisition geometry (ntr trace headers, big-endian words, host). */
int kpstm_lsm_geometry(kpstm_ctx *ctx, const int32_t *hdr_be, int64_t ntr);
/* Migration: d_model = L^T d_data. */
int kpstm_lsm_adjoint(kpstm_ctx *ctx, const float *d_data, float *d_model);
/* Demigration: d_data = L d_model (traces outside every class or the slab
   cull get zeros). */
int kpstm_lsm_forward(kpstm_ctx *ctx, const float *d_model, float *d_data);
/* Conjugate gradients on min ||L m - d||^2 (CGLS) from m = 0, niter
   iterations (niter applications of L and of L^T: the last iteration skips
   the next search direction), dot products and step lengths in FP64.  With
   KPSTM_PREC_BF16_KAHAN the data-domain vectors (d, residual) are stored
   as bf16 with a per-trace scale.  resid (nullable, niter + 1 values)
   receives ||d - L m_k||. */
int kpstm_lsm_cg(kpstm_ctx *ctx, const float *d_data, int32_t niter, float *d_model, double *resid);
/* Called by kpstm_lsm_cg_ex after iteration k (1 .. niter) has updated the
   model: d_model (device memory) holds the iterate m_k and resid_k =
   ||d - L m_k||.  Device work the monitor queues on the context's stream
   (kpstm_set_stream) sees m_k; the next iteration starts after the monitor
   returns.  A nonzero return ends the solve after this iteration. */
typedef int (*kpstm_cg_monitor)(int32_t iteration, const float *d_model, double resid_k, void *user);
/* kpstm_lsm_cg with a monitor (nullable): snapshots, wall-clock marks or a
   stopping rule per iteration. */
int kpstm_lsm_cg_ex(kpstm_ctx *ctx, const float *d_data, int32_t niter, float *d_model, double *resid,
                    kpstm_cg_monitor monitor, void *user);
/* Pairs (trace, in-aperture column, sample) of one operator application,
   counted by the last kpstm_lsm_adjoint (L visits the same pairs). */
int kpstm_lsm_pair_count(kpstm_ctx *ctx, int64_t *pairs);

/* ---- finishing without device allocation ------------------------------------ */

/* Largest image (nx*ny*nh*ns samples) and largest ns kpstm_finish_noalloc
   accepts (ns: the low-pass convolution keeps 10 ns floats in one CTA's
   shared memory). */
#define KPSTM_NOALLOC_MAX_SAMPLES 4194304
#define KPSTM_NOALLOC_MAX_NS 5600

/* The finishing step of kpstm_finish for callers that must not allocate
   device memory.  No counterpart in the reference (it has no device).

   Some callers cannot call cudaMalloc: a process whose framework allocator
   has already reserved the device memory it is allowed to use, or a
   pipelined service that must not let cudaMalloc/cudaFree synchronise the
   device between jobs.  This entry point allocates nothing: the caller
   passes the accumulators and the output, all in device memory and in the
   layout kpstm_get_accumulators returns ([nx][ny][nh][ns]; fold as floats,
   1 + contributing traces), and the intermediate derivative traces and the
   low-pass impulse response live in one fixed array compiled into the
   library - about 17 MB that every GPU which loads the library holds until
   the process exits.  Images larger than KPSTM_NOALLOC_MAX_SAMPLES samples
   or with more than KPSTM_NOALLOC_MAX_NS samples per trace are refused with
   KPSTM_ERR_TOO_LARGE; params are checked as in kpstm_create (no context is
   needed).

   The first call on a device looks up that array's device address (with
   the device current); make that first call before any stream capture.
   The address is kept for the life of the process and does not survive
   cudaDeviceReset.  The low-pass response is computed on the host and
   copied into the array (from a static host buffer) when ns, dt or the
   cutoff differ from the previous call on the device.
   Work is queued on cuda_stream (NULL: the default stream) and the call
   returns without waiting; synchronise before reading d_out.  All calls on
   a device share the one array, so calls whose work overlaps on the GPU
   (other streams, other host threads) race and must be serialised by the
   caller. */
int kpstm_finish_noalloc(const kpstm_params *params, const float *d_km, const float *d_fold,
                         float *d_out, void *cuda_stream);

/* ---- test hooks --------------------------------------------------------------- */
/* No counterpart in the reference, which exits on every error
   (Kirchhoff.c:462-467) and ignores short reads (:1280-1281).  They let
   tests drive the error paths without faulting a device. */

/* The stage waits of the imaging kernel give up after `polls` polls (0: at
   once; default 4194304) and report KPSTM_ERR_TIMEOUT at the next
   synchronising call; the kernel still waits, with the full bound, for its
   own copies in flight before it returns, and kpstm_reset clears the
   status.  Per context. */
int kpstm_debug_wait_limit(kpstm_ctx *ctx, uint32_t polls);
/* The nth device allocation from now (0: the next) made by kpstm_create or
   by the staging buffers of kpstm_add_traces* fails as if the device were
   out of memory (KPSTM_ERR_OUT_OF_MEMORY); -1 disarms.  Process-wide, one
   shot. */
int kpstm_debug_fail_alloc(int32_t nth);
/* The imaging kernel leaves out of an image tile's trace list, for one time
   window, every trace whose traveltimes to all of the tile's columns lie
   past the trace end at every sample of the window (a lower bound of the
   double-square-root time with a relative margin of 2^-12, so that only
   pairs the kernel would skip anyway are left out).  enable = 0 turns this
   off, so that a test can show the images are bit-identical either way.
   Per context; default on. */
int kpstm_debug_trace_cull(kpstm_ctx *ctx, int32_t enable);

/* ---- stand-alone set-up helpers (host only) -------------------------------- */

/* create_aliasfilter, Kirchhoff.c:380-441: trangeMax and the low-pass
   spectrum anti_alias[ns] (including the reference's mirror of the upper
   half, which zeroes bins ns/2 and ns/2+1 for odd ns). */
int kpstm_aliasfilter(int32_t ns, float dt, double iline_distance, double xline_distance,
                      double anti_alias_cutoff, int32_t *trange_max, float *anti_alias);

/* IBM System/360 single precision (big-endian words) to IEEE float, exactly
   as Kirchhoff.c:1284-1290 computes it. */
int kpstm_ibm_to_ieee(const uint32_t *ibm_be, float *out, int64_t n);

/* Sampling of a SEG-Y file image in memory, count_size_file
   (Kirchhoff.c:650-661): ns and dt from the first trace header, number of
   traces from the size. */
int kpstm_segy_info(const void *file_bytes, int64_t nbytes, int32_t *ns, float *dt,
                    int64_t *ntraces);

/* The gridded v_rms model from a velocity SEG-Y file image in memory,
   build_vel_model (Kirchhoff.c:447-626): header words 47/48 (iline, xline)
   pick the cell (truncating division, as :539), samples IBM-decoded; a later
   trace overwrites an earlier one, unreached cells are 0.  vrms receives
   [n_iline][n_xline][nsm] floats (nsm from kpstm_segy_info), ready for
   kpstm_velocity.vrms.  Needs no device. */
int kpstm_velocity_from_segy(const void *file_bytes, int64_t nbytes, int32_t n_iline, int32_t n_xline,
                             int32_t o_iline, int32_t o_xline, int32_t d_iline, int32_t d_xline, float *vrms,
                             int64_t vrms_elems);

/* SU trace records of a finished image, Kirchhoff.c:1482-1593: 240-byte
   big-endian header plus ns big-endian floats per output trace, traces in
   xc, yc, class order.  dst must hold dims.nx*dims.ny*nh*(240+4*ns) bytes. */
int kpstm_write_su(const kpstm_ctx *ctx, const float *image, void *dst, int64_t dst_bytes);

/* Front headers of the output SEG-Y file, write_segy_ebdic_header
   (Kirchhoff.c:729-814): 3200 text bytes and the 400-byte binary header
   (sample interval, samples per trace, format 5 = IEEE float).  The
   reference's combine script (Kirchhoff.c:821-874) writes them followed by
   the slabs' SU records (kpstm_write_su) in job order.  dst must hold 3600
   bytes.  Needs no device. */
int kpstm_segy_front_headers(const kpstm_params *params, void *dst, int64_t dst_bytes);

const char *kpstm_strerror(int status);
int kpstm_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KPSTM_H */
