/*
 * Single-communicator MPI stand-in used ONLY to compile the reference
 * Kirchhoff.c as a CPU oracle / CPU baseline (test infrastructure, never
 * linked into the product library).
 *
 * The reference uses MPI for rank ids, a 1-D Cartesian communicator,
 * barriers and wall clocks (Kirchhoff.c:223-243, 317, 331, 352, 370) and
 * never moves data.  This header supplies exactly those calls.  The rank and
 * size come from the environment (KPSTM_REF_RANK / KPSTM_REF_SIZE, default
 * 0 / 1) so that P independent processes reproduce the reference's
 * round-robin job loop `for (job = rank; job < no_job; job += size)`
 * (Kirchhoff.c:347) without an MPI runtime.  Barriers are no-ops: the
 * reference exchanges no data, so the only effect of a barrier is ordering
 * of log lines and of rank 0's header files, which the harness creates
 * before it starts the ranks.
 */
#ifndef KPSTM_ORACLE_MPI_STUB_H
#define KPSTM_ORACLE_MPI_STUB_H

#include <stdlib.h>
#include <time.h>

typedef int MPI_Comm;
#define MPI_COMM_WORLD 0

static int kref_env_int(const char *name, int dflt)
{
    const char *s = getenv(name);
    return (s && *s) ? atoi(s) : dflt;
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = kref_env_int("KPSTM_REF_RANK", 0); return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = kref_env_int("KPSTM_REF_SIZE", 1); return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Cart_create(MPI_Comm old, int ndims, int *dims, int *periods,
                                  int reorder, MPI_Comm *out)
{
    (void)ndims; (void)dims; (void)periods; (void)reorder;
    *out = old;
    return 0;
}
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
