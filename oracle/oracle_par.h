/*
 * oracle_par.h — TEST INFRASTRUCTURE ONLY: threads for the CPU oracle.
 *
 * The reference's parallel build (molsim_par) is MPI with replicated data:
 * every particle loop is split into contiguous rank ranges (LoadBalance,
 * nlist.F90:344-375), each rank accumulates its own force array and energy
 * partial sums, and mpi_allreduce SUM combines them (energy.F90:392-401,
 * parallel.F90:483-505).  The oracle restates that with threads: thread t of
 * nt takes the t-th contiguous range and the partial arrays are summed in
 * thread order, so a given thread count gives the same bits on every run.
 * One thread (the default) runs the serial code path unchanged.
 */
#ifndef ORACLE_PAR_H
#define ORACLE_PAR_H
#include <pthread.h>

#define ORC_MAX_THREADS 64

int orc_threads(void);   /* the count set by orc_set_threads (molsim_oracle.c) */

typedef void (*orc_task_fn)(void *ctx, int t, int nt);

typedef struct {
    orc_task_fn fn;
    void *ctx;
    int t, nt;
} orc_job;

static void *orc_job_entry(void *p) {
    orc_job *j = (orc_job *)p;
    j->fn(j->ctx, j->t, j->nt);
    return 0;
}

/* run fn(ctx, t, nt) for t = 0..nt-1, t = 0 on the calling thread */
static inline void orc_par_run(orc_task_fn fn, void *ctx, int nt) {
    if (nt <= 1) {
        fn(ctx, 0, 1);
        return;
    }
    pthread_t th[ORC_MAX_THREADS];
    orc_job jobs[ORC_MAX_THREADS];
    int started[ORC_MAX_THREADS];
    for (int t = 1; t < nt; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].t = t;
        jobs[t].nt = nt;
        started[t] = pthread_create(&th[t], 0, orc_job_entry, &jobs[t]) == 0;
        if (!started[t]) fn(ctx, t, nt);   /* no thread: run it here */
    }
    fn(ctx, 0, nt);
    for (int t = 1; t < nt; ++t)
        if (started[t]) pthread_join(th[t], 0);
}

/* the t-th of nt contiguous ranges of [0, n) */
static inline void orc_range(long n, int t, int nt, long *lo, long *hi) {
    *lo = n * t / nt;
    *hi = n * (t + 1) / nt;
}

#endif
