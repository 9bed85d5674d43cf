/*
 * gbmd_serve.h -- serving engine: many independent MD jobs resident on one
 * GPU, admitted by device-memory footprint and advanced together.
 *
 * CabanaMD runs one system per process (src/cabanamd_impl.h:70-432: init,
 * then the timestep loop).  The engine keeps that per-system semantics --
 * each job is exactly one CbnMD run (same step order, same rebuild and
 * thermo cadence, same results as gbmd_md_init + gbmd_md_run on a context)
 * -- and adds continuous batching:
 *  - jobs are submitted with their initial state at any time and wait in a
 *    FIFO queue;
 *  - gbmd_engine_step() admits queued jobs while a job slot and the device
 *    memory budget allow, then advances every running job by one chunk of
 *    timesteps; per phase of a timestep, the jobs that share a kernel form
 *    one launch over a job table (per-job cell grids, lists and parameters);
 *  - a job that reaches its step count is retired at the end of the chunk,
 *    its final state and thermo rows kept for gbmd_job_result(), and its
 *    slot and memory go to the next queued job.
 * A job's result does not depend on which other jobs ran beside it.
 */
#ifndef GBMD_SERVE_H
#define GBMD_SERVE_H

#include <stdint.h>

#include "gbmd.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbmd_engine gbmd_engine;

#define GBMD_JOB_QUEUED 0
#define GBMD_JOB_RUNNING 1
#define GBMD_JOB_DONE 2
#define GBMD_JOB_FAILED 3

/* One MD job: what an input deck gives CbnMD (src/inputFile_impl.h:125-534)
 * for a single-type LJ or single-element NNP system. */
typedef struct
{
    int force_type;     /* GBMD_FORCE_LJ or GBMD_FORCE_NNP */
    int precision;      /* GBMD_PREC_FP64 or GBMD_PREC_MIXED */
    double lo[3], hi[3];
    double boltz, mvv2e, dt; /* units (src/inputFile_impl.h:146-182) */
    double mass;        /* the one type's mass */
    double lj_epsilon, lj_sigma, lj_cut; /* LJ: pair_coeff 1 1 */
    const char *nnp_dir; /* NNP: input.nn, scaling.data, weights.%03d.data */
    double nnp_cflength, nnp_cfenergy;
    gbmd_md_params md;  /* cutoff, skin, list kind, rebuild / thermo cadence */
    int64_t nsteps;     /* timesteps to run */
} gbmd_job_spec;

typedef struct
{
    int64_t submitted, admitted, finished, failed;
    int64_t running, queued;
    uint64_t budget_bytes, used_bytes, peak_used_bytes;
    int64_t atom_steps;   /* summed over finished jobs */
    int64_t chunks;       /* gbmd_engine_step calls that ran work */
    int64_t launches;     /* kernel launches issued by the engine's jobs */
    double busy_seconds;  /* wall time inside gbmd_engine_step */
    int64_t atom_steps_run; /* atom-steps advanced so far (all jobs, as run) */
    int64_t cancelled;      /* jobs ended by gbmd_job_cancel (also counted in failed) */
    /* where busy_seconds went on the host: admission (context set-up,
     * upload, md_init), waits for the GPU (rebuilt lists, the end of each
     * chunk) and retirement (download, reordering by id); the rest is the
     * launching of work */
    double admit_seconds, wait_seconds, retire_seconds;
    /* job rebuilds (wrap, cell sort, list build) that ran in job-table
     * launches shared with the other jobs of their stream */
    int64_t batched_rebuilds;
} gbmd_engine_stats;

/* device: CUDA device; budget_bytes: device memory the running jobs may hold
 * (estimated at admission, then measured); max_running: job slots; chunk:
 * timesteps per gbmd_engine_step (0: 10). */
int gbmd_engine_create( gbmd_engine **out, int device, uint64_t budget_bytes, int max_running,
                        int chunk );
void gbmd_engine_destroy( gbmd_engine *e );
const char *gbmd_engine_last_error( const gbmd_engine *e );

/* Seconds since the engine was created (the clock of all job times). */
double gbmd_engine_now( const gbmd_engine *e );

/* Queue a job.  Host arrays as for gbmd_upload_atoms (copied; the caller may
 * free them on return).  arrival: engine-clock time the request arrived
 * (<= now; a negative value means now).  The job's id goes to *job_id. */
int gbmd_job_submit( gbmd_engine *e, const gbmd_job_spec *spec, int64_t n, const double *x,
                     const double *v, const int *type, const int *id, double arrival,
                     int64_t *job_id );

/* Admit what fits, advance running jobs by one chunk, retire finished jobs.
 * Optional outputs: jobs running and queued after the call, jobs finished by
 * the call. */
int gbmd_engine_step( gbmd_engine *e, int *running, int *queued, int *finished );

/* state: GBMD_JOB_*; error: the job's GBMD_ERR_* code (0 unless FAILED);
 * times (optional, 3 doubles): arrival, admission, finish (engine clock,
 * -1 where not reached). */
int gbmd_job_poll( gbmd_engine *e, int64_t job_id, int *state, int *error, double *times );
const char *gbmd_job_error( gbmd_engine *e, int64_t job_id );

/* Final state of a DONE job, in the order of its ids (any pointer may be
 * NULL), and its thermo rows [step, T, PE/N, KE/N] (src/cabanamd_impl.h:
 * 365-372) including step 0. */
int gbmd_job_result( gbmd_engine *e, int64_t job_id, int64_t *n, double *x, double *v,
                     double *f, int *type, int *id, double *thermo, int max_rows, int *nrows );

/* Cancel a queued or running job: a queued job leaves the queue; a running
 * one (between gbmd_engine_step calls no kernel of it is in flight) frees
 * its device memory and slot for the next queued job.  The job ends FAILED
 * with error GBMD_ERR_CANCELLED; the other jobs are untouched.  A job that
 * has already finished is an error. */
int gbmd_job_cancel( gbmd_engine *e, int64_t job_id );

/* Forget a finished (DONE or FAILED) job's stored result. */
int gbmd_job_release( gbmd_engine *e, int64_t job_id );

int gbmd_engine_get_stats( const gbmd_engine *e, gbmd_engine_stats *out );

#ifdef __cplusplus
}
#endif

#endif /* GBMD_SERVE_H */
