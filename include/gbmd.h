/*
 * gbmd.h -- C ABI of the GB300 backend for CabanaMD's per-timestep MD hot
 * path (cell binning + Verlet list, LJ and NNP forces, velocity-Verlet NVE,
 * thermo reductions).
 *
 * Every entry point replaces one call of CabanaMD's C++ module interfaces;
 * the comment above each names the reference interface (path inside the
 * CabanaMD project, file:line).  The reference's interfaces are C++
 * templates with no ABI of their own, so the C++ adapter classes in
 * cabanamd_gb300/host/ implement Force / Neighbor / Integrator / System /
 * Binning / Comm on top of these functions.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Host arrays are [n][3] row-major double
 *    for positions, velocities and forces, int32 for type (0-based) and id.
 *  - Every function returns GBMD_OK (0) or a GBMD_ERR_* code;
 *    gbmd_last_error() returns the message.  Errors are never fatal to the
 *    process: a caller such as the C++ adapter turns them into exceptions,
 *    which is what the reference's log_err does (src/output.h:37-54).
 *  - One context owns every device buffer of one system and one CUDA stream.
 *    Contexts are independent; a context is not thread-safe.
 *  - Nothing here falls back to the CPU: a context cannot be created without
 *    a CUDA device.
 */
#ifndef GBMD_H
#define GBMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes */
#define GBMD_OK 0
#define GBMD_ERR_ARG 1       /* bad argument or call order */
#define GBMD_ERR_CUDA 2      /* CUDA runtime error */
#define GBMD_ERR_CAPACITY 3  /* fixed capacity exceeded (caller may retry) */
#define GBMD_ERR_LOST_ATOM 4 /* atom left the periodic images (NaN or > 1 box) */
#define GBMD_ERR_TIMEOUT 5   /* a bounded device wait gave up */
#define GBMD_ERR_IO 6        /* file read / parse error */
#define GBMD_ERR_NODEVICE 7  /* no CUDA device */
#define GBMD_ERR_CANCELLED 8 /* serving job cancelled (gbmd_serve.h) */

/* Precision modes */
#define GBMD_PREC_FP64 0  /* plain FP64 everywhere (correctness form) */
#define GBMD_PREC_MIXED 1 /* FP32 pair math / symmetry functions, BF16 MLP,
                             FP64 positions, velocities, accumulation */

/* Force types (src/types.h ForceType) */
#define GBMD_FORCE_LJ 0
#define GBMD_FORCE_NNP 1

/* Kernel timers (gbmd_kernel_time) */
#define GBMD_KT_FORCE 0
#define GBMD_KT_NEIGH 1
#define GBMD_KT_SORT 2
#define GBMD_KT_INTEGRATE 3
#define GBMD_KT_THERMO 4
#define GBMD_KT_NNP_SF 5
#define GBMD_KT_NNP_MLP 6
#define GBMD_KT_NNP_FORCE 7
#define GBMD_KT_COUNT 8

typedef struct gbmd_ctx gbmd_ctx;

/* Parameters of the CbnMD timestep loop (src/cabanamd_impl.h:70-399;
 * input deck: pair_style cutoff, neighbor skin, neigh_modify every/one,
 * thermo, newton on|off). */
typedef struct
{
    double force_cut;     /* pair cutoff (largest over type pairs) */
    double skin;          /* neighbor skin; list cutoff = force_cut + skin */
    int half;             /* 1: half list + Newton 3 (newton on) */
    int rebuild_every;    /* comm_exchange_rate (neigh_modify every) */
    int thermo_every;     /* thermo_rate; 0 disables thermo */
    int max_neigh_guess;  /* neigh_modify one; grown automatically */
} gbmd_md_params;

/* ---- context (CbnMD owns System/modules: src/cabanamd.h:82-88) ---- */
int gbmd_create( gbmd_ctx **out, int device );
void gbmd_destroy( gbmd_ctx *ctx );
const char *gbmd_last_error( const gbmd_ctx *ctx );
int gbmd_version( void );

/* ---- System (src/system.h:65-136) ---- */
/* units: src/inputFile_impl.h:146-182 */
int gbmd_set_units( gbmd_ctx *ctx, double boltz, double mvv2e, double dt );
/* global mesh low/high corners: SystemCommon::create_domain, system.h:143-192 */
int gbmd_set_box( gbmd_ctx *ctx, const double lo[3], const double hi[3] );
/* ntypes + System::mass (system.h:81-85) */
int gbmd_set_types( gbmd_ctx *ctx, int ntypes, const double *mass );
int gbmd_set_precision( gbmd_ctx *ctx, int precision );
/* System::resize + deep_copy from host (inputFile_impl.h:791,849,865;
 * read_data.h:164-275).  Host arrays are copied; any may not be NULL except
 * v (zero velocities). */
int gbmd_upload_atoms( gbmd_ctx *ctx, int64_t n, const double *x,
                       const double *v, const int32_t *type,
                       const int32_t *id );
/* Page-lock (pin) and map caller-owned host memory; no reference
 * counterpart (the reference's deep_copy of its host mirrors,
 * inputFile_impl.h:849,865).  gbmd_upload_atoms / gbmd_download_atoms read
 * and write arrays that lie wholly inside one range registered here in place,
 * with one kernel each over the host link; other arrays go through staged
 * copies.  Register the host mirrors once, before the run; registering a
 * range that is already registered elsewhere is not an error (it is then
 * pinned but moved by copies).  Unregister before freeing. */
int gbmd_host_register( const void *p, size_t bytes );
int gbmd_host_unregister( const void *p );
/* deep_copy to host in the current (cell-sorted) order; NULL skips. */
int gbmd_download_atoms( gbmd_ctx *ctx, double *x, double *v, double *f,
                         int32_t *type, int32_t *id );
int gbmd_num_atoms( const gbmd_ctx *ctx, int64_t *n );

/* ---- Comm, single rank (src/comm_mpi.h:141-168, comm_mpi_impl.h:191-278) */
/* Comm::exchange: wrap positions into the periodic box. */
int gbmd_exchange( gbmd_ctx *ctx );

/* ---- Binning (src/binning_cabana.h:64-66, binning_cabana_impl.h:57-113) */
/* Binning::create_binning(..., sort=true): counting sort by cell (edge >=
 * neigh_cut), stable by id inside a cell; permutes x, v, type, id. */
int gbmd_binning( gbmd_ctx *ctx, double neigh_cut );

/* ---- Neighbor (src/neighbor.h:54-75, neighbor_types/neighbor_verlet.h:43-62)
 * Neighbor::create: Verlet list of every local atom over all periodic
 * images within neigh_cut (Comm::exchange_halo's ghost set,
 * comm_mpi.h:241-353), d^2 <= neigh_cut^2.  half=1 keeps a pair only at the
 * atom whose partner image is lexicographically greater (x, y, z).  Needs a
 * prior gbmd_binning with the same cut. */
int gbmd_neigh_build( gbmd_ctx *ctx, double neigh_cut, int half,
                      int max_neigh_guess );
/* Periodic images in the lists built from now on (every gbmd_neigh_build,
 * and the rebuilds of gbmd_md_init / gbmd_md_run).  periodic = 1 (default):
 * the Verlet lists above.  periodic = 0: the pairs among the atoms
 * themselves, no images -- what CabanaMD's tree lists hold
 * (neighbor_types/neighbor_tree.h:43-58: makeNeighborList over the N_local
 * atoms, without the ghosts), for vacuum or open systems (--vacuum,
 * inputFile_impl.h:553-559). */
int gbmd_set_list_images( gbmd_ctx *ctx, int periodic );
/* List size: total entries and the largest per-atom count
 * (NeighborList::maxNeighbor, neighbor_verlet.h:58-61). */
int gbmd_neigh_size( gbmd_ctx *ctx, int64_t *total, int32_t *max_count );
/* Copy the list to host CSR form: counts[n]; j_out/img_out[total] hold
 * the partner's current index and its image code (sx+1)+3(sy+1)+9(sz+1). */
int gbmd_neigh_download( gbmd_ctx *ctx, int32_t *counts, int32_t *j_out,
                         int8_t *img_out );

/* ---- Force (src/force.h:57-74) ---- */
/* ForceLJ::init_coeff row "pair_coeff i j eps sigma cut" (1-based types,
 * force_lj_cabana_neigh_impl.h:62-89). */
int gbmd_lj_coeff( gbmd_ctx *ctx, int itype, int jtype, double eps,
                   double sigma, double cut );
int gbmd_set_force_type( gbmd_ctx *ctx, int force_type );
/* f = 0 (cabanamd_impl.h:336-338) */
int gbmd_zero_force( gbmd_ctx *ctx );
/* Force::compute: accumulate forces (Newton 3 folded into the owner of each
 * image, i.e. Comm::update_force is included). */
int gbmd_force_compute( gbmd_ctx *ctx );
/* Force::compute_energy: total potential energy (not divided by N). */
int gbmd_force_energy( gbmd_ctx *ctx, double *pe );

/* ---- Integrator (src/integrator_nve.h:56-111) ---- */
int gbmd_integrate_initial( gbmd_ctx *ctx );
int gbmd_integrate_final( gbmd_ctx *ctx );

/* v *= factor for every atom (the velocity rescale of create_lattice,
 * src/inputFile_impl.h:854-864, and the velocity reversal of
 * unit_test/tstIntegrator.hpp:106-113). */
int gbmd_scale_velocities( gbmd_ctx *ctx, double factor );

/* ---- Thermo (src/property_temperature_impl.h:55-77,
 *      property_kine_impl.h:55-76): T and total KE. */
int gbmd_thermo( gbmd_ctx *ctx, double *temperature, double *kinetic );

/* Temperature and kinetic energy without allocating any GPU memory.
 * No counterpart in the reference: this is an extra entry point for callers
 * that cannot call cudaMalloc -- hosts that own all device memory through
 * their own pool and forbid other allocations, real-time loops that must
 * stay out of the driver's allocator (its calls can block).  It computes
 * what gbmd_thermo computes, from caller-owned device arrays: v_dev is
 * [3][n] (all x, then all y, then all z), type_dev [n] 0-based, mass_dev
 * [ntypes]; out_dev[0] receives T and out_dev[1] the total kinetic energy.
 * Work is queued on `stream` (a cudaStream_t; NULL = legacy default
 * stream) and nothing is synchronised.
 * Limits and sharing: the partial sums live in one fixed 512 KiB device
 * array per GPU, held for as long as the library is loaded, so n must be at
 * most 16,777,216 (GBMD_ERR_CAPACITY otherwise).  All calls share that
 * array: calls whose kernels overlap on the GPU race and return wrong
 * values, so serialise them.  The first call on each device looks the
 * array's address up (cudaGetSymbolAddress) with that device current; make
 * that first call before starting any stream capture.  A CUDA error already
 * pending in the calling thread makes the call return GBMD_ERR_CUDA before
 * it launches anything, and the error is left pending for its owner. */
int gbmd_thermo_noalloc( const double *v_dev, const int32_t *type_dev,
                         const double *mass_dev, int64_t n, double mvv2e,
                         double boltz, void *stream, double *out_dev );

/* ---- Whole timestep loop (CbnMD::init/run, src/cabanamd_impl.h:70-399) */
/* init: wrap, sort, list, f = 0, force; writes the step-0 thermo row
 * (step, T, PE/N, KE/N) into thermo0[4] when thermo_every > 0. */
int gbmd_md_init( gbmd_ctx *ctx, const gbmd_md_params *p, double *thermo0 );
/* run nsteps further steps; thermo rows (step, T, PE/N, KE/N) for every
 * step % thermo_every == 0 go to thermo[max_rows][4]. */
int gbmd_md_run( gbmd_ctx *ctx, int nsteps, double *thermo, int max_rows,
                 int *nrows );
int gbmd_md_step_count( const gbmd_ctx *ctx, int64_t *step );
/* Device time of the last gbmd_md_run (CUDA events recorded on the context
 * stream around the whole loop) and how many kernels it launched.  The
 * reference reports Atomsteps/s = N * nsteps / loop time
 * (src/cabanamd_impl.h:401-420). */
int gbmd_md_last_run( const gbmd_ctx *ctx, double *device_ms,
                      int64_t *launches );
/* CUDA graphs in gbmd_md_run (CbnMD::run's step loop, cabanamd_impl.h:
 * 284-399; on by default): between thermo steps and list rebuilds the steps
 * (fused LJ steps; force + integrator launches for NNP and half lists) are
 * captured once per run of steps and replayed, keyed on every launch
 * argument, so a changed dt, coefficient, potential or buffer captures
 * anew.  Results are bit-identical to direct launches.  gbmd_graph_replays
 * counts graph launches since the context was created. */
int gbmd_set_graphs( gbmd_ctx *ctx, int on );
int gbmd_graph_replays( const gbmd_ctx *ctx, int64_t *replays );

/* ---- Tile shapes (no reference counterpart: CabanaMD fixes its Kokkos
 * team and vector sizes at compile time, src/CMakeLists.txt) ----
 * The kernels are compiled for a few tile shapes: LJ atoms per block
 * (64, 128, 256) with, in mixed precision, the list rows' L2 prefetch
 * distance, and the list build's home cells per block x list slots per lane
 * staged in shared memory ((12, 32), (8, 32), (16, 24), (8, 48)).  No shape
 * changes a result.  mode 1 (the default): gbmd_md_init times the
 * candidates on the system after its first list build and keeps the fastest,
 * cached for the process per class of system (force, precision, list kind,
 * size and density classes).  mode 0: the shapes stay as set. */
int gbmd_set_tuning( gbmd_ctx *ctx, int mode );
/* Fix the shapes (and switch tuning off): lj_threads 64 | 128 | 256,
 * lj_prefetch 0..64 rows, (nb_warps, nb_out) one of the pairs above. */
int gbmd_set_shapes( gbmd_ctx *ctx, int lj_threads, int lj_prefetch, int nb_warps,
                     int nb_out );
/* shapes[5]: lj_threads, lj_prefetch, nb_warps, nb_out, and 1 when the
 * autotuner chose them (0: defaults or set by gbmd_set_shapes). */
int gbmd_get_shapes( const gbmd_ctx *ctx, int *shapes );

/* ---- NNP (src/force_types/force_nnp_cabana_neigh_impl.h:41-130) ---- */
/* ForceNNP::init_coeff: load input.nn, scaling.data and weights.%03d.data
 * from directory dir (n2p2 file formats).  cflength / cfenergy are the
 * pair_style unit conversions. */
int gbmd_nnp_load( gbmd_ctx *ctx, const char *dir, double cflength,
                   double cfenergy );
/* Per-atom symmetry functions G[n][nsf] (raw, unscaled) and energies E[n]
 * of the last force evaluation, for testing; NULL skips. */
int gbmd_nnp_download( gbmd_ctx *ctx, double *G, double *E, int *nsf );

/* ---- Kernel timing (CUDA events on the context stream) ---- */
int gbmd_set_profiling( gbmd_ctx *ctx, int on );
int gbmd_kernel_time( gbmd_ctx *ctx, int which, double *ms_total,
                      int64_t *launches );
int gbmd_synchronize( gbmd_ctx *ctx );

/* ---- Failure detection ----
 * Every device-side wait (the mbarrier waits of the tensor-core MLP) is
 * bounded: on expiry the kernel sets a context flag, frees what it holds and
 * returns, and the next call that reads the flags returns GBMD_ERR_TIMEOUT;
 * gbmd_md_init clears the flags.  This call runs that path on purpose: one
 * CTA waits on an mbarrier that nothing arrives on, for at most `seconds`
 * (clamped to 0.001 .. 2) of SM clock, then reports GBMD_ERR_TIMEOUT with
 * the context still usable.  No fault, no unbounded wait. */
int gbmd_check_bounded_wait( gbmd_ctx *ctx, double seconds );

#ifdef __cplusplus
}
#endif
#endif
