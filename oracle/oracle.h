/*
 * oracle.h -- FP64 CPU restatement of CabanaMD's per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs may load it.  The product path
 * (libgbmd.so, include/gbmd.h) never calls into it.
 *
 * Parity status: the LJ / neighbour / integrator / thermo semantics below
 * are pinned against the reference's own known-answer tests
 * (unit_test/tstNeighbor.hpp brute-force list, unit_test/tstIntegrator.hpp
 * reversibility), re-run in tests/test_oracle.py.  The reference itself
 * cannot be compiled here (Kokkos, Cabana, MPI, n2p2 absent), so there is no
 * oracle/_ref.  The NNP arithmetic lives in the third-party n2p2 library
 * (v2.0.1, not vendored); the restatement follows the published
 * Behler-Parrinello definitions and is "parity unpinned".
 *
 * All arithmetic that decides a neighbour pair or an integrator update is
 * written so that the compiler may not contract it (built with
 * -ffp-contract=off): the GPU's FP64 path performs the identical IEEE
 * operation sequence, so neighbour sets and integrator updates match bit
 * for bit.
 *
 * Array conventions: positions, velocities and forces are [n][3] row-major
 * doubles; type is 0-based int32; id is 1-based int32.
 */
#ifndef GBMD_ORACLE_H
#define GBMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXTYPES 8

/* Image code of a periodic shift s in {-1,0,1}^3. */
#define ORC_IMG(sx, sy, sz) ((int8_t)(((sx) + 1) + 3 * ((sy) + 1) + 9 * ((sz) + 1)))
#define ORC_IMG_ZERO 13

typedef struct
{
    int nc[3];      /* cells per dimension */
    double h[3];    /* cell edge */
    double lo[3];   /* box low corner */
    double L[3];    /* box extent (global_mesh_x/y/z) */
} orc_grid;

typedef struct
{
    int ntypes;
    double lj1[ORC_MAXTYPES * ORC_MAXTYPES];
    double lj2[ORC_MAXTYPES * ORC_MAXTYPES];
    double cutsq[ORC_MAXTYPES * ORC_MAXTYPES];
} orc_lj;

/* CSR neighbour list over local atoms.  Entry k of atom i is the image
 * (j[k], img[k]) of local atom j[k] shifted by img[k] box lengths. */
typedef struct
{
    int64_t n;
    int64_t *off; /* n + 1 */
    int32_t *j;
    int8_t *img;
} orc_list;

void orc_free( void *p );
void orc_list_free( orc_list *l );

/* Comm::exchange on a single rank: wrap into the periodic box. */
void orc_exchange_self( int64_t n, double *x, const double L[3] );

/* Cell grid used for sorting and list building (cell edge >= cut). */
void orc_make_grid( const double lo[3], const double hi[3], double cut,
                    orc_grid *g );
int64_t orc_cell_index( const orc_grid *g, const double *xi );

/* Binning::create_binning(sort=true): stable order by (cell, id).
 * perm_out (optional, n) receives old index of each new slot. */
void orc_sort_atoms( int64_t n, const orc_grid *g, double *x, double *v,
                     double *f, int32_t *type, int32_t *id,
                     int64_t *perm_out );

/* Comm::exchange_halo on a single rank (6 phases).  Returns the ghost count;
 * *src and *img (malloc'd) give each ghost's source local atom and shift. */
int64_t orc_halo( int64_t n, const double *x, const double lo[3],
                  const double hi[3], double depth, int32_t **src,
                  int8_t **img );

/* Brute-force list (tstNeighbor.hpp:76-141) of the first n of ntot explicit
 * particles (locals first, then ghosts) over all ntot; j indexes x. */
int orc_neigh_brute( int64_t n, int64_t ntot, const double *x, double cut,
                     int half, orc_list *out );

/* Explicit ghost coordinates of orc_halo's (src, img) images: a copy of the
 * source coordinate and one "-= L" or "+= L" per shifted dimension. */
void orc_image_positions( int64_t nghost, const double *x,
                          const int32_t *src, const int8_t *img,
                          const double L[3], double *xg );

/* Cell-stencil list in the canonical order the GPU builder produces. */
int orc_neigh_cells( int64_t n, const double *x, const orc_grid *g,
                     const double hi[3], double depth, double cut, int half,
                     int nthreads, orc_list *out );

/* LJ */
void orc_lj_init( orc_lj *p, int ntypes );
void orc_lj_coeff( orc_lj *p, int i, int j, double eps, double sigma,
                   double cut );
/* Accumulate forces into f (caller zeroes).  Half lists apply Newton's
 * third law to the image's owner (Comm::update_force folded in). */
void orc_lj_force( int64_t n, const double *x, const int32_t *type,
                   const orc_lj *p, const orc_list *l, const double L[3],
                   int half, int nthreads, double *f );
double orc_lj_energy( int64_t n, const double *x, const int32_t *type,
                      const orc_lj *p, const orc_list *l, const double L[3],
                      int half, int nthreads );

/* IntegratorNVE */
void orc_nve_initial( int64_t n, double *x, double *v, const double *f,
                      const int32_t *type, const double *mass, double dt,
                      double mvv2e, int nthreads );
void orc_nve_final( int64_t n, double *v, const double *f,
                    const int32_t *type, const double *mass, double dt,
                    double mvv2e, int nthreads );

/* sum_i m_i |v_i|^2 */
double orc_sum_mv2( int64_t n, const double *v, const int32_t *type,
                    const double *mass, int nthreads );

/* Whole CbnMD::init + CbnMD::run for the LJ force (single rank). */
typedef struct
{
    double force_cut;
    double skin;
    int half;
    int rebuild_every; /* comm_exchange_rate */
    int thermo_every;  /* thermo_rate */
    int nsteps;
    int nthreads;
    double boltz, mvv2e, dt;
    int ntypes;
    double mass[ORC_MAXTYPES];
    int time_from_step;  /* loop_seconds covers steps > time_from_step */
    double loop_seconds; /* output: wall time of the timed steps */
} orc_run_cfg;

/* thermo: rows of (step, T, PE/N, KE/N); returns row count or -1. */
int orc_run_lj( int64_t n, double *x, double *v, double *f, int32_t *type,
                int32_t *id, const double lo[3], const double hi[3],
                const orc_lj *p, orc_run_cfg *cfg, double *thermo,
                int max_rows );

#ifdef __cplusplus
}
#endif
#endif
