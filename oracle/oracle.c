/*
 * oracle.c -- FP64 CPU restatement of CabanaMD's per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Build with -ffp-contract=off.
 *
 * Reference files followed (paths inside the CabanaMD project):
 *   wrap            src/comm_mpi.h:141-168 (TagExchangeSelf)
 *   halo / images   src/comm_mpi.h:241-353, src/comm_mpi_impl.h:280-441
 *   sort            src/binning_cabana_impl.h:57-113
 *   lists           unit_test/tstNeighbor.hpp:76-141 (d^2 <= rc^2, self
 *                   excluded), src/neighbor_types/neighbor_verlet.h:43-62;
 *                   half-list ownership from Cabana 0.6.1's VerletList
 *                   (third-party, not vendored): a pair (p, n) is stored
 *                   at p only when n's coordinates are lexicographically
 *                   greater than p's (x, then y, then z).
 *   LJ              src/force_types/force_lj_cabana_neigh_impl.h:62-89,151-377
 *   NVE             src/integrator_nve.h:91-110, src/integrator_nve_impl.h:49-54
 *   thermo          src/property_kine_impl.h:55-76,
 *                   src/property_temperature_impl.h:55-77
 *   step order      src/cabanamd_impl.h:70-255 (init), 284-399 (run)
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

void orc_free( void *p ) { free( p ); }

static double wall_seconds( void )
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

void orc_list_free( orc_list *l )
{
    if ( !l )
        return;
    free( l->off );
    free( l->j );
    free( l->img );
    l->off = NULL;
    l->j = NULL;
    l->img = NULL;
    l->n = 0;
}

static inline int img_s( int8_t code, int d )
{
    int c = code;
    for ( int k = 0; k < d; k++ )
        c /= 3;
    return c % 3 - 1;
}

/* Position of an image: the reference's ghost gets a copy of its source's
 * coordinate and then one "x -= L" or "x += L" (comm_mpi.h:324-353). */
static inline double img_coord( double xs, int s, double L )
{
    if ( s < 0 )
        return xs - L;
    if ( s > 0 )
        return xs + L;
    return xs;
}

/* comm_mpi.h:141-168 -- each test uses the coordinate before wrapping. */
void orc_exchange_self( int64_t n, double *x, const double L[3] )
{
    for ( int64_t i = 0; i < n; i++ )
        for ( int d = 0; d < 3; d++ )
        {
            const double x1 = x[3 * i + d];
            if ( x1 > L[d] )
                x[3 * i + d] -= L[d];
            if ( x1 < 0 )
                x[3 * i + d] += L[d];
        }
}

void orc_make_grid( const double lo[3], const double hi[3], double cut,
                    orc_grid *g )
{
    for ( int d = 0; d < 3; d++ )
    {
        g->lo[d] = lo[d];
        g->L[d] = hi[d] - lo[d];
        int nc = (int)floor( g->L[d] / ( cut * ( 1.0 + 1e-10 ) ) );
        if ( nc < 1 )
            nc = 1;
        g->nc[d] = nc;
        g->h[d] = g->L[d] / nc;
    }
}

static inline int cell_1d( const orc_grid *g, double xd, int d )
{
    double t = floor( ( xd - g->lo[d] ) / g->h[d] );
    int c = ( t < 0.0 ) ? 0 : ( t > (double)( g->nc[d] - 1 ) ? g->nc[d] - 1 : (int)t );
    return c;
}

int64_t orc_cell_index( const orc_grid *g, const double *xi )
{
    int cx = cell_1d( g, xi[0], 0 );
    int cy = cell_1d( g, xi[1], 1 );
    int cz = cell_1d( g, xi[2], 2 );
    return (int64_t)cx + (int64_t)g->nc[0] * ( cy + (int64_t)g->nc[1] * cz );
}

typedef struct
{
    int64_t key;
    int32_t id;
    int64_t idx;
} sort_item;

static int cmp_item( const void *a, const void *b )
{
    const sort_item *p = (const sort_item *)a, *q = (const sort_item *)b;
    if ( p->key != q->key )
        return p->key < q->key ? -1 : 1;
    if ( p->id != q->id )
        return p->id < q->id ? -1 : 1;
    return ( p->idx < q->idx ) ? -1 : ( p->idx > q->idx );
}

static void permute_d3( int64_t n, double *a, const sort_item *it )
{
    if ( !a )
        return;
    double *t = (double *)malloc( sizeof( double ) * 3 * n );
    for ( int64_t k = 0; k < n; k++ )
        memcpy( t + 3 * k, a + 3 * it[k].idx, 3 * sizeof( double ) );
    memcpy( a, t, sizeof( double ) * 3 * n );
    free( t );
}

static void permute_i( int64_t n, int32_t *a, const sort_item *it )
{
    if ( !a )
        return;
    int32_t *t = (int32_t *)malloc( sizeof( int32_t ) * n );
    for ( int64_t k = 0; k < n; k++ )
        t[k] = a[it[k].idx];
    memcpy( a, t, sizeof( int32_t ) * n );
    free( t );
}

/* binning_cabana_impl.h:57-113 sorts local atoms into cell order and
 * permutes every per-atom array.  Order inside a cell is by id, which makes
 * the permutation deterministic on every backend. */
void orc_sort_atoms( int64_t n, const orc_grid *g, double *x, double *v,
                     double *f, int32_t *type, int32_t *id,
                     int64_t *perm_out )
{
    sort_item *it = (sort_item *)malloc( sizeof( sort_item ) * ( n ? n : 1 ) );
    for ( int64_t i = 0; i < n; i++ )
    {
        it[i].key = orc_cell_index( g, x + 3 * i );
        it[i].id = id ? id[i] : (int32_t)i;
        it[i].idx = i;
    }
    qsort( it, (size_t)n, sizeof( sort_item ), cmp_item );
    permute_d3( n, x, it );
    permute_d3( n, v, it );
    permute_d3( n, f, it );
    permute_i( n, type, it );
    permute_i( n, id, it );
    if ( perm_out )
        for ( int64_t k = 0; k < n; k++ )
            perm_out[k] = it[k].idx;
    free( it );
}

/* comm_mpi_impl.h:280-367 with the pack test of comm_mpi.h:240-319 and the
 * periodic shift of comm_mpi.h:324-353, on a single rank (every phase sends
 * to itself).  Phase p looks at locals plus the ghosts made by earlier
 * phases, except that an odd phase skips the ghosts of the phase just
 * before it. */
int64_t orc_halo( int64_t n, const double *x, const double lo[3],
                  const double hi[3], double depth, int32_t **src_out,
                  int8_t **img_out )
{
    int64_t cap = n + 16, ng = 0;
    int32_t *src = (int32_t *)malloc( sizeof( int32_t ) * cap );
    int8_t *sh = (int8_t *)malloc( 3 * cap ); /* per-dim shift */
    double *gx = (double *)malloc( sizeof( double ) * 3 * cap );
    int64_t recv_prev = 0;
    for ( int phase = 0; phase < 6; phase++ )
    {
        const int d = phase / 2;
        const int64_t total = n + ng;
        const int64_t np = total - ( ( phase % 2 == 1 ) ? recv_prev : 0 );
        int64_t count = 0;
        for ( int64_t p = 0; p < np; p++ )
        {
            const double *xp = ( p < n ) ? x + 3 * p : gx + 3 * ( p - n );
            int sel = ( phase % 2 == 0 ) ? ( xp[d] >= hi[d] - depth )
                                         : ( xp[d] <= lo[d] + depth );
            if ( !sel )
                continue;
            if ( ng + 1 > cap )
            {
                cap = cap * 2;
                src = (int32_t *)realloc( src, sizeof( int32_t ) * cap );
                sh = (int8_t *)realloc( sh, 3 * cap );
                gx = (double *)realloc( gx, sizeof( double ) * 3 * cap );
            }
            const int64_t gnew = ng;
            if ( p < n )
            {
                src[gnew] = (int32_t)p;
                sh[3 * gnew] = sh[3 * gnew + 1] = sh[3 * gnew + 2] = 0;
            }
            else
            {
                src[gnew] = src[p - n];
                memcpy( sh + 3 * gnew, sh + 3 * ( p - n ), 3 );
            }
            memcpy( gx + 3 * gnew, xp, 3 * sizeof( double ) );
            /* Single rank: proc_pos == 0 == proc_grid - 1. */
            if ( phase % 2 == 0 )
            {
                gx[3 * gnew + d] -= hi[d] - lo[d];
                sh[3 * gnew + d] = -1;
            }
            else
            {
                gx[3 * gnew + d] += hi[d] - lo[d];
                sh[3 * gnew + d] = 1;
            }
            ng++;
            count++;
        }
        recv_prev = count;
    }
    int8_t *img = (int8_t *)malloc( ng ? ng : 1 );
    for ( int64_t g = 0; g < ng; g++ )
        img[g] = ORC_IMG( sh[3 * g], sh[3 * g + 1], sh[3 * g + 2] );
    free( sh );
    free( gx );
    *src_out = src;
    *img_out = img;
    return ng;
}

void orc_image_positions( int64_t nghost, const double *x,
                          const int32_t *src, const int8_t *img,
                          const double L[3], double *xg )
{
    for ( int64_t g = 0; g < nghost; g++ )
        for ( int d = 0; d < 3; d++ )
            xg[3 * g + d] =
                img_coord( x[3 * src[g] + d], img_s( img[g], d ), L[d] );
}

static inline int half_keep( const double *xp, const double *xn )
{
    return ( xn[0] > xp[0] ) ||
           ( ( xn[0] == xp[0] ) &&
             ( ( xn[1] > xp[1] ) || ( ( xn[1] == xp[1] ) && ( xn[2] > xp[2] ) ) ) );
}

static inline double dist2( const double *a, const double *b )
{
    const double dx = a[0] - b[0];
    const double dy = a[1] - b[1];
    const double dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;
}

/* unit_test/tstNeighbor.hpp:76-141: every particle p != i with
 * d^2 <= cut^2, lists for the first nlocal particles only. */
int orc_neigh_brute( int64_t n, int64_t ntot, const double *x, double cut,
                     int half, orc_list *out )
{
    const double rsq = cut * cut;
    int64_t *off = (int64_t *)calloc( n + 1, sizeof( int64_t ) );
    int64_t cap = 1024, cnt = 0;
    int32_t *jj = (int32_t *)malloc( sizeof( int32_t ) * cap );
    int8_t *im = (int8_t *)malloc( cap );
    for ( int64_t i = 0; i < n; i++ )
    {
        const double *xi = x + 3 * i;
        for ( int64_t p = 0; p < ntot; p++ )
        {
            if ( p == i )
                continue;
            const double *xn = x + 3 * p;
            if ( dist2( xi, xn ) <= rsq )
            {
                if ( half && !half_keep( xi, xn ) )
                    continue;
                if ( cnt == cap )
                {
                    cap *= 2;
                    jj = (int32_t *)realloc( jj, sizeof( int32_t ) * cap );
                    im = (int8_t *)realloc( im, cap );
                }
                jj[cnt] = (int32_t)p;
                im[cnt] = ORC_IMG_ZERO;
                cnt++;
            }
        }
        off[i + 1] = cnt;
    }
    out->n = n;
    out->off = off;
    out->j = jj;
    out->img = im;
    return 0;
}

/* Walk the 27 (cell, shift) stencil of atom i in the canonical order
 * (dz, dy, dx nested, dx fastest; atoms of a cell in sorted order). */
typedef struct
{
    const double *x;
    const orc_grid *g;
    const int64_t *cstart; /* ncell + 1 */
    double thr_hi[3], thr_lo[3];
    double rsq;
    int half;
} cell_ctx;

static int64_t walk_atom( const cell_ctx *c, int64_t i, int32_t *jj,
                          int8_t *im )
{
    const orc_grid *g = c->g;
    const double *xi = c->x + 3 * i;
    int ci[3];
    for ( int d = 0; d < 3; d++ )
        ci[d] = cell_1d( g, xi[d], d );
    int64_t cnt = 0;
    for ( int dz = -1; dz <= 1; dz++ )
        for ( int dy = -1; dy <= 1; dy++ )
            for ( int dx = -1; dx <= 1; dx++ )
            {
                const int dd[3] = { dx, dy, dz };
                int cc[3], s[3];
                for ( int d = 0; d < 3; d++ )
                {
                    int t = ci[d] + dd[d];
                    s[d] = ( t < 0 ) ? -1 : ( t >= g->nc[d] ? 1 : 0 );
                    cc[d] = t - s[d] * g->nc[d];
                }
                const int64_t cell =
                    cc[0] + (int64_t)g->nc[0] * ( cc[1] + (int64_t)g->nc[1] * cc[2] );
                const int8_t code = ORC_IMG( s[0], s[1], s[2] );
                for ( int64_t j = c->cstart[cell]; j < c->cstart[cell + 1]; j++ )
                {
                    if ( j == i && code == ORC_IMG_ZERO )
                        continue;
                    const double *xj = c->x + 3 * j;
                    int ok = 1;
                    for ( int d = 0; d < 3; d++ )
                    {
                        if ( s[d] < 0 && !( xj[d] >= c->thr_hi[d] ) )
                            ok = 0;
                        if ( s[d] > 0 && !( xj[d] <= c->thr_lo[d] ) )
                            ok = 0;
                    }
                    if ( !ok )
                        continue;
                    double xn[3];
                    for ( int d = 0; d < 3; d++ )
                        xn[d] = img_coord( xj[d], s[d], g->L[d] );
                    if ( !( dist2( xi, xn ) <= c->rsq ) )
                        continue;
                    if ( c->half && !half_keep( xi, xn ) )
                        continue;
                    if ( jj )
                    {
                        jj[cnt] = (int32_t)j;
                        im[cnt] = code;
                    }
                    cnt++;
                }
            }
    return cnt;
}

int orc_neigh_cells( int64_t n, const double *x, const orc_grid *g,
                     const double hi[3], double depth, double cut, int half,
                     int nthreads, orc_list *out )
{
    const int64_t ncell = (int64_t)g->nc[0] * g->nc[1] * g->nc[2];
    int64_t *cstart = (int64_t *)calloc( ncell + 1, sizeof( int64_t ) );
    int64_t prev = -1;
    for ( int64_t i = 0; i < n; i++ )
    {
        int64_t k = orc_cell_index( g, x + 3 * i );
        if ( k < prev )
        {
            free( cstart );
            return -1; /* atoms are not in cell order */
        }
        prev = k;
        cstart[k + 1]++;
    }
    for ( int64_t k = 0; k < ncell; k++ )
        cstart[k + 1] += cstart[k];
    cell_ctx c;
    c.x = x;
    c.g = g;
    c.cstart = cstart;
    c.rsq = cut * cut;
    c.half = half;
    for ( int d = 0; d < 3; d++ )
    {
        c.thr_hi[d] = hi[d] - depth;
        c.thr_lo[d] = g->lo[d] + depth;
    }
    int64_t *off = (int64_t *)calloc( n + 1, sizeof( int64_t ) );
    (void)nthreads;
#pragma omp parallel for schedule( dynamic, 256 ) num_threads( nthreads > 0 ? nthreads : 1 )
    for ( int64_t i = 0; i < n; i++ )
        off[i + 1] = walk_atom( &c, i, NULL, NULL );
    for ( int64_t i = 0; i < n; i++ )
        off[i + 1] += off[i];
    const int64_t tot = off[n];
    int32_t *jj = (int32_t *)malloc( sizeof( int32_t ) * ( tot ? tot : 1 ) );
    int8_t *im = (int8_t *)malloc( tot ? tot : 1 );
#pragma omp parallel for schedule( dynamic, 256 ) num_threads( nthreads > 0 ? nthreads : 1 )
    for ( int64_t i = 0; i < n; i++ )
        walk_atom( &c, i, jj + off[i], im + off[i] );
    free( cstart );
    out->n = n;
    out->off = off;
    out->j = jj;
    out->img = im;
    return 0;
}

/* force_lj_cabana_neigh_impl.h:62-89 */
void orc_lj_init( orc_lj *p, int ntypes )
{
    memset( p, 0, sizeof( *p ) );
    p->ntypes = ntypes;
}

void orc_lj_coeff( orc_lj *p, int i, int j, double eps, double sigma,
                   double cut )
{
    const int T = ORC_MAXTYPES;
    p->lj1[i * T + j] = 48.0 * eps * pow( sigma, 12.0 );
    p->lj2[i * T + j] = 24.0 * eps * pow( sigma, 6.0 );
    p->cutsq[i * T + j] = cut * cut;
    p->lj1[j * T + i] = p->lj1[i * T + j];
    p->lj2[j * T + i] = p->lj2[i * T + j];
    p->cutsq[j * T + i] = p->cutsq[i * T + j];
}

/* force_lj_cabana_neigh_impl.h:151-259.  For each list entry the reference
 * adds (fxi, fyi, fzi) -- zero when rsq >= cutsq -- into f(i); the half list
 * also subtracts the pair force from the image, whose force
 * Comm::update_force later adds to the owner. */
void orc_lj_force( int64_t n, const double *x, const int32_t *type,
                   const orc_lj *p, const orc_list *l, const double L[3],
                   int half, int nthreads, double *f )
{
    const int T = ORC_MAXTYPES;
    (void)nthreads;
#pragma omp parallel for schedule( static ) num_threads( nthreads > 0 ? nthreads : 1 ) if ( !half || nthreads > 1 )
    for ( int64_t i = 0; i < n; i++ )
    {
        const double x_i = x[3 * i], y_i = x[3 * i + 1], z_i = x[3 * i + 2];
        const int ti = type[i];
        for ( int64_t k = l->off[i]; k < l->off[i + 1]; k++ )
        {
            const int32_t j = l->j[k];
            const int8_t code = l->img[k];
            const double dx = x_i - img_coord( x[3 * j], img_s( code, 0 ), L[0] );
            const double dy = y_i - img_coord( x[3 * j + 1], img_s( code, 1 ), L[1] );
            const double dz = z_i - img_coord( x[3 * j + 2], img_s( code, 2 ), L[2] );
            const int tj = type[j];
            const double rsq = dx * dx + dy * dy + dz * dz;
            double fxi = 0.0, fyi = 0.0, fzi = 0.0;
            if ( rsq < p->cutsq[ti * T + tj] )
            {
                const double lj1 = p->lj1[ti * T + tj];
                const double lj2 = p->lj2[ti * T + tj];
                const double r2inv = 1.0 / rsq;
                const double r6inv = r2inv * r2inv * r2inv;
                const double fpair = ( r6inv * ( lj1 * r6inv - lj2 ) ) * r2inv;
                fxi += dx * fpair;
                fyi += dy * fpair;
                fzi += dz * fpair;
                if ( half )
                {
                    const double ax = dx * fpair, ay = dy * fpair, az = dz * fpair;
#pragma omp atomic
                    f[3 * j] -= ax;
#pragma omp atomic
                    f[3 * j + 1] -= ay;
#pragma omp atomic
                    f[3 * j + 2] -= az;
                }
            }
            if ( half )
            {
#pragma omp atomic
                f[3 * i] += fxi;
#pragma omp atomic
                f[3 * i + 1] += fyi;
#pragma omp atomic
                f[3 * i + 2] += fzi;
            }
            else
            {
                f[3 * i] += fxi;
                f[3 * i + 1] += fyi;
                f[3 * i + 2] += fzi;
            }
        }
    }
}

/* force_lj_cabana_neigh_impl.h:261-377 (shift_flag is always true). */
double orc_lj_energy( int64_t n, const double *x, const int32_t *type,
                      const orc_lj *p, const orc_list *l, const double L[3],
                      int half, int nthreads )
{
    const int T = ORC_MAXTYPES;
    double PE = 0.0;
    (void)nthreads;
#pragma omp parallel for schedule( static ) num_threads( nthreads > 0 ? nthreads : 1 ) reduction( + : PE )
    for ( int64_t i = 0; i < n; i++ )
    {
        const double x_i = x[3 * i], y_i = x[3 * i + 1], z_i = x[3 * i + 2];
        const int ti = type[i];
        double pe = 0.0;
        for ( int64_t k = l->off[i]; k < l->off[i + 1]; k++ )
        {
            const int32_t j = l->j[k];
            const int8_t code = l->img[k];
            const double dx = x_i - img_coord( x[3 * j], img_s( code, 0 ), L[0] );
            const double dy = y_i - img_coord( x[3 * j + 1], img_s( code, 1 ), L[1] );
            const double dz = z_i - img_coord( x[3 * j + 2], img_s( code, 2 ), L[2] );
            const int tj = type[j];
            const double rsq = dx * dx + dy * dy + dz * dz;
            const double cutsq = p->cutsq[ti * T + tj];
            if ( rsq < cutsq )
            {
                const double lj1 = p->lj1[ti * T + tj];
                const double lj2 = p->lj2[ti * T + tj];
                const double r2inv = 1.0 / rsq;
                const double r6inv = r2inv * r2inv * r2inv;
                const double r2invc = 1.0 / cutsq;
                const double r6invc = r2invc * r2invc * r2invc;
                if ( !half )
                {
                    pe += 0.5 * r6inv * ( 0.5 * lj1 * r6inv - lj2 ) / 6.0;
                    pe -= 0.5 * r6invc * ( 0.5 * lj1 * r6invc - lj2 ) / 6.0;
                }
                else
                {
                    const double fac = ( code == ORC_IMG_ZERO ) ? 1.0 : 0.5;
                    pe += fac * r6inv * ( 0.5 * lj1 * r6inv - lj2 ) / 6.0;
                    pe -= fac * r6invc * ( 0.5 * lj1 * r6invc - lj2 ) / 6.0;
                }
            }
        }
        PE += pe;
    }
    return PE;
}

/* integrator_nve.h:91-110, integrator_nve_impl.h:49-54 */
void orc_nve_initial( int64_t n, double *x, double *v, const double *f,
                      const int32_t *type, const double *mass, double dt,
                      double mvv2e, int nthreads )
{
    const double dtf = 0.5 * dt / mvv2e;
    const double dtv = dt;
    (void)nthreads;
#pragma omp parallel for schedule( static ) num_threads( nthreads > 0 ? nthreads : 1 )
    for ( int64_t i = 0; i < n; i++ )
    {
        const double dtfm = dtf / mass[type[i]];
        v[3 * i] += dtfm * f[3 * i];
        v[3 * i + 1] += dtfm * f[3 * i + 1];
        v[3 * i + 2] += dtfm * f[3 * i + 2];
        x[3 * i] += dtv * v[3 * i];
        x[3 * i + 1] += dtv * v[3 * i + 1];
        x[3 * i + 2] += dtv * v[3 * i + 2];
    }
}

void orc_nve_final( int64_t n, double *v, const double *f,
                    const int32_t *type, const double *mass, double dt,
                    double mvv2e, int nthreads )
{
    const double dtf = 0.5 * dt / mvv2e;
    (void)nthreads;
#pragma omp parallel for schedule( static ) num_threads( nthreads > 0 ? nthreads : 1 )
    for ( int64_t i = 0; i < n; i++ )
    {
        const double dtfm = dtf / mass[type[i]];
        v[3 * i] += dtfm * f[3 * i];
        v[3 * i + 1] += dtfm * f[3 * i + 1];
        v[3 * i + 2] += dtfm * f[3 * i + 2];
    }
}

/* property_kine.h:72-78 */
double orc_sum_mv2( int64_t n, const double *v, const int32_t *type,
                    const double *mass, int nthreads )
{
    double s = 0.0;
    (void)nthreads;
#pragma omp parallel for schedule( static ) num_threads( nthreads > 0 ? nthreads : 1 ) reduction( + : s )
    for ( int64_t i = 0; i < n; i++ )
        s += ( v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
               v[3 * i + 2] * v[3 * i + 2] ) *
             mass[type[i]];
    return s;
}

static void thermo_row( int64_t n, const double *x, const double *v,
                        const int32_t *type, const orc_lj *p,
                        const orc_list *l, const double L[3],
                        const orc_run_cfg *cfg, int step, double *row )
{
    const double smv2 = orc_sum_mv2( n, v, type, cfg->mass, cfg->nthreads );
    /* property_temperature_impl.h:66-76, property_kine_impl.h:66-75 */
    const int64_t dof = 3 * n - 3;
    const double T = smv2 * ( cfg->mvv2e / ( 1.0 * dof * cfg->boltz ) );
    const double KE = smv2 * ( 0.5 * cfg->mvv2e );
    const double PE = orc_lj_energy( n, x, type, p, l, L, cfg->half, cfg->nthreads );
    row[0] = step;
    row[1] = T;
    row[2] = PE / n;
    row[3] = KE / n;
}

/* cabanamd_impl.h:70-255 (init) and 284-399 (run), one rank, LJ force. */
int orc_run_lj( int64_t n, double *x, double *v, double *f, int32_t *type,
                int32_t *id, const double lo[3], const double hi[3],
                const orc_lj *p, orc_run_cfg *cfg, double *thermo,
                int max_rows )
{
    const double neigh_cut = cfg->force_cut + cfg->skin;
    double t_start = 0.0;
    cfg->loop_seconds = 0.0;
    orc_grid g;
    orc_make_grid( lo, hi, neigh_cut, &g );
    const double *L = g.L;
    orc_list l = { 0, NULL, NULL, NULL };
    int rows = 0;

    orc_exchange_self( n, x, L );
    orc_sort_atoms( n, &g, x, v, f, type, id, NULL );
    if ( orc_neigh_cells( n, x, &g, hi, neigh_cut, neigh_cut, cfg->half,
                          cfg->nthreads, &l ) )
        return -1;
    memset( f, 0, sizeof( double ) * 3 * n );
    orc_lj_force( n, x, type, p, &l, L, cfg->half, cfg->nthreads, f );
    if ( cfg->thermo_every > 0 && rows < max_rows )
        thermo_row( n, x, v, type, p, &l, L, cfg, 0, thermo + 4 * rows++ );

    for ( int step = 1; step <= cfg->nsteps; step++ )
    {
        if ( step == cfg->time_from_step + 1 )
            t_start = wall_seconds();
        orc_nve_initial( n, x, v, f, type, cfg->mass, cfg->dt, cfg->mvv2e,
                         cfg->nthreads );
        if ( step % cfg->rebuild_every == 0 )
        {
            orc_exchange_self( n, x, L );
            orc_sort_atoms( n, &g, x, v, f, type, id, NULL );
            orc_list_free( &l );
            if ( orc_neigh_cells( n, x, &g, hi, neigh_cut, neigh_cut,
                                  cfg->half, cfg->nthreads, &l ) )
                return -1;
        }
        memset( f, 0, sizeof( double ) * 3 * n );
        orc_lj_force( n, x, type, p, &l, L, cfg->half, cfg->nthreads, f );
        orc_nve_final( n, v, f, type, cfg->mass, cfg->dt, cfg->mvv2e,
                       cfg->nthreads );
        if ( cfg->thermo_every > 0 && step % cfg->thermo_every == 0 &&
             rows < max_rows )
            thermo_row( n, x, v, type, p, &l, L, cfg, step,
                        thermo + 4 * rows++ );
    }
    if ( cfg->nsteps > cfg->time_from_step )
        cfg->loop_seconds = wall_seconds() - t_start;
    orc_list_free( &l );
    return rows;
}
