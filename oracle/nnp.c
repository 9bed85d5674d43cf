/*
 * nnp.c -- FP64 CPU restatement of the neural-network potential path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Build with -ffp-contract=off.
 *
 * The arithmetic of this path lives in n2p2 v2.0.1 (CompPhysVienna/n2p2,
 * pinned by the reference's CI, .github/workflows/CI.yml:126-128), which is
 * not vendored.  It is restated from the published Behler-Parrinello
 * definitions and n2p2's documented file formats; parity is UNPINNED (no
 * reference test exercises NNP results).  Reference call sites:
 *   src/force_types/force_nnp_cabana_neigh_impl.h:41-66  (init_coeff: load
 *        input.nn, scaling.data, weights.%03zu.data)
 *   :68-99   compute: calculateSymmetryFunctionGroups ->
 *            calculateAtomicNeuralNetworks -> calculateForces
 *   :101-130 compute_energy: ((sum E_i + N_local * atomicEnergyOffset)
 *            / convEnergy + N * meanEnergy) * 27.211384021355236
 *
 * Definitions (n2p2 symmetry function types 2 and 3, cutoff type 1):
 *   fc(r)   = 0.5 (cos(pi r / rc) + 1)                      r < rc, else 0
 *   G2_i    = sum_j exp(-eta (r_ij - rs)^2) fc(r_ij)
 *   G3_i    = 2^(1-zeta) sum_{j<k} (1 + lambda cos t_ijk)^zeta
 *             exp(-eta (r_ij^2 + r_ik^2 + r_jk^2)) fc(r_ij) fc(r_ik) fc(r_jk)
 *   scaled  = smin + (smax - smin) (G - Gmin) / (Gmax - Gmin)
 *   E_i     = NN(scaled G_i); f = -dE/dx through G.
 * With several elements, atom i uses its element's functions and network;
 * a radial function sums neighbours j of element e1 only, an angular one
 * the pairs (j, k) whose elements are {e1, e2} in either order.
 */
#include "nnp.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

static double omp_wall( void )
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

static inline double fc_cos( double r, double rc )
{
    if ( r >= rc )
        return 0.0;
    return 0.5 * ( cos( ORC_PI * r / rc ) + 1.0 );
}

static inline double dfc_cos( double r, double rc )
{
    if ( r >= rc )
        return 0.0;
    return -0.5 * ORC_PI / rc * sin( ORC_PI * r / rc );
}

static inline int img_s( int8_t code, int d )
{
    int c = code;
    for ( int k = 0; k < d; k++ )
        c /= 3;
    return c % 3 - 1;
}

static inline double img_coord( double xs, int s, double L )
{
    if ( s < 0 )
        return xs - L;
    if ( s > 0 )
        return xs + L;
    return xs;
}

static double act( char a, double x )
{
    switch ( a )
    {
    case 't':
        return tanh( x );
    case 'p': /* softplus */
        return x > 30.0 ? x : log1p( exp( x ) );
    case 's': /* logistic */
        return 1.0 / ( 1.0 + exp( -x ) );
    default: /* 'l' linear */
        return x;
    }
}

static double dact( char a, double x )
{
    switch ( a )
    {
    case 't':
    {
        const double t = tanh( x );
        return 1.0 - t * t;
    }
    case 'p':
        return 1.0 / ( 1.0 + exp( -x ) );
    case 's':
    {
        const double s = 1.0 / ( 1.0 + exp( -x ) );
        return s * ( 1.0 - s );
    }
    default:
        return 1.0;
    }
}

/* Neighbours of atom i inside the largest SF cutoff, as displacement
 * vectors r_ij = x_img(j) - x_i with their owners. */
typedef struct
{
    int n;
    int cap;
    double *d; /* [cap][3] */
    double *r;
    int32_t *j;
    int32_t *t; /* neighbour element */
} nbr_buf;

static void gather_neighbours( int64_t i, const double *x, const int32_t *type,
                               const orc_list *l, const double L[3], double rc, nbr_buf *b )
{
    b->n = 0;
    const int64_t cnt = l->off[i + 1] - l->off[i];
    if ( cnt > b->cap )
    {
        b->cap = (int)cnt + 16;
        b->d = (double *)realloc( b->d, sizeof( double ) * 3 * b->cap );
        b->r = (double *)realloc( b->r, sizeof( double ) * b->cap );
        b->j = (int32_t *)realloc( b->j, sizeof( int32_t ) * b->cap );
        b->t = (int32_t *)realloc( b->t, sizeof( int32_t ) * b->cap );
    }
    for ( int64_t k = l->off[i]; k < l->off[i + 1]; k++ )
    {
        const int32_t j = l->j[k];
        const int8_t code = l->img[k];
        double dv[3];
        for ( int d = 0; d < 3; d++ )
            dv[d] = img_coord( x[3 * j + d], img_s( code, d ), L[d] ) - x[3 * i + d];
        const double r2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
        const double r = sqrt( r2 );
        if ( !( r < rc ) )
            continue;
        memcpy( b->d + 3 * b->n, dv, sizeof( dv ) );
        b->r[b->n] = r;
        b->j[b->n] = j;
        b->t[b->n] = type ? type[j] : 0;
        b->n++;
    }
}

static double max_cutoff( const orc_nnp *m, int nelem )
{
    double rc = 0.0;
    for ( int e = 0; e < nelem; e++ )
        for ( int s = 0; s < m[e].nsf; s++ )
            if ( m[e].rc[s] > rc )
                rc = m[e].rc[s];
    return rc;
}

static inline int pair_match( const orc_nnp *m, int s, int ta, int tb )
{
    return ( ta == m->e1[s] && tb == m->e2[s] ) || ( ta == m->e2[s] && tb == m->e1[s] );
}

/* Raw symmetry functions of one atom. */
static void sf_atom( const orc_nnp *m, const nbr_buf *b, double *G )
{
    for ( int s = 0; s < m->nsf; s++ )
        G[s] = 0.0;
    for ( int a = 0; a < b->n; a++ )
    {
        const double rij = b->r[a];
        for ( int s = 0; s < m->nsf; s++ )
            if ( m->type[s] == 2 && rij < m->rc[s] && b->t[a] == m->e1[s] )
            {
                const double dr = rij - m->rs[s];
                G[s] += exp( -m->eta[s] * dr * dr ) * fc_cos( rij, m->rc[s] );
            }
    }
    for ( int a = 0; a < b->n; a++ )
        for ( int c = a + 1; c < b->n; c++ )
        {
            const double *dj = b->d + 3 * a, *dk = b->d + 3 * c;
            const double rij = b->r[a], rik = b->r[c];
            const double djk[3] = { dk[0] - dj[0], dk[1] - dj[1], dk[2] - dj[2] };
            const double rjk2 = djk[0] * djk[0] + djk[1] * djk[1] + djk[2] * djk[2];
            const double rjk = sqrt( rjk2 );
            const double cs = ( dj[0] * dk[0] + dj[1] * dk[1] + dj[2] * dk[2] ) / ( rij * rik );
            const double R2 = rij * rij + rik * rik + rjk2;
            for ( int s = 0; s < m->nsf; s++ )
            {
                if ( m->type[s] != 3 || !pair_match( m, s, b->t[a], b->t[c] ) )
                    continue;
                const double rc = m->rc[s];
                if ( !( rij < rc && rik < rc && rjk < rc ) )
                    continue;
                const double base = 1.0 + m->lambda[s] * cs;
                const double F = fc_cos( rij, rc ) * fc_cos( rik, rc ) * fc_cos( rjk, rc );
                G[s] += pow( 2.0, 1.0 - m->zeta[s] ) * pow( base, m->zeta[s] ) *
                        exp( -m->eta[s] * R2 ) * F;
            }
        }
}

/* NN forward + backward: E and dE/dG (raw G units). */
static double nn_atom( const orc_nnp *m, const double *G, double *dEdG )
{
    double y[ORC_NNP_MAXNODES], z[ORC_NNP_MAXLAYERS + 1][ORC_NNP_MAXNODES],
        a[ORC_NNP_MAXLAYERS + 1][ORC_NNP_MAXNODES];
    const int L = m->nlayers; /* weight layers; nodes[0] = nsf */
    for ( int s = 0; s < m->nsf; s++ )
    {
        const double den = m->gmax[s] - m->gmin[s];
        a[0][s] = m->smin + ( m->smax - m->smin ) * ( G[s] - m->gmin[s] ) / den;
    }
    for ( int l = 1; l <= L; l++ )
    {
        const double *W = m->w + m->woff[l];
        const double *B = m->b + m->boff[l];
        for ( int jn = 0; jn < m->nodes[l]; jn++ )
        {
            double acc = B[jn];
            for ( int in = 0; in < m->nodes[l - 1]; in++ )
                acc += W[jn * m->nodes[l - 1] + in] * a[l - 1][in];
            z[l][jn] = acc;
            a[l][jn] = act( m->act[l], acc );
        }
    }
    const double E = a[L][0];
    /* backward */
    double g[ORC_NNP_MAXNODES];
    g[0] = dact( m->act[L], z[L][0] );
    for ( int l = L; l >= 1; l-- )
    {
        const double *W = m->w + m->woff[l];
        for ( int in = 0; in < m->nodes[l - 1]; in++ )
        {
            double acc = 0.0;
            for ( int jn = 0; jn < m->nodes[l]; jn++ )
                acc += W[jn * m->nodes[l - 1] + in] * g[jn];
            y[in] = acc;
        }
        for ( int in = 0; in < m->nodes[l - 1]; in++ )
            g[in] = ( l > 1 ) ? y[in] * dact( m->act[l - 1], z[l - 1][in] ) : y[in];
    }
    for ( int s = 0; s < m->nsf; s++ )
        dEdG[s] = g[s] * ( m->smax - m->smin ) / ( m->gmax[s] - m->gmin[s] );
    return E;
}

/* Force contributions of one atom's SFs: f_m -= sum_s dEdG_s dG_s/dx_m. */
static void force_atom( const orc_nnp *m, int64_t i, const nbr_buf *b, const double *dEdG,
                        double *f )
{
    double fi[3] = { 0, 0, 0 };
    for ( int a = 0; a < b->n; a++ )
    {
        const double rij = b->r[a];
        double coef = 0.0; /* dE/dr_ij */
        for ( int s = 0; s < m->nsf; s++ )
            if ( m->type[s] == 2 && rij < m->rc[s] && b->t[a] == m->e1[s] )
            {
                const double dr = rij - m->rs[s];
                const double e = exp( -m->eta[s] * dr * dr );
                coef += dEdG[s] * e *
                        ( -2.0 * m->eta[s] * dr * fc_cos( rij, m->rc[s] ) +
                          dfc_cos( rij, m->rc[s] ) );
            }
        /* r_ij = x_j - x_i: dr/dx_j = d/r, dr/dx_i = -d/r */
        const double *d = b->d + 3 * a;
        const int32_t j = b->j[a];
        for ( int k = 0; k < 3; k++ )
        {
            const double g = coef * d[k] / rij;
            f[3 * j + k] -= g;
            fi[k] += g;
        }
    }
    for ( int a = 0; a < b->n; a++ )
        for ( int c = a + 1; c < b->n; c++ )
        {
            const double *dj = b->d + 3 * a, *dk = b->d + 3 * c;
            const double rij = b->r[a], rik = b->r[c];
            const double djk[3] = { dk[0] - dj[0], dk[1] - dj[1], dk[2] - dj[2] };
            const double rjk2 = djk[0] * djk[0] + djk[1] * djk[1] + djk[2] * djk[2];
            const double rjk = sqrt( rjk2 );
            const double cs = ( dj[0] * dk[0] + dj[1] * dk[1] + dj[2] * dk[2] ) / ( rij * rik );
            const double R2 = rij * rij + rik * rik + rjk2;
            /* accumulate dE/dc, dE/dR2-weighted, dE/dfc pieces over SFs */
            double gj[3] = { 0, 0, 0 }, gk[3] = { 0, 0, 0 };
            for ( int s = 0; s < m->nsf; s++ )
            {
                if ( m->type[s] != 3 || !pair_match( m, s, b->t[a], b->t[c] ) )
                    continue;
                const double rc = m->rc[s];
                if ( !( rij < rc && rik < rc && rjk < rc ) )
                    continue;
                const double lam = m->lambda[s], zeta = m->zeta[s], eta = m->eta[s];
                const double base = 1.0 + lam * cs;
                const double pre = pow( 2.0, 1.0 - zeta );
                const double A = pow( base, zeta );
                const double dA = zeta * pow( base, zeta - 1.0 ) * lam;
                const double Ex = exp( -eta * R2 );
                const double fij = fc_cos( rij, rc ), fik = fc_cos( rik, rc ),
                             fjk = fc_cos( rjk, rc );
                const double F = fij * fik * fjk;
                const double w = dEdG[s] * pre;
                /* d/dx_j and d/dx_k of A(c) E(R2) F(rij, rik, rjk) */
                for ( int q = 0; q < 3; q++ )
                {
                    const double dcj = dk[q] / ( rij * rik ) - cs * dj[q] / ( rij * rij );
                    const double dck = dj[q] / ( rij * rik ) - cs * dk[q] / ( rik * rik );
                    const double dEj = Ex * ( -eta ) * ( 2.0 * dj[q] - 2.0 * djk[q] );
                    const double dEk = Ex * ( -eta ) * ( 2.0 * dk[q] + 2.0 * djk[q] );
                    const double dFj = dfc_cos( rij, rc ) * dj[q] / rij * fik * fjk -
                                       fij * fik * dfc_cos( rjk, rc ) * djk[q] / rjk;
                    const double dFk = fij * dfc_cos( rik, rc ) * dk[q] / rik * fjk +
                                       fij * fik * dfc_cos( rjk, rc ) * djk[q] / rjk;
                    gj[q] += w * ( dA * dcj * Ex * F + A * dEj * F + A * Ex * dFj );
                    gk[q] += w * ( dA * dck * Ex * F + A * dEk * F + A * Ex * dFk );
                }
            }
            const int32_t j = b->j[a], k = b->j[c];
            for ( int q = 0; q < 3; q++ )
            {
                f[3 * j + q] -= gj[q];
                f[3 * k + q] -= gk[q];
                fi[q] += gj[q] + gk[q]; /* dG/dx_i = -(dG/dx_j + dG/dx_k) */
            }
        }
    for ( int q = 0; q < 3; q++ )
        f[3 * i + q] += fi[q];
}

static void nbr_free( nbr_buf *b )
{
    free( b->d );
    free( b->r );
    free( b->j );
    free( b->t );
}

double orc_nnp_compute_multi_mt( int64_t n, const double *x, const int32_t *type,
                                 const orc_list *l, const double L[3], const orc_nnp *models,
                                 int nelem, int gstride, double *G, double *E, double *dEdG,
                                 double *f, int nthreads )
{
    const double rc = max_cutoff( models, nelem );
    double esum = 0.0;
    const size_t rows = (size_t)( n ? n : 1 ) * gstride;
    double *dE = dEdG ? dEdG : (double *)calloc( rows, sizeof( double ) );
    double *g = G ? G : (double *)calloc( rows, sizeof( double ) );
    double *e_at = (double *)calloc( n ? n : 1, sizeof( double ) );
    if ( nthreads < 1 )
        nthreads = 1;
    /* symmetry functions and networks: independent per atom */
#pragma omp parallel num_threads( nthreads )
    {
        nbr_buf b = { 0, 0, NULL, NULL, NULL, NULL };
#pragma omp for schedule( static )
        for ( int64_t i = 0; i < n; i++ )
        {
            const orc_nnp *m = models + ( type ? type[i] : 0 );
            gather_neighbours( i, x, type, l, L, rc, &b );
            sf_atom( m, &b, g + (size_t)gstride * i );
            e_at[i] = nn_atom( m, g + (size_t)gstride * i, dE + (size_t)gstride * i );
        }
        nbr_free( &b );
    }
    /* the energy sum in atom order, whatever the thread count */
    for ( int64_t i = 0; i < n; i++ )
    {
        if ( E )
            E[i] = e_at[i];
        esum += e_at[i];
    }
    free( e_at );
    if ( f && nthreads == 1 )
    {
        nbr_buf b = { 0, 0, NULL, NULL, NULL, NULL };
        for ( int64_t i = 0; i < n; i++ )
        {
            const orc_nnp *m = models + ( type ? type[i] : 0 );
            gather_neighbours( i, x, type, l, L, rc, &b );
            force_atom( m, i, &b, dE + (size_t)gstride * i, f );
        }
        nbr_free( &b );
    }
    else if ( f )
    {
        /* a private force array per thread (contributions scatter onto
         * neighbours), added into f in thread order */
        double *ft = (double *)calloc( (size_t)nthreads * 3 * ( n ? n : 1 ), sizeof( double ) );
#pragma omp parallel num_threads( nthreads )
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double *fl = ft + (size_t)t * 3 * n;
            nbr_buf b = { 0, 0, NULL, NULL, NULL, NULL };
#pragma omp for schedule( static )
            for ( int64_t i = 0; i < n; i++ )
            {
                const orc_nnp *m = models + ( type ? type[i] : 0 );
                gather_neighbours( i, x, type, l, L, rc, &b );
                force_atom( m, i, &b, dE + (size_t)gstride * i, fl );
            }
            nbr_free( &b );
        }
        for ( int t = 0; t < nthreads; t++ )
            for ( int64_t k = 0; k < 3 * n; k++ )
                f[k] += ft[(size_t)t * 3 * n + k];
        free( ft );
    }
    if ( !dEdG )
        free( dE );
    if ( !G )
        free( g );
    return esum;
}

double orc_nnp_compute_multi( int64_t n, const double *x, const int32_t *type, const orc_list *l,
                              const double L[3], const orc_nnp *models, int nelem, int gstride,
                              double *G, double *E, double *dEdG, double *f )
{
    return orc_nnp_compute_multi_mt( n, x, type, l, L, models, nelem, gstride, G, E, dEdG, f,
                                     1 );
}

double orc_nnp_compute( int64_t n, const double *x, const orc_list *l, const double L[3],
                        const orc_nnp *m, double *G, double *E, double *dEdG, double *f )
{
    return orc_nnp_compute_multi( n, x, NULL, l, L, m, 1, m->nsf, G, E, dEdG, f );
}

/* force_nnp_cabana_neigh_impl.h:101-130 */
double orc_nnp_energy( int64_t n, double esum, const orc_nnp *m )
{
    double e = esum;
    e += n * m->e_offset;
    e /= m->conv_energy;
    e += n * m->mean_energy;
    e *= 27.211384021355236;
    return e;
}

/* CbnMD::init + CbnMD::run with the NNP force on one rank
 * (cabanamd_impl.h:70-255, 284-399): wrap, sort and a full list of cutoff
 * force_cut + skin at start and every rebuild_every steps; each step
 * initial_integrate, [rebuild], f = 0, compute (the forces on ghost images
 * folded into their owners, Comm::update_force, :348), final_integrate, and
 * every thermo_every steps a row (step, T, PE/N, KE/N) with
 * PE = ForceNNP::compute_energy of the same evaluation.  Atoms use
 * models[type[i]].  When snap_step >= 0, the state after that step
 * (positions, velocities, forces in the current order, ids) is copied to
 * snap_x / snap_v / snap_f / snap_id.  Returns the row count, or -1. */
int orc_run_nnp( int64_t n, double *x, double *v, double *f, int32_t *type, int32_t *id,
                 const double lo[3], const double hi[3], const orc_nnp *models, int nelem,
                 orc_run_cfg *cfg, double *thermo, int max_rows, int snap_step, double *snap_x,
                 double *snap_v, double *snap_f, int32_t *snap_id )
{
    const double neigh_cut = cfg->force_cut + cfg->skin;
    orc_grid g;
    orc_make_grid( lo, hi, neigh_cut, &g );
    const double *L = g.L;
    orc_list l = { 0, NULL, NULL, NULL };
    int gstride = 0;
    for ( int e = 0; e < nelem; e++ )
        if ( models[e].nsf > gstride )
            gstride = models[e].nsf;
    int rows = 0;
    double t_start = 0.0;
    cfg->loop_seconds = 0.0;

    orc_exchange_self( n, x, L );
    orc_sort_atoms( n, &g, x, v, f, type, id, NULL );
    if ( orc_neigh_cells( n, x, &g, hi, neigh_cut, neigh_cut, 0, cfg->nthreads, &l ) )
        return -1;
    for ( int step = 0; step <= cfg->nsteps; step++ )
    {
        if ( step == cfg->time_from_step + 1 )
            t_start = omp_wall();
        if ( step > 0 )
        {
            orc_nve_initial( n, x, v, f, type, cfg->mass, cfg->dt, cfg->mvv2e, cfg->nthreads );
            if ( step % cfg->rebuild_every == 0 )
            {
                orc_exchange_self( n, x, L );
                orc_sort_atoms( n, &g, x, v, f, type, id, NULL );
                orc_list_free( &l );
                if ( orc_neigh_cells( n, x, &g, hi, neigh_cut, neigh_cut, 0, cfg->nthreads,
                                      &l ) )
                    return -1;
            }
        }
        memset( f, 0, sizeof( double ) * 3 * n );
        const double esum = orc_nnp_compute_multi_mt( n, x, type, &l, L, models, nelem, gstride,
                                                      NULL, NULL, NULL, f, cfg->nthreads );
        if ( step > 0 )
            orc_nve_final( n, v, f, type, cfg->mass, cfg->dt, cfg->mvv2e, cfg->nthreads );
        if ( cfg->thermo_every > 0 && step % cfg->thermo_every == 0 && rows < max_rows )
        {
            const double smv2 = orc_sum_mv2( n, v, type, cfg->mass, cfg->nthreads );
            /* property_temperature_impl.h:66-76, property_kine_impl.h:66-75 */
            const int64_t dof = 3 * n - 3;
            double *row = thermo + 4 * rows++;
            row[0] = step;
            row[1] = smv2 * ( cfg->mvv2e / ( 1.0 * dof * cfg->boltz ) );
            row[2] = orc_nnp_energy( n, esum, models ) / n;
            row[3] = smv2 * ( 0.5 * cfg->mvv2e ) / n;
        }
        if ( step == snap_step )
        {
            if ( snap_x )
                memcpy( snap_x, x, sizeof( double ) * 3 * n );
            if ( snap_v )
                memcpy( snap_v, v, sizeof( double ) * 3 * n );
            if ( snap_f )
                memcpy( snap_f, f, sizeof( double ) * 3 * n );
            if ( snap_id )
                memcpy( snap_id, id, sizeof( int32_t ) * n );
        }
    }
    if ( cfg->nsteps > cfg->time_from_step )
        cfg->loop_seconds = omp_wall() - t_start;
    orc_list_free( &l );
    return rows;
}
