// gbmd_lj.cu -- Lennard-Jones 12-6 pair force and energy over the
// transposed Verlet list, one thread per atom, optionally fused with the
// velocity-Verlet updates around it.
//
// Reference: src/force_types/force_lj_cabana_neigh_impl.h (paths inside the
// CabanaMD project)
//   full list force   :151-203   f_i += dx * fpair for rsq < cutsq
//   half list force   :205-259   plus f_j -= dx * fpair (Newton 3); the
//                                ghost force reaches its owner through
//                                Comm::update_force (comm_mpi_impl.h:410-441)
//   energy full/half  :261-377   shifted LJ, factor 1/2 (full) or 1 / 1/2
//                                for a local / ghost partner (half)
//   step order        src/cabanamd_impl.h:336-367 (zero f, force, final
//                                integrate, thermo) then :289 (next initial)
//
// FP64 path: the reference's operation sequence with every multiply, add
// and divide rounded separately (no contraction), summed in list order, so a
// full-list force is bit-identical to a sequential CPU evaluation of the
// same list.  GB300's FP64 pipe is ~1/64 of its FP32 rate, so this path is
// FP64-issue bound by design.
//
// Mixed path: pair math in FP32 on home-cell-relative coordinates (one
// 16-byte gather per neighbour), Kahan-compensated FP32 sums, FP64 force
// output; FP64 appears only per atom (epilogue) and for the rare pairs that
// sit within the FP32 rounding band of the cutoff.
//
// MODE_STEP fuses, for a full list, the force of step n with final_integrate
// of step n, the thermo sums of step n, and initial_integrate of step n+1:
// positions are double-buffered (neighbours read x / xr, the atom's own
// update goes to x_next / xr_next), so the per-step velocity and position
// traffic is paid once.  The update sequence is the reference's, so the FP64
// trajectory stays bit-identical.
#include "gbmd_internal.cuh"

#include <cmath>

constexpr int LJ_THREADS = 128;
constexpr int LJ_BATCH = 4;

enum
{
    MODE_ACC = 0, // f += force           (Force::compute on a zeroed f)
    MODE_SET = 1, // f  = force           (full list, f overwritten)
    MODE_STEP = 2 // f = force, final, thermo, optional next initial
};

struct LjArgs
{
    int n;
    int ntypes;
    int half;
    double L[3];
    double lo[3], h[3];
    int nc[3];
    float hf[3];
    float band; // relative half-width of the exact-decision band around rc^2
    size_t pstride; // partial sums slot stride
};

// Two block sums at once (potential energy, sum m v^2).
__device__ __forceinline__ void block_sum2( double &a, double &b, double *red )
{
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
    {
        a += __shfl_xor_sync( 0xffffffffu, a, o );
        b += __shfl_xor_sync( 0xffffffffu, b, o );
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if ( lane == 0 )
    {
        red[2 * w] = a;
        red[2 * w + 1] = b;
    }
    __syncthreads();
    if ( threadIdx.x == 0 )
    {
        double sa = 0.0, sb = 0.0;
        for ( int k = 0; k < (int)( blockDim.x >> 5 ); k++ )
        {
            sa += red[2 * k];
            sb += red[2 * k + 1];
        }
        a = sa;
        b = sb;
    }
}

// final_integrate (step n) + sum m v^2 + initial_integrate (step n+1) of
// atom i, exactly the reference's operation sequence
// (integrator_nve.h:91-110, property_kine.h:72-78).
template <bool EFLAG, bool MIXED>
__device__ __forceinline__ void step_epilogue( int i, const LjArgs &a, const StepArgs &s,
                                               double fx, double fy, double fz, double4 xi,
                                               int t, int hp, double *__restrict__ v,
                                               double4 *__restrict__ x_next,
                                               float4 *__restrict__ xr_next, double &mv2 )
{
    const int n = a.n;
    const double dtfm = s.dtfm[t];
    double vx = v[i], vy = v[n + i], vz = v[2 * n + i];
    vx = dadd( vx, dmul( dtfm, fx ) );
    vy = dadd( vy, dmul( dtfm, fy ) );
    vz = dadd( vz, dmul( dtfm, fz ) );
    if ( EFLAG )
        mv2 = dmul( dadd( dadd( dmul( vx, vx ), dmul( vy, vy ) ), dmul( vz, vz ) ), s.mass[t] );
    if ( s.next )
    {
        vx = dadd( vx, dmul( dtfm, fx ) );
        vy = dadd( vy, dmul( dtfm, fy ) );
        vz = dadd( vz, dmul( dtfm, fz ) );
        xi.x = dadd( xi.x, dmul( s.dtv, vx ) );
        xi.y = dadd( xi.y, dmul( s.dtv, vy ) );
        xi.z = dadd( xi.z, dmul( s.dtv, vz ) );
        x_next[i] = xi;
        if ( MIXED )
        {
            const double ox = a.lo[0] + unpack_home( hp, 0 ) * a.h[0];
            const double oy = a.lo[1] + unpack_home( hp, 1 ) * a.h[1];
            const double oz = a.lo[2] + unpack_home( hp, 2 ) * a.h[2];
            xr_next[i] = make_float4( (float)( xi.x - ox ), (float)( xi.y - oy ),
                                      (float)( xi.z - oz ), __int_as_float( t ) );
        }
    }
    v[i] = vx;
    v[n + i] = vy;
    v[2 * n + i] = vz;
}

// ---------------------------------------------------------------------------
// FP64
template <bool FORCE, bool EFLAG, bool HALF, int MODE>
__global__ void __launch_bounds__( LJ_THREADS )
    k_lj_fp64( const double4 *__restrict__ x, const int *__restrict__ home,
               const uint32_t *__restrict__ nlist, const int *__restrict__ nnum,
               const GbmdLJ *__restrict__ prm, LjArgs a, double *__restrict__ f,
               double *__restrict__ partials, StepArgs s, double *__restrict__ v,
               double4 *__restrict__ x_next )
{
    __shared__ double s_lj1[GBMD_MAXT * GBMD_MAXT], s_lj2[GBMD_MAXT * GBMD_MAXT],
        s_cut[GBMD_MAXT * GBMD_MAXT], s_esh[GBMD_MAXT * GBMD_MAXT];
    __shared__ double red[2 * LJ_THREADS / 32];
    for ( int k = threadIdx.x; k < GBMD_MAXT * GBMD_MAXT; k += blockDim.x )
    {
        s_lj1[k] = prm->lj1[k];
        s_lj2[k] = prm->lj2[k];
        s_cut[k] = prm->cutsq[k];
        s_esh[k] = prm->eshift[k];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, mv2 = 0.0;
    if ( i < a.n )
    {
        const double4 xi = x[i];
        const int ti = (int)xi.w;
        const int hp = home[i];
        const int hc[3] = { unpack_home( hp, 0 ), unpack_home( hp, 1 ), unpack_home( hp, 2 ) };
        const int cnt = nnum[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for ( int k = 0; k < cnt; k++ )
        {
            const uint32_t e = __ldg( &nlist[(size_t)k * a.n + i] );
            const int j = (int)( e & GBMD_JMASK );
            const int sc = (int)( e >> 27 );
            const double4 xj = x[j];
            const int s0 = image_shift( hc[0], sc % 3 - 1, a.nc[0] );
            const int s1 = image_shift( hc[1], ( sc / 3 ) % 3 - 1, a.nc[1] );
            const int s2 = image_shift( hc[2], sc / 9 - 1, a.nc[2] );
            const double dx = dsub( xi.x, img_coord( xj.x, s0, a.L[0] ) );
            const double dy = dsub( xi.y, img_coord( xj.y, s1, a.L[1] ) );
            const double dz = dsub( xi.z, img_coord( xj.z, s2, a.L[2] ) );
            const int tp = ti * GBMD_MAXT + (int)xj.w;
            const double rsq = dadd( dadd( dmul( dx, dx ), dmul( dy, dy ) ), dmul( dz, dz ) );
            if ( rsq < s_cut[tp] )
            {
                const double lj1 = s_lj1[tp], lj2 = s_lj2[tp];
                // correctly rounded reciprocal == the reference's 1.0 / rsq
                const double r2inv = __drcp_rn( rsq );
                const double r6inv = dmul( dmul( r2inv, r2inv ), r2inv );
                if ( FORCE )
                {
                    const double fpair =
                        dmul( dmul( r6inv, dsub( dmul( lj1, r6inv ), lj2 ) ), r2inv );
                    const double ax = dmul( dx, fpair ), ay = dmul( dy, fpair ),
                                 az = dmul( dz, fpair );
                    fx = dadd( fx, ax );
                    fy = dadd( fy, ay );
                    fz = dadd( fz, az );
                    if ( HALF )
                    {
                        atomicAdd( &f[j], -ax );
                        atomicAdd( &f[a.n + j], -ay );
                        atomicAdd( &f[2 * a.n + j], -az );
                    }
                }
                if ( EFLAG )
                {
                    double fac = 0.5;
                    if ( HALF )
                        fac = ( s0 | s1 | s2 ) ? 0.5 : 1.0;
                    // PE += fac r6inv (0.5 lj1 r6inv - lj2) / 6; PE -= fac E(rc)
                    pe = dadd( pe, ddiv( dmul( dmul( fac, r6inv ),
                                               dsub( dmul( dmul( 0.5, lj1 ), r6inv ), lj2 ) ),
                                         6.0 ) );
                    pe = dsub( pe, dmul( fac, s_esh[tp] ) );
                }
            }
        }
        if ( FORCE )
        {
            if ( HALF )
            {
                atomicAdd( &f[i], fx );
                atomicAdd( &f[a.n + i], fy );
                atomicAdd( &f[2 * a.n + i], fz );
            }
            else if ( MODE == MODE_ACC )
            {
                f[i] = dadd( f[i], fx );
                f[a.n + i] = dadd( f[a.n + i], fy );
                f[2 * a.n + i] = dadd( f[2 * a.n + i], fz );
            }
            else
            {
                f[i] = fx;
                f[a.n + i] = fy;
                f[2 * a.n + i] = fz;
                if ( MODE == MODE_STEP )
                    step_epilogue<EFLAG, false>( i, a, s, fx, fy, fz, xi, ti, hp, v, x_next,
                                                 nullptr, mv2 );
            }
        }
    }
    if ( EFLAG )
    {
        block_sum2( pe, mv2, red );
        if ( threadIdx.x == 0 )
        {
            partials[a.pstride + blockIdx.x] = pe;
            if ( MODE == MODE_STEP )
                partials[blockIdx.x] = mv2;
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed precision
__device__ __forceinline__ void kahan_add( float &s, float &c, float v )
{
    const float y = v - c;
    const float t = s + y;
    c = ( t - s ) - y;
    s = t;
}

struct MixAcc
{
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float ps = 0.f, pc = 0.f; // potential energy
};

// One pair in mixed precision.  The cutoff test is decided in FP32 except
// inside a narrow band around rc^2 (set from the FP32 rounding bound), where
// the exact FP64 test of the FP64 path decides: the LJ force jumps at rc, so
// a pair on the wrong side would cost a whole F(rc) of error.
template <bool FORCE, bool EFLAG, bool HALF>
__device__ __forceinline__ void lj_pair_mixed(
    const float4 &xi, const float4 &xj, uint32_t e, int i, int ti, const int *hc,
    const double4 *__restrict__ x, const float *s_lj1, const float *s_lj2,
    const float *s_cut, const float *s_esh, const double *s_cut64, const LjArgs &a,
    MixAcc &acc, double *__restrict__ f )
{
    const int j = (int)( e & GBMD_JMASK );
    const int sc = (int)( e >> 27 );
    const int o0 = sc % 3 - 1, o1 = ( sc / 3 ) % 3 - 1, o2 = sc / 9 - 1;
    const float dx = xi.x - xj.x - (float)o0 * a.hf[0];
    const float dy = xi.y - xj.y - (float)o1 * a.hf[1];
    const float dz = xi.z - xj.z - (float)o2 * a.hf[2];
    const int tp = ti * GBMD_MAXT + __float_as_int( xj.w );
    const float rsq = dx * dx + dy * dy + dz * dz;
    const float cutsq = s_cut[tp];
    bool in = rsq < cutsq;
    if ( fabsf( rsq - cutsq ) <= a.band * cutsq )
    {
        const double4 p = x[i], q = x[j];
        const int s0 = image_shift( hc[0], o0, a.nc[0] );
        const int s1 = image_shift( hc[1], o1, a.nc[1] );
        const int s2 = image_shift( hc[2], o2, a.nc[2] );
        const double ex = dsub( p.x, img_coord( q.x, s0, a.L[0] ) );
        const double ey = dsub( p.y, img_coord( q.y, s1, a.L[1] ) );
        const double ez = dsub( p.z, img_coord( q.z, s2, a.L[2] ) );
        const double r64 = dadd( dadd( dmul( ex, ex ), dmul( ey, ey ) ), dmul( ez, ez ) );
        in = r64 < s_cut64[tp];
    }
    if ( in )
    {
        const float lj1 = s_lj1[tp], lj2 = s_lj2[tp];
        const float r2inv = 1.0f / rsq;
        const float r6inv = r2inv * r2inv * r2inv;
        if ( FORCE )
        {
            const float fpair = r6inv * ( lj1 * r6inv - lj2 ) * r2inv;
            kahan_add( acc.sx, acc.cx, dx * fpair );
            kahan_add( acc.sy, acc.cy, dy * fpair );
            kahan_add( acc.sz, acc.cz, dz * fpair );
            if ( HALF )
            {
                atomicAdd( &f[j], -(double)( dx * fpair ) );
                atomicAdd( &f[a.n + j], -(double)( dy * fpair ) );
                atomicAdd( &f[2 * a.n + j], -(double)( dz * fpair ) );
            }
        }
        if ( EFLAG )
        {
            float fac = 0.5f;
            if ( HALF )
            {
                const int g0 = image_shift( hc[0], o0, a.nc[0] );
                const int g1 = image_shift( hc[1], o1, a.nc[1] );
                const int g2 = image_shift( hc[2], o2, a.nc[2] );
                fac = ( g0 | g1 | g2 ) ? 0.5f : 1.0f;
            }
            kahan_add( acc.ps, acc.pc,
                       fac * ( r6inv * ( 0.5f * lj1 * r6inv - lj2 ) * ( 1.0f / 6.0f ) -
                               s_esh[tp] ) );
        }
    }
}

template <bool FORCE, bool EFLAG, bool HALF, int MODE>
__global__ void __launch_bounds__( LJ_THREADS )
    k_lj_mixed( const float4 *__restrict__ xr, const double4 *__restrict__ x,
                const int *__restrict__ home, const uint32_t *__restrict__ nlist,
                const int *__restrict__ nnum, const GbmdLJ *__restrict__ prm, LjArgs a,
                double *__restrict__ f, double *__restrict__ partials, StepArgs s,
                double *__restrict__ v, double4 *__restrict__ x_next,
                float4 *__restrict__ xr_next )
{
    __shared__ float s_lj1[GBMD_MAXT * GBMD_MAXT], s_lj2[GBMD_MAXT * GBMD_MAXT],
        s_cut[GBMD_MAXT * GBMD_MAXT], s_esh[GBMD_MAXT * GBMD_MAXT];
    __shared__ double s_cut64[GBMD_MAXT * GBMD_MAXT];
    __shared__ double red[2 * LJ_THREADS / 32];
    for ( int k = threadIdx.x; k < GBMD_MAXT * GBMD_MAXT; k += blockDim.x )
    {
        s_lj1[k] = prm->lj1f[k];
        s_lj2[k] = prm->lj2f[k];
        s_cut[k] = prm->cutsqf[k];
        s_esh[k] = prm->eshiftf[k];
        s_cut64[k] = prm->cutsq[k];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, mv2 = 0.0;
    if ( i < a.n )
    {
        const float4 xi = xr[i];
        const int ti = __float_as_int( xi.w );
        const int hp = home[i];
        const int hc[3] = { unpack_home( hp, 0 ), unpack_home( hp, 1 ), unpack_home( hp, 2 ) };
        const int cnt = nnum[i];
        MixAcc acc;
        const uint32_t *lp = nlist + i;
        const size_t stride = (size_t)a.n;
        int k = 0;
        // Batches of independent list loads then gathers: LJ_BATCH memory
        // requests in flight per thread instead of one dependent chain.
        for ( ; k + LJ_BATCH <= cnt; k += LJ_BATCH )
        {
            uint32_t e[LJ_BATCH];
            float4 xj[LJ_BATCH];
#pragma unroll
            for ( int u = 0; u < LJ_BATCH; u++ )
                e[u] = __ldg( lp + ( k + u ) * stride );
#pragma unroll
            for ( int u = 0; u < LJ_BATCH; u++ )
                xj[u] = __ldg( &xr[e[u] & GBMD_JMASK] );
#pragma unroll
            for ( int u = 0; u < LJ_BATCH; u++ )
                lj_pair_mixed<FORCE, EFLAG, HALF>( xi, xj[u], e[u], i, ti, hc, x, s_lj1, s_lj2,
                                                   s_cut, s_esh, s_cut64, a, acc, f );
        }
        for ( ; k < cnt; k++ )
        {
            const uint32_t e = __ldg( lp + k * stride );
            const float4 xj = __ldg( &xr[e & GBMD_JMASK] );
            lj_pair_mixed<FORCE, EFLAG, HALF>( xi, xj, e, i, ti, hc, x, s_lj1, s_lj2, s_cut,
                                               s_esh, s_cut64, a, acc, f );
        }
        if ( EFLAG )
            pe = (double)acc.ps - (double)acc.pc;
        if ( FORCE )
        {
            const double fx = (double)acc.sx - (double)acc.cx;
            const double fy = (double)acc.sy - (double)acc.cy;
            const double fz = (double)acc.sz - (double)acc.cz;
            if ( HALF )
            {
                atomicAdd( &f[i], fx );
                atomicAdd( &f[a.n + i], fy );
                atomicAdd( &f[2 * a.n + i], fz );
            }
            else if ( MODE == MODE_ACC )
            {
                f[i] += fx;
                f[a.n + i] += fy;
                f[2 * a.n + i] += fz;
            }
            else
            {
                f[i] = fx;
                f[a.n + i] = fy;
                f[2 * a.n + i] = fz;
                if ( MODE == MODE_STEP )
                    step_epilogue<EFLAG, true>( i, a, s, fx, fy, fz, x[i], ti, hp, v, x_next,
                                                xr_next, mv2 );
            }
        }
    }
    if ( EFLAG )
    {
        block_sum2( pe, mv2, red );
        if ( threadIdx.x == 0 )
        {
            partials[a.pstride + blockIdx.x] = pe;
            if ( MODE == MODE_STEP )
                partials[blockIdx.x] = mv2;
        }
    }
}

// ---------------------------------------------------------------------------
static LjArgs make_args( const gbmd_ctx *c, size_t stride )
{
    LjArgs a;
    a.n = (int)c->n;
    a.ntypes = c->ntypes;
    a.half = c->half;
    for ( int d = 0; d < 3; d++ )
    {
        a.L[d] = c->geom.L[d];
        a.lo[d] = c->geom.lo[d];
        a.h[d] = c->geom.h[d];
        a.nc[d] = c->geom.nc[d];
        a.hf[d] = c->geom.hf[d];
    }
    // band from the smallest pair cutoff in use (the bound grows as rc shrinks)
    double rcmin = 0.0;
    for ( int ti = 0; ti < c->ntypes; ti++ )
        for ( int tj = 0; tj < c->ntypes; tj++ )
        {
            const double cs = c->lj.cutsq[ti * GBMD_MAXT + tj];
            if ( cs > 0 && ( rcmin == 0.0 || cs < rcmin * rcmin ) )
                rcmin = std::sqrt( cs );
        }
    a.band = (float)gbmd_fp32_band( c->geom, rcmin > 0 ? rcmin : c->neigh_cut );
    a.pstride = stride; // slot 1: potential energy
    return a;
}

StepArgs gbmd_step_args( const gbmd_ctx *c, bool next )
{
    StepArgs s;
    const double dtf = 0.5 * c->dt / c->mvv2e;
    for ( int t = 0; t < GBMD_MAXT; t++ )
    {
        s.mass[t] = c->mass[t];
        s.dtfm[t] = dtf / c->mass[t]; // integrator_nve.h:96
    }
    s.dtv = c->dt;
    s.next = next ? 1 : 0;
    return s;
}

template <bool FORCE, bool EFLAG, bool HALF, int MODE>
static void launch_one( gbmd_ctx *c, int blocks, GbmdLJ *ljd, const LjArgs &a,
                        const StepArgs &s )
{
    if ( c->precision == GBMD_PREC_FP64 )
        k_lj_fp64<FORCE, EFLAG, HALF, MODE><<<blocks, LJ_THREADS, 0, c->stream>>>(
            c->x.p, c->home.p, c->nlist.p, c->nnum.p, ljd, a, c->f.p, c->partials.p, s,
            c->v.p, c->x_alt.p );
    else
        k_lj_mixed<FORCE, EFLAG, HALF, MODE><<<blocks, LJ_THREADS, 0, c->stream>>>(
            c->xr.p, c->x.p, c->home.p, c->nlist.p, c->nnum.p, ljd, a, c->f.p,
            c->partials.p, s, c->v.p, c->x_alt.p, c->xr_alt.p );
}

int gbmd_lj_launch( gbmd_ctx *c, bool eflag, bool zero_first )
{
    const int n = (int)c->n;
    if ( n == 0 )
        return GBMD_OK;
    size_t stride;
    GbmdLJ *ljd;
    int rc = gbmd_partials_prepare( c, n, &stride, &ljd );
    if ( rc )
        return rc;
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, false );
    const bool half = c->half != 0;
    if ( half && zero_first )
        GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * n, c->stream ) );
    const int blocks = ( n + LJ_THREADS - 1 ) / LJ_THREADS;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_FORCE, &t0 );
    if ( half )
    {
        if ( eflag )
            launch_one<true, true, true, MODE_ACC>( c, blocks, ljd, a, s );
        else
            launch_one<true, false, true, MODE_ACC>( c, blocks, ljd, a, s );
    }
    else if ( zero_first )
    {
        if ( eflag )
            launch_one<true, true, false, MODE_SET>( c, blocks, ljd, a, s );
        else
            launch_one<true, false, false, MODE_SET>( c, blocks, ljd, a, s );
    }
    else
    {
        if ( eflag )
            launch_one<true, true, false, MODE_ACC>( c, blocks, ljd, a, s );
        else
            launch_one<true, false, false, MODE_ACC>( c, blocks, ljd, a, s );
    }
    GBMD_LAUNCH_CHECK( c, "lj force" );
    gbmd_ktime_end( c, GBMD_KT_FORCE, t0 );
    if ( eflag )
        return gbmd_reduce_partials( c, blocks, 1 );
    return GBMD_OK;
}

// Fused step for a full list: force(n) + final(n) [+ thermo(n)] [+ initial(n+1)].
int gbmd_lj_step_launch( gbmd_ctx *c, bool thermo, bool next )
{
    const int n = (int)c->n;
    if ( n == 0 )
        return GBMD_OK;
    size_t stride;
    GbmdLJ *ljd;
    int rc = gbmd_partials_prepare( c, n, &stride, &ljd );
    if ( rc )
        return rc;
    if ( ( rc = gbmd_reserve( c, c->xr_alt, n, "xr_alt" ) ) )
        return rc;
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, next );
    const int blocks = ( n + LJ_THREADS - 1 ) / LJ_THREADS;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_FORCE, &t0 );
    if ( thermo )
        launch_one<true, true, false, MODE_STEP>( c, blocks, ljd, a, s );
    else
        launch_one<true, false, false, MODE_STEP>( c, blocks, ljd, a, s );
    GBMD_LAUNCH_CHECK( c, "lj step" );
    gbmd_ktime_end( c, GBMD_KT_FORCE, t0 );
    if ( next )
    {
        std::swap( c->x, c->x_alt );
        if ( c->precision == GBMD_PREC_MIXED )
            std::swap( c->xr, c->xr_alt );
    }
    if ( thermo )
    {
        if ( ( rc = gbmd_reduce_partials( c, blocks, 0 ) ) )
            return rc;
        return gbmd_reduce_partials( c, blocks, 1 );
    }
    return GBMD_OK;
}

int gbmd_lj_energy_launch( gbmd_ctx *c )
{
    const int n = (int)c->n;
    size_t stride;
    GbmdLJ *ljd;
    int rc = gbmd_partials_prepare( c, n, &stride, &ljd );
    if ( rc )
        return rc;
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, false );
    const int blocks = ( n + LJ_THREADS - 1 ) / LJ_THREADS;
    if ( c->half )
        launch_one<false, true, true, MODE_ACC>( c, blocks, ljd, a, s );
    else
        launch_one<false, true, false, MODE_ACC>( c, blocks, ljd, a, s );
    GBMD_LAUNCH_CHECK( c, "lj energy" );
    return gbmd_reduce_partials( c, blocks, 1 );
}
