// gbmd_lj.cu -- Lennard-Jones 12-6 pair force and energy over the
// transposed Verlet list, one thread per atom.
//
// Reference: src/force_types/force_lj_cabana_neigh_impl.h (paths inside the
// CabanaMD project)
//   full list force   :151-203   f_i += dx * fpair for rsq < cutsq
//   half list force   :205-259   plus f_j -= dx * fpair (Newton 3); the
//                                ghost force reaches its owner through
//                                Comm::update_force (comm_mpi_impl.h:410-441)
//   energy full/half  :261-377   shifted LJ, factor 1/2 (full) or 1 / 1/2
//                                for a local / ghost partner (half)
//
// FP64 path: the reference's operation sequence with every multiply, add
// and divide rounded separately (no contraction), summed in list order, so a
// full-list force is bit-identical to a sequential CPU evaluation of the
// same list.  Mixed path: pair math in FP32 on cell-relative coordinates
// (one 16-byte gather per neighbour), Kahan-compensated FP32 accumulation,
// FP64 force output.
#include "gbmd_internal.cuh"

constexpr int LJ_THREADS = 128;

struct LjArgs
{
    int n;
    int ntypes;
    int half;
    double L[3];
    int nc[3];
    float hf[3];
    size_t pstride; // partial sums slot stride
};

template <int NT> struct LjShared
{
    double lj1[NT], lj2[NT], cutsq[NT];
    float lj1f[NT], lj2f[NT], cutsqf[NT];
};

__device__ __forceinline__ double block_sum( double v, double *red )
{
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        v += __shfl_xor_sync( 0xffffffffu, v, o );
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if ( lane == 0 )
        red[w] = v;
    __syncthreads();
    double s = 0.0;
    if ( threadIdx.x == 0 )
        for ( int k = 0; k < (int)( blockDim.x >> 5 ); k++ )
            s += red[k];
    return s;
}

// FP64, full or half list.  FORCE: write forces; EFLAG: per-block PE partial.
template <bool FORCE, bool EFLAG, bool HALF, bool ZERO>
__global__ void __launch_bounds__( LJ_THREADS )
    k_lj_fp64( const double4 *__restrict__ x, const int *__restrict__ home,
               const uint32_t *__restrict__ nlist, const int *__restrict__ nnum,
               const GbmdLJ *__restrict__ prm, LjArgs a, double *__restrict__ f,
               double *__restrict__ partials )
{
    __shared__ LjShared<GBMD_MAXT * GBMD_MAXT> sp;
    __shared__ double red[LJ_THREADS / 32];
    for ( int k = threadIdx.x; k < GBMD_MAXT * GBMD_MAXT; k += blockDim.x )
    {
        sp.lj1[k] = prm->lj1[k];
        sp.lj2[k] = prm->lj2[k];
        sp.cutsq[k] = prm->cutsq[k];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0;
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
            const uint32_t e = nlist[(size_t)k * a.n + i];
            const int j = (int)( e & GBMD_JMASK );
            const int sc = (int)( e >> 27 );
            const double4 xj = x[j];
            const int s0 = image_shift( hc[0], sc % 3 - 1, a.nc[0] );
            const int s1 = image_shift( hc[1], ( sc / 3 ) % 3 - 1, a.nc[1] );
            const int s2 = image_shift( hc[2], sc / 9 - 1, a.nc[2] );
            const double dx = dsub( xi.x, img_coord( xj.x, s0, a.L[0] ) );
            const double dy = dsub( xi.y, img_coord( xj.y, s1, a.L[1] ) );
            const double dz = dsub( xi.z, img_coord( xj.z, s2, a.L[2] ) );
            const int tj = (int)xj.w;
            const int tp = ti * GBMD_MAXT + tj;
            const double rsq = dadd( dadd( dmul( dx, dx ), dmul( dy, dy ) ), dmul( dz, dz ) );
            const double cutsq = sp.cutsq[tp];
            if ( rsq < cutsq )
            {
                const double lj1 = sp.lj1[tp], lj2 = sp.lj2[tp];
                const double r2inv = ddiv( 1.0, rsq );
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
                    const double r2invc = ddiv( 1.0, cutsq );
                    const double r6invc = dmul( dmul( r2invc, r2invc ), r2invc );
                    double fac = 0.5;
                    if ( HALF )
                        fac = ( s0 | s1 | s2 ) ? 0.5 : 1.0;
                    pe = dadd( pe, ddiv( dmul( dmul( fac, r6inv ),
                                               dsub( dmul( dmul( 0.5, lj1 ), r6inv ), lj2 ) ),
                                         6.0 ) );
                    pe = dsub( pe, ddiv( dmul( dmul( fac, r6invc ),
                                               dsub( dmul( dmul( 0.5, lj1 ), r6invc ), lj2 ) ),
                                         6.0 ) );
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
            else if ( ZERO )
            {
                f[i] = fx;
                f[a.n + i] = fy;
                f[2 * a.n + i] = fz;
            }
            else
            {
                f[i] = dadd( f[i], fx );
                f[a.n + i] = dadd( f[a.n + i], fy );
                f[2 * a.n + i] = dadd( f[2 * a.n + i], fz );
            }
        }
    }
    if ( EFLAG )
    {
        const double s = block_sum( pe, red );
        if ( threadIdx.x == 0 )
            partials[a.pstride + blockIdx.x] = s;
    }
}

// Mixed precision: FP32 pair math on home-cell-relative coordinates.
__device__ __forceinline__ void kahan_add( float &s, float &c, float v )
{
    const float y = v - c;
    const float t = s + y;
    c = ( t - s ) - y;
    s = t;
}

template <bool FORCE, bool EFLAG, bool HALF, bool ZERO>
__global__ void __launch_bounds__( LJ_THREADS )
    k_lj_mixed( const float4 *__restrict__ xr, const int *__restrict__ home,
                const uint32_t *__restrict__ nlist, const int *__restrict__ nnum,
                const GbmdLJ *__restrict__ prm, LjArgs a, double *__restrict__ f,
                double *__restrict__ partials )
{
    __shared__ float s_lj1[GBMD_MAXT * GBMD_MAXT], s_lj2[GBMD_MAXT * GBMD_MAXT],
        s_cut[GBMD_MAXT * GBMD_MAXT];
    __shared__ double red[LJ_THREADS / 32];
    for ( int k = threadIdx.x; k < GBMD_MAXT * GBMD_MAXT; k += blockDim.x )
    {
        s_lj1[k] = prm->lj1f[k];
        s_lj2[k] = prm->lj2f[k];
        s_cut[k] = prm->cutsqf[k];
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0;
    if ( i < a.n )
    {
        const float4 xi = xr[i];
        const int ti = __float_as_int( xi.w );
        int hc[3];
        if ( HALF && EFLAG )
        {
            const int hp = home[i];
            hc[0] = unpack_home( hp, 0 );
            hc[1] = unpack_home( hp, 1 );
            hc[2] = unpack_home( hp, 2 );
        }
        const int cnt = nnum[i];
        float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
        for ( int k = 0; k < cnt; k++ )
        {
            const uint32_t e = __ldg( &nlist[(size_t)k * a.n + i] );
            const int j = (int)( e & GBMD_JMASK );
            const int sc = (int)( e >> 27 );
            const float4 xj = __ldg( &xr[j] );
            const int o0 = sc % 3 - 1, o1 = ( sc / 3 ) % 3 - 1, o2 = sc / 9 - 1;
            const float dx = xi.x - xj.x - (float)o0 * a.hf[0];
            const float dy = xi.y - xj.y - (float)o1 * a.hf[1];
            const float dz = xi.z - xj.z - (float)o2 * a.hf[2];
            const int tp = ti * GBMD_MAXT + __float_as_int( xj.w );
            const float rsq = dx * dx + dy * dy + dz * dz;
            const float cutsq = s_cut[tp];
            if ( rsq < cutsq )
            {
                const float lj1 = s_lj1[tp], lj2 = s_lj2[tp];
                const float r2inv = 1.0f / rsq;
                const float r6inv = r2inv * r2inv * r2inv;
                if ( FORCE )
                {
                    const float fpair = r6inv * ( lj1 * r6inv - lj2 ) * r2inv;
                    kahan_add( sx, cx, dx * fpair );
                    kahan_add( sy, cy, dy * fpair );
                    kahan_add( sz, cz, dz * fpair );
                    if ( HALF )
                    {
                        atomicAdd( &f[j], -(double)( dx * fpair ) );
                        atomicAdd( &f[a.n + j], -(double)( dy * fpair ) );
                        atomicAdd( &f[2 * a.n + j], -(double)( dz * fpair ) );
                    }
                }
                if ( EFLAG )
                {
                    const float r2invc = 1.0f / cutsq;
                    const float r6invc = r2invc * r2invc * r2invc;
                    float fac = 0.5f;
                    if ( HALF )
                    {
                        const int g0 = image_shift( hc[0], o0, a.nc[0] );
                        const int g1 = image_shift( hc[1], o1, a.nc[1] );
                        const int g2 = image_shift( hc[2], o2, a.nc[2] );
                        fac = ( g0 | g1 | g2 ) ? 0.5f : 1.0f;
                    }
                    pe += (double)( fac * r6inv * ( 0.5f * lj1 * r6inv - lj2 ) / 6.0f ) -
                          (double)( fac * r6invc * ( 0.5f * lj1 * r6invc - lj2 ) / 6.0f );
                }
            }
        }
        if ( FORCE )
        {
            const double fx = (double)sx - (double)cx;
            const double fy = (double)sy - (double)cy;
            const double fz = (double)sz - (double)cz;
            if ( HALF )
            {
                atomicAdd( &f[i], fx );
                atomicAdd( &f[a.n + i], fy );
                atomicAdd( &f[2 * a.n + i], fz );
            }
            else if ( ZERO )
            {
                f[i] = fx;
                f[a.n + i] = fy;
                f[2 * a.n + i] = fz;
            }
            else
            {
                f[i] += fx;
                f[a.n + i] += fy;
                f[2 * a.n + i] += fz;
            }
        }
    }
    if ( EFLAG )
    {
        const double s = block_sum( pe, red );
        if ( threadIdx.x == 0 )
            partials[a.pstride + blockIdx.x] = s;
    }
}

// ---------------------------------------------------------------------------
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
    LjArgs a;
    a.n = n;
    a.ntypes = c->ntypes;
    a.half = c->half;
    for ( int d = 0; d < 3; d++ )
    {
        a.L[d] = c->geom.L[d];
        a.nc[d] = c->geom.nc[d];
        a.hf[d] = c->geom.hf[d];
    }
    a.pstride = stride; // slot 1: potential energy
    const bool half = c->half != 0;
    if ( half && zero_first )
        GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * n, c->stream ) );
    const int blocks = ( n + LJ_THREADS - 1 ) / LJ_THREADS;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_FORCE, &t0 );
#define LJ_ARGS c->nlist.p, c->nnum.p, ljd, a, c->f.p, c->partials.p
    if ( c->precision == GBMD_PREC_FP64 )
    {
        if ( half )
        {
            if ( eflag )
                k_lj_fp64<true, true, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
            else
                k_lj_fp64<true, false, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
        }
        else if ( zero_first )
        {
            if ( eflag )
                k_lj_fp64<true, true, false, true><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
            else
                k_lj_fp64<true, false, false, true><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
        }
        else
        {
            if ( eflag )
                k_lj_fp64<true, true, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
            else
                k_lj_fp64<true, false, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
        }
    }
    else
    {
        if ( half )
        {
            if ( eflag )
                k_lj_mixed<true, true, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
            else
                k_lj_mixed<true, false, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
        }
        else if ( zero_first )
        {
            if ( eflag )
                k_lj_mixed<true, true, false, true><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
            else
                k_lj_mixed<true, false, false, true><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
        }
        else
        {
            if ( eflag )
                k_lj_mixed<true, true, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
            else
                k_lj_mixed<true, false, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
        }
    }
    GBMD_LAUNCH_CHECK( c, "lj force" );
    gbmd_ktime_end( c, GBMD_KT_FORCE, t0 );
    if ( eflag )
        return gbmd_reduce_partials( c, blocks, 1 );
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
    LjArgs a;
    a.n = n;
    a.ntypes = c->ntypes;
    a.half = c->half;
    for ( int d = 0; d < 3; d++ )
    {
        a.L[d] = c->geom.L[d];
        a.nc[d] = c->geom.nc[d];
        a.hf[d] = c->geom.hf[d];
    }
    a.pstride = stride;
    const int blocks = ( n + LJ_THREADS - 1 ) / LJ_THREADS;
    if ( c->precision == GBMD_PREC_FP64 )
    {
        if ( c->half )
            k_lj_fp64<false, true, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
        else
            k_lj_fp64<false, true, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->x.p, c->home.p, LJ_ARGS );
    }
    else
    {
        if ( c->half )
            k_lj_mixed<false, true, true, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
        else
            k_lj_mixed<false, true, false, false><<<blocks, LJ_THREADS, 0, c->stream>>>( c->xr.p, c->home.p, LJ_ARGS );
    }
#undef LJ_ARGS
    GBMD_LAUNCH_CHECK( c, "lj energy" );
    return gbmd_reduce_partials( c, blocks, 1 );
}
