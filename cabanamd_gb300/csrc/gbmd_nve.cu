// gbmd_nve.cu -- velocity-Verlet NVE integration and the thermo
// reductions, with deterministic two-level sums.
//
// Reference (paths inside the CabanaMD project):
//   src/integrator_nve.h:91-110     initial: v += dtf/m f; x += dt v
//                                   final:   v += dtf/m f
//   src/integrator_nve_impl.h:49-54 dtf = 0.5 dt / mvv2e, dtv = dt
//   src/property_kine.h:72-78       sum (v.v) m
//   src/property_temperature.h:73-79
//
// The FP64 updates round every multiply and add separately, exactly like the
// reference's scalar code, so trajectories are bit-identical to a CPU run
// of the same forces.  dtf / m is taken from a per-type table computed on
// the host (the same correctly rounded quotient), because an FP64 divide is
// a long instruction sequence on GB300's narrow FP64 pipe.  In mixed
// precision the initial kernel also refreshes the FP32 home-cell-relative
// position shadow read by the force kernels.
#include "gbmd_internal.cuh"
#include "gbmd_nnp.cuh"

constexpr int NVE_THREADS = 256;
static_assert( NVE_THREADS == NNP_NVE_THREADS, "the NNP job tables count integrator blocks" );

__device__ __forceinline__ double block_sum_nve( double v, double *red )
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

__device__ __forceinline__ float4 shadow_of( const double4 &p, int hp, int t, const GbmdGeom &g )
{
    const double ox = g.lo[0] + ( unpack_home( hp, 0 ) + 0.5 ) * g.h[0];
    const double oy = g.lo[1] + ( unpack_home( hp, 1 ) + 0.5 ) * g.h[1];
    const double oz = g.lo[2] + ( unpack_home( hp, 2 ) + 0.5 ) * g.h[2];
    return make_float4( (float)( p.x - ox ), (float)( p.y - oy ), (float)( p.z - oz ),
                        __int_as_float( t ) );
}

// FINAL: final_integrate of the current step first (with optional sum m v^2
// between the two half kicks) -- the half-list path's fused step tail.
// (The bodies take the block index explicitly: the serving job-table kernel
// runs them for the block's index inside its job.)
template <bool MIXED, bool FINAL, bool THERMO>
__device__ __forceinline__ void
    nve_initial_body( int n, double4 *__restrict__ x, double *__restrict__ v,
                      const double *__restrict__ f, const int *__restrict__ type,
                      const StepArgs &s, const int *__restrict__ home, float4 *__restrict__ xr,
                      const GbmdGeom &g, double *__restrict__ partials, const int bid )
{
    __shared__ double red[NVE_THREADS / 32];
    const int i = bid * blockDim.x + threadIdx.x;
    double mv2 = 0.0;
    if ( i < n )
    {
        const int t = type[i];
        const double dtfm = s.dtfm[t];
        const double fx = f[i], fy = f[n + i], fz = f[2 * n + i];
        double vx = v[i], vy = v[n + i], vz = v[2 * n + i];
        if ( FINAL )
        {
            vx = dadd( vx, dmul( dtfm, fx ) );
            vy = dadd( vy, dmul( dtfm, fy ) );
            vz = dadd( vz, dmul( dtfm, fz ) );
            if ( THERMO )
                mv2 = dmul( dadd( dadd( dmul( vx, vx ), dmul( vy, vy ) ), dmul( vz, vz ) ),
                            s.mass[t] );
        }
        double4 p = x[i];
        vx = dadd( vx, dmul( dtfm, fx ) );
        vy = dadd( vy, dmul( dtfm, fy ) );
        vz = dadd( vz, dmul( dtfm, fz ) );
        p.x = dadd( p.x, dmul( s.dtv, vx ) );
        p.y = dadd( p.y, dmul( s.dtv, vy ) );
        p.z = dadd( p.z, dmul( s.dtv, vz ) );
        v[i] = vx;
        v[n + i] = vy;
        v[2 * n + i] = vz;
        x[i] = p;
        if ( MIXED )
            xr[i] = shadow_of( p, home[i], t, g );
    }
    if ( THERMO )
    {
        const double b = block_sum_nve( mv2, red );
        if ( threadIdx.x == 0 )
            partials[bid] = b;
    }
}

template <bool MIXED, bool FINAL, bool THERMO>
__global__ void __launch_bounds__( NVE_THREADS )
    k_nve_initial( int n, double4 *__restrict__ x, double *__restrict__ v,
                   const double *__restrict__ f, const int *__restrict__ type, StepArgs s,
                   const int *__restrict__ home, float4 *__restrict__ xr, GbmdGeom g,
                   double *__restrict__ partials )
{
    nve_initial_body<MIXED, FINAL, THERMO>( n, x, v, f, type, s, home, xr, g, partials,
                                            (int)blockIdx.x );
}

template <bool UPDATE, bool THERMO>
__device__ __forceinline__ void nve_final_body( int n, double *__restrict__ v,
                                                const double *__restrict__ f,
                                                const int *__restrict__ type, const StepArgs &s,
                                                double *__restrict__ partials, const int bid )
{
    __shared__ double red[NVE_THREADS / 32];
    const int i = bid * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if ( i < n )
    {
        const int t = type[i];
        double vx = v[i], vy = v[n + i], vz = v[2 * n + i];
        if ( UPDATE )
        {
            const double dtfm = s.dtfm[t];
            vx = dadd( vx, dmul( dtfm, f[i] ) );
            vy = dadd( vy, dmul( dtfm, f[n + i] ) );
            vz = dadd( vz, dmul( dtfm, f[2 * n + i] ) );
            v[i] = vx;
            v[n + i] = vy;
            v[2 * n + i] = vz;
        }
        if ( THERMO )
            acc = dmul( dadd( dadd( dmul( vx, vx ), dmul( vy, vy ) ), dmul( vz, vz ) ),
                        s.mass[t] );
    }
    if ( THERMO )
    {
        const double b = block_sum_nve( acc, red );
        if ( threadIdx.x == 0 )
            partials[bid] = b;
    }
}

template <bool UPDATE, bool THERMO>
__global__ void __launch_bounds__( NVE_THREADS )
    k_nve_final( int n, double *__restrict__ v, const double *__restrict__ f,
                 const int *__restrict__ type, StepArgs s, double *__restrict__ partials )
{
    nve_final_body<UPDATE, THERMO>( n, v, f, type, s, partials, (int)blockIdx.x );
}

// Serving: final integrate (+ sum m v^2 where the job is at a thermo step)
// and, unless the job is at its last step, the next initial integrate, for
// every NNP job of the table (mixed precision: the position shadow is
// refreshed too) -- what gbmd_nve_step_tail_launch / gbmd_nve_final_launch
// do for one job.
__global__ void __launch_bounds__( NVE_THREADS ) k_nve_jobs( const __grid_constant__ NnpJobTable t )
{
    const int j = nnp_job_of( t.b_nve, t.njobs, (int)blockIdx.x );
    const NnpJobArgs &J = t.job[j];
    const int bid = (int)blockIdx.x - t.b_nve[j];
    if ( J.last )
    {
        if ( J.thermo )
            nve_final_body<true, true>( J.n, J.v, J.f, J.type, J.s, J.partials, bid );
        else
            nve_final_body<true, false>( J.n, J.v, J.f, J.type, J.s, J.partials, bid );
    }
    else if ( J.thermo )
        nve_initial_body<true, true, true>( J.n, J.x, J.v, J.f, J.type, J.s, J.home, J.xr_out,
                                            J.g, J.partials, bid );
    else
        nve_initial_body<true, true, false>( J.n, J.x, J.v, J.f, J.type, J.s, J.home, J.xr_out,
                                             J.g, J.partials, bid );
}

int gbmd_nve_jobs_launch( const NnpJobTable &t, cudaStream_t st )
{
    k_nve_jobs<<<t.b_nve[t.njobs], NVE_THREADS, 0, st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

// Fixed-order sum of partial sums (per block or per warp) in one launch:
// each block sums one contiguous range (four load-and-add chains per thread,
// then a fixed tree), writes its sum, and the last block to finish (an
// atomic ticket) adds the block sums in index order and resets the ticket.
// The grid depends only on nparts, so the rounding is the same every time.
constexpr int RED_THREADS = 512;
constexpr int RED_BLOCKS_MAX = 64;
static_assert( GBMD_RED_WORDS >= GBMD_RED_RESULTS + RED_BLOCKS_MAX + 1, "red_out too small" );

static int reduce_blocks( int nparts )
{
    const int b = ( nparts + 4095 ) / 4096;
    return b < 1 ? 1 : ( b > RED_BLOCKS_MAX ? RED_BLOCKS_MAX : b );
}

__global__ void __launch_bounds__( RED_THREADS )
    k_reduce_partials( const double *__restrict__ partials, int nparts, double *__restrict__ out,
                       double *__restrict__ block_sums, unsigned *__restrict__ ticket )
{
    __shared__ double red[RED_THREADS / 32];
    __shared__ bool last;
    const int chunk = ( nparts + gridDim.x - 1 ) / gridDim.x;
    const int b0 = blockIdx.x * chunk;
    const int b1 = min( nparts, b0 + chunk );
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    const int bd = blockDim.x;
    int k = b0 + threadIdx.x;
    for ( ; k + 3 * bd < b1; k += 4 * bd )
    {
        s0 += partials[k];
        s1 += partials[k + bd];
        s2 += partials[k + 2 * bd];
        s3 += partials[k + 3 * bd];
    }
    for ( ; k < b1; k += bd )
        s0 += partials[k];
    double s = ( s0 + s1 ) + ( s2 + s3 );
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        s += __shfl_xor_sync( 0xffffffffu, s, o );
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if ( lane == 0 )
        red[w] = s;
    __syncthreads();
    if ( threadIdx.x == 0 )
    {
        double t = 0.0;
        for ( int q = 0; q < bd >> 5; q++ )
            t += red[q];
        block_sums[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd( ticket, 1u ) == gridDim.x - 1;
    }
    __syncthreads();
    if ( !last || w != 0 )
        return;
    __threadfence();
    double t = 0.0;
    for ( int q = lane; q < (int)gridDim.x; q += 32 )
        t += __ldcg( &block_sums[q] );
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        t += __shfl_xor_sync( 0xffffffffu, t, o );
    if ( lane == 0 )
    {
        *out = t;
        *ticket = 0u;
    }
}

int gbmd_partials_prepare( gbmd_ctx *c, int64_t n_items, size_t *slot_stride,
                           GbmdLJ **lj_dev )
{
    const size_t want = (size_t)( n_items / 32 ) + 1024;
    const size_t words_lj = ( sizeof( GbmdLJ ) + sizeof( double ) - 1 ) / sizeof( double );
    if ( c->part_stride < want || !c->partials.p )
    {
        gbmd_release( c, c->partials );
        int rc = gbmd_reserve( c, c->partials, 2 * want + words_lj, "partials" );
        if ( rc )
            return rc;
        c->part_stride = want;
        c->lj_dirty = true;
    }
    GbmdLJ *ljd = (GbmdLJ *)( c->partials.p + 2 * c->part_stride );
    if ( c->lj_dirty )
    {
        GBMD_CUDA( c, cudaMemcpyAsync( ljd, &c->lj, sizeof( GbmdLJ ),
                                       cudaMemcpyHostToDevice, c->stream ) );
        GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
        c->lj_dirty = false;
    }
    if ( slot_stride )
        *slot_stride = c->part_stride;
    if ( lj_dev )
        *lj_dev = ljd;
    return GBMD_OK;
}

int gbmd_reduce_partials( gbmd_ctx *c, int nparts, int slot )
{
    // red_out holds the results [0, 8), the block sums [8, 8 + 64) and the
    // ticket (zero between launches) after them
    double *scratch = c->red_out.p + GBMD_RED_RESULTS;
    unsigned *ticket = reinterpret_cast<unsigned *>( scratch + RED_BLOCKS_MAX );
    k_reduce_partials<<<reduce_blocks( nparts ), RED_THREADS, 0, c->stream>>>(
        c->partials.p + slot * c->part_stride, nparts, c->red_out.p + slot, scratch, ticket );
    GBMD_LAUNCH_CHECK( c, "reduce partials" );
    return GBMD_OK;
}

template <bool FINAL, bool THERMO>
static void launch_initial( gbmd_ctx *c, int blocks, const StepArgs &s, bool mixed )
{
    if ( mixed )
        k_nve_initial<true, FINAL, THERMO><<<blocks, NVE_THREADS, 0, c->stream>>>(
            (int)c->n, c->x.p, c->v.p, c->f.p, c->type.p, s, c->home.p, c->xr.p, c->geom,
            c->partials.p );
    else
        k_nve_initial<false, FINAL, THERMO><<<blocks, NVE_THREADS, 0, c->stream>>>(
            (int)c->n, c->x.p, c->v.p, c->f.p, c->type.p, s, nullptr, nullptr, c->geom,
            c->partials.p );
}

// initial_integrate; with with_final, final_integrate of the previous force
// first (and its thermo sum when thermo is set).
int gbmd_nve_step_tail_launch( gbmd_ctx *c, bool with_final, bool thermo )
{
    const int n = (int)c->n;
    if ( n == 0 )
        return GBMD_OK;
    size_t stride;
    int rc = gbmd_partials_prepare( c, n, &stride, nullptr );
    if ( rc )
        return rc;
    const StepArgs s = gbmd_step_args( c, true );
    const int blocks = ( n + NVE_THREADS - 1 ) / NVE_THREADS;
    const bool mixed = c->precision == GBMD_PREC_MIXED && c->sorted;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_INTEGRATE, &t0 );
    if ( !with_final )
        launch_initial<false, false>( c, blocks, s, mixed );
    else if ( thermo )
        launch_initial<true, true>( c, blocks, s, mixed );
    else
        launch_initial<true, false>( c, blocks, s, mixed );
    GBMD_LAUNCH_CHECK( c, "nve initial" );
    gbmd_ktime_end( c, GBMD_KT_INTEGRATE, t0 );
    if ( with_final && thermo )
        return gbmd_reduce_partials( c, blocks, 0 );
    return GBMD_OK;
}

int gbmd_nve_initial_launch( gbmd_ctx *c ) { return gbmd_nve_step_tail_launch( c, false, false ); }

int gbmd_nve_final_launch( gbmd_ctx *c, bool thermo )
{
    const int n = (int)c->n;
    if ( n == 0 )
        return GBMD_OK;
    size_t stride;
    int rc = gbmd_partials_prepare( c, n, &stride, nullptr );
    if ( rc )
        return rc;
    const StepArgs s = gbmd_step_args( c, false );
    const int blocks = ( n + NVE_THREADS - 1 ) / NVE_THREADS;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_INTEGRATE, &t0 );
    if ( thermo )
        k_nve_final<true, true><<<blocks, NVE_THREADS, 0, c->stream>>>(
            n, c->v.p, c->f.p, c->type.p, s, c->partials.p );
    else
        k_nve_final<true, false><<<blocks, NVE_THREADS, 0, c->stream>>>(
            n, c->v.p, c->f.p, c->type.p, s, c->partials.p );
    GBMD_LAUNCH_CHECK( c, "nve final" );
    gbmd_ktime_end( c, GBMD_KT_INTEGRATE, t0 );
    if ( thermo )
        return gbmd_reduce_partials( c, blocks, 0 );
    return GBMD_OK;
}

int gbmd_mv2_launch( gbmd_ctx *c )
{
    const int n = (int)c->n;
    size_t stride;
    int rc = gbmd_partials_prepare( c, n, &stride, nullptr );
    if ( rc )
        return rc;
    const StepArgs s = gbmd_step_args( c, false );
    const int blocks = ( n + NVE_THREADS - 1 ) / NVE_THREADS;
    if ( n > 0 )
    {
        k_nve_final<false, true><<<blocks, NVE_THREADS, 0, c->stream>>>(
            n, c->v.p, c->f.p, c->type.p, s, c->partials.p );
        GBMD_LAUNCH_CHECK( c, "sum m v^2" );
    }
    return gbmd_reduce_partials( c, blocks, 0 );
}

// Refresh the mixed-precision shadow from the FP64 positions.
__global__ void k_shadow( int n, const double4 *__restrict__ x, const int *__restrict__ type,
                          const int *__restrict__ home, float4 *__restrict__ xr, GbmdGeom g )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    xr[i] = shadow_of( x[i], home[i], type[i], g );
}

int gbmd_update_shadow_launch( gbmd_ctx *c )
{
    const int n = (int)c->n;
    if ( n == 0 || !c->sorted )
        return GBMD_OK;
    k_shadow<<<( n + 255 ) / 256, 256, 0, c->stream>>>( n, c->x.p, c->type.p, c->home.p,
                                                         c->xr.p, c->geom );
    GBMD_LAUNCH_CHECK( c, "shadow" );
    return GBMD_OK;
}
