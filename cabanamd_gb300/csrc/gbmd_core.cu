// gbmd_core.cu -- context, System storage, Comm (single-rank wrap), Binning
// (counting sort by cell), the CbnMD timestep loop and the C ABI glue.
//
// Reference behaviour restated here (paths inside the CabanaMD project):
//   Comm::exchange single rank     src/comm_mpi.h:141-168
//   Binning::create_binning        src/binning_cabana_impl.h:57-113
//   CbnMD::init / CbnMD::run       src/cabanamd_impl.h:70-255, 284-399
//   thermo                         src/property_temperature_impl.h:55-77,
//                                  src/property_kine_impl.h:55-76
#include "gbmd_internal.cuh"
#include "gbmd_nnp.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

extern "C" {
static void graph_cache_clear( gbmd_ctx *c ); // md_run's CUDA graphs
}

// ---------------------------------------------------------------------------
// errors
int gbmd_fail( gbmd_ctx *c, int code, const std::string &msg )
{
    if ( c )
        c->err = msg;
    return code;
}

int gbmd_cuda_check( gbmd_ctx *c, cudaError_t e, const char *what )
{
    if ( e == cudaSuccess )
        return GBMD_OK;
    std::string m = std::string( "CUDA error in " ) + what + ": " +
                    cudaGetErrorString( e );
    // The failed call left its error pending in this thread; it is reported
    // here, so clear it (a sticky error stays), or the next launch check of
    // any context would report it again.
    cudaGetLastError();
    return gbmd_fail( c, GBMD_ERR_CUDA, m );
}

// ---------------------------------------------------------------------------
// kernel timing
void gbmd_ktime_begin( gbmd_ctx *c, int which, cudaEvent_t *start )
{
    (void)which;
    *start = nullptr;
    if ( !c->profiling )
        return;
    cudaEvent_t e;
    if ( !c->ev_pool.empty() )
    {
        e = c->ev_pool.back();
        c->ev_pool.pop_back();
    }
    else
        cudaEventCreate( &e );
    cudaEventRecord( e, c->stream );
    *start = e;
}

void gbmd_ktime_end( gbmd_ctx *c, int which, cudaEvent_t start )
{
    if ( !c->profiling || !start )
        return;
    cudaEvent_t e;
    if ( !c->ev_pool.empty() )
    {
        e = c->ev_pool.back();
        c->ev_pool.pop_back();
    }
    else
        cudaEventCreate( &e );
    cudaEventRecord( e, c->stream );
    c->ev_pending.push_back( { which, { start, e } } );
}

static void ktime_resolve( gbmd_ctx *c )
{
    for ( auto &p : c->ev_pending )
    {
        float ms = 0.f;
        cudaEventSynchronize( p.second.second );
        cudaEventElapsedTime( &ms, p.second.first, p.second.second );
        c->ktime_ms[p.first] += ms;
        c->kcount[p.first] += 1;
        c->ev_pool.push_back( p.second.first );
        c->ev_pool.push_back( p.second.second );
    }
    c->ev_pending.clear();
}

// ---------------------------------------------------------------------------
// exclusive scan of int counts: out[0..n] with out[n] = total
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_scan_tile( const int *__restrict__ in, int *__restrict__ out,
                             int *__restrict__ tile_sums, int n )
{
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for ( int k = 0; k < SCAN_ITEMS; k++ )
    {
        v[k] = ( base + k < n ) ? in[base + k] : 0;
        s += v[k];
    }
    // inclusive warp scan of per-thread sums
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = s;
#pragma unroll
    for ( int o = 1; o < 32; o <<= 1 )
    {
        int t = __shfl_up_sync( 0xffffffffu, incl, o );
        if ( lane >= o )
            incl += t;
    }
    if ( lane == 31 )
        warp_tot[wid] = incl;
    __syncthreads();
    if ( wid == 0 )
    {
        int w = warp_tot[lane];
        int wi = w;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            int t = __shfl_up_sync( 0xffffffffu, wi, o );
            if ( lane >= o )
                wi += t;
        }
        warp_tot[lane] = wi - w; // exclusive
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - s;
#pragma unroll
    for ( int k = 0; k < SCAN_ITEMS; k++ )
    {
        if ( base + k < n )
            out[base + k] = run;
        run += v[k];
    }
    if ( threadIdx.x == SCAN_THREADS - 1 && tile_sums )
        tile_sums[blockIdx.x] = run;
}

__global__ void k_scan_add( int *__restrict__ out, const int *__restrict__ tile_off,
                            int n )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i < n )
        out[i] += tile_off[i / SCAN_TILE];
}

__global__ void k_set_total( int *out, const int *in, int n )
{
    // out[n] = out[n-1] + in[n-1]
    if ( n > 0 )
        out[n] = out[n - 1] + in[n - 1];
    else
        out[0] = 0;
}

// Recursive exclusive scan; tmp must hold enough tile sums for all levels.
static int scan_exclusive( gbmd_ctx *c, const int *in, int *out, int n,
                           int *tmp )
{
    const int tiles = ( n + SCAN_TILE - 1 ) / SCAN_TILE;
    if ( n == 0 )
    {
        k_set_total<<<1, 1, 0, c->stream>>>( out, in, 0 );
        GBMD_LAUNCH_CHECK( c, "scan" );
        return GBMD_OK;
    }
    if ( tiles == 1 )
    {
        k_scan_tile<<<1, SCAN_THREADS, 0, c->stream>>>( in, out, nullptr, n );
    }
    else
    {
        int *sums = tmp;
        int *offs = tmp + tiles + 1;
        k_scan_tile<<<tiles, SCAN_THREADS, 0, c->stream>>>( in, out, sums, n );
        GBMD_LAUNCH_CHECK( c, "scan tile" );
        int rc = scan_exclusive( c, sums, offs, tiles, offs + tiles + 1 );
        if ( rc )
            return rc;
        k_scan_add<<<( n + 255 ) / 256, 256, 0, c->stream>>>( out, offs, n );
    }
    GBMD_LAUNCH_CHECK( c, "scan" );
    k_set_total<<<1, 1, 0, c->stream>>>( out, in, n );
    GBMD_LAUNCH_CHECK( c, "scan total" );
    return GBMD_OK;
}

// ---------------------------------------------------------------------------
// Comm::exchange (comm_mpi.h:141-168): x > L -> x - L, x < 0 -> x + L per
// dimension; every test reads the pre-wrap value, and only wrapped atoms are
// stored.  Flags atoms that are NaN or outside [lo - L, lo + 2L] afterwards
// (the image model of a single-rank halo cannot hold them); the bounds come
// from the host (2L is exact, so they equal the per-atom expressions).
// An int64 whose signed order is the numeric order of finite doubles: the
// bits of x, with the magnitude bits of negative values flipped (sign-
// magnitude to two's complement) and -0 taken as +0.  NaNs map beyond the
// infinities, so no comparison with finite bounds accepts them -- as no IEEE
// comparison does.  GB300's FP64 pipe runs at ~1/64 of its FP32 rate, so the
// rebuild's per-atom compares use these keys on the integer pipes.
__device__ __forceinline__ long long dkey( double x )
{
    long long b = __double_as_longlong( x );
    b = b == (long long)0x8000000000000000ull ? 0 : b;
    return b ^ ( ( b >> 63 ) & 0x7fffffffffffffffll );
}

// Wraps atom i in place and returns its position after the wrap.
__device__ __forceinline__ double4 wrap_atom( double4 *__restrict__ x, int i, double Lx,
                                              double Ly, double Lz, double3 blo, double3 bhi,
                                              int *__restrict__ flags )
{
    double4 p = x[i];
    // x > L and x < 0 on the keys (the same outcomes as the FP64 compares;
    // a NaN may be "moved", staying NaN, and is flagged below either way)
    const long long kx = dkey( p.x ), ky = dkey( p.y ), kz = dkey( p.z );
    bool moved = false;
    if ( kx > dkey( Lx ) )
    {
        p.x = dsub( p.x, Lx );
        moved = true;
    }
    if ( kx < 0 )
    {
        p.x = dadd( p.x, Lx );
        moved = true;
    }
    if ( ky > dkey( Ly ) )
    {
        p.y = dsub( p.y, Ly );
        moved = true;
    }
    if ( ky < 0 )
    {
        p.y = dadd( p.y, Ly );
        moved = true;
    }
    if ( kz > dkey( Lz ) )
    {
        p.z = dsub( p.z, Lz );
        moved = true;
    }
    if ( kz < 0 )
    {
        p.z = dadd( p.z, Lz );
        moved = true;
    }
    long long qx = kx, qy = ky, qz = kz;
    if ( moved )
    {
        x[i] = p;
        qx = dkey( p.x );
        qy = dkey( p.y );
        qz = dkey( p.z );
    }
    const bool bad = !( qx >= dkey( blo.x ) && qx <= dkey( bhi.x ) ) ||
                     !( qy >= dkey( blo.y ) && qy <= dkey( bhi.y ) ) ||
                     !( qz >= dkey( blo.z ) && qz <= dkey( bhi.z ) );
    if ( bad )
        atomicAdd( &flags[1], 1 );
    return p;
}

__global__ void k_wrap( double4 *__restrict__ x, int n, double Lx, double Ly, double Lz,
                        double3 blo, double3 bhi, int *__restrict__ flags )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    wrap_atom( x, i, Lx, Ly, Lz, blo, bhi, flags );
}

// Cell index floor((x - lo) / h), clamped to [0, nc), exactly as the FP64
// division gives it (binning_cabana_impl.h:57-113 bins by that quotient).
// The FP32 estimate t = (float)(x - lo) * (float)(1 / h) is within
// 3 * 2^-24 |t| (+ second order) of the FP64 quotient, i.e. below 1e-3 for
// |t| < 4096 (at most 1024 cells per dimension).  So when t is further than
// 1e-3 from an integer its floor is the FP64 one; otherwise (and for NaN,
// infinity or |t| >= 4096) the correctly rounded FP64 division decides.
// This keeps the FP64 pipe (1/64 of the FP32 rate) to one subtraction and one
// conversion per coordinate instead of a division.
__device__ __forceinline__ int cell_1d( double xd, double lo, double h, float hinv_f, int nc )
{
    const double d = dsub( xd, lo );
    const float tf = (float)d * hinv_f;
    if ( fabsf( tf - rintf( tf ) ) > 1.0e-3f && fabsf( tf ) < 4096.0f )
    {
        const int c = (int)floorf( tf );
        return c < 0 ? 0 : ( c > nc - 1 ? nc - 1 : c );
    }
    const double t = floor( ddiv( d, h ) );
    return t < 0.0 ? 0 : ( t > (double)( nc - 1 ) ? nc - 1 : (int)t );
}

// Add one per lane to counter[k], aggregated over the lanes of the warp that
// share k (atoms arrive nearly cell-sorted from the previous binning, so a
// warp's 32 atoms fall in two or three cells); returns the lane's old value
// plus its rank among those lanes.  valid = false lanes take part in the
// match but add nothing.
__device__ __forceinline__ int warp_count_add( int *counter, int k, bool valid )
{
    const int lane = threadIdx.x & 31;
    const unsigned same = __match_any_sync( 0xffffffffu, valid ? k : -1 );
    const int leader = __ffs( same ) - 1;
    int base = 0;
    if ( valid && lane == leader )
        base = atomicAdd( &counter[k], __popc( same ) );
    base = __shfl_sync( 0xffffffffu, base, leader );
    return base + __popc( same & ( ( 1u << lane ) - 1u ) );
}

// Cell key of atom i at position p, counted into its cell; every lane of
// the warp takes part (valid = false lanes add nothing).
__device__ __forceinline__ void cell_count_atom( double4 p, bool valid, int i, const GbmdGeom &g,
                                                 int *__restrict__ key, int *__restrict__ count )
{
    int k = 0;
    if ( valid )
    {
        const int cx = cell_1d( p.x, g.lo[0], g.h[0], g.hinv_f[0], g.nc[0] );
        const int cy = cell_1d( p.y, g.lo[1], g.h[1], g.hinv_f[1], g.nc[1] );
        const int cz = cell_1d( p.z, g.lo[2], g.h[2], g.hinv_f[2], g.nc[2] );
        k = cx + g.nc[0] * ( cy + g.nc[1] * cz );
        key[i] = k;
    }
    warp_count_add( count, k, valid );
}

__global__ void k_cell_count( const double4 *__restrict__ x, int n, GbmdGeom g,
                              int *__restrict__ key, int *__restrict__ count )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const double4 p = valid ? x[i] : make_double4( 0.0, 0.0, 0.0, 0.0 );
    cell_count_atom( p, valid, i, g, key, count );
}

__device__ __forceinline__ void cell_fill_atom( const int *__restrict__ key, int n,
                                                const int *__restrict__ start,
                                                int *__restrict__ fill,
                                                int *__restrict__ slot_atom, int i )
{
    const bool valid = i < n;
    const int k = valid ? key[i] : 0;
    const int s = warp_count_add( fill, k, valid );
    if ( valid )
        slot_atom[start[k] + s] = i;
}

__global__ void k_cell_fill( const int *__restrict__ key, int n,
                             const int *__restrict__ start, int *__restrict__ fill,
                             int *__restrict__ slot_atom )
{
    cell_fill_atom( key, n, start, fill, slot_atom, blockIdx.x * blockDim.x + threadIdx.x );
}

// One warp per cell: rank the cell's atoms by (id, old index) so the order
// inside a cell does not depend on atomic arrival order.
__device__ __forceinline__ void cell_order_warp( const int *__restrict__ start,
                                                 const int *__restrict__ slot_atom,
                                                 const int *__restrict__ id, int ncell, int nc0,
                                                 int nc1, int *__restrict__ perm,
                                                 int *__restrict__ home, int warp )
{
    const int lane = threadIdx.x & 31;
    if ( warp >= ncell )
        return;
    const int b = start[warp], e = start[warp + 1];
    // the cell's coordinates, packed, for every slot it owns (the permute
    // kernel reads them instead of binning the position again)
    const int hp = ( warp % nc0 ) | ( ( ( warp / nc0 ) % nc1 ) << 10 ) |
                   ( ( warp / ( nc0 * nc1 ) ) << 20 );
    for ( int a = b + lane; a < e; a += 32 )
        home[a] = hp;
    for ( int a = b + lane; a < e; a += 32 )
    {
        const int ia = slot_atom[a];
        const int ida = id[ia];
        int rank = 0;
        for ( int q = b; q < e; q++ )
        {
            const int iq = slot_atom[q];
            const int idq = id[iq];
            rank += ( idq < ida ) || ( idq == ida && iq < ia );
        }
        perm[b + rank] = ia;
    }
}

__global__ void k_cell_order( const int *__restrict__ start,
                              const int *__restrict__ slot_atom,
                              const int *__restrict__ id, int ncell, int nc0, int nc1,
                              int *__restrict__ perm, int *__restrict__ home )
{
    cell_order_warp( start, slot_atom, id, ncell, nc0, nc1, perm, home,
                     ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5 );
}

// Gather every per-atom array into cell order and set the home cell and
// the mixed-precision shadow.
__device__ __forceinline__ void permute_atom( const int *__restrict__ perm, int n,
                                              const GbmdGeom &g,
                                              const double4 *__restrict__ x_in,
                                              double4 *__restrict__ x_out,
                                              const double *__restrict__ v_in,
                                              double *__restrict__ v_out,
                                              const int *__restrict__ t_in,
                                              int *__restrict__ t_out,
                                              const int *__restrict__ id_in,
                                              int *__restrict__ id_out,
                                              const int *__restrict__ home,
                                              float4 *__restrict__ xr,
                                              float4 *__restrict__ xr_alt,
                                              uint8_t *__restrict__ gflag, int k )
{
    if ( k == 0 )
    {
        // Sentinel atom n of both shadow buffers: padded list rows point at
        // it; it lies outside every cutoff of every atom.
        const float far = 1.0e15f;
        xr[n] = make_float4( far, far, far, __int_as_float( 0 ) );
        xr_alt[n] = make_float4( far, far, far, __int_as_float( 0 ) );
    }
    if ( k >= n )
        return;
    const int o = perm[k];
    const double4 p = x_in[o];
    x_out[k] = p;
    const long long kx = dkey( p.x ), ky = dkey( p.y ), kz = dkey( p.z );
    gflag[k] = (uint8_t)( ( kx >= dkey( g.thr_hi[0] ) ) | ( ( kx <= dkey( g.thr_lo[0] ) ) << 1 ) |
                          ( ( ky >= dkey( g.thr_hi[1] ) ) << 2 ) |
                          ( ( ky <= dkey( g.thr_lo[1] ) ) << 3 ) |
                          ( ( kz >= dkey( g.thr_hi[2] ) ) << 4 ) |
                          ( ( kz <= dkey( g.thr_lo[2] ) ) << 5 ) );
    v_out[k] = v_in[o];
    v_out[n + k] = v_in[n + o];
    v_out[2 * n + k] = v_in[2 * n + o];
    const int t = t_in[o];
    t_out[k] = t;
    id_out[k] = id_in[o];
    // the destination slot's cell, written by k_cell_order (the cell the
    // binning gave this position)
    const int hp = home[k];
    const int cx = unpack_home( hp, 0 ), cy = unpack_home( hp, 1 ), cz = unpack_home( hp, 2 );
    {
        // relative to the home cell's centre: |xr| <= h/2 (+ motion), so
        // the FP32 rounding is half that of a corner origin
        const double ox = g.lo[0] + ( cx + 0.5 ) * g.h[0];
        const double oy = g.lo[1] + ( cy + 0.5 ) * g.h[1];
        const double oz = g.lo[2] + ( cz + 0.5 ) * g.h[2];
        xr[k] = make_float4( (float)( p.x - ox ), (float)( p.y - oy ),
                             (float)( p.z - oz ), __int_as_float( t ) );
    }
}

__global__ void k_permute( const int *__restrict__ perm, int n, GbmdGeom g,
                           const double4 *__restrict__ x_in, double4 *__restrict__ x_out,
                           const double *__restrict__ v_in, double *__restrict__ v_out,
                           const int *__restrict__ t_in, int *__restrict__ t_out,
                           const int *__restrict__ id_in, int *__restrict__ id_out,
                           const int *__restrict__ home, float4 *__restrict__ xr,
                           float4 *__restrict__ xr_alt, uint8_t *__restrict__ gflag )
{
    permute_atom( perm, n, g, x_in, x_out, v_in, v_out, t_in, t_out, id_in, id_out, home, xr,
                  xr_alt, gflag, blockIdx.x * blockDim.x + threadIdx.x );
}

// ---------------------------------------------------------------------------
static int blocks_for( int64_t n, int t ) { return (int)( ( n + t - 1 ) / t ); }

static void make_geom( gbmd_ctx *c, double cut )
{
    GbmdGeom &g = c->geom;
    g.ncell = 1;
    for ( int d = 0; d < 3; d++ )
    {
        g.lo[d] = c->lo[d];
        g.hi[d] = c->hi[d];
        g.L[d] = c->hi[d] - c->lo[d];
        int nc = (int)std::floor( g.L[d] / ( cut * ( 1.0 + 1e-10 ) ) );
        if ( nc < 1 )
            nc = 1;
        if ( nc > GBMD_MAX_CELLS_PER_DIM )
            nc = GBMD_MAX_CELLS_PER_DIM;
        g.nc[d] = nc;
        g.h[d] = g.L[d] / nc;
        g.hf[d] = (float)g.h[d];
        g.hinv_f[d] = (float)( 1.0 / g.h[d] );
        g.thr_hi[d] = c->hi[d] - cut;
        g.thr_lo[d] = c->lo[d] + cut;
        g.ncell *= nc;
    }
    c->grid_cut = cut;
}

static int do_exchange( gbmd_ctx *c )
{
    if ( c->n == 0 )
        return GBMD_OK;
    const double L[3] = { c->hi[0] - c->lo[0], c->hi[1] - c->lo[1],
                          c->hi[2] - c->lo[2] };
    const double3 blo = make_double3( c->lo[0] - L[0], c->lo[1] - L[1], c->lo[2] - L[2] );
    const double3 bhi = make_double3( c->lo[0] + 2.0 * L[0], c->lo[1] + 2.0 * L[1],
                                      c->lo[2] + 2.0 * L[2] );
    k_wrap<<<blocks_for( c->n, 256 ), 256, 0, c->stream>>>( c->x.p, (int)c->n, L[0], L[1], L[2],
                                                           blo, bhi, c->flags.p );
    GBMD_LAUNCH_CHECK( c, "wrap" );
    return GBMD_OK;
}

// The binning's grid and buffers for cutoff cut (host side; allocations are
// ordered on the context's stream).
static int binning_prepare( gbmd_ctx *c, double cut )
{
    make_geom( c, cut );
    const int n = (int)c->n;
    const int ncell = c->geom.ncell;
    int rc;
    if ( ( rc = gbmd_reserve( c, c->cell_key, n, "cell_key" ) ) ||
         ( rc = gbmd_reserve( c, c->cell_count, ncell + 1, "cell_count" ) ) ||
         ( rc = gbmd_reserve( c, c->cell_fill, ncell + 1, "cell_fill" ) ) ||
         ( rc = gbmd_reserve( c, c->cell_start, ncell + 1, "cell_start" ) ) ||
         ( rc = gbmd_reserve( c, c->perm, n, "perm" ) ) ||
         ( rc = gbmd_reserve( c, c->scan_tmp, ncell / 1024 + 64, "scan_tmp" ) ) ||
         ( rc = gbmd_reserve( c, c->x_alt, n, "x_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->v_alt, 3 * (size_t)n, "v_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->type_alt, n, "type_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->id_alt, n, "id_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->home, n, "home" ) ) ||
         ( rc = gbmd_reserve( c, c->xr, n + 1, "xr" ) ) ||
         ( rc = gbmd_reserve( c, c->xr_alt, n + 1, "xr_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->gflag, n, "gflag" ) ) )
        return rc;
    return GBMD_OK;
}

static int do_binning( gbmd_ctx *c, double cut )
{
    int rc;
    if ( ( rc = binning_prepare( c, cut ) ) )
        return rc;
    const int n = (int)c->n;
    const int ncell = c->geom.ncell;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_SORT, &t0 );
    GBMD_CUDA( c, cudaMemsetAsync( c->cell_count.p, 0, sizeof( int ) * ( ncell + 1 ),
                                   c->stream ) );
    GBMD_CUDA( c, cudaMemsetAsync( c->cell_fill.p, 0, sizeof( int ) * ( ncell + 1 ),
                                   c->stream ) );
    if ( n > 0 )
    {
        k_cell_count<<<blocks_for( n, 256 ), 256, 0, c->stream>>>(
            c->x.p, n, c->geom, c->cell_key.p, c->cell_count.p );
        GBMD_LAUNCH_CHECK( c, "cell_count" );
    }
    if ( ( rc = scan_exclusive( c, c->cell_count.p, c->cell_start.p, ncell,
                                c->scan_tmp.p ) ) )
        return rc;
    if ( n > 0 )
    {
        // perm doubles as the unordered slot->atom map, then cell_key's
        // storage receives the ordered permutation.
        k_cell_fill<<<blocks_for( n, 256 ), 256, 0, c->stream>>>(
            c->cell_key.p, n, c->cell_start.p, c->cell_fill.p, c->perm.p );
        GBMD_LAUNCH_CHECK( c, "cell_fill" );
        k_cell_order<<<blocks_for( (int64_t)ncell * 32, 256 ), 256, 0, c->stream>>>(
            c->cell_start.p, c->perm.p, c->id.p, ncell, c->geom.nc[0], c->geom.nc[1],
            c->cell_key.p, c->home.p );
        GBMD_LAUNCH_CHECK( c, "cell_order" );
        k_permute<<<blocks_for( n, 256 ), 256, 0, c->stream>>>(
            c->cell_key.p, n, c->geom, c->x.p, c->x_alt.p, c->v.p, c->v_alt.p,
            c->type.p, c->type_alt.p, c->id.p, c->id_alt.p, c->home.p, c->xr.p,
            c->xr_alt.p, c->gflag.p );
        GBMD_LAUNCH_CHECK( c, "permute" );
        std::swap( c->x, c->x_alt );
        std::swap( c->v, c->v_alt );
        std::swap( c->type, c->type_alt );
        std::swap( c->id, c->id_alt );
    }
    gbmd_ktime_end( c, GBMD_KT_SORT, t0 );
    c->sorted = true;
    c->have_list = false;
    return GBMD_OK;
}

int gbmd_rebuild( gbmd_ctx *c )
{
    const double cut = c->md.force_cut + c->md.skin;
    int rc;
    if ( ( rc = do_exchange( c ) ) )
        return rc;
    if ( ( rc = do_binning( c, cut ) ) )
        return rc;
    c->half = c->md.half;
    c->neigh_cut = cut;
    if ( c->md.max_neigh_guess > c->max_neigh_guess )
        c->max_neigh_guess = c->md.max_neigh_guess;
    if ( ( rc = gbmd_build_list( c ) ) )
        return rc;
    c->rebuilds++;
    return GBMD_OK;
}

// ---------------------------------------------------------------------------
// Rebuilds of several systems that share one stream (the serving engine's
// jobs), batched into job-table launches.  Each phase of gbmd_rebuild_launch
// -- zeroing of the cell counters, wrap (fused with the cell count), scan,
// fill, in-cell order, permute, then the list build (gbmd_neigh.cu) -- is one
// launch for all the jobs.  Every block finds its job in the table (binary
// search over per-job block offsets) and runs the single-system kernel's
// body on that job's arrays, so each job's order, shadow and list are those
// its own launches would give.
constexpr int RB_JOBS = 32;           // jobs per job-table launch
constexpr int RB_MAX_CELLS = 1 << 18; // cells whose counts one block scans

struct RbJob
{
    double4 *x, *x_alt;
    double *v, *v_alt;
    int *type, *type_alt, *id, *id_alt;
    int *cell_key, *cell_count, *cell_fill, *cell_start, *perm, *home;
    float4 *xr, *xr_alt;
    uint8_t *gflag;
    int *flags;
    GbmdGeom g;
    double3 blo, bhi; // bounds outside which a wrapped atom is lost
    int n;
};

struct RbTable
{
    int njobs;
    int block0[RB_JOBS + 1]; // first block of each job in this launch
    RbJob job[RB_JOBS];
};
static_assert( sizeof( RbTable ) <= 32764, "job table exceeds the kernel parameter space" );

__device__ __forceinline__ const RbJob &rb_job( const RbTable &t, int &local )
{
    int lo = 0, hi = t.njobs - 1;
    while ( lo < hi )
    {
        const int mid = ( lo + hi + 1 ) >> 1;
        if ( t.block0[mid] <= (int)blockIdx.x )
            lo = mid;
        else
            hi = mid - 1;
    }
    local = (int)blockIdx.x - t.block0[lo];
    return t.job[lo];
}

// cell_count = cell_fill = 0 (ncell + 1 entries), list row maximum = 0
__global__ void __launch_bounds__( 256 ) k_rb_zero( const __grid_constant__ RbTable t )
{
    int lb;
    const RbJob &J = rb_job( t, lb );
    const int k = lb * 256 + (int)threadIdx.x;
    if ( k <= J.g.ncell )
    {
        J.cell_count[k] = 0;
        J.cell_fill[k] = 0;
    }
    if ( k == 0 )
        J.flags[0] = 0;
}

// Comm::exchange's wrap, then the cell count of the wrapped position
__global__ void __launch_bounds__( 256 ) k_rb_wrap_count( const __grid_constant__ RbTable t )
{
    int lb;
    const RbJob &J = rb_job( t, lb );
    const int i = lb * 256 + (int)threadIdx.x;
    const bool valid = i < J.n;
    double4 p = make_double4( 0.0, 0.0, 0.0, 0.0 );
    if ( valid )
        p = wrap_atom( J.x, i, J.g.L[0], J.g.L[1], J.g.L[2], J.blo, J.bhi, J.flags );
    cell_count_atom( p, valid, i, J.g, J.cell_key, J.cell_count );
}

// Exclusive scan of one job's cell counts per block, tile after tile with a
// running carry (k_scan_tile's arithmetic); cell_start[ncell] = the total.
__global__ void __launch_bounds__( SCAN_THREADS ) k_rb_scan( const __grid_constant__ RbTable t )
{
    const RbJob &J = t.job[blockIdx.x];
    const int n = J.g.ncell;
    const int *__restrict__ in = J.cell_count;
    int *__restrict__ out = J.cell_start;
    __shared__ int warp_tot[SCAN_THREADS / 32];
    __shared__ int tile_total;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int carry = 0;
    for ( int t0 = 0; t0 < n; t0 += SCAN_TILE )
    {
        const int base = t0 + (int)threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int s = 0;
#pragma unroll
        for ( int k = 0; k < SCAN_ITEMS; k++ )
        {
            v[k] = ( base + k < n ) ? in[base + k] : 0;
            s += v[k];
        }
        int incl = s;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            const int u = __shfl_up_sync( 0xffffffffu, incl, o );
            if ( lane >= o )
                incl += u;
        }
        if ( lane == 31 )
            warp_tot[wid] = incl;
        __syncthreads();
        if ( wid == 0 )
        {
            const int w = warp_tot[lane];
            int wi = w;
#pragma unroll
            for ( int o = 1; o < 32; o <<= 1 )
            {
                const int u = __shfl_up_sync( 0xffffffffu, wi, o );
                if ( lane >= o )
                    wi += u;
            }
            warp_tot[lane] = wi - w; // exclusive
            if ( lane == 31 )
                tile_total = wi;
        }
        __syncthreads();
        int run = carry + warp_tot[wid] + incl - s;
#pragma unroll
        for ( int k = 0; k < SCAN_ITEMS; k++ )
        {
            if ( base + k < n )
                out[base + k] = run;
            run += v[k];
        }
        carry += tile_total;
        __syncthreads(); // warp_tot and tile_total are rewritten by the next tile
    }
    if ( threadIdx.x == 0 )
        out[n] = carry;
}

__global__ void __launch_bounds__( 256 ) k_rb_fill( const __grid_constant__ RbTable t )
{
    int lb;
    const RbJob &J = rb_job( t, lb );
    cell_fill_atom( J.cell_key, J.n, J.cell_start, J.cell_fill, J.perm,
                    lb * 256 + (int)threadIdx.x );
}

__global__ void __launch_bounds__( 256 ) k_rb_order( const __grid_constant__ RbTable t )
{
    int lb;
    const RbJob &J = rb_job( t, lb );
    cell_order_warp( J.cell_start, J.perm, J.id, J.g.ncell, J.g.nc[0], J.g.nc[1], J.cell_key,
                     J.home, ( lb * 256 + (int)threadIdx.x ) >> 5 );
}

__global__ void __launch_bounds__( 256 ) k_rb_permute( const __grid_constant__ RbTable t )
{
    int lb;
    const RbJob &J = rb_job( t, lb );
    permute_atom( J.cell_key, J.n, J.g, J.x, J.x_alt, J.v, J.v_alt, J.type, J.type_alt, J.id,
                  J.id_alt, J.home, J.xr, J.xr_alt, J.gflag, lb * 256 + (int)threadIdx.x );
}

// Cells of the grid make_geom builds for cutoff cut (no side effects).
static int64_t grid_cells( const gbmd_ctx *c, double cut )
{
    int64_t cells = 1;
    for ( int d = 0; d < 3; d++ )
    {
        int nc = (int)std::floor( ( c->hi[d] - c->lo[d] ) / ( cut * ( 1.0 + 1e-10 ) ) );
        nc = std::min( std::max( nc, 1 ), GBMD_MAX_CELLS_PER_DIM );
        cells *= nc;
    }
    return cells;
}

bool gbmd_rebuild_batchable( const gbmd_ctx *c )
{
    return c->n > 0 && !c->profiling &&
           grid_cells( c, c->md.force_cut + c->md.skin ) <= RB_MAX_CELLS;
}

int gbmd_rebuild_prepare( gbmd_ctx *c )
{
    const double cut = c->md.force_cut + c->md.skin;
    int rc;
    if ( ( rc = binning_prepare( c, cut ) ) )
        return rc;
    c->half = c->md.half;
    c->neigh_cut = cut;
    if ( c->md.max_neigh_guess > c->max_neigh_guess )
        c->max_neigh_guess = c->md.max_neigh_guess;
    c->nl_attempts = 0;
    return gbmd_build_list_prepare( c );
}

int gbmd_rebuild_batch_launch( gbmd_ctx *const *cs, int count, int64_t *launches )
{
    if ( count <= 0 )
        return GBMD_OK;
    const cudaStream_t st = cs[0]->stream;
    RbTable t;
    std::memset( &t, 0, sizeof t );
    // per-job blocks of a phase: 0 = cells + 1, 1 = atoms, 2 = a warp per cell
    auto set_blocks = [&]( int nj, int kind ) -> int {
        int tot = 0;
        for ( int q = 0; q < nj; q++ )
        {
            const RbJob &J = t.job[q];
            t.block0[q] = tot;
            tot += kind == 0 ? blocks_for( (int64_t)J.g.ncell + 1, 256 )
                             : ( kind == 1 ? blocks_for( J.n, 256 )
                                           : blocks_for( (int64_t)J.g.ncell * 32, 256 ) );
        }
        t.block0[nj] = tot;
        return tot;
    };
    auto check = [&]( const char *what ) -> int {
        ( *launches )++;
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GBMD_OK : gbmd_cuda_check( cs[0], e, what );
    };
    int rc;
    for ( int b = 0; b < count; b += RB_JOBS )
    {
        const int nj = std::min( RB_JOBS, count - b );
        t.njobs = nj;
        for ( int q = 0; q < nj; q++ )
        {
            gbmd_ctx *c = cs[b + q];
            RbJob &J = t.job[q];
            J.x = c->x.p;
            J.x_alt = c->x_alt.p;
            J.v = c->v.p;
            J.v_alt = c->v_alt.p;
            J.type = c->type.p;
            J.type_alt = c->type_alt.p;
            J.id = c->id.p;
            J.id_alt = c->id_alt.p;
            J.cell_key = c->cell_key.p;
            J.cell_count = c->cell_count.p;
            J.cell_fill = c->cell_fill.p;
            J.cell_start = c->cell_start.p;
            J.perm = c->perm.p;
            J.home = c->home.p;
            J.xr = c->xr.p;
            J.xr_alt = c->xr_alt.p;
            J.gflag = c->gflag.p;
            J.flags = c->flags.p;
            J.g = c->geom;
            const double L[3] = { c->hi[0] - c->lo[0], c->hi[1] - c->lo[1],
                                  c->hi[2] - c->lo[2] };
            J.blo = make_double3( c->lo[0] - L[0], c->lo[1] - L[1], c->lo[2] - L[2] );
            J.bhi = make_double3( c->lo[0] + 2.0 * L[0], c->lo[1] + 2.0 * L[1],
                                  c->lo[2] + 2.0 * L[2] );
            J.n = (int)c->n;
        }
        k_rb_zero<<<set_blocks( nj, 0 ), 256, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: zero" ) ) )
            return rc;
        k_rb_wrap_count<<<set_blocks( nj, 1 ), 256, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: wrap and count" ) ) )
            return rc;
        k_rb_scan<<<nj, SCAN_THREADS, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: scan" ) ) )
            return rc;
        k_rb_fill<<<set_blocks( nj, 1 ), 256, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: fill" ) ) )
            return rc;
        k_rb_order<<<set_blocks( nj, 2 ), 256, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: order" ) ) )
            return rc;
        k_rb_permute<<<set_blocks( nj, 1 ), 256, 0, st>>>( t );
        if ( ( rc = check( "rebuild batch: permute" ) ) )
            return rc;
    }
    for ( int q = 0; q < count; q++ )
    {
        gbmd_ctx *c = cs[q];
        std::swap( c->x, c->x_alt );
        std::swap( c->v, c->v_alt );
        std::swap( c->type, c->type_alt );
        std::swap( c->id, c->id_alt );
        c->sorted = true;
        c->have_list = false;
    }
    return gbmd_build_list_batch( cs, count, launches );
}

int gbmd_rebuild_check( gbmd_ctx *c, bool *again )
{
    int rc = gbmd_build_list_check( c, again );
    if ( rc == GBMD_OK && !*again )
        c->rebuilds++;
    return rc;
}

// ---------------------------------------------------------------------------
// Force dispatch
static int force_launch( gbmd_ctx *c, bool eflag, bool zero_first )
{
    if ( !c->have_list )
        return gbmd_fail( c, GBMD_ERR_ARG, "force: no neighbor list (call gbmd_neigh_build)" );
    if ( c->force_type == GBMD_FORCE_LJ )
    {
        if ( !c->lj_set )
            return gbmd_fail( c, GBMD_ERR_ARG, "force: LJ coefficients not set" );
        return gbmd_lj_launch( c, eflag, zero_first );
    }
    if ( c->force_type == GBMD_FORCE_NNP )
    {
        if ( !c->nnp )
            return gbmd_fail( c, GBMD_ERR_ARG, "force: NNP potential not loaded" );
        if ( zero_first )
            GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * c->n,
                                           c->stream ) );
        return gbmd_nnp_launch( c, eflag, true );
    }
    return gbmd_fail( c, GBMD_ERR_ARG, "force: unknown force type" );
}

// Device-side error flags (already copied to h_flags).
static int check_flags( gbmd_ctx *c )
{
    if ( c->h_flags[1] )
        return gbmd_fail( c, GBMD_ERR_LOST_ATOM,
                          "atoms lost: position NaN or more than one box outside" );
    if ( c->h_flags[2] )
        return gbmd_fail( c, GBMD_ERR_CAPACITY,
                          "nnp: an atom has more than " +
                              std::to_string( c->nl_maxc > NNP_MAXNBR ? NNP_MAXNBR_LARGE
                                                                      : NNP_MAXNBR ) +
                              " neighbours inside the NNP cutoff (" +
                              std::to_string( c->h_flags[2] ) + ")" );
    if ( c->h_flags[3] )
        return gbmd_fail( c, GBMD_ERR_TIMEOUT, "a bounded device wait timed out" );
    return GBMD_OK;
}

static int read_reductions( gbmd_ctx *c )
{
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_red, c->red_out.p, 4 * sizeof( double ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, 4 * sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return check_flags( c );
}

// Force::compute_energy from the reduced sum in red_out[1]: the LJ kernels
// reduce the energy itself; the NNP kernels reduce sum E_i, which
// ForceNNP::compute_energy turns into the reported total.
static double potential_energy_from( const gbmd_ctx *c, const double *red )
{
    if ( c->force_type == GBMD_FORCE_NNP && c->nnp )
        return gbmd_nnp_total_energy( c, red[1] );
    return red[1];
}

static double potential_energy( const gbmd_ctx *c ) { return potential_energy_from( c, c->h_red ); }

// Thermo row [step, T, PE/N, KE/N] from reduced sums red[0] = sum m v^2 and
// red[1] = the force's energy sum (cabanamd_impl.h:365-372).
void gbmd_thermo_row_from( const gbmd_ctx *c, int64_t step, const double *red, double *row )
{
    const double smv2 = red[0];
    const int64_t dof = 3 * c->n - 3;
    const double T = smv2 * ( c->mvv2e / ( 1.0 * dof * c->boltz ) );
    const double KE = smv2 * ( 0.5 * c->mvv2e );
    const double PE = potential_energy_from( c, red );
    row[0] = (double)step;
    row[1] = T;
    row[2] = PE / c->n;
    row[3] = KE / c->n;
}

static void thermo_row( gbmd_ctx *c, int64_t step, double *row )
{
    gbmd_thermo_row_from( c, step, c->h_red, row );
}

// Serving-engine halves of one timestep (gbmd_serve.cu).  A rebuild is
// launched for many jobs before one synchronisation, then finished (list
// capacity checked, grown and relaunched where needed).
int gbmd_rebuild_launch( gbmd_ctx *c )
{
    const double cut = c->md.force_cut + c->md.skin;
    int rc;
    if ( ( rc = do_exchange( c ) ) )
        return rc;
    if ( ( rc = do_binning( c, cut ) ) )
        return rc;
    c->half = c->md.half;
    c->neigh_cut = cut;
    if ( c->md.max_neigh_guess > c->max_neigh_guess )
        c->max_neigh_guess = c->md.max_neigh_guess;
    c->nl_attempts = 0;
    return gbmd_build_list_launch( c );
}

int gbmd_rebuild_finish( gbmd_ctx *c, bool *again )
{
    int rc = gbmd_build_list_finish( c, again );
    if ( rc == GBMD_OK && !*again )
        c->rebuilds++;
    return rc;
}

// force + final integrate (+ the next step's initial integrate unless last)
// [+ thermo sums into red_out] for one job: the body of gbmd_md_run's step
// after the rebuild.
int gbmd_job_force_step( gbmd_ctx *c, bool thermo, bool last )
{
    int rc;
    if ( c->force_type == GBMD_FORCE_LJ && !c->md.half )
        return gbmd_lj_step_launch( c, thermo, !last );
    if ( ( rc = force_launch( c, thermo, true ) ) )
        return rc;
    return last ? gbmd_nve_final_launch( c, thermo ) : gbmd_nve_step_tail_launch( c, true, thermo );
}

int gbmd_check_flags( gbmd_ctx *c ) { return check_flags( c ); }

// ---------------------------------------------------------------------------
// C ABI
extern "C" {

int gbmd_version( void ) { return 1; }

static int ctx_init( gbmd_ctx **out, int device, cudaStream_t stream, double *h_red,
                     int *h_flags )
{
    if ( !out )
        return GBMD_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if ( cudaGetDeviceCount( &ndev ) != cudaSuccess || ndev <= 0 )
        return GBMD_ERR_NODEVICE;
    if ( device < 0 || device >= ndev )
        return GBMD_ERR_ARG;
    gbmd_ctx *c = new gbmd_ctx();
    c->device = device;
    int rc;
    if ( cudaSetDevice( device ) != cudaSuccess )
    {
        delete c;
        return GBMD_ERR_CUDA;
    }
    {
        // keep freed stream-ordered allocations in the pool for reuse
        cudaMemPool_t pool;
        if ( cudaDeviceGetDefaultMemPool( &pool, device ) == cudaSuccess )
        {
            uint64_t keep = ~(uint64_t)0;
            cudaMemPoolSetAttribute( pool, cudaMemPoolAttrReleaseThreshold, &keep );
        }
    }
    if ( stream )
    {
        c->stream = stream;
        c->owns_stream = false;
    }
    else if ( cudaStreamCreateWithFlags( &c->stream, cudaStreamNonBlocking ) != cudaSuccess )
    {
        delete c;
        return GBMD_ERR_CUDA;
    }
    if ( h_red && h_flags )
    {
        c->h_red = h_red;
        c->h_flags = h_flags;
        c->owns_host = false;
    }
    else if ( cudaMallocHost( (void **)&c->h_red, 8 * sizeof( double ) ) != cudaSuccess ||
              cudaMallocHost( (void **)&c->h_flags, 8 * sizeof( int ) ) != cudaSuccess )
    {
        gbmd_destroy( c );
        return GBMD_ERR_CUDA;
    }
    // device address of the pinned host flags (batched rebuilds write the
    // list's row maximum there); none if the memory is not mapped
    if ( cudaHostGetDevicePointer( (void **)&c->h_flags_dev, c->h_flags, 0 ) != cudaSuccess )
    {
        c->h_flags_dev = nullptr;
        cudaGetLastError(); // that error is answered here
    }
    if ( ( rc = gbmd_reserve( c, c->flags, 8, "flags" ) ) ||
         ( rc = gbmd_reserve( c, c->red_out, GBMD_RED_WORDS, "red_out" ) ) ||
         ( rc = gbmd_reserve( c, c->mass_d, GBMD_MAXT, "mass" ) ) )
    {
        gbmd_destroy( c );
        return rc;
    }
    for ( int t = 0; t < GBMD_MAXT; t++ )
        c->mass[t] = 1.0;
    if ( cudaMemsetAsync( c->flags.p, 0, 8 * sizeof( int ), c->stream ) != cudaSuccess ||
         cudaMemsetAsync( c->red_out.p, 0, GBMD_RED_WORDS * sizeof( double ), c->stream ) !=
             cudaSuccess ||
         cudaMemcpyAsync( c->mass_d.p, c->mass, sizeof( c->mass ), cudaMemcpyHostToDevice,
                          c->stream ) != cudaSuccess ||
         cudaStreamSynchronize( c->stream ) != cudaSuccess )
    {
        gbmd_destroy( c );
        return GBMD_ERR_CUDA;
    }
    *out = c;
    return GBMD_OK;
}

int gbmd_create( gbmd_ctx **out, int device )
{
    return ctx_init( out, device, nullptr, nullptr, nullptr );
}

void gbmd_destroy( gbmd_ctx *c )
{
    if ( !c )
        return;
    cudaSetDevice( c->device );
    if ( c->stream && c->owns_stream )
        cudaStreamSynchronize( c->stream );
    ktime_resolve( c );
    for ( auto e : c->ev_pool )
        cudaEventDestroy( e );
    graph_cache_clear( c );
    gbmd_nnp_free( c );
    gbmd_release( c, c->x );
    gbmd_release( c, c->x_alt );
    gbmd_release( c, c->xr );
    gbmd_release( c, c->v );
    gbmd_release( c, c->v_alt );
    gbmd_release( c, c->f );
    gbmd_release( c, c->f4 );
    gbmd_release( c, c->type );
    gbmd_release( c, c->type_alt );
    gbmd_release( c, c->id );
    gbmd_release( c, c->id_alt );
    gbmd_release( c, c->home );
    gbmd_release( c, c->gflag );
    gbmd_release( c, c->xr_alt );
    gbmd_release( c, c->mass_d );
    gbmd_release( c, c->cell_key );
    gbmd_release( c, c->cell_count );
    gbmd_release( c, c->cell_start );
    gbmd_release( c, c->cell_fill );
    gbmd_release( c, c->perm );
    gbmd_release( c, c->scan_tmp );
    gbmd_release( c, c->nlist );
    gbmd_release( c, c->nnum );
    gbmd_release( c, c->flags );
    gbmd_release( c, c->partials );
    gbmd_release( c, c->red_out );
    gbmd_release( c, c->stage );
    if ( c->owns_host )
    {
        if ( c->h_red )
            cudaFreeHost( c->h_red );
        if ( c->h_flags )
            cudaFreeHost( c->h_flags );
    }
    if ( c->stream && c->owns_stream )
    {
        cudaStreamSynchronize( c->stream );
        cudaStreamDestroy( c->stream );
    }
    delete c;
}

const char *gbmd_last_error( const gbmd_ctx *c )
{
    return c ? c->err.c_str() : "null context";
}

int gbmd_set_units( gbmd_ctx *c, double boltz, double mvv2e, double dt )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( !( boltz > 0 ) || !( mvv2e > 0 ) || !( dt > 0 ) )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_units: boltz, mvv2e and dt must be > 0" );
    c->boltz = boltz;
    c->mvv2e = mvv2e;
    c->dt = dt;
    return GBMD_OK;
}

int gbmd_set_box( gbmd_ctx *c, const double lo[3], const double hi[3] )
{
    if ( !c || !lo || !hi )
        return GBMD_ERR_ARG;
    for ( int d = 0; d < 3; d++ )
        if ( !( hi[d] > lo[d] ) )
            return gbmd_fail( c, GBMD_ERR_ARG, "set_box: hi must exceed lo" );
    for ( int d = 0; d < 3; d++ )
    {
        c->lo[d] = lo[d];
        c->hi[d] = hi[d];
    }
    c->sorted = false;
    c->have_list = false;
    return GBMD_OK;
}

int gbmd_set_types( gbmd_ctx *c, int ntypes, const double *mass )
{
    if ( !c || !mass )
        return GBMD_ERR_ARG;
    if ( ntypes < 1 || ntypes > GBMD_MAXT )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_types: 1 <= ntypes <= 8" );
    c->ntypes = ntypes;
    for ( int t = 0; t < ntypes; t++ )
    {
        if ( !( mass[t] > 0 ) )
            return gbmd_fail( c, GBMD_ERR_ARG, "set_types: masses must be > 0" );
        c->mass[t] = mass[t];
    }
    GBMD_CUDA( c, cudaMemcpyAsync( c->mass_d.p, c->mass, sizeof( c->mass ),
                                   cudaMemcpyHostToDevice, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_set_precision( gbmd_ctx *c, int precision )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( precision != GBMD_PREC_FP64 && precision != GBMD_PREC_MIXED )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_precision: unknown mode" );
    c->precision = precision;
    return GBMD_OK;
}

__global__ void k_scale( double *__restrict__ a, int n, double s )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i < n )
        a[i] = dmul( a[i], s );
}

// Host arrays (copied into device staging) -> the device layout.  Types
// outside [0, ntypes) are counted in bad_type instead of being stored.
__global__ void k_upload_pack( const double *__restrict__ xh, const int *__restrict__ t,
                               int n, int ntypes, double4 *__restrict__ x,
                               const double *__restrict__ vh, double *__restrict__ v,
                               int *__restrict__ bad_type )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    int ti = t[i];
    if ( ti < 0 || ti >= ntypes )
    {
        atomicAdd( bad_type, 1 );
        ti = 0;
    }
    x[i] = make_double4( xh[3 * i], xh[3 * i + 1], xh[3 * i + 2], (double)ti );
    if ( vh )
    {
        v[i] = vh[3 * i];
        v[n + i] = vh[3 * i + 1];
        v[2 * n + i] = vh[3 * i + 2];
    }
    else
    {
        v[i] = 0.0;
        v[n + i] = 0.0;
        v[2 * n + i] = 0.0;
    }
}

__global__ void k_download_unpack( const double4 *__restrict__ x,
                                   const double *__restrict__ v,
                                   const double *__restrict__ f, int n,
                                   double *__restrict__ xo, double *__restrict__ vo,
                                   double *__restrict__ fo )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    const double4 p = x[i];
    xo[3 * i] = p.x;
    xo[3 * i + 1] = p.y;
    xo[3 * i + 2] = p.z;
    vo[3 * i] = v[i];
    vo[3 * i + 1] = v[n + i];
    vo[3 * i + 2] = v[2 * n + i];
    fo[3 * i] = f[i];
    fo[3 * i + 1] = f[n + i];
    fo[3 * i + 2] = f[2 * n + i];
}

// Host ranges pinned and mapped by gbmd_host_register, with their device
// addresses.  Uploads from, and downloads into, arrays that lie wholly inside
// one of them are done by kernels that read or write the mapped host memory
// directly over the host link (one pass, no staging copy); anything else takes
// the copy path.
namespace
{
struct HostRange
{
    const char *h;
    size_t bytes;
    char *d;
};
std::mutex g_host_mutex;
std::vector<HostRange> g_host_ranges;
} // namespace

// Device address of host array [p, p + bytes), or null unless it lies inside
// one range registered here.
static void *host_mapped( const void *p, size_t bytes )
{
    if ( !p )
        return nullptr;
    const char *q = static_cast<const char *>( p );
    std::lock_guard<std::mutex> lock( g_host_mutex );
    for ( const HostRange &r : g_host_ranges )
        if ( q >= r.h && bytes <= r.bytes && (size_t)( q - r.h ) <= r.bytes - bytes )
            return r.d + ( q - r.h );
    return nullptr;
}

// Direct transfers between the device arrays and mapped host arrays (the
// caller's xyz-per-atom layout), 256 atoms per block: each block moves its
// atoms' 768 coordinates as whole contiguous rows through shared memory, so
// the host link sees full-line reads and writes.
constexpr int XFER_ATOMS = 256;

__global__ void __launch_bounds__( XFER_ATOMS )
    k_upload_direct( const double *__restrict__ xh, const double *__restrict__ vh,
                     const int *__restrict__ th, const int *__restrict__ idh, int n, int ntypes,
                     double4 *__restrict__ x, double *__restrict__ v, int *__restrict__ type,
                     int *__restrict__ id, int *__restrict__ bad_type )
{
    __shared__ double sx[3 * XFER_ATOMS], sv[3 * XFER_ATOMS];
    const int t = threadIdx.x;
    const int base = blockIdx.x * XFER_ATOMS;
    const int na = min( XFER_ATOMS, n - base );
    for ( int k = t; k < 3 * na; k += XFER_ATOMS )
    {
        sx[k] = xh[3 * (size_t)base + k];
        sv[k] = vh ? vh[3 * (size_t)base + k] : 0.0;
    }
    __syncthreads();
    if ( t >= na )
        return;
    const int i = base + t;
    const int traw = th[i];
    int ti = traw;
    if ( ti < 0 || ti >= ntypes )
    {
        atomicAdd( bad_type, 1 );
        ti = 0;
    }
    type[i] = traw;
    id[i] = idh[i];
    x[i] = make_double4( sx[3 * t], sx[3 * t + 1], sx[3 * t + 2], (double)ti );
    v[i] = sv[3 * t];
    v[n + i] = sv[3 * t + 1];
    v[2 * n + i] = sv[3 * t + 2];
}

__global__ void __launch_bounds__( XFER_ATOMS )
    k_download_direct( const double4 *__restrict__ x, const double *__restrict__ v,
                       const double *__restrict__ f, const int *__restrict__ type,
                       const int *__restrict__ id, int n, double *__restrict__ xo,
                       double *__restrict__ vo, double *__restrict__ fo, int *__restrict__ to,
                       int *__restrict__ ido )
{
    __shared__ double s[3 * XFER_ATOMS];
    const int t = threadIdx.x;
    const int base = blockIdx.x * XFER_ATOMS;
    const int na = min( XFER_ATOMS, n - base );
    const int i = base + t;
    const bool live = t < na;
    // one xyz array at a time: gather per atom, write whole rows
    auto put = [&]( double *out, double a, double b, double c ) {
        if ( live )
        {
            s[3 * t] = a;
            s[3 * t + 1] = b;
            s[3 * t + 2] = c;
        }
        __syncthreads();
        for ( int k = t; k < 3 * na; k += XFER_ATOMS )
            out[3 * (size_t)base + k] = s[k];
        __syncthreads();
    };
    if ( xo )
    {
        const double4 p = live ? x[i] : make_double4( 0.0, 0.0, 0.0, 0.0 );
        put( xo, p.x, p.y, p.z );
    }
    if ( vo )
        put( vo, live ? v[i] : 0.0, live ? v[n + i] : 0.0, live ? v[2 * n + i] : 0.0 );
    if ( fo )
        put( fo, live ? f[i] : 0.0, live ? f[n + i] : 0.0, live ? f[2 * n + i] : 0.0 );
    if ( live && to )
        to[i] = type[i];
    if ( live && ido )
        ido[i] = id[i];
}

int gbmd_upload_atoms( gbmd_ctx *c, int64_t n, const double *x,
                       const double *v, const int32_t *type,
                       const int32_t *id )
{
    if ( !c || n < 0 || ( n > 0 && ( !x || !type || !id ) ) )
        return c ? gbmd_fail( c, GBMD_ERR_ARG, "upload_atoms: bad arguments" ) : GBMD_ERR_ARG;
    if ( n > GBMD_MAX_ATOMS )
        return gbmd_fail( c, GBMD_ERR_CAPACITY, "upload_atoms: more than 2^27-2 atoms" );
    int rc;
    if ( ( rc = gbmd_reserve( c, c->x, n, "x" ) ) ||
         ( rc = gbmd_reserve( c, c->v, 3 * n, "v" ) ) ||
         ( rc = gbmd_reserve( c, c->f, 3 * n, "f" ) ) ||
         ( rc = gbmd_reserve( c, c->type, n, "type" ) ) ||
         ( rc = gbmd_reserve( c, c->id, n, "id" ) ) ||
         ( rc = gbmd_reserve( c, c->x_alt, n, "x_alt" ) ) ||
         ( rc = gbmd_reserve( c, c->v_alt, 3 * n, "v_alt" ) ) )
        return rc;
    c->n = n;
    c->sorted = false;
    c->have_list = false;
    c->md_ready = false;
    if ( n == 0 )
        return GBMD_OK;
    GBMD_CUDA( c, cudaMemsetAsync( c->flags.p + 4, 0, sizeof( int ), c->stream ) );
    // Arrays registered with gbmd_host_register are read in place by one
    // kernel over the host link.  Otherwise the host arrays are staged
    // through the alt buffers (x_alt holds 4n doubles >= 3n) by copies, DMA
    // from pinned memory, through the driver's staging from pageable memory.
    // Types are checked on the device either way.
    const double *xd = (const double *)host_mapped( x, sizeof( double ) * 3 * n );
    const double *vd = v ? (const double *)host_mapped( v, sizeof( double ) * 3 * n ) : nullptr;
    const int *td = (const int *)host_mapped( type, sizeof( int ) * n );
    const int *idd = (const int *)host_mapped( id, sizeof( int ) * n );
    if ( xd && td && idd && ( !v || vd ) )
    {
        k_upload_direct<<<blocks_for( n, XFER_ATOMS ), XFER_ATOMS, 0, c->stream>>>(
            xd, vd, td, idd, (int)n, c->ntypes, c->x.p, c->v.p, c->type.p, c->id.p,
            c->flags.p + 4 );
        GBMD_LAUNCH_CHECK( c, "upload_direct" );
    }
    else
    {
        double *xs = (double *)c->x_alt.p;
        GBMD_CUDA( c, cudaMemcpyAsync( xs, x, sizeof( double ) * 3 * n,
                                       cudaMemcpyHostToDevice, c->stream ) );
        if ( v )
            GBMD_CUDA( c, cudaMemcpyAsync( c->v_alt.p, v, sizeof( double ) * 3 * n,
                                           cudaMemcpyHostToDevice, c->stream ) );
        GBMD_CUDA( c, cudaMemcpyAsync( c->type.p, type, sizeof( int ) * n,
                                       cudaMemcpyHostToDevice, c->stream ) );
        GBMD_CUDA( c, cudaMemcpyAsync( c->id.p, id, sizeof( int ) * n,
                                       cudaMemcpyHostToDevice, c->stream ) );
        k_upload_pack<<<blocks_for( n, 256 ), 256, 0, c->stream>>>(
            xs, c->type.p, (int)n, c->ntypes, c->x.p, v ? c->v_alt.p : nullptr, c->v.p,
            c->flags.p + 4 );
        GBMD_LAUNCH_CHECK( c, "upload_pack" );
    }
    GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * n, c->stream ) );
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags + 4, c->flags.p + 4, sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    if ( c->h_flags[4] )
    {
        c->n = 0; // nothing usable was uploaded
        return gbmd_fail( c, GBMD_ERR_ARG, "upload_atoms: type out of range (" +
                                               std::to_string( c->h_flags[4] ) + " atoms)" );
    }
    return GBMD_OK;
}

int gbmd_host_register( const void *p, size_t bytes )
{
    if ( !p || bytes == 0 )
        return GBMD_ERR_ARG;
    const cudaError_t e = cudaHostRegister( const_cast<void *>( p ), bytes,
                                            cudaHostRegisterMapped | cudaHostRegisterPortable );
    if ( e == cudaErrorHostMemoryAlreadyRegistered )
    {
        cudaGetLastError(); // pinned already (not recorded: its extent is not known here)
        return GBMD_OK;
    }
    if ( e != cudaSuccess )
        return GBMD_ERR_CUDA;
    void *d = nullptr;
    if ( cudaHostGetDevicePointer( &d, const_cast<void *>( p ), 0 ) == cudaSuccess && d )
    {
        std::lock_guard<std::mutex> lock( g_host_mutex );
        g_host_ranges.push_back( { static_cast<const char *>( p ), bytes, static_cast<char *>( d ) } );
    }
    else
        cudaGetLastError(); // pinned, not mapped: copies only
    return GBMD_OK;
}

int gbmd_host_unregister( const void *p )
{
    if ( !p )
        return GBMD_ERR_ARG;
    {
        std::lock_guard<std::mutex> lock( g_host_mutex );
        g_host_ranges.erase( std::remove_if( g_host_ranges.begin(), g_host_ranges.end(),
                                             [&]( const HostRange &r ) { return r.h == p; } ),
                             g_host_ranges.end() );
    }
    const cudaError_t e = cudaHostUnregister( const_cast<void *>( p ) );
    if ( e == cudaErrorHostMemoryNotRegistered )
    {
        cudaGetLastError();
        return GBMD_ERR_ARG;
    }
    return e == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

int gbmd_download_atoms( gbmd_ctx *c, double *x, double *v, double *f,
                         int32_t *type, int32_t *id )
{
    if ( !c )
        return GBMD_ERR_ARG;
    const int64_t n = c->n;
    if ( n == 0 )
        return GBMD_OK;
    // Into arrays registered with gbmd_host_register: one kernel writes them
    // in place over the host link.
    {
        double *xd = (double *)host_mapped( x, sizeof( double ) * 3 * n );
        double *vd = (double *)host_mapped( v, sizeof( double ) * 3 * n );
        double *fd = (double *)host_mapped( f, sizeof( double ) * 3 * n );
        int *td = (int *)host_mapped( type, sizeof( int ) * n );
        int *idd = (int *)host_mapped( id, sizeof( int ) * n );
        if ( ( !x || xd ) && ( !v || vd ) && ( !f || fd ) && ( !type || td ) && ( !id || idd ) )
        {
            k_download_direct<<<blocks_for( n, XFER_ATOMS ), XFER_ATOMS, 0, c->stream>>>(
                c->x.p, c->v.p, c->f.p, c->type.p, c->id.p, (int)n, xd, vd, fd, td, idd );
            GBMD_LAUNCH_CHECK( c, "download_direct" );
            GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
            return GBMD_OK;
        }
    }
    // Otherwise unpack into the context's staging buffer (kept for later
    // calls), then one copy per array.
    int rc;
    if ( ( rc = gbmd_reserve( c, c->stage, 9 * (size_t)n, "download stage" ) ) )
        return rc;
    double *stage = c->stage.p;
    k_download_unpack<<<blocks_for( n, 256 ), 256, 0, c->stream>>>(
        c->x.p, c->v.p, c->f.p, (int)n, stage, stage + 3 * n, stage + 6 * n );
    GBMD_LAUNCH_CHECK( c, "download_unpack" );
    if ( x )
        GBMD_CUDA( c, cudaMemcpyAsync( x, stage, sizeof( double ) * 3 * n,
                                       cudaMemcpyDeviceToHost, c->stream ) );
    if ( v )
        GBMD_CUDA( c, cudaMemcpyAsync( v, stage + 3 * n, sizeof( double ) * 3 * n,
                                       cudaMemcpyDeviceToHost, c->stream ) );
    if ( f )
        GBMD_CUDA( c, cudaMemcpyAsync( f, stage + 6 * n, sizeof( double ) * 3 * n,
                                       cudaMemcpyDeviceToHost, c->stream ) );
    if ( type )
        GBMD_CUDA( c, cudaMemcpyAsync( type, c->type.p, sizeof( int ) * n,
                                       cudaMemcpyDeviceToHost, c->stream ) );
    if ( id )
        GBMD_CUDA( c, cudaMemcpyAsync( id, c->id.p, sizeof( int ) * n,
                                       cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_num_atoms( const gbmd_ctx *c, int64_t *n )
{
    if ( !c || !n )
        return GBMD_ERR_ARG;
    *n = c->n;
    return GBMD_OK;
}

int gbmd_exchange( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    int rc = do_exchange( c );
    if ( rc )
        return rc;
    c->sorted = false;
    c->have_list = false;
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, 4 * sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    if ( c->h_flags[1] )
        return gbmd_fail( c, GBMD_ERR_LOST_ATOM,
                          "exchange: atom NaN or more than one box outside" );
    return GBMD_OK;
}

int gbmd_binning( gbmd_ctx *c, double neigh_cut )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( !( neigh_cut > 0 ) )
        return gbmd_fail( c, GBMD_ERR_ARG, "binning: cut must be > 0" );
    if ( !( c->hi[0] > c->lo[0] ) )
        return gbmd_fail( c, GBMD_ERR_ARG, "binning: box not set" );
    int rc = do_binning( c, neigh_cut );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_neigh_build( gbmd_ctx *c, double neigh_cut, int half,
                      int max_neigh_guess )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( !c->sorted || c->grid_cut != neigh_cut )
        return gbmd_fail( c, GBMD_ERR_ARG,
                          "neigh_build: call gbmd_binning with the same cut first" );
    c->half = half ? 1 : 0;
    c->neigh_cut = neigh_cut;
    if ( max_neigh_guess > c->max_neigh_guess )
        c->max_neigh_guess = max_neigh_guess;
    int rc = gbmd_build_list( c );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_lj_coeff( gbmd_ctx *c, int itype, int jtype, double eps, double sigma,
                   double cut )
{
    if ( !c )
        return GBMD_ERR_ARG;
    const int i = itype - 1, j = jtype - 1;
    if ( i < 0 || j < 0 || i >= GBMD_MAXT || j >= GBMD_MAXT )
        return gbmd_fail( c, GBMD_ERR_ARG, "lj_coeff: type out of range" );
    GbmdLJ &p = c->lj;
    const int T = GBMD_MAXT;
    // force_lj_cabana_neigh_impl.h:77-84
    p.lj1[i * T + j] = 48.0 * eps * std::pow( sigma, 12.0 );
    p.lj2[i * T + j] = 24.0 * eps * std::pow( sigma, 6.0 );
    p.cutsq[i * T + j] = cut * cut;
    p.lj1[j * T + i] = p.lj1[i * T + j];
    p.lj2[j * T + i] = p.lj2[i * T + j];
    p.cutsq[j * T + i] = p.cutsq[i * T + j];
    for ( int k = 0; k < T * T; k++ )
    {
        // energy at the cutoff, in the reference's expression order
        // (force_lj_cabana_neigh_impl.h:301-306 without the factor, which is
        // 1/2 or 1 and so scales the rounded value exactly)
        double esh = 0.0;
        if ( p.cutsq[k] > 0.0 )
        {
            const double r2invc = 1.0 / p.cutsq[k];
            const double r6invc = r2invc * r2invc * r2invc;
            esh = r6invc * ( 0.5 * p.lj1[k] * r6invc - p.lj2[k] ) / 6.0;
        }
        p.eshift[k] = esh;
        p.lj1f[k] = (float)p.lj1[k];
        p.lj2f[k] = (float)p.lj2[k];
        p.cutsqf[k] = (float)p.cutsq[k];
        p.eshiftf[k] = (float)esh;
    }
    c->lj_set = true;
    c->lj_dirty = true;
    return GBMD_OK;
}

int gbmd_set_force_type( gbmd_ctx *c, int force_type )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( force_type != GBMD_FORCE_LJ && force_type != GBMD_FORCE_NNP )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_force_type: unknown force" );
    c->force_type = force_type;
    return GBMD_OK;
}

int gbmd_zero_force( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n )
        GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * c->n,
                                       c->stream ) );
    return GBMD_OK;
}

int gbmd_force_compute( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n == 0 )
        return GBMD_OK;
    int rc = force_launch( c, false, false );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, 4 * sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return check_flags( c );
}

int gbmd_force_energy( gbmd_ctx *c, double *pe )
{
    if ( !c || !pe )
        return GBMD_ERR_ARG;
    if ( c->n == 0 )
    {
        *pe = 0.0;
        return GBMD_OK;
    }
    if ( !c->have_list )
        return gbmd_fail( c, GBMD_ERR_ARG, "force_energy: no neighbor list" );
    int rc;
    if ( c->force_type == GBMD_FORCE_LJ )
    {
        if ( !c->lj_set )
            return gbmd_fail( c, GBMD_ERR_ARG, "force_energy: LJ coefficients not set" );
        rc = gbmd_lj_energy_launch( c );
    }
    else
    {
        if ( !c->nnp )
            return gbmd_fail( c, GBMD_ERR_ARG, "force_energy: NNP not loaded" );
        // force_nnp_cabana_neigh_impl.h:101-130 sums the stored E_i; the
        // symmetry functions and the MLP are re-evaluated at the current
        // positions (no force pass).
        rc = gbmd_nnp_launch( c, true, false );
    }
    if ( rc )
        return rc;
    if ( ( rc = read_reductions( c ) ) )
        return rc;
    *pe = potential_energy( c );
    return GBMD_OK;
}

int gbmd_integrate_initial( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n == 0 )
        return GBMD_OK;
    int rc = gbmd_nve_initial_launch( c );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_integrate_final( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n == 0 )
        return GBMD_OK;
    int rc = gbmd_nve_final_launch( c, false );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_scale_velocities( gbmd_ctx *c, double factor )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n == 0 )
        return GBMD_OK;
    const int n3 = (int)( 3 * c->n );
    k_scale<<<blocks_for( n3, 256 ), 256, 0, c->stream>>>( c->v.p, n3, factor );
    GBMD_LAUNCH_CHECK( c, "scale velocities" );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

int gbmd_thermo( gbmd_ctx *c, double *temperature, double *kinetic )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( c->n < 2 )
        return gbmd_fail( c, GBMD_ERR_ARG, "thermo: need at least 2 atoms" );
    int rc = gbmd_mv2_launch( c );
    if ( rc )
        return rc;
    if ( ( rc = read_reductions( c ) ) )
        return rc;
    double row[4];
    thermo_row( c, 0, row );
    if ( temperature )
        *temperature = row[1];
    if ( kinetic )
        *kinetic = row[3] * c->n;
    return GBMD_OK;
}

int gbmd_md_init( gbmd_ctx *c, const gbmd_md_params *p, double *thermo0 )
{
    if ( !c || !p )
        return GBMD_ERR_ARG;
    if ( !( p->force_cut > 0 ) || p->skin < 0 || p->rebuild_every < 1 ||
         p->thermo_every < 0 )
        return gbmd_fail( c, GBMD_ERR_ARG, "md_init: bad parameters" );
    if ( c->n < 2 )
        return gbmd_fail( c, GBMD_ERR_ARG, "md_init: need at least 2 atoms" );
    if ( c->force_type == GBMD_FORCE_NNP && p->half )
        return gbmd_fail( c, GBMD_ERR_ARG,
                          "Half neighbor list not implemented for the neural "
                          "network potential." );
    c->md = *p;
    c->step = 0;
    GBMD_CUDA( c, cudaMemsetAsync( c->flags.p, 0, 8 * sizeof( int ), c->stream ) );
    gbmd_pretune( c );
    int rc;
    if ( ( rc = gbmd_rebuild( c ) ) )
        return rc;
    // tile shapes for this system (timed on it, or from the process cache)
    if ( ( rc = gbmd_autotune( c ) ) )
        return rc;
    const bool thermo = p->thermo_every > 0;
    if ( ( rc = force_launch( c, thermo, true ) ) )
        return rc;
    if ( thermo )
    {
        if ( ( rc = gbmd_mv2_launch( c ) ) )
            return rc;
        if ( ( rc = read_reductions( c ) ) )
            return rc;
        if ( thermo0 )
            thermo_row( c, 0, thermo0 );
    }
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    c->md_ready = true;
    return GBMD_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs of md_run's steps.  Between two host synchronisations (a
// thermo read-back or a list rebuild) md_run issues the same launches step
// after step: the fused LJ step kernel (full lists), or force + the
// integrator's fused final/initial kernel (NNP, half lists).  A run of k of
// them is captured once into a graph and replayed whenever the same k steps
// recur with the same arguments (the fused LJ steps alternate the position
// buffers, so a few graphs cover a whole run).
constexpr int GBMD_GRAPH_MIN_STEPS = 2;
constexpr size_t GBMD_GRAPH_CACHE = 8;

static void graph_cache_clear( gbmd_ctx *c )
{
    for ( auto &e : c->graph_cache )
        cudaGraphExecDestroy( e.second );
    c->graph_cache.clear();
    c->graph_launches.clear();
}

static void key_bytes( std::string &key, const void *p, size_t bytes )
{
    key.append( static_cast<const char *>( p ), bytes );
}
#define key_add( key, v ) key_bytes( ( key ), &( v ), sizeof( v ) )

// The launch arguments of a force + integrator step (NNP, half lists), as
// bytes: every buffer and value the launches read from the context.
static int plain_step_key( gbmd_ctx *c, std::string &key )
{
    key.clear();
    const void *ptrs[] = { c->x.p,    c->xr.p,       c->v.p,    c->f.p,       c->f4.p,
                           c->type.p, c->home.p,     c->nlist.p, c->nnum.p,   c->partials.p,
                           c->flags.p, c->red_out.p, c->mass_d.p };
    key_add( key, ptrs );
    const int64_t ints[] = { c->n,     (int64_t)c->nl_stride, c->nl_cap,   c->nl_maxc,
                             c->precision, c->force_type,    c->half,     c->ntypes,
                             (int64_t)c->part_stride, c->sorted ? 1 : 0, c->no_images };
    key_add( key, ints );
    key_add( key, c->geom );
    key_add( key, c->lj );
    key_add( key, c->tune );
    const StepArgs s = gbmd_step_args( c, true );
    key_add( key, s );
    key_add( key, c->neigh_cut );
    if ( c->nnp )
        gbmd_nnp_key( c, key );
    return GBMD_OK;
}

// One step of the run (not a rebuild, not a thermo step, followed by
// another step), as md_run's direct path launches it.
static int plain_step_launch( gbmd_ctx *c, bool fused )
{
    if ( fused )
        return gbmd_lj_step_launch( c, false, true );
    int rc = force_launch( c, false, true );
    if ( rc )
        return rc;
    return gbmd_nve_step_tail_launch( c, true, false );
}

// k steps as md_run's direct path would launch them.  Capture problems fall
// back to direct launches and switch graphs off for the context.
static int run_step_graph( gbmd_ctx *c, int k, bool fused )
{
    std::string key;
    int rc = fused ? gbmd_lj_step_key( c, key ) : plain_step_key( c, key );
    if ( rc )
        return rc;
    key.append( reinterpret_cast<const char *>( &k ), sizeof k );
    key.push_back( fused ? 'f' : 'p' );
    const bool mixed = c->precision == GBMD_PREC_MIXED;
    // the fused steps alternate the position buffers
    const bool swaps = fused && ( k & 1 );
    for ( auto &e : c->graph_cache )
        if ( e.first == key )
        {
            GBMD_CUDA( c, cudaGraphLaunch( e.second, c->stream ) );
            if ( swaps ) // the buffer swaps of k steps
            {
                std::swap( c->x, c->x_alt );
                if ( mixed )
                    std::swap( c->xr, c->xr_alt );
            }
            c->launches += c->graph_launches[e.first];
            c->graph_replays++;
            return GBMD_OK;
        }
    if ( c->graph_cache.size() >= GBMD_GRAPH_CACHE )
        graph_cache_clear( c );
    // An error already pending in this thread is reported, not swallowed by
    // the capture fallback below (which clears only the capture's own error).
    GBMD_CUDA( c, cudaPeekAtLastError() );
    const DevBuf<double4> x0 = c->x, xa0 = c->x_alt;
    const DevBuf<float4> r0 = c->xr, ra0 = c->xr_alt;
    const int64_t launches0 = c->launches;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaStreamBeginCapture( c->stream, cudaStreamCaptureModeThreadLocal );
    if ( e == cudaSuccess )
    {
        for ( int j = 0; j < k && !rc; j++ )
            rc = plain_step_launch( c, fused );
        e = cudaStreamEndCapture( c->stream, &g );
        if ( !rc && e == cudaSuccess && g )
            e = cudaGraphInstantiate( &ex, g, 0 );
        if ( g )
            cudaGraphDestroy( g );
    }
    if ( rc || e != cudaSuccess || !ex )
    {
        cudaGetLastError(); // the capture's error, not a kernel's
        c->x = x0;
        c->x_alt = xa0;
        c->xr = r0;
        c->xr_alt = ra0;
        c->launches = launches0;
        c->graphs = false;
        for ( int j = 0; j < k; j++ )
            if ( ( rc = plain_step_launch( c, fused ) ) )
                return rc;
        return GBMD_OK;
    }
    c->graph_cache.push_back( { key, ex } );
    c->graph_launches[key] = c->launches - launches0;
    GBMD_CUDA( c, cudaGraphLaunch( ex, c->stream ) );
    c->graph_replays++;
    return GBMD_OK;
}

int gbmd_set_graphs( gbmd_ctx *c, int on )
{
    if ( !c )
        return GBMD_ERR_ARG;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    graph_cache_clear( c );
    c->graphs = on != 0;
    return GBMD_OK;
}

int gbmd_graph_replays( const gbmd_ctx *c, int64_t *replays )
{
    if ( !c || !replays )
        return GBMD_ERR_ARG;
    *replays = c->graph_replays;
    return GBMD_OK;
}

int gbmd_md_run( gbmd_ctx *c, int nsteps, double *thermo, int max_rows,
                 int *nrows )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( nrows )
        *nrows = 0;
    if ( !c->md_ready )
        return gbmd_fail( c, GBMD_ERR_ARG, "md_run: call gbmd_md_init first" );
    int rows = 0, rc;
    cudaEvent_t ev0, ev1;
    GBMD_CUDA( c, cudaEventCreate( &ev0 ) );
    GBMD_CUDA( c, cudaEventCreate( &ev1 ) );
    const int64_t launches0 = c->launches;
    GBMD_CUDA( c, cudaEventRecord( ev0, c->stream ) );
    // The step sequence is the reference's (cabanamd_impl.h:284-399): initial
    // integrate, [rebuild], force, final integrate, [thermo].  Kernels fuse
    // across step boundaries: final(n) and initial(n+1) run in one pass over
    // the atoms (inside the force kernel for a full LJ list), so only the
    // first step of each call launches initial_integrate on its own.
    const bool fused_force = c->force_type == GBMD_FORCE_LJ && !c->md.half;
    NvtxRange run_range( "gbmd.md_run" );
    if ( nsteps > 0 && ( rc = gbmd_nve_initial_launch( c ) ) )
        return rc;
    const bool use_graphs = c->graphs && !c->profiling;
    for ( int s = 0; s < nsteps; s++ )
    {
        if ( use_graphs && c->graphs )
        {
            // the steps from here that are neither a rebuild, a thermo step
            // nor the call's last one
            int k = 0;
            while ( s + k < nsteps - 1 )
            {
                const int64_t st = c->step + 1 + k;
                if ( st % c->md.rebuild_every == 0 ||
                     ( c->md.thermo_every > 0 && st % c->md.thermo_every == 0 ) )
                    break;
                k++;
            }
            if ( k >= GBMD_GRAPH_MIN_STEPS )
            {
                if ( fused_force && ( !c->have_list || !c->lj_set ) )
                    return gbmd_fail( c, GBMD_ERR_ARG, "md_run: no list or LJ coefficients" );
                NvtxRange graph_range( "gbmd.step_graph" );
                if ( ( rc = run_step_graph( c, k, fused_force ) ) )
                    return rc;
                c->step += k;
                s += k - 1;
                continue;
            }
        }
        const int64_t step = ++c->step;
        const bool last = s == nsteps - 1;
        if ( step % c->md.rebuild_every == 0 )
        {
            NvtxRange r( "gbmd.rebuild" );
            if ( ( rc = gbmd_rebuild( c ) ) )
                return rc;
        }
        NvtxRange step_range( "gbmd.step" );
        const bool th = c->md.thermo_every > 0 && step % c->md.thermo_every == 0;
        if ( fused_force )
        {
            if ( !c->have_list || !c->lj_set )
                return gbmd_fail( c, GBMD_ERR_ARG, "md_run: no list or LJ coefficients" );
            if ( ( rc = gbmd_lj_step_launch( c, th, !last ) ) )
                return rc;
        }
        else
        {
            if ( ( rc = force_launch( c, th, true ) ) )
                return rc;
            if ( last )
                rc = gbmd_nve_final_launch( c, th );
            else
                rc = gbmd_nve_step_tail_launch( c, true, th );
            if ( rc )
                return rc;
        }
        if ( th )
        {
            if ( ( rc = read_reductions( c ) ) )
                return rc;
            if ( thermo && rows < max_rows )
                thermo_row( c, step, thermo + 4 * rows++ );
        }
    }
    GBMD_CUDA( c, cudaEventRecord( ev1, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    float ms = 0.f;
    cudaEventElapsedTime( &ms, ev0, ev1 );
    cudaEventDestroy( ev0 );
    cudaEventDestroy( ev1 );
    c->last_run_ms = ms;
    c->last_run_launches = c->launches - launches0;
    GBMD_CUDA( c, cudaMemcpy( c->h_flags, c->flags.p, 4 * sizeof( int ),
                              cudaMemcpyDeviceToHost ) );
    if ( ( rc = check_flags( c ) ) )
        return rc;
    if ( nrows )
        *nrows = rows;
    return GBMD_OK;
}

int gbmd_md_last_run( const gbmd_ctx *c, double *device_ms, int64_t *launches )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( device_ms )
        *device_ms = c->last_run_ms;
    if ( launches )
        *launches = c->last_run_launches;
    return GBMD_OK;
}

int gbmd_md_step_count( const gbmd_ctx *c, int64_t *step )
{
    if ( !c || !step )
        return GBMD_ERR_ARG;
    *step = c->step;
    return GBMD_OK;
}

int gbmd_set_profiling( gbmd_ctx *c, int on )
{
    if ( !c )
        return GBMD_ERR_ARG;
    cudaStreamSynchronize( c->stream );
    ktime_resolve( c );
    c->profiling = on != 0;
    for ( int k = 0; k < GBMD_KT_COUNT; k++ )
    {
        c->ktime_ms[k] = 0;
        c->kcount[k] = 0;
    }
    return GBMD_OK;
}

int gbmd_kernel_time( gbmd_ctx *c, int which, double *ms_total, int64_t *launches )
{
    if ( !c || which < 0 || which >= GBMD_KT_COUNT )
        return GBMD_ERR_ARG;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    ktime_resolve( c );
    if ( ms_total )
        *ms_total = c->ktime_ms[which];
    if ( launches )
        *launches = c->kcount[which];
    return GBMD_OK;
}

int gbmd_synchronize( gbmd_ctx *c )
{
    if ( !c )
        return GBMD_ERR_ARG;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return GBMD_OK;
}

} // extern "C"

int gbmd_create_on_stream( gbmd_ctx **out, int device, cudaStream_t stream, double *h_red,
                           int *h_flags )
{
    if ( !stream || !h_red || !h_flags )
        return GBMD_ERR_ARG;
    return ctx_init( out, device, stream, h_red, h_flags );
}

size_t gbmd_ctx_device_bytes( const gbmd_ctx *c )
{
    size_t b = gbmd_bytes( c->x ) + gbmd_bytes( c->x_alt ) + gbmd_bytes( c->xr ) +
               gbmd_bytes( c->xr_alt ) + gbmd_bytes( c->v ) + gbmd_bytes( c->v_alt ) +
               gbmd_bytes( c->f ) + gbmd_bytes( c->f4 ) + gbmd_bytes( c->type ) + gbmd_bytes( c->type_alt ) +
               gbmd_bytes( c->id ) + gbmd_bytes( c->id_alt ) + gbmd_bytes( c->home ) +
               gbmd_bytes( c->gflag ) + gbmd_bytes( c->mass_d ) + gbmd_bytes( c->cell_key ) +
               gbmd_bytes( c->cell_count ) + gbmd_bytes( c->cell_start ) +
               gbmd_bytes( c->cell_fill ) + gbmd_bytes( c->perm ) + gbmd_bytes( c->scan_tmp ) +
               gbmd_bytes( c->nlist ) + gbmd_bytes( c->nnum ) + gbmd_bytes( c->flags ) +
               gbmd_bytes( c->partials ) + gbmd_bytes( c->red_out );
    return b + gbmd_nnp_device_bytes( c );
}

// ---------------------------------------------------------------------------
// Failure-detection check: a bounded wait that nothing completes.
__global__ void k_wait_expires( long long limit, int *__restrict__ flags )
{
    __shared__ __align__( 8 ) uint64_t bar;
    if ( threadIdx.x == 0 )
    {
        mbar_init( &bar, 1 ); // one arrival expected, none made
        mbar_fence_init();
    }
    __syncthreads();
    const bool done = mbar_wait_bounded( &bar, 0, limit );
    if ( !__syncthreads_or( !done ) )
        return;
    if ( threadIdx.x == 0 )
        atomicExch( &flags[3], 1 );
}

extern "C" int gbmd_check_bounded_wait( gbmd_ctx *c, double seconds )
{
    if ( !c )
        return GBMD_ERR_ARG;
    int khz = 0;
    GBMD_CUDA( c, cudaDeviceGetAttribute( &khz, cudaDevAttrClockRate, c->device ) );
    const double s = std::min( 2.0, std::max( 0.001, seconds ) );
    const long long limit = (long long)( s * 1e3 * ( khz > 0 ? khz : 2000000 ) );
    k_wait_expires<<<1, 32, 0, c->stream>>>( limit, c->flags.p );
    GBMD_LAUNCH_CHECK( c, "bounded wait check" );
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, 4 * sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    return check_flags( c );
}

