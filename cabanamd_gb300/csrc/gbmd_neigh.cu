// gbmd_neigh.cu -- Verlet list build: one warp per home cell, the 27
// (cell, periodic shift) stencil neighbours staged in shared memory.
//
// Semantics (paths inside the CabanaMD project):
//   src/neighbor_types/neighbor_verlet.h:43-62 builds a Cabana::VerletList of
//   local atoms over locals + ghosts with d^2 <= neigh_cut^2 (the same test
//   as unit_test/tstNeighbor.hpp:87-139).  The ghosts are the single-rank
//   halo of src/comm_mpi.h:241-353: an image shifted by -L in dimension d
//   exists when the source has x_d >= hi_d - neigh_cut, by +L when
//   x_d <= lo_d + neigh_cut.  Half lists (Cabana 0.6.1 VerletList,
//   HalfNeighborTag) keep the pair at the atom whose partner image is
//   lexicographically greater in (x, y, z).
//
// GB300 design: GB300 issues FP64 at ~1/64 of its FP32 rate, so the build
// runs on FP32 home-cell-relative coordinates (the 16-byte shadow written
// by the sort) and touches FP64 only to settle the rare pairs whose FP32
// squared distance, or whose FP32 coordinate comparison for the half-list
// rule, lies within the FP32 rounding bound of the decision.  The resulting
// sets equal those of an all-FP64 build.  Ghost existence comes from
// per-atom bits computed once per sort.  Each warp appends its lanes'
// entries to per-lane windows of rows in shared memory and writes the
// windows out row by row, so every row of the transposed list
// (nlist[slot * n + atom]) is written coalesced.
#include "gbmd_internal.cuh"

#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

// A warp stages each lane's entries in a window of NOUT rows in shared
// memory and writes the windows out, row by row, whenever one of them could
// overflow, and at the end of its home atoms.  Fewer rows per window buy
// occupancy, more rows fewer write-outs.  The shape (warps NW per block,
// rows NOUT) is the context's tile shape: one of GBMD_NB_SHAPES, fixed or
// picked by the autotuner (gbmd_tune.cu); the list it builds is the same for
// every shape.  Per rebuild of the 4,000,000-atom LJ melt the tuner picks
// (8, 48): 2.44 ms (2.84 ms when only the first NOUT entries were staged and
// later ones went to the list as scattered 4-byte stores).
constexpr int NB_CHUNK = 128; // staged candidates per warp

struct NbParams
{
    GbmdGeom g;
    double rsq;
    float rsq_lo, rsq_hi;
    float eps_half; // FP32 coordinate-comparison margin for the half rule
    int stride;     // row stride of the transposed list (atoms, padded)
    int cap;
    int half;
    int no_images;  // skip stencil cells reached through a periodic image
};

template <int NOUT> struct NbWarpSmem
{
    // staged candidates relative to the home cell centre, as separate x, y, z
    // arrays (four consecutive candidates are one 16-byte load per
    // coordinate); +4: far padding to a multiple of 4
    float rx[NB_CHUNK + 4], ry[NB_CHUNK + 4], rz[NB_CHUNK + 4];
    uint32_t ent[NB_CHUNK + 4]; // their list entries (j | stencil code << 27)
    uint32_t out[NOUT][32];     // the lanes' first NOUT entries
    // the home cell's 27 stencil cells: first and end atom, ghost-existence
    // bits a partner must carry, FP32 shift of the cell centre
    int2 span[27];
    uint32_t need[27];
    float4 shift[27];
};

// Exact FP64 image of partner j (stencil code sc) seen from home cell hc.
__device__ __forceinline__ double3 exact_image( const double4 *__restrict__ x, int j, int sc,
                                                const int *hc, const GbmdGeom &g )
{
    const double4 q = x[j];
    const int s0 = image_shift( hc[0], sc % 3 - 1, g.nc[0] );
    const int s1 = image_shift( hc[1], ( sc / 3 ) % 3 - 1, g.nc[1] );
    const int s2 = image_shift( hc[2], sc / 9 - 1, g.nc[2] );
    return make_double3( img_coord( q.x, s0, g.L[0] ), img_coord( q.y, s1, g.L[1] ),
                         img_coord( q.z, s2, g.L[2] ) );
}

// The exact decision for a pair the FP32 test left open: the FP64 squared
// distance when the FP32 one lies in the rounding band of the cutoff
// (near_cut), the FP64 lexicographic half rule when the two x coordinates
// lie within the FP32 bound of each other (undecided).
__device__ __noinline__ bool nb_exact_keep( const double4 *__restrict__ x, int i, uint32_t e,
                                            const int *hc, const GbmdGeom &g, double rsq,
                                            bool near_cut, bool undecided )
{
    const double4 pi = x[i];
    const double3 q = exact_image( x, (int)( e & GBMD_JMASK ), (int)( e >> 27 ), hc, g );
    if ( near_cut )
    {
        const double ex = dsub( pi.x, q.x );
        const double ey = dsub( pi.y, q.y );
        const double ez = dsub( pi.z, q.z );
        const double dd = dadd( dadd( dmul( ex, ex ), dmul( ey, ey ) ), dmul( ez, ez ) );
        if ( !( dd <= rsq ) )
            return false;
    }
    if ( undecided )
        return ( q.x > pi.x ) ||
               ( ( q.x == pi.x ) && ( ( q.y > pi.y ) || ( ( q.y == pi.y ) && ( q.z > pi.z ) ) ) );
    return true;
}

// One warp per home cell, in chunks of up to 32 home atoms (one per lane).
// The stencil's candidates are staged in shared memory in list order
// (stencil code, then atom index), up to NB_CHUNK at a time, skipping those
// beyond the cutoff from the chunk's bounding box; every lane then walks the
// staged candidates in that order and appends its neighbours.
// The body takes its block index explicitly: k_neigh_build runs it for one
// system (bid = blockIdx.x), k_neigh_build_jobs for the block's job in a
// batch of serving jobs.
template <int NW, int NOUT, bool HALF>
__device__ __forceinline__ void
    neigh_build_block( const double4 *__restrict__ x, const float4 *__restrict__ xr,
                       const uint8_t *__restrict__ gflag, const int *__restrict__ cstart,
                       const NbParams &p, uint32_t *__restrict__ nlist, int *__restrict__ nnum,
                       int *__restrict__ flags, const int bid )
{
    extern __shared__ __align__( 16 ) unsigned char nb_smem_raw[];
    NbWarpSmem<NOUT> &W = reinterpret_cast<NbWarpSmem<NOUT> *>( nb_smem_raw )[threadIdx.x >> 5];
    const int wib = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int cell = bid * NW + wib;
    if ( cell >= p.g.ncell )
        return;
    const GbmdGeom &g = p.g;
    const int hc[3] = { cell % g.nc[0], ( cell / g.nc[0] ) % g.nc[1],
                        cell / ( g.nc[0] * g.nc[1] ) };
    const int hb = cstart[cell], he = cstart[cell + 1];
    const float rsq_lo = p.rsq_lo, rsq_hi = p.rsq_hi;
    int warp_max = 0;

    // The 27 stencil cells of the home cell, one per lane (lanes 0..26); a
    // cell reached through a periodic image is empty when images are off.
    if ( lane < 27 )
    {
        const int o[3] = { lane % 3 - 1, ( lane / 3 ) % 3 - 1, lane / 9 - 1 };
        int cc[3], sf[3];
        uint32_t need = 0;
#pragma unroll
        for ( int d = 0; d < 3; d++ )
        {
            sf[d] = image_shift( hc[d], o[d], g.nc[d] );
            cc[d] = hc[d] + o[d] - sf[d] * g.nc[d];
            if ( sf[d] < 0 )
                need |= 1u << ( 2 * d );
            if ( sf[d] > 0 )
                need |= 1u << ( 2 * d + 1 );
        }
        const int ncellid = cc[0] + g.nc[0] * ( cc[1] + g.nc[1] * cc[2] );
        int cb = cstart[ncellid], ce = cstart[ncellid + 1];
        if ( p.no_images && ( sf[0] | sf[1] | sf[2] ) )
            ce = cb; // nothing to stage
        W.span[lane] = make_int2( cb, ce );
        W.need[lane] = need;
        W.shift[lane] = make_float4( (float)o[0] * g.hf[0], (float)o[1] * g.hf[1],
                                     (float)o[2] * g.hf[2], 0.f );
    }
    __syncwarp();

    for ( int base = hb; base < he; base += 32 )
    {
        const int i = base + lane;
        const bool active = i < he;
        float4 xi = make_float4( 0.f, 0.f, 0.f, 0.f );
        if ( active )
            xi = xr[i];
        int cnt = 0;
        int flushed = 0; // this lane's entries already written to the list
        int nst = 0;
        const unsigned amask = __ballot_sync( 0xffffffffu, active );
        // Bounding box of this chunk's home atoms: a candidate farther than
        // the cutoff from the box is no lane's neighbour and is not staged.
        // About a quarter of the 27-cell stencil volume lies beyond the
        // cutoff from a cell-sized box.  The 1e-3 relative margin on r^2
        // (on top of the FP32 band) dwarfs the FP32 rounding of the test,
        // so no pair that the exact test would keep is dropped.
        float blo[3] = { active ? xi.x : 3.0e38f, active ? xi.y : 3.0e38f,
                         active ? xi.z : 3.0e38f };
        float bhi[3] = { active ? xi.x : -3.0e38f, active ? xi.y : -3.0e38f,
                         active ? xi.z : -3.0e38f };
#pragma unroll
        for ( int d = 0; d < 3; d++ )
#pragma unroll
            for ( int o = 16; o; o >>= 1 )
            {
                blo[d] = fminf( blo[d], __shfl_xor_sync( 0xffffffffu, blo[d], o ) );
                bhi[d] = fmaxf( bhi[d], __shfl_xor_sync( 0xffffffffu, bhi[d], o ) );
            }
        const float prune2 = rsq_hi * 1.001f;
        const uint32_t self = (uint32_t)i | ( 13u << 27 );
        // Each lane (home atom) walks the staged candidates in staging order,
        // four at a time: packed FP32 distances of two candidates per
        // instruction, the tests on the squared distance's bits (for d2 >= 0
        // the unsigned order of the bits is the float order), the exact FP64
        // test only when a lane's pair sits in the rounding band of the cutoff
        // (or, for half lists, its two x coordinates are too close for FP32 to
        // order them; or d2 == 0, where the atom itself is told from a partner
        // on top of it), then predicated appends -- no branch per candidate.
        const float2 nxi = make_float2( -xi.x, -xi.x ), nyi = make_float2( -xi.y, -xi.y ),
                     nzi = make_float2( -xi.z, -xi.z );
        const uint32_t b_hi = __float_as_uint( rsq_hi );
        const uint32_t b_lo1 = __float_as_uint( rsq_lo ) - 1u;
        // Entries are appended to the lane's window of NOUT rows in shared
        // memory; when a lane's window could overflow within the next four
        // candidates, every active lane writes its window out.  The write-out
        // walks list rows, so the lanes holding row r store it together (one
        // coalesced segment per row), and entries past the capacity are
        // counted but not stored.
        auto flush_rows = [&]() {
            const int r0 = __reduce_min_sync( amask, flushed );
            const int r1 = __reduce_max_sync( amask, cnt );
            for ( int r = r0; r < r1; r++ )
                if ( r >= flushed && r < cnt && r < p.cap )
                    nlist[(size_t)r * p.stride + i] = W.out[r - flushed][lane];
            flushed = cnt;
        };
        auto process = [&]( int count ) {
            if ( lane < 4 ) // pad to a multiple of 4 with points outside every cutoff
            {
                W.rx[count + lane] = W.ry[count + lane] = W.rz[count + lane] = 3.0e18f;
                W.ent[count + lane] = 0xffffffffu;
            }
            __syncwarp();
            if ( active )
            {
                for ( int k = 0; k < count; k += 4 )
                {
                    if ( __any_sync( amask, cnt - flushed > NOUT - 4 ) )
                        flush_rows();
                    const float4 X = *reinterpret_cast<const float4 *>( &W.rx[k] );
                    const float4 Y = *reinterpret_cast<const float4 *>( &W.ry[k] );
                    const float4 Z = *reinterpret_cast<const float4 *>( &W.rz[k] );
                    const uint4 e4 = *reinterpret_cast<const uint4 *>( &W.ent[k] );
                    const uint32_t ev[4] = { e4.x, e4.y, e4.z, e4.w };
                    // candidate minus home atom (the sign does not enter d2)
                    const float2 dx01 = __fadd2_rn( make_float2( X.x, X.y ), nxi );
                    const float2 dx23 = __fadd2_rn( make_float2( X.z, X.w ), nxi );
                    const float2 dy01 = __fadd2_rn( make_float2( Y.x, Y.y ), nyi );
                    const float2 dy23 = __fadd2_rn( make_float2( Y.z, Y.w ), nyi );
                    const float2 dz01 = __fadd2_rn( make_float2( Z.x, Z.y ), nzi );
                    const float2 dz23 = __fadd2_rn( make_float2( Z.z, Z.w ), nzi );
                    const float2 s01 = __ffma2_rn(
                        dz01, dz01, __ffma2_rn( dy01, dy01, __fmul2_rn( dx01, dx01 ) ) );
                    const float2 s23 = __ffma2_rn(
                        dz23, dz23, __ffma2_rn( dy23, dy23, __fmul2_rn( dx23, dx23 ) ) );
                    const float d2[4] = { s01.x, s01.y, s23.x, s23.y };
                    const float ax[4] = { dx01.x, dx01.y, dx23.x, dx23.y };
                    bool acc[4];
                    unsigned open = 0; // candidates the FP32 test leaves to FP64
#pragma unroll
                    for ( int u = 0; u < 4; u++ )
                    {
                        const uint32_t ub = __float_as_uint( d2[u] );
                        const bool cand = ub <= b_hi;
                        // d2 == 0 or d2 >= rsq_lo
                        bool rare = cand && ub - 1u >= b_lo1;
                        acc[u] = cand && !rare;
                        if ( HALF )
                        {
                            rare = rare || ( cand && !( ax[u] > p.eps_half ) );
                            acc[u] = acc[u] && ax[u] > p.eps_half;
                        }
                        if ( rare )
                            open |= 1u << u;
                    }
                    if ( open ) // rare
                    {
#pragma unroll
                        for ( int u = 0; u < 4; u++ )
                            if ( ( open >> u ) & 1u )
                            {
                                bool keep = ev[u] != self;
                                if ( keep && HALF && ax[u] < -p.eps_half )
                                    keep = false; // the half rule decides: not this atom's pair
                                if ( keep )
                                {
                                    const bool near_cut = d2[u] >= rsq_lo;
                                    const bool und = HALF && !( ax[u] > p.eps_half );
                                    if ( near_cut || und )
                                        keep = nb_exact_keep( x, i, ev[u], hc, g, p.rsq, near_cut,
                                                              und );
                                }
                                acc[u] = keep;
                            }
                    }
#pragma unroll
                    for ( int u = 0; u < 4; u++ )
                    {
                        if ( acc[u] )
                            W.out[cnt - flushed][lane] = ev[u];
                        cnt += acc[u] ? 1 : 0;
                    }
                }
            }
            __syncwarp();
        };

        for ( int sc = 0; sc < 27; sc++ )
        {
            const int2 span = W.span[sc];
            const int cb = span.x, ce = span.y;
            const uint32_t need = W.need[sc];
            for ( int a = cb; a < ce; a += 32 )
            {
                const int j = a + lane;
                bool valid = j < ce;
                float px = 0.f, py = 0.f, pz = 0.f;
                if ( valid )
                {
                    const float4 xj = xr[j];
                    if ( need && ( gflag[j] & need ) != need )
                        valid = false;
                    const float4 sh = W.shift[sc];
                    px = xj.x + sh.x;
                    py = xj.y + sh.y;
                    pz = xj.z + sh.z;
                    const float ex = fmaxf( fmaxf( blo[0] - px, px - bhi[0] ), 0.f );
                    const float ey = fmaxf( fmaxf( blo[1] - py, py - bhi[1] ), 0.f );
                    const float ez = fmaxf( fmaxf( blo[2] - pz, pz - bhi[2] ), 0.f );
                    if ( ex * ex + ey * ey + ez * ez > prune2 )
                        valid = false;
                }
                const unsigned m = __ballot_sync( 0xffffffffu, valid );
                const int add = __popc( m );
                if ( nst + add > NB_CHUNK )
                {
                    process( nst );
                    nst = 0;
                }
                if ( valid )
                {
                    const int slot = nst + __popc( m & ( ( 1u << lane ) - 1u ) );
                    W.rx[slot] = px;
                    W.ry[slot] = py;
                    W.rz[slot] = pz;
                    W.ent[slot] = (uint32_t)j | ( (uint32_t)sc << 27 );
                }
                nst += add;
            }
        }
        if ( nst )
            process( nst );
        if ( active )
        {
            nnum[i] = cnt;
            flush_rows(); // the rest of the windows
        }
        __syncwarp();
        warp_max = max( warp_max, active ? cnt : 0 );
    }
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        warp_max = max( warp_max, __shfl_xor_sync( 0xffffffffu, warp_max, o ) );
    if ( lane == 0 && warp_max > 0 )
        atomicMax( &flags[0], warp_max );
}

template <int NW, int NOUT, bool HALF>
__global__ void __launch_bounds__( NW * 32 )
    k_neigh_build( const double4 *__restrict__ x, const float4 *__restrict__ xr,
                   const uint8_t *__restrict__ gflag, const int *__restrict__ cstart,
                   const __grid_constant__ NbParams p, uint32_t *__restrict__ nlist,
                   int *__restrict__ nnum, int *__restrict__ flags )
{
    neigh_build_block<NW, NOUT, HALF>( x, xr, gflag, cstart, p, nlist, nnum, flags,
                                       (int)blockIdx.x );
}

// List builds of several systems sharing a stream in one launch per shape:
// the table (up to NB_JOBS jobs of pointers and parameters) travels in the
// launch parameters and each block finds its job by binary search over the
// per-job block offsets.
constexpr int NB_JOBS = 32;

struct NbJob
{
    const double4 *x;
    const float4 *xr;
    const uint8_t *gflag;
    const int *cstart;
    uint32_t *nlist;
    int *nnum;
    int *flags;
    int *h_max; // the job's pinned host flags, device-mapped (row maximum -> [0])
    NbParams p;
};

struct NbJobTable
{
    int njobs;
    int block0[NB_JOBS + 1];
    NbJob job[NB_JOBS];
};
static_assert( sizeof( NbJobTable ) <= 32764, "job table exceeds the kernel parameter space" );

template <int NW, int NOUT, bool HALF>
__global__ void __launch_bounds__( NW * 32 ) k_neigh_build_jobs( const __grid_constant__ NbJobTable t )
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
    const NbJob &J = t.job[lo];
    neigh_build_block<NW, NOUT, HALF>( J.x, J.xr, J.gflag, J.cstart, J.p, J.nlist, J.nnum,
                                       J.flags, (int)blockIdx.x - t.block0[lo] );
}

// Each job's largest row count to its pinned host flags (one thread per job).
__global__ void k_nb_publish_jobs( const __grid_constant__ NbJobTable t )
{
    const int q = (int)threadIdx.x;
    if ( q < t.njobs )
        t.job[q].h_max[0] = t.job[q].flags[0];
}

// Pad every atom's list rows up to its warp's largest count, rounded up to
// GBMD_ROW_PAD, with the sentinel entry (atom n, stencil code 0,0,0), so the
// mixed force kernel walks a warp's rows with no per-lane bound.  Threads
// cover whole warps up to roundup(n, 32) <= the row stride.
__device__ __forceinline__ void pad_list_rows( const int *__restrict__ nnum, int n, int stride,
                                               uint32_t *__restrict__ nlist, int i )
{
    const int cnt = i < n ? nnum[i] : 0;
    int wmax = __reduce_max_sync( 0xffffffffu, cnt );
    wmax = ( wmax + GBMD_ROW_PAD - 1 ) / GBMD_ROW_PAD * GBMD_ROW_PAD;
    const uint32_t sentinel = (uint32_t)n | ( 13u << 27 );
    for ( int sl = cnt; sl < wmax; sl++ )
        nlist[(size_t)sl * stride + i] = sentinel;
}

__global__ void k_pad_lists( const int *__restrict__ nnum, int n, int stride,
                             uint32_t *__restrict__ nlist )
{
    pad_list_rows( nnum, n, stride, nlist, blockIdx.x * blockDim.x + threadIdx.x );
}

struct PadJob
{
    const int *nnum;
    uint32_t *nlist;
    int n, stride;
};

struct PadTable
{
    int njobs;
    int block0[NB_JOBS + 1];
    PadJob job[NB_JOBS];
};

__global__ void __launch_bounds__( 128 ) k_pad_lists_jobs( const __grid_constant__ PadTable t )
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
    const PadJob &J = t.job[lo];
    pad_list_rows( J.nnum, J.n, J.stride, J.nlist,
                   ( (int)blockIdx.x - t.block0[lo] ) * 128 + (int)threadIdx.x );
}

// Half-width of the FP32 decision band, relative to rc^2 (see header).
double gbmd_fp32_band( const GbmdGeom &g, double rc )
{
    double hmax = fmax( g.h[0], fmax( g.h[1], g.h[2] ) );
    const double R = 2.0 * hmax + rc;
    const double u = std::ldexp( 1.0, -24 );
    const double bound = u * ( 3.5 * ( 2.0 * R + rc ) / rc + 3.0 );
    return fmax( 1e-5, 8.0 * bound );
}

// The build kernel in shape (NW warps per block, NOUT staged slots).
template <int NW, int NOUT, bool HALF> static int nb_launch_kind( gbmd_ctx *c, const NbParams &p )
{
    constexpr size_t smem = sizeof( NbWarpSmem<NOUT> ) * NW;
    // attribute set, one bit per device (atomic: contexts may build lists
    // from several host threads)
    static std::atomic<unsigned> ready{ 0 };
    const unsigned bit = c->device < 32 ? 1u << c->device : 0u;
    if ( !( ready.load( std::memory_order_acquire ) & bit ) )
    {
        GBMD_CUDA( c, cudaFuncSetAttribute( k_neigh_build<NW, NOUT, HALF>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem ) );
        ready.fetch_or( bit, std::memory_order_release );
    }
    const int blocks = ( c->geom.ncell + NW - 1 ) / NW;
    k_neigh_build<NW, NOUT, HALF><<<blocks, NW * 32, smem, c->stream>>>(
        c->x.p, c->xr.p, c->gflag.p, c->cell_start.p, p, c->nlist.p, c->nnum.p, c->flags.p );
    GBMD_LAUNCH_CHECK( c, "neigh_build" );
    return GBMD_OK;
}

template <int NW, int NOUT> static int nb_launch_shape( gbmd_ctx *c, const NbParams &p )
{
    return p.half ? nb_launch_kind<NW, NOUT, true>( c, p ) : nb_launch_kind<NW, NOUT, false>( c, p );
}

// The compiled list-build shapes (warps per block, staged slots per lane);
// the first is the default.
static const int nb_shapes[GBMD_NB_NSHAPES][2] = { { 12, 32 }, { 8, 32 }, { 16, 24 }, { 8, 48 } };

bool gbmd_nb_shape_ok( int nw, int nout )
{
    for ( const auto &sh : nb_shapes )
        if ( sh[0] == nw && sh[1] == nout )
            return true;
    return false;
}

void gbmd_nb_shape( int k, int *nw, int *nout )
{
    *nw = nb_shapes[k][0];
    *nout = nb_shapes[k][1];
}

static int nb_launch( gbmd_ctx *c, const NbParams &p )
{
    const int nw = c->tune.nb_warps, no = c->tune.nb_out;
    if ( nw == 8 && no == 32 )
        return nb_launch_shape<8, 32>( c, p );
    if ( nw == 16 && no == 24 )
        return nb_launch_shape<16, 24>( c, p );
    if ( nw == 8 && no == 48 )
        return nb_launch_shape<8, 48>( c, p );
    return nb_launch_shape<12, 32>( c, p );
}

// List build in two halves so that a caller with many systems can launch
// all their builds and check all capacities after one synchronisation:
// _launch sizes the list and launches the build (the maximum row count goes
// to h_flags[0] asynchronously); _finish, after the stream has drained,
// pads the rows or grows the capacity and asks for another launch.
// _prepare is the sizing alone (host side: list capacity, row stride and
// buffers, allocations ordered on the context's stream).
int gbmd_build_list_prepare( gbmd_ctx *c )
{
    const int n = (int)c->n;
    int rc;
    if ( ( rc = gbmd_reserve( c, c->nnum, n, "nnum" ) ) )
        return rc;
    if ( c->nl_cap == 0 && n > 0 )
    {
        // First build: size from the mean density so the list rarely needs
        // a second pass (the guess still grows like neighbor_verlet.h:58-61).
        const double vol = c->geom.L[0] * c->geom.L[1] * c->geom.L[2];
        const double rc = c->neigh_cut;
        double expect = n / vol * 4.18879020478639 * rc * rc * rc;
        if ( c->half )
            expect *= 0.5;
        const int est = (int)( expect * 1.4 ) + 16;
        if ( est > c->max_neigh_guess )
            c->max_neigh_guess = est;
    }
    if ( c->nl_cap < c->max_neigh_guess )
        c->nl_cap = ( c->max_neigh_guess + 3 ) & ~3;
    // Rows padded to whole 128-atom blocks: a block's slice of a row is one
    // 512-byte, 16-byte-aligned bulk copy for the force kernels.
    c->nl_stride = ( (size_t)n + 127 ) / 128 * 128;
    if ( c->nl_stride == 0 )
        c->nl_stride = 128;
    return gbmd_reserve( c, c->nlist, (size_t)c->nl_cap * c->nl_stride, "nlist" );
}

// The build's parameters for the context's grid, cutoff and list sizing.
static NbParams nb_params( const gbmd_ctx *c )
{
    NbParams p;
    std::memset( &p, 0, sizeof p );
    p.g = c->geom;
    p.rsq = c->neigh_cut * c->neigh_cut;
    const double band = gbmd_fp32_band( c->geom, c->neigh_cut );
    p.rsq_lo = (float)( p.rsq * ( 1.0 - band ) );
    p.rsq_hi = (float)( p.rsq * ( 1.0 + band ) );
    p.stride = (int)c->nl_stride;
    p.half = c->half;
    p.no_images = c->no_images;
    {
        // |FP32 relative coordinate - exact| <= u (|x| + |shift|) with
        // |x| <= 2h + rc; 8x margin for the difference of two.
        const double hmax = fmax( c->geom.h[0], fmax( c->geom.h[1], c->geom.h[2] ) );
        p.eps_half = (float)( 8.0 * std::ldexp( 1.0, -24 ) * ( 3.0 * hmax + c->neigh_cut ) );
    }
    p.cap = c->nl_cap;
    return p;
}

int gbmd_build_list_launch( gbmd_ctx *c )
{
    const int n = (int)c->n;
    int rc;
    if ( ( rc = gbmd_build_list_prepare( c ) ) )
        return rc;
    const NbParams p = nb_params( c );
    GBMD_CUDA( c, cudaMemsetAsync( c->flags.p, 0, sizeof( int ), c->stream ) );
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_NEIGH, &t0 );
    if ( n > 0 && ( rc = nb_launch( c, p ) ) )
        return rc;
    gbmd_ktime_end( c, GBMD_KT_NEIGH, t0 );
    GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, sizeof( int ),
                                   cudaMemcpyDeviceToHost, c->stream ) );
    c->nl_attempts++;
    return GBMD_OK;
}

// Index of the context's list-build shape among the compiled ones (an
// unknown shape runs the default, as nb_launch does).
static int nb_shape_index( const gbmd_ctx *c )
{
    for ( int k = 0; k < GBMD_NB_NSHAPES; k++ )
        if ( nb_shapes[k][0] == c->tune.nb_warps && nb_shapes[k][1] == c->tune.nb_out )
            return k;
    return 0;
}

template <int NW, int NOUT, bool HALF>
static int nb_jobs_launch_kind( gbmd_ctx *c0, const NbJobTable &t, int blocks )
{
    constexpr size_t smem = sizeof( NbWarpSmem<NOUT> ) * NW;
    static std::atomic<unsigned> ready{ 0 }; // attribute set, one bit per device
    const unsigned bit = c0->device < 32 ? 1u << c0->device : 0u;
    if ( !( ready.load( std::memory_order_acquire ) & bit ) )
    {
        GBMD_CUDA( c0, cudaFuncSetAttribute( k_neigh_build_jobs<NW, NOUT, HALF>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem ) );
        ready.fetch_or( bit, std::memory_order_release );
    }
    k_neigh_build_jobs<NW, NOUT, HALF><<<blocks, NW * 32, smem, c0->stream>>>( t );
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBMD_OK : gbmd_cuda_check( c0, e, "neigh_build batch" );
}

template <int NW, int NOUT>
static int nb_jobs_launch_shape( gbmd_ctx *c0, const NbJobTable &t, int blocks, bool half )
{
    return half ? nb_jobs_launch_kind<NW, NOUT, true>( c0, t, blocks )
                : nb_jobs_launch_kind<NW, NOUT, false>( c0, t, blocks );
}

static int nb_jobs_launch( gbmd_ctx *c0, int shape, bool half, const NbJobTable &t, int blocks )
{
    switch ( shape )
    {
    case 1:
        return nb_jobs_launch_shape<8, 32>( c0, t, blocks, half );
    case 2:
        return nb_jobs_launch_shape<16, 24>( c0, t, blocks, half );
    case 3:
        return nb_jobs_launch_shape<8, 48>( c0, t, blocks, half );
    default:
        return nb_jobs_launch_shape<12, 32>( c0, t, blocks, half );
    }
}

// The list builds of sorted contexts sharing one stream (prepared with
// gbmd_build_list_prepare, flags[0] zeroed): one job-table launch per
// (shape, half) group, then one launch that copies every job's largest row
// count to its pinned host flags.
int gbmd_build_list_batch( gbmd_ctx *const *cs, int count, int64_t *launches )
{
    if ( count <= 0 )
        return GBMD_OK;
    gbmd_ctx *c0 = cs[0];
    NbJobTable t;
    std::memset( &t, 0, sizeof t );
    auto fill = [&]( int q, gbmd_ctx *c ) {
        NbJob &J = t.job[q];
        J.x = c->x.p;
        J.xr = c->xr.p;
        J.gflag = c->gflag.p;
        J.cstart = c->cell_start.p;
        J.nlist = c->nlist.p;
        J.nnum = c->nnum.p;
        J.flags = c->flags.p;
        J.h_max = c->h_flags_dev;
        J.p = nb_params( c );
    };
    int rc;
    for ( int shape = 0; shape < GBMD_NB_NSHAPES; shape++ )
        for ( int half = 0; half < 2; half++ )
        {
            int nw, nout;
            gbmd_nb_shape( shape, &nw, &nout );
            std::vector<gbmd_ctx *> grp;
            for ( int q = 0; q < count; q++ )
                if ( nb_shape_index( cs[q] ) == shape && ( cs[q]->half != 0 ) == ( half != 0 ) )
                    grp.push_back( cs[q] );
            for ( size_t b = 0; b < grp.size(); b += NB_JOBS )
            {
                const int nj = (int)std::min( grp.size() - b, (size_t)NB_JOBS );
                int blocks = 0;
                t.njobs = nj;
                for ( int q = 0; q < nj; q++ )
                {
                    fill( q, grp[b + q] );
                    t.block0[q] = blocks;
                    blocks += ( grp[b + q]->geom.ncell + nw - 1 ) / nw;
                }
                t.block0[nj] = blocks;
                if ( ( rc = nb_jobs_launch( c0, shape, half != 0, t, blocks ) ) )
                    return rc;
                ( *launches )++;
            }
        }
    // row maxima to the host: mapped pinned flags in one launch, or a copy
    // per job where the host flags have no device mapping
    std::vector<gbmd_ctx *> mapped;
    for ( int q = 0; q < count; q++ )
    {
        gbmd_ctx *c = cs[q];
        if ( c->h_flags_dev )
            mapped.push_back( c );
        else
            GBMD_CUDA( c, cudaMemcpyAsync( c->h_flags, c->flags.p, sizeof( int ),
                                           cudaMemcpyDeviceToHost, c->stream ) );
        c->nl_attempts++;
    }
    for ( size_t b = 0; b < mapped.size(); b += NB_JOBS )
    {
        const int nj = (int)std::min( mapped.size() - b, (size_t)NB_JOBS );
        t.njobs = nj;
        for ( int q = 0; q < nj; q++ )
        {
            t.job[q].flags = mapped[b + q]->flags.p;
            t.job[q].h_max = mapped[b + q]->h_flags_dev;
        }
        k_nb_publish_jobs<<<1, NB_JOBS, 0, c0->stream>>>( t );
        const cudaError_t e = cudaGetLastError();
        if ( e != cudaSuccess )
            return gbmd_cuda_check( c0, e, "neigh_build batch: row maxima" );
        ( *launches )++;
    }
    return GBMD_OK;
}

// Capacity check of a launched build (its largest row count in h_flags[0],
// the stream drained): accepts the list, whose rows the caller then pads, or
// grows the capacity and asks for another launch.
int gbmd_build_list_check( gbmd_ctx *c, bool *again )
{
    const int maxc = c->h_flags[0];
    *again = false;
    if ( maxc <= c->nl_cap )
    {
        c->nl_maxc = maxc;
        // neighbor_verlet.h:58-61 grows the guess by 10% past the max
        if ( maxc > c->max_neigh_guess )
            c->max_neigh_guess = (int)( maxc * 1.1 );
        c->have_list = true;
        c->nl_attempts = 0;
        return GBMD_OK;
    }
    if ( c->nl_attempts >= 4 )
        return gbmd_fail( c, GBMD_ERR_CAPACITY, "neigh_build: list capacity did not converge" );
    c->max_neigh_guess = (int)( maxc * 1.1 ) + 1;
    c->nl_cap = ( c->max_neigh_guess + 3 ) & ~3;
    *again = true;
    return GBMD_OK;
}

int gbmd_build_list_finish( gbmd_ctx *c, bool *again )
{
    const int n = (int)c->n;
    int rc = gbmd_build_list_check( c, again );
    if ( rc || *again )
        return rc;
    if ( n > 0 )
    {
        const int nw = ( n + 31 ) / 32 * 32; // whole warps, <= nl_stride
        k_pad_lists<<<( nw + 127 ) / 128, 128, 0, c->stream>>>( c->nnum.p, n, (int)c->nl_stride,
                                                               c->nlist.p );
        GBMD_LAUNCH_CHECK( c, "pad lists" );
    }
    return GBMD_OK;
}

// Row padding of accepted lists of contexts sharing one stream, in job-table
// launches.
int gbmd_pad_lists_batch( gbmd_ctx *const *cs, int count, int64_t *launches )
{
    PadTable t;
    std::memset( &t, 0, sizeof t );
    std::vector<gbmd_ctx *> live;
    for ( int q = 0; q < count; q++ )
        if ( cs[q]->n > 0 )
            live.push_back( cs[q] );
    for ( size_t b = 0; b < live.size(); b += NB_JOBS )
    {
        const int nj = (int)std::min( live.size() - b, (size_t)NB_JOBS );
        int blocks = 0;
        t.njobs = nj;
        for ( int q = 0; q < nj; q++ )
        {
            const gbmd_ctx *c = live[b + q];
            PadJob &J = t.job[q];
            J.nnum = c->nnum.p;
            J.nlist = c->nlist.p;
            J.n = (int)c->n;
            J.stride = (int)c->nl_stride;
            t.block0[q] = blocks;
            blocks += ( ( J.n + 31 ) / 32 * 32 + 127 ) / 128;
        }
        t.block0[nj] = blocks;
        k_pad_lists_jobs<<<blocks, 128, 0, live[0]->stream>>>( t );
        const cudaError_t e = cudaGetLastError();
        if ( e != cudaSuccess )
            return gbmd_cuda_check( live[0], e, "pad lists batch" );
        ( *launches )++;
    }
    return GBMD_OK;
}

int gbmd_build_list( gbmd_ctx *c )
{
    c->nl_attempts = 0;
    for ( ;; )
    {
        int rc = gbmd_build_list_launch( c );
        if ( rc )
            return rc;
        GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
        bool again = false;
        if ( ( rc = gbmd_build_list_finish( c, &again ) ) )
            return rc;
        if ( !again )
            return GBMD_OK;
    }
}

extern "C" int gbmd_neigh_size( gbmd_ctx *c, int64_t *total, int32_t *max_count )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( !c->have_list )
        return gbmd_fail( c, GBMD_ERR_ARG, "neigh_size: no list" );
    std::vector<int> cnt( c->n );
    if ( c->n )
        GBMD_CUDA( c, cudaMemcpy( cnt.data(), c->nnum.p, sizeof( int ) * c->n,
                                  cudaMemcpyDeviceToHost ) );
    int64_t t = 0;
    int m = 0;
    for ( int v : cnt )
    {
        t += v;
        m = v > m ? v : m;
    }
    if ( total )
        *total = t;
    if ( max_count )
        *max_count = m;
    return GBMD_OK;
}

extern "C" int gbmd_neigh_download( gbmd_ctx *c, int32_t *counts, int32_t *j_out,
                                    int8_t *img_out )
{
    if ( !c || !counts )
        return GBMD_ERR_ARG;
    if ( !c->have_list )
        return gbmd_fail( c, GBMD_ERR_ARG, "neigh_download: no list" );
    const int64_t n = c->n;
    if ( n == 0 )
        return GBMD_OK;
    std::vector<int> cnt( n ), home( n );
    std::vector<uint32_t> nl( (size_t)c->nl_cap * c->nl_stride );
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    GBMD_CUDA( c, cudaMemcpy( cnt.data(), c->nnum.p, sizeof( int ) * n,
                              cudaMemcpyDeviceToHost ) );
    GBMD_CUDA( c, cudaMemcpy( home.data(), c->home.p, sizeof( int ) * n,
                              cudaMemcpyDeviceToHost ) );
    GBMD_CUDA( c, cudaMemcpy( nl.data(), c->nlist.p, sizeof( uint32_t ) * nl.size(),
                              cudaMemcpyDeviceToHost ) );
    int64_t k = 0;
    for ( int64_t i = 0; i < n; i++ )
    {
        counts[i] = cnt[i];
        for ( int s = 0; s < cnt[i]; s++ )
        {
            const uint32_t e = nl[(size_t)s * c->nl_stride + i];
            const int sc = (int)( e >> 27 );
            int code = 0, mul = 1;
            for ( int d = 0; d < 3; d++ )
            {
                const int sh = image_shift( unpack_home( home[i], d ),
                                            stencil_d( sc, d ), c->geom.nc[d] );
                code += ( sh + 1 ) * mul;
                mul *= 3;
            }
            if ( j_out )
                j_out[k] = (int32_t)( e & GBMD_JMASK );
            if ( img_out )
                img_out[k] = (int8_t)code;
            k++;
        }
    }
    return GBMD_OK;
}

extern "C" int gbmd_set_list_images( gbmd_ctx *c, int periodic )
{
    if ( !c )
        return GBMD_ERR_ARG;
    const int ni = periodic ? 0 : 1;
    if ( ni != c->no_images )
        c->have_list = false;
    c->no_images = ni;
    return GBMD_OK;
}

