// gbmd_nnp_mlp_tc.cu -- the per-element atomic MLP of the NNP (energy E_i
// and dE_i/dG) as 5th-generation tensor-core GEMM tiles over atoms.
//
// Reference: n2p2 calculateAtomicNeuralNetworks, called from
// src/force_types/force_nnp_cabana_neigh_impl.h:96 (paths inside the
// CabanaMD project): scaled G -> hidden layers -> E_i, and the backward
// pass dE/dG that calculateForces chains into forces.
//
// One CTA (4 warps, one atom row per thread) runs tiles of 128 atoms through
// four M=128, N=32 GEMMs issued by one thread with tcgen05.mma (kind::f16,
// BF16 operands, FP32 accumulators in tensor memory):
//   forward   z1 = x0 W1^T,   z2 = a1 W2^T
//   backward  g1 = d2 W2,     dx0 = d1 W1
// and reads every accumulator back with tcgen05.ld for the FP32 epilogue
// (bias, activation and its derivative, the linear output layer, BF16
// packing of the next operand).  Operands are split three ways in BF16,
// x = hi + mid + lo (8 significand bits each, 24 in all), and laid out along
// K = 192 as A = [hi | hi | mid | hi | lo | mid] against
// B = [hi | mid | hi | lo | hi | mid], so each GEMM accumulates, in FP32,
// hi*hi + hi*mid + mid*hi + hi*lo + lo*hi + mid*mid: every product down to
// 2^-24 relative, i.e. FP32-accurate GEMMs on BF16 tensor cores.  (A two-way
// split keeps 2^-16, and the input scaling of the symmetry functions
// amplifies that to ~1e-4 in the forces.)
// The weight operands arrive in shared memory by one TMA bulk copy; every
// mbarrier wait is bounded and reports a timeout through the context flags.
#include "gbmd_nnp.cuh"

#include <cuda_bf16.h>

#include <cstring>

constexpr int TC_M = 128;
constexpr int TC_KC = 24;                     // core matrices along K = 192
constexpr int TC_A_BYTES = 16 * TC_KC * 128; // 128 rows x 192 K of BF16
constexpr int TC_SMEM = TC_A_BYTES + 4 * TC_B_BYTES + 64;
constexpr uint32_t TC_TMEM_COLS = 128; // four 32-column FP32 accumulators

// ---------------------------------------------------------------------------
// host: operand images
static uint16_t f2bf( float f )
{
    uint32_t u;
    std::memcpy( &u, &f, 4 );
    if ( ( u & 0x7fffffffu ) > 0x7f800000u )
        return 0x7fc0;
    return (uint16_t)( ( u + 0x7fffu + ( ( u >> 16 ) & 1u ) ) >> 16 );
}

static float bf2f( uint16_t h )
{
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy( &f, &u, 4 );
    return f;
}

static size_t core_offset( int row, int k ) // bytes, TC_KC core matrices along K
{
    return ( ( row / 8 ) * TC_KC + k / 8 ) * 128 + ( row % 8 ) * 16 + ( k % 8 ) * 2;
}

// B (32 x 32 logical, B[n][k]) -> [hi | mid | hi | lo | hi | mid] image
static void put_b( uint16_t *img, int n, int k, double val )
{
    const float f = (float)val;
    const uint16_t hi = f2bf( f );
    const float r = f - bf2f( hi );
    const uint16_t mid = f2bf( r );
    const uint16_t lo = f2bf( r - bf2f( mid ) );
    const uint16_t part[6] = { hi, mid, hi, lo, hi, mid };
    for ( int q = 0; q < 6; q++ )
        img[core_offset( n, 32 * q + k ) / 2] = part[q];
}

bool gbmd_tc_model_build( const NnpParams &p, const std::vector<double> &w,
                          const std::vector<double> &b, TcModel &out )
{
    if ( p.nl != 3 || p.nsf > 32 || p.nodes[1] > 32 || p.nodes[2] > 32 || p.nodes[3] != 1 ||
         p.act[3] != 'l' )
        return false;
    std::memset( &out, 0, sizeof( out ) );
    const int nsf = p.nsf, h1 = p.nodes[1], h2 = p.nodes[2];
    const double *W1 = w.data() + p.woff[1]; // [h1][nsf]
    const double *W2 = w.data() + p.woff[2]; // [h2][h1]
    const double *W3 = w.data() + p.woff[3]; // [1][h2]
    for ( int j = 0; j < h1; j++ )
        for ( int s = 0; s < nsf; s++ )
        {
            put_b( out.img[0], j, s, W1[j * nsf + s] ); // forward:  B[n=j][k=s]
            put_b( out.img[3], s, j, W1[j * nsf + s] ); // backward: B[n=s][k=j]
        }
    for ( int j = 0; j < h2; j++ )
        for ( int i = 0; i < h1; i++ )
        {
            put_b( out.img[1], j, i, W2[j * h1 + i] ); // forward:  B[n=j][k=i]
            put_b( out.img[2], i, j, W2[j * h1 + i] ); // backward: B[n=i][k=j]
        }
    for ( int j = 0; j < h1; j++ )
        out.b1[j] = (float)b[p.boff[1] + j];
    for ( int j = 0; j < h2; j++ )
    {
        out.b2[j] = (float)b[p.boff[2] + j];
        out.w3[j] = (float)W3[j];
    }
    out.b3 = (float)b[p.boff[3]];
    for ( int s = 0; s < nsf; s++ )
    {
        out.gmin[s] = (float)p.gmin[s];
        out.gscale[s] = (float)p.gscale[s];
    }
    out.smin = (float)p.smin;
    out.nsf = nsf;
    out.h1 = h1;
    out.h2 = h2;
    out.act1 = p.act[1];
    out.act2 = p.act[2];
    return true;
}

// ---------------------------------------------------------------------------
// device: tcgen05 wrappers (inline PTX)
__device__ __forceinline__ void tmem_alloc( uint32_t *slot, uint32_t ncols )
{
    asm volatile( "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                      smem_u32( slot ) ),
                  "r"( ncols )
                  : "memory" );
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile( "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory" );
}

__device__ __forceinline__ void tmem_dealloc( uint32_t taddr, uint32_t ncols )
{
    asm volatile( "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"( taddr ),
                  "r"( ncols )
                  : "memory" );
}

__device__ __forceinline__ void tc_fence_before() { asm volatile( "tcgen05.fence::before_thread_sync;" ::: "memory" ); }
__device__ __forceinline__ void tc_fence_after() { asm volatile( "tcgen05.fence::after_thread_sync;" ::: "memory" ); }
__device__ __forceinline__ void fence_async_smem() { asm volatile( "fence.proxy.async.shared::cta;" ::: "memory" ); }

// D[tmem] (+)= A[smem] x B[smem], M=128, N=32, K=16, BF16 in, FP32 out.
__device__ __forceinline__ void umma_bf16( uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                           uint32_t idesc, uint32_t accumulate )
{
    asm volatile( "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"( d_tmem ),
                  "l"( adesc ), "l"( bdesc ), "r"( idesc ), "r"( accumulate )
                  : "memory" );
}

__device__ __forceinline__ void umma_commit( uint64_t *bar )
{
    asm volatile( "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                      smem_u32( bar ) )
                  : "memory" );
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32( uint32_t taddr, float *v )
{
    uint32_t r[32];
    asm volatile( "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                  "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                  "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                  : "=r"( r[0] ), "=r"( r[1] ), "=r"( r[2] ), "=r"( r[3] ), "=r"( r[4] ),
                    "=r"( r[5] ), "=r"( r[6] ), "=r"( r[7] ), "=r"( r[8] ), "=r"( r[9] ),
                    "=r"( r[10] ), "=r"( r[11] ), "=r"( r[12] ), "=r"( r[13] ), "=r"( r[14] ),
                    "=r"( r[15] ), "=r"( r[16] ), "=r"( r[17] ), "=r"( r[18] ), "=r"( r[19] ),
                    "=r"( r[20] ), "=r"( r[21] ), "=r"( r[22] ), "=r"( r[23] ), "=r"( r[24] ),
                    "=r"( r[25] ), "=r"( r[26] ), "=r"( r[27] ), "=r"( r[28] ), "=r"( r[29] ),
                    "=r"( r[30] ), "=r"( r[31] )
                  : "r"( taddr )
                  : "memory" );
    asm volatile( "tcgen05.wait::ld.sync.aligned;" ::: "memory" );
#pragma unroll
    for ( int k = 0; k < 32; k++ )
        v[k] = __uint_as_float( r[k] );
}

// Shared memory matrix descriptor: no swizzle, K-major core matrices of
// 8 rows x 16 bytes; LBO = distance between core matrices along K (128 B),
// SBO = distance between 8-row groups (TC_KC * 128 B); descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc( uint32_t addr )
{
    const uint64_t lbo = 128, sbo = TC_KC * 128;
    return (uint64_t)( ( addr & 0x3FFFFu ) >> 4 ) | ( ( lbo >> 4 ) << 16 ) |
           ( ( sbo >> 4 ) << 32 ) | ( 1ull << 46 );
}

// Instruction descriptor: D FP32, A and B BF16, both K-major, N = 32, M = 128.
constexpr uint32_t TC_IDESC = ( 1u << 4 ) | ( 1u << 7 ) | ( 1u << 10 ) | ( ( 32u >> 3 ) << 17 ) |
                              ( ( 128u >> 4 ) << 24 );

// An activation and its derivative at x: 't' tanh, 'p' softplus
// log(1 + e^x) (x beyond 20: x), 's' sigmoid, 'l' linear.  The values are
// the same operations as one evaluation per function would give (tanh and
// the sigmoid computed once for both), so the network's outputs do not
// depend on this sharing.
template <char A> __device__ __forceinline__ void act_both( float x, float &a, float &d )
{
    if constexpr ( A == 't' )
    {
        const float t = tanhf( x );
        a = t;
        d = 1.f - t * t;
    }
    else if constexpr ( A == 'p' )
    {
        a = x > 20.f ? x : log1pf( __expf( x ) );
        d = 1.f / ( 1.f + __expf( -x ) );
    }
    else if constexpr ( A == 's' )
    {
        const float sg = 1.f / ( 1.f + __expf( -x ) );
        a = sg;
        d = sg * ( 1.f - sg );
    }
    else
    {
        a = x;
        d = 1.f;
    }
}

// Hidden layer 1 at one row: v = act(z + b1), d1 = act'(z + b1) (zero past h1).
template <char A>
__device__ __forceinline__ void layer1_rows( const float *z, const TcModel *__restrict__ M, int h1,
                                             float *v, float *d1 )
{
#pragma unroll
    for ( int j = 0; j < 32; j++ )
    {
        float a = 0.f, d = 0.f;
        if ( j < h1 )
            act_both<A>( z[j] + M->b1[j], a, d );
        v[j] = a;
        d1[j] = d;
    }
}

// Hidden layer 2 at one row: the atom's energy e += w3 . act(z + b2) and
// v = w3 * act'(z + b2) = dE/dz2 (linear output layer).
template <char A>
__device__ __forceinline__ void layer2_rows( const float *z, const TcModel *__restrict__ M, int h2,
                                             float &e, float *v )
{
#pragma unroll
    for ( int j = 0; j < 32; j++ )
    {
        float a = 0.f, d = 0.f;
        if ( j < h2 )
            act_both<A>( z[j] + M->b2[j], a, d );
        const float w3 = j < h2 ? M->w3[j] : 0.f;
        e += w3 * a;
        v[j] = w3 * d;
    }
}

// Row `row` of the A operand: [hi | hi | mid | hi | lo | mid] of 32 FP32
// values (three-way BF16 split).
__device__ __forceinline__ void write_a_row( uint8_t *A, int row, const float *v )
{
#pragma unroll
    for ( int kc = 0; kc < 4; kc++ )
    {
        uint32_t hw[4], mw[4], lw[4];
#pragma unroll
        for ( int q = 0; q < 4; q++ )
        {
            uint32_t h2 = 0, m2 = 0, l2 = 0;
#pragma unroll
            for ( int e = 0; e < 2; e++ )
            {
                const float a = v[kc * 8 + 2 * q + e];
                const __nv_bfloat16 h = __float2bfloat16_rn( a );
                const float r = a - __bfloat162float( h );
                const __nv_bfloat16 m = __float2bfloat16_rn( r );
                const __nv_bfloat16 l = __float2bfloat16_rn( r - __bfloat162float( m ) );
                h2 |= (uint32_t)__bfloat16_as_ushort( h ) << ( 16 * e );
                m2 |= (uint32_t)__bfloat16_as_ushort( m ) << ( 16 * e );
                l2 |= (uint32_t)__bfloat16_as_ushort( l ) << ( 16 * e );
            }
            hw[q] = h2;
            mw[q] = m2;
            lw[q] = l2;
        }
        const uint4 H = make_uint4( hw[0], hw[1], hw[2], hw[3] );
        const uint4 Mi = make_uint4( mw[0], mw[1], mw[2], mw[3] );
        const uint4 Lo = make_uint4( lw[0], lw[1], lw[2], lw[3] );
        uint8_t *base = A + ( row / 8 ) * TC_KC * 128 + ( row % 8 ) * 16 + kc * 128;
        *reinterpret_cast<uint4 *>( base + 0 * 512 ) = H;
        *reinterpret_cast<uint4 *>( base + 1 * 512 ) = H;
        *reinterpret_cast<uint4 *>( base + 2 * 512 ) = Mi;
        *reinterpret_cast<uint4 *>( base + 3 * 512 ) = H;
        *reinterpret_cast<uint4 *>( base + 4 * 512 ) = Lo;
        *reinterpret_cast<uint4 *>( base + 5 * 512 ) = Mi;
    }
}

// Shared state of one CTA: operand buffers, barriers, TMEM and the phase of
// the MMA-completion barrier.
struct MlpCta
{
    uint8_t *A, *B;
    uint64_t *bar;
    uint32_t a_addr, b_addr, tbase, tlane, phase;
    int tid, warp;
    double *red;
};

// Set-up shared by the kernels: barriers, TMEM allocation (four 32-column
// accumulators); the weights are loaded by mlp_load_weights.
__device__ __forceinline__ void mlp_setup( MlpCta &x, uint8_t *sm, double *red,
                                           uint32_t *&tslot )
{
    x.A = sm;
    x.B = sm + TC_A_BYTES;
    x.bar = reinterpret_cast<uint64_t *>( sm + TC_A_BYTES + 4 * TC_B_BYTES );
    tslot = reinterpret_cast<uint32_t *>( x.bar + 2 );
    x.red = red;
    x.tid = threadIdx.x;
    x.warp = x.tid >> 5;
    x.phase = 0;
    if ( x.tid == 0 )
    {
        mbar_init( &x.bar[0], 1 ); // weights landed
        mbar_init( &x.bar[1], 1 ); // an MMA chain finished
        mbar_fence_init();
    }
    __syncthreads();
}

// Weight images of model M into B by one TMA bulk copy; bounded wait on
// barrier 0 with parity `wphase`.  Block-uniform result.
__device__ __forceinline__ bool mlp_load_weights( MlpCta &x, const TcModel *M, uint32_t wphase )
{
    if ( x.tid == 0 )
    {
        mbar_arrive_expect_tx( &x.bar[0], 4 * TC_B_BYTES );
        tma_load_1d( x.B, M->img, 4 * TC_B_BYTES, &x.bar[0] );
    }
    return __syncthreads_and( mbar_wait_bounded( &x.bar[0], wphase ) ) != 0;
}

// One GEMM chain: K = 192 in twelve K16 steps into accumulator column block
// `blk` with B image `img`, then a bounded wait for its completion.
__device__ __forceinline__ bool mlp_gemm( MlpCta &x, int img, int blk )
{
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if ( x.tid == 0 )
    {
#pragma unroll
        for ( int ks = 0; ks < 12; ks++ )
            umma_bf16( x.tbase + 32u * blk, smem_desc( x.a_addr + ks * 256 ),
                       smem_desc( x.b_addr + img * TC_B_BYTES + ks * 256 ), TC_IDESC, ks > 0 );
        umma_commit( &x.bar[1] );
    }
    const bool done = mbar_wait_bounded( &x.bar[1], x.phase );
    x.phase ^= 1u;
    tc_fence_after();
    // block-uniform verdict, so no thread leaves while others wait
    return __syncthreads_and( done ) != 0;
}

// One tile of 128 atoms: forward and backward pass, E_i, dE/dG and the
// tile's energy partial.  Returns false when a bounded wait gave up.
__device__ __forceinline__ bool mlp_tile( MlpCta &x, const float *__restrict__ G, int n,
                                          const TcModel *__restrict__ M,
                                          float *__restrict__ dEdG, double *__restrict__ E,
                                          double *__restrict__ partials, int G_scaled,
                                          const ElemAtoms &ea, int gstride, int tile )
{
    const int tid = x.tid, warp = x.warp;
    // tile rows: atoms in order (one element) or the element group's atoms.
    // A tile past the group's atoms (the grid covers all n) has no rows:
    // block-uniform skip, its energy partial is zero.
    if ( ea.atom( tile * TC_M, n ) < 0 )
    {
        if ( tid == 0 )
            partials[tile] = 0.0;
        return true;
    }
    const int nsf = M->nsf, h1 = M->h1, h2 = M->h2;
    const char act1 = M->act1, act2 = M->act2;
    const int atom = ea.atom( tile * TC_M + tid, n );
    const bool live = atom >= 0;
    const size_t row = live ? (size_t)atom * gstride : 0;
    // One element with 32-float rows: the tile's rows are one contiguous
    // block, so each warp moves its 32 rows as whole 16-byte pieces through
    // shared memory (the A operand's space, free between tiles; rows padded
    // to 33 floats so the per-row reads do not conflict).  Otherwise each
    // thread reads its own row.
    const bool block_rows = !ea.atoms && gstride == 32;
    float *stage = reinterpret_cast<float *>( x.A ) + warp * 32 * 33;
    const int lane = tid & 31;
    const int row0 = tile * TC_M + warp * 32; // first row of this warp
    float v[32];
    if ( block_rows )
    {
#pragma unroll
        for ( int q = 0; q < 8; q++ )
        {
            const int f4 = q * 32 + lane; // float4 index inside the warp's rows
            const int r = f4 >> 3, c = ( f4 & 7 ) * 4;
            float4 g4 = make_float4( 0.f, 0.f, 0.f, 0.f );
            if ( row0 + r < n )
                g4 = __ldg( reinterpret_cast<const float4 *>( G + (size_t)( row0 + r ) * 32 ) +
                            ( f4 & 7 ) );
            stage[r * 33 + c] = g4.x;
            stage[r * 33 + c + 1] = g4.y;
            stage[r * 33 + c + 2] = g4.z;
            stage[r * 33 + c + 3] = g4.w;
        }
        __syncwarp();
#pragma unroll
        for ( int s = 0; s < 32; s++ )
        {
            const float gv = stage[lane * 33 + s];
            v[s] = ( live && s < nsf )
                       ? ( G_scaled ? gv : M->smin + ( gv - M->gmin[s] ) * M->gscale[s] )
                       : 0.f;
        }
        __syncthreads(); // every warp has its rows before A is overwritten
    }
    else
    {
#pragma unroll
        for ( int s = 0; s < 32; s++ )
            v[s] = ( live && s < nsf )
                       ? ( G_scaled ? G[row + s]
                                    : M->smin + ( G[row + s] - M->gmin[s] ) * M->gscale[s] )
                       : 0.f;
    }
    write_a_row( x.A, tid, v );
    if ( !mlp_gemm( x, 0, 0 ) )
        return false;
    float z[32], d1[32];
    tmem_ld32( x.tlane + 0, z );
    switch ( act1 ) // block-uniform
    {
    case 't': layer1_rows<'t'>( z, M, h1, v, d1 ); break;
    case 'p': layer1_rows<'p'>( z, M, h1, v, d1 ); break;
    case 's': layer1_rows<'s'>( z, M, h1, v, d1 ); break;
    default: layer1_rows<'l'>( z, M, h1, v, d1 ); break;
    }
    write_a_row( x.A, tid, v );
    if ( !mlp_gemm( x, 1, 1 ) )
        return false;
    tmem_ld32( x.tlane + 32, z );
    float e = M->b3;
    switch ( act2 ) // block-uniform
    {
    case 't': layer2_rows<'t'>( z, M, h2, e, v ); break;
    case 'p': layer2_rows<'p'>( z, M, h2, e, v ); break;
    case 's': layer2_rows<'s'>( z, M, h2, e, v ); break;
    default: layer2_rows<'l'>( z, M, h2, e, v ); break;
    }
    write_a_row( x.A, tid, v );
    if ( !mlp_gemm( x, 2, 2 ) )
        return false;
    tmem_ld32( x.tlane + 64, z );
#pragma unroll
    for ( int j = 0; j < 32; j++ )
        v[j] = z[j] * d1[j]; // dE/dz1
    write_a_row( x.A, tid, v );
    if ( !mlp_gemm( x, 3, 3 ) )
        return false;
    tmem_ld32( x.tlane + 96, z );
    if ( block_rows )
    {
        // the MMAs are done with A (mlp_gemm waited): rows back through the
        // same staging, stored as whole 16-byte pieces (columns past nsf
        // are zero: gscale is zero there)
#pragma unroll
        for ( int s = 0; s < 32; s++ )
            stage[lane * 33 + s] = z[s] * M->gscale[s];
        __syncwarp();
#pragma unroll
        for ( int q = 0; q < 8; q++ )
        {
            const int f4 = q * 32 + lane;
            const int r = f4 >> 3, c = ( f4 & 7 ) * 4;
            if ( row0 + r < n )
                reinterpret_cast<float4 *>( dEdG + (size_t)( row0 + r ) * 32 )[f4 & 7] =
                    make_float4( stage[r * 33 + c], stage[r * 33 + c + 1],
                                 stage[r * 33 + c + 2], stage[r * 33 + c + 3] );
        }
        if ( live )
            E[atom] = (double)e;
    }
    else if ( live )
    {
#pragma unroll
        for ( int s = 0; s < 32; s++ )
            if ( s < nsf )
                dEdG[row + s] = z[s] * M->gscale[s];
        E[atom] = (double)e;
    }
    // per-tile energy sum (potential-energy slot)
    double ev = live ? (double)e : 0.0;
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        ev += __shfl_xor_sync( 0xffffffffu, ev, o );
    if ( ( tid & 31 ) == 0 )
        x.red[warp] = ev;
    __syncthreads();
    if ( tid == 0 )
        partials[tile] = x.red[0] + x.red[1] + x.red[2] + x.red[3];
    return true;
}

// TMEM columns for this CTA, after the weights' copy was issued.
__device__ __forceinline__ void mlp_tmem( MlpCta &x, uint32_t *tslot )
{
    if ( x.warp == 0 )
    {
        tmem_alloc( tslot, TC_TMEM_COLS );
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    x.tbase = *tslot;
    x.tlane = x.tbase + ( (uint32_t)( x.warp * 32 ) << 16 ); // this warp's lanes
    x.a_addr = smem_u32( x.A );
    x.b_addr = smem_u32( x.B );
}

__device__ __forceinline__ void mlp_teardown( MlpCta &x, bool ok, int *flags )
{
    if ( !ok && x.tid == 0 )
        atomicExch( &flags[3], 1 );
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if ( x.warp == 0 )
        tmem_dealloc( x.tbase, TC_TMEM_COLS );
}

__global__ void __launch_bounds__( TC_M, 1 )
    k_nnp_mlp_tc( const float *__restrict__ G, int n, const TcModel *__restrict__ M,
                  float *__restrict__ dEdG, double *__restrict__ E, double *__restrict__ partials,
                  int G_scaled, int *__restrict__ flags, ElemAtoms ea, int gstride )
{
    extern __shared__ __align__( 1024 ) uint8_t sm[];
    __shared__ double red[TC_M / 32];
    MlpCta x;
    uint32_t *tslot;
    mlp_setup( x, sm, red, tslot );
    if ( x.tid == 0 )
    {
        mbar_arrive_expect_tx( &x.bar[0], 4 * TC_B_BYTES );
        tma_load_1d( x.B, M->img, 4 * TC_B_BYTES, &x.bar[0] );
    }
    mlp_tmem( x, tslot );
    bool ok = __syncthreads_and( mbar_wait_bounded( &x.bar[0], 0 ) ) != 0;
    const int ntiles = ( n + TC_M - 1 ) / TC_M;
    for ( int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x )
        ok = mlp_tile( x, G, n, M, dEdG, E, partials, G_scaled, ea, gstride, tile );
    mlp_teardown( x, ok, flags );
}

// Serving: the tiles of every job of the table, persistent over the grid.
// Each CTA takes a contiguous range of tiles, so consecutive tiles mostly
// belong to one job, and it reloads the weight images only when a tile's
// job has another model.
__global__ void __launch_bounds__( TC_M, 1 ) k_nnp_mlp_tc_jobs( const __grid_constant__ NnpJobTable t )
{
    extern __shared__ __align__( 1024 ) uint8_t sm[];
    __shared__ double red[TC_M / 32];
    MlpCta x;
    uint32_t *tslot;
    mlp_setup( x, sm, red, tslot );
    mlp_tmem( x, tslot );
    bool ok = true;
    const TcModel *loaded = nullptr;
    uint32_t wphase = 0;
    int *flags = t.job[0].flags;
    const int ntiles = t.b_mlp[t.njobs];
    const int per = ( ntiles + gridDim.x - 1 ) / gridDim.x;
    const int g0 = blockIdx.x * per, g1 = min( ntiles, g0 + per );
    for ( int gt = g0; gt < g1 && ok; gt++ )
    {
        const int j = nnp_job_of( t.b_mlp, t.njobs, gt );
        const NnpJobArgs &J = t.job[j];
        flags = J.flags;
        if ( J.tcm != loaded )
        {
            // the previous tile's MMAs completed (mlp_gemm waited), so B is free
            if ( !( ok = mlp_load_weights( x, J.tcm, wphase ) ) )
                break;
            wphase ^= 1u;
            loaded = J.tcm;
        }
        ok = mlp_tile( x, J.G, J.n, J.tcm, J.dEdG, J.E, J.pe_part, 1, ElemAtoms(), J.gstride,
                       gt - t.b_mlp[j] );
    }
    mlp_teardown( x, ok, flags );
}

int gbmd_nnp_mlp_tc_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st )
{
    int nsm = 0;
    cudaDeviceGetAttribute( &nsm, cudaDevAttrMultiProcessorCount, device );
    const int ntiles = t.b_mlp[t.njobs];
    if ( ntiles == 0 )
        return GBMD_OK;
    const int grid = ntiles < 2 * nsm ? ntiles : 2 * nsm;
    if ( cudaFuncSetAttribute( k_nnp_mlp_tc_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               TC_SMEM ) != cudaSuccess )
        return GBMD_ERR_CUDA;
    k_nnp_mlp_tc_jobs<<<grid, TC_M, TC_SMEM, st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

int gbmd_nnp_mlp_tc_launch( gbmd_ctx *c, const TcModel *dev, const float *G, float *dEdG,
                            double *E, int n, double *partials, int G_scaled,
                            const ElemAtoms &ea, int gstride )
{
    if ( n == 0 )
        return GBMD_OK;
    int nsm = 0;
    cudaDeviceGetAttribute( &nsm, cudaDevAttrMultiProcessorCount, c->device );
    const int ntiles = ( n + TC_M - 1 ) / TC_M;
    // persistent: up to two CTAs per SM (96 KB of shared memory each; 2 x 128
    // TMEM columns of the 512, so no allocation ever waits)
    const int grid = ntiles < 2 * nsm ? ntiles : 2 * nsm;
    GBMD_CUDA( c, cudaFuncSetAttribute( k_nnp_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        TC_SMEM ) );
    k_nnp_mlp_tc<<<grid, TC_M, TC_SMEM, c->stream>>>( G, n, dev, dEdG, E, partials, G_scaled,
                                                      c->flags.p, ea, gstride );
    GBMD_LAUNCH_CHECK( c, "nnp mlp tensor core" );
    return GBMD_OK;
}
