// gbmd_nnp_f32.cu -- mixed-precision NNP symmetry functions and forces for
// the common n2p2 form: angular functions with lambda = +-1 and zeta a power
// of two (the reference's fixture input/nnp/input.nn and the synthetic Cu
// potential both use zeta in {1, 2, 4, 16}).
//
// Same mathematics as gbmd_nnp.cu (G2/G3 of n2p2 v2.0.1, cosine cutoff,
// forces through dE/dG), organised for the SIMT pipes of GB300:
//  - One warp per atom.  The neighbours inside rc are gathered into shared
//    memory as three 16-byte records each -- (dx, dy, dz, r), (1/r, fc, dfc,
//    owner) and the gradient accumulated on it -- so a triplet reads its two
//    neighbours with four 128-bit shared loads.
//  - Triplets are compacted before any arithmetic: the warp walks the j<k
//    pairs row by row, 32 candidates per step, tests r_jk < rc and appends
//    the survivors (packed slot pairs) to a 512-entry shared buffer; the
//    triplet body then runs with every lane busy.  (Without compaction about
//    half the lanes idle: half the candidate pairs fail r_jk < rc.)  With
//    several elements the gathered neighbours are first grouped by element,
//    and each element pair (channel) walks only its own block of pairs.
//  - (1 + lambda cos)^zeta for every zeta = 2^m is a squaring ladder of
//    1 - cos and 1 + cos; its derivative lambda zeta b^(zeta-1) uses the
//    products b^(2^m - 1) = b b^2 ... b^(2^(m-1)).  The lambda = -1 / +1
//    halves of the ladder and of every accumulator are one float2, computed
//    with Blackwell's packed FP32 instructions (two lanes of arithmetic per
//    issue slot: __fmul2_rn, __ffma2_rn, __fadd2_rn).
//  - Forces: a triplet's gradients on its two neighbours are
//      g_j = A_j d_j + U d_k,   g_k = U d_j + B_k d_k
//    (the chain rule through cos, R^2 and the three cutoffs, collected on
//    the two displacement vectors).  Gradients on the first neighbour are
//    reduced over the lanes that share it (they are contiguous: the buffer
//    is in row order) with a segmented shuffle reduction; gradients on the
//    second neighbour go to shared memory one row segment at a time.  The
//    warp's per-neighbour sums reach the owners as 64-bit fixed-point
//    integer atomics (2^-32 eV/A resolution), which are order-independent,
//    so the forces are bit-reproducible; a last pass adds them to f in FP64.
//  - Two neighbour capacities: 192 inside rc (the common case, five blocks
//    per SM) and 448 for dense states (an atom's list count -- neighbours
//    inside rc + skin, an upper bound of those inside rc -- decides at each
//    rebuild; more than 448 inside rc is a capacity error).
#include <atomic>
#include <cmath>
#include <cstddef>
#include <type_traits>

#include "gbmd_internal.cuh"
#include "gbmd_nnp.cuh"

#define NNP_TB 512 // compacted triplets staged per warp
constexpr int NNP_F32_WARPS = 4;
constexpr int NNP_CAP_SMALL = NNP_MAXNBR;       // 192
constexpr int NNP_CAP_LARGE = NNP_MAXNBR_LARGE; // 448
// minimum resident blocks per SM requested from the compiler for the
// 192-neighbour kernels (caps the registers per thread; 0: no cap)
#ifndef GBMD_NNP_MINB
#define GBMD_NNP_MINB 5
#endif
// compensated (Kahan) merge of the per-buffer partial sums in the
// symmetry-function kernel
#ifndef GBMD_NNP_KAHAN
#define GBMD_NNP_KAHAN 0
#endif
// Exponential of the angular terms (one per triplet and eta):
//  - default: the hardware approximation __expf.  Its error, a few ulp at
//    the arguments here (|eta R2| < 10), is far below the BF16-split MLP's.
//    Measured at 256k atoms: NNP step 10.93 vs 11.13 ms, max force error
//    2.9e-5 vs 3.1e-5 relative to the RMS force.
//  - GBMD_NNP_FASTEXP=0: the accurate expf.
#ifndef GBMD_NNP_FASTEXP
#define GBMD_NNP_FASTEXP 1
#endif
__device__ __forceinline__ float tri_exp( float v )
{
#if GBMD_NNP_FASTEXP
    return __expf( v );
#else
    return expf( v );
#endif
}
template <int CAP, int MINB> struct NnpMinBlocks
{
    static constexpr int value = CAP <= NNP_CAP_SMALL ? MINB : 1;
};
#define NNP_F32_BOUNDS( CAP )                                                                      \
    __launch_bounds__( NNP_F32_WARPS * 32, ( NnpMinBlocks<CAP, GBMD_NNP_MINB>::value ) )
// The symmetry-function kernel's buffers carry no gradients, so shared
// memory would hold more of its blocks than of the force kernel's; its
// registers still allow five.  Measured at 256k atoms: 3.26 ms per launch at
// five blocks per SM (91 registers) against 3.49 ms at six (80 registers).
#ifndef GBMD_NNP_SF_MINB
#define GBMD_NNP_SF_MINB 5
#endif
#define NNP_SF_BOUNDS( CAP )                                                                       \
    __launch_bounds__( NNP_F32_WARPS * 32, ( NnpMinBlocks<CAP, GBMD_NNP_SF_MINB>::value ) )
constexpr float FQ_SCALE = 4294967296.0f; // 2^32
constexpr double FQ_INV = 1.0 / 4294967296.0;

__device__ __forceinline__ float2 f2( float a, float b ) { return make_float2( a, b ); }
__device__ __forceinline__ float2 f2s( float a ) { return make_float2( a, a ); }

// Per-warp neighbour buffer for CAP neighbours.  ME (several elements) adds
// each neighbour's element and the slots grouped by element (perm[es[e] ..
// es[e + 1]) holds element e's, in slot order).  Triplets are stored as slot
// pairs a | c << TB_SHIFT.
template <bool ME, int CAP> struct NbrF
{
    static constexpr int NG = ME ? CAP : 1;
    using TbT = typename std::conditional<( CAP <= 256 ), uint16_t, uint32_t>::type;
    using PermT = typename std::conditional<( CAP <= 256 ), uint8_t, uint16_t>::type;
    static constexpr int TB_SHIFT = CAP <= 256 ? 8 : 16;
    static constexpr unsigned TB_MASK = ( 1u << TB_SHIFT ) - 1u;
    float4 g[CAP]; // dx, dy, dz, r
    float4 h[CAP]; // 1/r, fc, dfc, owner index (int bits)
    TbT tb[NNP_TB];
    uint8_t el[NG];
    PermT perm[NG];
    int es[ME ? NNP_MAXELEM + 1 : 1];
    // last, so that the symmetry-function kernel, which has no gradients,
    // allocates its warps' buffers without it
    float4 f[CAP]; // accumulated -dE/dx of the neighbour (x, y, z, unused)
};

// Bytes of one warp's buffer (GRAD: with the gradient array) and of a
// block's buffers.
template <bool ME, int CAP, bool GRAD> constexpr size_t nbr_stride()
{
    using NB = NbrF<ME, CAP>;
    return GRAD ? sizeof( NB ) : ( offsetof( NB, f ) + 15 ) / 16 * 16;
}
template <bool ME, int CAP, bool GRAD> constexpr size_t nbr_smem_bytes()
{
    return nbr_stride<ME, CAP, GRAD>() * NNP_F32_WARPS;
}

// The warps' neighbour buffers live in dynamic shared memory (the 448
// capacity needs more than the 48 KB of static shared memory).
extern __shared__ float4 nnp_dyn_smem[];

// ME: a potential with several elements.  The kernels then cover one
// element's atom group per launch, filter radial sums by neighbour element,
// and run the triplet compaction and sums once per channel (unordered
// neighbour-element pair) with that channel's power-ladder map; each channel
// walks only its own pairs of the element-grouped neighbours.
template <bool ME> struct NnpF32Const
{
    static constexpr int CH = ME ? NNP_MAXCH : 1;
    float eta_r[16], rs_r[16];
    float eta_u[NNP_MAXETA];
    int lad_sf[CH][NNP_MAXETA][2][6];
    int rad_e1[16];
    int nch, ch_e1[NNP_MAXCH], ch_e2[NNP_MAXCH];
    int nrad, nsf, neta;
    float rc, hpirc, cfl; // hpirc = pi / (2 rc)
    double conv; // cflength / cfenergy
    int nelem;
};

template <bool ME>
__device__ __forceinline__ void load_f32_const( const NnpParams *Pg, NnpF32Const<ME> &K )
{
    const int t = threadIdx.x;
    if ( t < 16 )
    {
        K.eta_r[t] = (float)Pg->eta_r[t];
        K.rs_r[t] = (float)Pg->rs_r[t];
        K.rad_e1[t] = Pg->rad_e1[t];
    }
    if ( t < NNP_MAXETA )
        K.eta_u[t] = (float)Pg->eta_u[t];
    for ( int k = t; k < NnpF32Const<ME>::CH * NNP_MAXETA * 2 * 6; k += blockDim.x )
        ( &K.lad_sf[0][0][0][0] )[k] = ( &Pg->lad_sf[0][0][0][0] )[k];
    if ( t < NNP_MAXCH )
    {
        K.ch_e1[t] = Pg->ch_e1[t];
        K.ch_e2[t] = Pg->ch_e2[t];
    }
    if ( t == 0 )
    {
        K.nch = ME ? Pg->nch : 1;
        K.nelem = ME ? Pg->nelem : 1;
        K.nrad = Pg->nrad;
        K.nsf = Pg->nsf;
        K.neta = Pg->neta;
        K.rc = (float)Pg->rc;
        K.hpirc = (float)( 0.5 * M_PI / Pg->rc );
        K.cfl = (float)Pg->cflength;
        K.conv = Pg->cflength / Pg->cfenergy;
    }
}

// Work item w -> atom (or -1): every atom for one element, the element
// group's atoms otherwise.
template <bool ME>
__device__ __forceinline__ int f32_atom( const ElemAtoms &ea, int w, int n )
{
    return ME ? ea.atom( w, n ) : ( w < n ? w : -1 );
}

constexpr int popc_c( int v ) { return v ? ( v & 1 ) + popc_c( v >> 1 ) : 0; }
constexpr int top_bit( int v ) { return v > 1 ? 1 + top_bit( v >> 1 ) : 0; }

// 2^(1 - 2^m), the G3 prefactor 2^(1 - zeta) for zeta = 2^m
__device__ __forceinline__ float ladder_pre( int m )
{
    return __int_as_float( ( 127 + 1 - ( 1 << m ) ) << 23 );
}

// Gather atom i's neighbours inside rc (list order) into S; returns the
// count, capped at CAP (overflow flagged in flags[2]).
template <bool ME, int CAP, bool ZF>
__device__ int gather_f( const float4 *__restrict__ xr, const uint32_t *__restrict__ nlist,
                         size_t stride, int i, int cnt, const GbmdGeom &g,
                         const NnpF32Const<ME> &K, NbrF<ME, CAP> &S, int *flags,
                         const int *__restrict__ type )
{
    const int lane = threadIdx.x & 31;
    const float4 p = xr[i];
    int base = 0;
    for ( int k0 = 0; k0 < cnt; k0 += 32 )
    {
        const int k = k0 + lane;
        bool in = false;
        float dx = 0.f, dy = 0.f, dz = 0.f, r = 0.f;
        int j = 0;
        if ( k < cnt )
        {
            const uint32_t e = nlist[(size_t)k * stride + i];
            j = (int)( e & GBMD_JMASK );
            const int sc = (int)( e >> 27 );
            const float4 q = xr[j];
            dx = ( q.x + (float)( sc % 3 - 1 ) * g.hf[0] - p.x ) * K.cfl;
            dy = ( q.y + (float)( ( sc / 3 ) % 3 - 1 ) * g.hf[1] - p.y ) * K.cfl;
            dz = ( q.z + (float)( sc / 9 - 1 ) * g.hf[2] - p.z ) * K.cfl;
            r = sqrtf( dx * dx + dy * dy + dz * dz );
            in = r < K.rc && r > 0.f;
        }
        const unsigned m = __ballot_sync( 0xffffffffu, in );
        const int pos = base + __popc( m & ( ( 1u << lane ) - 1u ) );
        if ( in && pos < CAP )
        {
            float fc, dfc;
            fc_dfc_f32( r, K.hpirc, fc, dfc );
            S.g[pos] = make_float4( dx, dy, dz, r );
            S.h[pos] = make_float4( 1.0f / r, fc, dfc, __int_as_float( j ) );
            if constexpr ( ZF )
                S.f[pos] = make_float4( 0.f, 0.f, 0.f, 0.f );
            if ( ME )
                S.el[pos] = (uint8_t)type[j];
        }
        base += __popc( m );
    }
    if ( base > CAP )
    {
        if ( lane == 0 )
            atomicMax( &flags[2], base );
        base = CAP;
    }
    __syncwarp();
    return base;
}

// Several elements: group the gathered neighbours by element (a stable
// counting sort of slot indices into S.perm, one ballot per element and 32
// slots), so that each channel's pairs form one block of rows.
template <bool ME, int CAP>
__device__ __forceinline__ void group_by_element( NbrF<ME, CAP> &S, int np, int nelem )
{
    if ( !ME )
        return;
    using PermT = typename NbrF<ME, CAP>::PermT;
    const int lane = threadIdx.x & 31;
    const unsigned lt = ( 1u << lane ) - 1u;
    int base = 0;
    for ( int e = 0; e < nelem; e++ )
    {
        if ( lane == 0 )
            S.es[e] = base;
        for ( int a0 = 0; a0 < np; a0 += 32 )
        {
            const int a = a0 + lane;
            const bool in = a < np && S.el[a] == e;
            const unsigned m = __ballot_sync( 0xffffffffu, in );
            if ( in )
                S.perm[base + __popc( m & lt )] = (PermT)a;
            base += __popc( m );
        }
    }
    if ( lane == 0 )
        S.es[nelem] = base;
    __syncwarp();
}

// Warp-uniform cursor over one channel's neighbour pairs (j < k); adv(u, v,
// k) moves a copy k pairs on, pair(u, v) names the two slots, and a copy
// past the last pair fails valid().
//  - One element: the triangle over the np neighbours (slots in list order)
//    walked by diagonals (v = 1 .. np-1, u = 0 .. np-1-v: pair (u, u + v)),
//    32 consecutive pairs at a time.  Inside one diagonal every pair has its
//    own first and its own second slot, so the force kernel adds the
//    gradients of a run of same-diagonal triplets to the neighbours without
//    reductions (in two phases: first slots, then second slots).
//  - Several: positions index S.perm, walked by rows.  The channel (e1, e2)
//    is the triangle over element e1's group when e1 = e2, else the
//    rectangle e1 x e2: rows u in [u, rowend), row u holding v in
//    [tri ? u + 1 : vs, v1).
template <bool ME> struct PairWalk;

template <> struct PairWalk<false>
{
    int u, v, np; // next lane group starts at pair (u, u + v)
    template <class NB>
    __device__ PairWalk( const NB &, int np_, int, int ) : u( 0 ), v( 1 ), np( np_ )
    {
    }
    __device__ __forceinline__ bool active() const { return v < np; }
    // next start: the pair after (u_last, v_last) in diagonal order
    __device__ __forceinline__ void set_after( int u_last, int v_last )
    {
        u = u_last + 1;
        v = v_last;
        if ( u >= np - v )
        {
            u = 0;
            v++;
        }
    }
};

template <> struct PairWalk<true>
{
    int u, v, rowend, v1, vs;
    bool tri;
    template <class NB> __device__ PairWalk( const NB &S, int, int c1, int c2 )
    {
        if ( c1 == c2 )
        {
            u = S.es[c1];
            v = u + 1;
            rowend = S.es[c1 + 1] - 1;
            v1 = S.es[c1 + 1];
            vs = 0;
            tri = true;
        }
        else
        {
            u = S.es[c1];
            rowend = S.es[c1 + 1];
            vs = S.es[c2];
            v1 = S.es[c2 + 1];
            v = vs;
            tri = false;
            if ( vs == v1 ) // no e2 neighbours: nothing to walk
                u = rowend;
        }
    }
    __device__ __forceinline__ bool active() const { return u < rowend; }
    __device__ __forceinline__ bool valid( int a, int c ) const { return a < rowend && c < v1; }
    __device__ __forceinline__ void adv( int &a, int &c, int k ) const
    {
        c += k;
        while ( c >= v1 && a < rowend - 1 )
        {
            c = c - v1 + ( tri ? a + 2 : vs );
            a++;
        }
    }
    __device__ __forceinline__ void set( int a, int c )
    {
        u = a;
        v = c;
        if ( !( c < v1 ) )
            u = rowend;
    }
    template <class NB> __device__ __forceinline__ void pair( const NB &S, int a, int c, int &j,
                                                              int &k ) const
    {
        j = S.perm[a];
        k = S.perm[c];
    }
};

// Append the channel's next pairs with r_jk^2 < rc^2 to S.tb (as slot
// pairs) until the buffer could not take another 32 or the pairs run out;
// returns the count and moves the cursor.
template <bool ME, int CAP>
__device__ __forceinline__ int fill_triplets( NbrF<ME, CAP> &S, PairWalk<ME> &w, float rc2 )
{
    using NB = NbrF<ME, CAP>;
    const int lane = threadIdx.x & 31;
    const unsigned lt = ( 1u << lane ) - 1u;
    int cnt = 0;
    if constexpr ( !ME )
    {
        // 32 consecutive pairs of the diagonal order per step, across
        // diagonal ends (lane l takes the l-th pair from the cursor), so the
        // short diagonals do not leave lanes idle
        while ( w.active() && cnt <= NNP_TB - 32 )
        {
            int u = w.u + lane, v = w.v;
            while ( v < w.np && u >= w.np - v )
            {
                u -= w.np - v;
                v++;
            }
            const int a = u, c = u + v;
            bool in = false;
            if ( v < w.np )
            {
                const float4 ga = S.g[a], gc = S.g[c];
                const float jx = gc.x - ga.x, jy = gc.y - ga.y, jz = gc.z - ga.z;
                in = jx * jx + jy * jy + jz * jz < rc2;
            }
            const unsigned m = __ballot_sync( 0xffffffffu, in );
            if ( in )
                S.tb[cnt + __popc( m & lt )] =
                    ( typename NB::TbT )( (unsigned)a | ( (unsigned)c << NB::TB_SHIFT ) );
            cnt += __popc( m );
            // the cursor moves past lane 31's pair
            w.set_after( __shfl_sync( 0xffffffffu, u, 31 ), __shfl_sync( 0xffffffffu, v, 31 ) );
        }
        __syncwarp();
        return cnt;
    }
    else
    {
    while ( w.active() && cnt <= NNP_TB - 32 )
    {
        int u = w.u, v = w.v;
        w.adv( u, v, lane );
        bool in = false;
        int a = 0, c = 0;
        if ( w.valid( u, v ) )
        {
            w.pair( S, u, v, a, c );
            const float4 ga = S.g[a], gc = S.g[c];
            const float jx = gc.x - ga.x, jy = gc.y - ga.y, jz = gc.z - ga.z;
            in = jx * jx + jy * jy + jz * jz < rc2;
        }
        const unsigned m = __ballot_sync( 0xffffffffu, in );
        if ( in )
            S.tb[cnt + __popc( m & lt )] =
                ( typename NB::TbT )( (unsigned)a | ( (unsigned)c << NB::TB_SHIFT ) );
        cnt += __popc( m );
        w.adv( u, v, 1 );
        w.set( __shfl_sync( 0xffffffffu, u, 31 ), __shfl_sync( 0xffffffffu, v, 31 ) );
    }
    __syncwarp();
    return cnt;
    }
}

// ---------------------------------------------------------------------------
// Symmetry functions.  The G values feed (G - Gmin) / (Gmax - Gmin): for a
// function that hardly varies over the fitted states the scaling multiplies
// any error of G by G / (Gmax - Gmin), often 10^2 - 10^3.  So the scaled
// input is formed in FP64 from the warp's sum (with `scaled` set the kernel
// writes smin + (G - Gmin) Gscale rather than G, so no FP32 rounding of G
// itself reaches the network).  Each lane sums one buffer of triplets
// (<= 16) in FP32 and merges it into its running sum (optionally Kahan-
// compensated: GBMD_NNP_KAHAN; measured, it does not change the force error,
// which FP32 geometry sets, and costs registers).
__device__ __forceinline__ void kahan_merge( float2 &s, float2 &c, float2 v )
{
#if GBMD_NNP_KAHAN
    const float2 y = make_float2( v.x - c.x, v.y - c.y );
    const float2 t = make_float2( s.x + y.x, s.y + y.y );
    c = make_float2( ( t.x - s.x ) - y.x, ( t.y - s.y ) - y.y );
    s = t;
#else
    s = __fadd2_rn( s, v );
#endif
}

// The kernel bodies take their block index explicitly: the single-system
// kernels run them with blockIdx.x, the serving job-table kernels with the
// block's index inside its job, on that job's arrays.  (The symmetry-function
// body takes it unsigned and the force body signed: measured at 256k atoms,
// each form is the faster one for its kernel, 3.32 against 3.67 ms and 3.81
// against 3.85 ms.)
template <int NRM, int ZM, int NE, bool ME, int CAP>
__device__ __forceinline__ void
    nnp_sf_body( const float4 *__restrict__ xr, const uint32_t *__restrict__ nlist,
                 const int *__restrict__ nnum, size_t stride, int n, const GbmdGeom &g,
                 const NnpParams *__restrict__ Pg, float *__restrict__ Gout, int scaled,
                 int *__restrict__ flags, const ElemAtoms &ea, int gstride,
                 const NnpTriCache &tc, const unsigned bid )
{
    using NB = NbrF<ME, CAP>;
    constexpr int NZ = popc_c( ZM ), MTOP = top_bit( ZM );
    __shared__ NnpF32Const<ME> K;
    load_f32_const<ME>( Pg, K );
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = f32_atom<ME>( ea, bid * NNP_F32_WARPS + warp, n );
    if ( i < 0 )
        return;
    NB &S = *reinterpret_cast<NB *>( reinterpret_cast<char *>( nnp_dyn_smem ) +
                                     warp * nbr_stride<ME, CAP, false>() );
    const int np =
        gather_f<ME, CAP, false>( xr, nlist, stride, i, nnum[i], g, K, S, flags, ea.type );
    group_by_element<ME, CAP>( S, np, K.nelem );
    float accr[NRM];
    float2 sum[NE][NZ], cmp[NE][NZ]; // (lambda = -1, lambda = +1)
#pragma unroll
    for ( int s = 0; s < NRM; s++ )
        accr[s] = 0.f;
    for ( int a = lane; a < np; a += 32 )
    {
        const float r = S.g[a].w, fc = S.h[a].y;
        const int el = ME ? S.el[a] : 0;
#pragma unroll
        for ( int s = 0; s < NRM; s++ )
            if ( s < K.nrad && ( !ME || el == K.rad_e1[s] ) )
            {
                const float dr = r - K.rs_r[s];
                accr[s] += expf( -K.eta_r[s] * dr * dr ) * fc;
            }
    }
    const float rc2 = K.rc * K.rc;
    const int nrad = K.nrad;
    int ntot = 0; // triplets so far (the cache holds them when they fit)
    // one pass per channel (one for a one-element potential); the radial
    // sums are stored with the first
    const int nch = ME ? K.nch : 1; // a compile-time 1 for one element
    for ( int ch = 0; ch < nch; ch++ )
    {
#pragma unroll
        for ( int e = 0; e < NE; e++ )
#pragma unroll
            for ( int z = 0; z < NZ; z++ )
            {
                sum[e][z] = f2( 0.f, 0.f );
                cmp[e][z] = f2( 0.f, 0.f );
            }
        const int c1 = ME ? K.ch_e1[ch] : 0, c2 = ME ? K.ch_e2[ch] : 0;
        // per-triplet constants in registers
        float eta[NE];
#pragma unroll
        for ( int e = 0; e < NE; e++ )
            eta[e] = -K.eta_u[e];
        const float hpirc = K.hpirc;
        PairWalk<ME> w( S, np, c1, c2 );
        while ( w.active() )
        {
            const int cnt = fill_triplets<ME, CAP>( S, w, rc2 );
            if ( !ME && CAP <= 256 && tc.t && ntot + cnt <= NNP_TCAP )
            {
                uint16_t *dst = tc.t + (size_t)i * NNP_TCAP + ntot;
                for ( int t = lane; t < cnt; t += 32 )
                    dst[t] = (uint16_t)S.tb[t];
            }
            ntot += cnt;
            float2 acc[NE][NZ];
#pragma unroll
            for ( int e = 0; e < NE; e++ )
#pragma unroll
                for ( int z = 0; z < NZ; z++ )
                    acc[e][z] = f2( 0.f, 0.f );
            for ( int t = lane; t < cnt; t += 32 )
            {
                const unsigned pk = S.tb[t];
                const int a = (int)( pk & NB::TB_MASK ), c = (int)( pk >> NB::TB_SHIFT );
                const float4 ga = S.g[a], gc = S.g[c];
                const float4 ha = S.h[a], hc = S.h[c];
                const float jx = gc.x - ga.x, jy = gc.y - ga.y, jz = gc.z - ga.z;
                const float rjk2 = jx * jx + jy * jy + jz * jz;
                const float rjk = rjk2 * rsqrtf( rjk2 ); // r_jk > 0: distinct neighbours
                const float cs = ( ga.x * gc.x + ga.y * gc.y + ga.z * gc.z ) * ( ha.x * hc.x );
                const float R2 = ga.w * ga.w + gc.w * gc.w + rjk2;
                const float F = ha.y * hc.y * fc_f32( rjk, hpirc );
                float2 pw[MTOP + 1];
                pw[0] = f2( 1.0f - cs, 1.0f + cs );
#pragma unroll
                for ( int m = 1; m <= MTOP; m++ )
                    pw[m] = __fmul2_rn( pw[m - 1], pw[m - 1] );
#pragma unroll
                for ( int e = 0; e < NE; e++ )
                {
                    const float2 ex = f2s( tri_exp( eta[e] * R2 ) * F );
                    int z = 0;
#pragma unroll
                    for ( int m = 0; m <= MTOP; m++ )
                        if ( ( ZM >> m ) & 1 )
                        {
                            acc[e][z] = __ffma2_rn( ex, pw[m], acc[e][z] );
                            z++;
                        }
                }
            }
#pragma unroll
            for ( int e = 0; e < NE; e++ )
#pragma unroll
                for ( int z = 0; z < NZ; z++ )
                    kahan_merge( sum[e][z], cmp[e][z], acc[e][z] );
            __syncwarp();
        }
        // warp sums, stored in n2p2 order (scaled or raw).  The accumulators
        // are laid out as [radial | angular (eta, lambda, m)] and reduced 32
        // at a time by a transpose reduction (lane k ends with the sum of
        // slot k: 31 shuffles per group instead of 5 per value); each lane
        // then forms its value's scaled input in FP64.
        constexpr int NACC = NRM + NE * 2 * NZ;
        constexpr int NGRP = ( NACC + 31 ) / 32;
#pragma unroll
        for ( int grp = 0; grp < NGRP; grp++ )
        {
            float v[32];
#pragma unroll
            for ( int k = 0; k < 32; k++ )
            {
                const int slot = grp * 32 + k;
                float x = 0.f;
                if ( slot < NRM )
                    x = accr[slot < NRM ? slot : 0];
                else if ( slot < NACC )
                {
                    const int t = slot - NRM;
                    const int e = t / ( 2 * NZ ), q = ( t / NZ ) % 2, z = t % NZ;
                    x = q ? sum[e][z].y - cmp[e][z].y : sum[e][z].x - cmp[e][z].x;
                }
                v[k] = x;
            }
#pragma unroll
            for ( int h = 16; h >= 1; h >>= 1 )
            {
                const bool up = ( lane & h ) != 0;
#pragma unroll
                for ( int k = 0; k < h; k++ )
                {
                    const float send = up ? v[k] : v[k + h];
                    const float keep = up ? v[k + h] : v[k];
                    v[k] = keep + __shfl_xor_sync( 0xffffffffu, send, h );
                }
            }
            // lane k holds slot grp * 32 + k
            const int slot = grp * 32 + lane;
            int out = -1;
            double val = (double)v[0];
            if ( slot < NRM )
                out = slot < nrad && ( !ME || ch == 0 ) ? slot : -1;
            else if ( slot < NACC )
            {
                const int t = slot - NRM;
                const int e = t / ( 2 * NZ ), q = ( t / NZ ) % 2, z = t % NZ;
                int m = 0, seen = 0;
                for ( int mm = 0; mm <= MTOP; mm++ ) // the z-th set bit of ZM
                    if ( ( ZM >> mm ) & 1 )
                    {
                        if ( seen == z )
                            m = mm;
                        seen++;
                    }
                const int sf = K.lad_sf[ME ? ch : 0][e][q][m];
                out = sf >= 0 ? nrad + sf : -1;
                val *= (double)ladder_pre( m );
            }
            if ( out >= 0 )
                Gout[(size_t)i * gstride + out] =
                    scaled ? (float)( Pg->smin + ( val - Pg->gmin[out] ) * Pg->gscale[out] )
                           : (float)val;
        }
    }
    if ( !ME && CAP <= 256 && tc.t && lane == 0 )
        tc.cnt[i] = ntot;
}

template <int NRM, int ZM, int NE, bool ME, int CAP>
__global__ void NNP_SF_BOUNDS( CAP )
    k_nnp_sf_f32( const float4 *__restrict__ xr, const uint32_t *__restrict__ nlist,
                  const int *__restrict__ nnum, size_t stride, int n, GbmdGeom g,
                  const NnpParams *__restrict__ Pg, float *__restrict__ Gout, int scaled,
                  int *__restrict__ flags, ElemAtoms ea, int gstride, NnpTriCache tc )
{
    nnp_sf_body<NRM, ZM, NE, ME, CAP>( xr, nlist, nnum, stride, n, g, Pg, Gout, scaled, flags,
                                       ea, gstride, tc, blockIdx.x );
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ void fq_add( unsigned long long *p, float v )
{
    atomicAdd( p, (unsigned long long)__float2ll_rn( v * FQ_SCALE ) );
}

template <int NRM, int ZM, int NE, bool ME, int CAP>
__device__ __forceinline__ void
    nnp_force_body( const float4 *__restrict__ xr, const uint32_t *__restrict__ nlist,
                    const int *__restrict__ nnum, size_t stride, int n, const GbmdGeom &g,
                    const NnpParams *__restrict__ Pg, const float *__restrict__ dEdG,
                    unsigned long long *__restrict__ fq, int *__restrict__ flags,
                    const ElemAtoms &ea, int gstride, const NnpTriCache &tc, const int bid )
{
    using NB = NbrF<ME, CAP>;
    constexpr int NZ = popc_c( ZM ), MTOP = top_bit( ZM );
    __shared__ NnpF32Const<ME> K;
    load_f32_const<ME>( Pg, K );
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = f32_atom<ME>( ea, bid * NNP_F32_WARPS + warp, n );
    if ( i < 0 )
        return;
    NB &S = *reinterpret_cast<NB *>( reinterpret_cast<char *>( nnp_dyn_smem ) +
                                     warp * nbr_stride<ME, CAP, true>() );
    const int np =
        gather_f<ME, CAP, true>( xr, nlist, stride, i, nnum[i], g, K, S, flags, ea.type );
    group_by_element<ME, CAP>( S, np, K.nelem );
    const int nrad = K.nrad;
    // dE/dG weights; the angular ones (per channel, below) carry the
    // 2^(1 - zeta) prefactor, as (lambda = -1, lambda = +1) pairs
    float wr[NRM];
    float2 wg[NE][NZ];
#pragma unroll
    for ( int s = 0; s < NRM; s++ )
        wr[s] = s < nrad ? dEdG[(size_t)i * gstride + s] : 0.f;
    // angular weights of channel ch (loaded here for one element, as the
    // loads then overlap the radial loop; per channel below otherwise)
    auto load_wg = [&]( int ch ) {
#pragma unroll
        for ( int e = 0; e < NE; e++ )
        {
            int z = 0;
#pragma unroll
            for ( int m = 0; m <= MTOP; m++ )
                if ( ( ZM >> m ) & 1 )
                {
                    float w2[2];
#pragma unroll
                    for ( int q = 0; q < 2; q++ )
                    {
                        const int sf = K.lad_sf[ME ? ch : 0][e][q][m];
                        w2[q] = sf >= 0 ? dEdG[(size_t)i * gstride + nrad + sf] * ladder_pre( m )
                                        : 0.f;
                    }
                    wg[e][z] = f2( w2[0], w2[1] );
                    z++;
                }
        }
    };
    if ( !ME )
        load_wg( 0 );
    float fix = 0.f, fiy = 0.f, fiz = 0.f;
    // radial: lanes over neighbours (each lane owns its neighbours' slots)
    for ( int a = lane; a < np; a += 32 )
    {
        const float4 ga = S.g[a], ha = S.h[a];
        const float r = ga.w, fc = ha.y, dfc = ha.z;
        const int el = ME ? S.el[a] : 0;
        float coef = 0.f;
#pragma unroll
        for ( int s = 0; s < NRM; s++ )
            if ( s < nrad && ( !ME || el == K.rad_e1[s] ) )
            {
                const float eta = K.eta_r[s];
                const float dr = r - K.rs_r[s];
                coef += wr[s] * expf( -eta * dr * dr ) * ( -2.0f * eta * dr * fc + dfc );
            }
        const float ri = ha.x;
        const float gx = coef * ga.x * ri, gy = coef * ga.y * ri, gz = coef * ga.z * ri;
        float4 fa = S.f[a];
        fa.x -= gx;
        fa.y -= gy;
        fa.z -= gz;
        S.f[a] = fa;
        fix += gx;
        fiy += gy;
        fiz += gz;
    }
    __syncwarp();
    const float rc2 = K.rc * K.rc;
    const unsigned lt = ( 1u << lane ) - 1u;
    // ladder derivative factors lambda 2^m as (lambda = -1, lambda = +1)
    float2 lz[MTOP + 1];
#pragma unroll
    for ( int m = 0; m <= MTOP; m++ )
        lz[m] = f2( -(float)( 1 << m ), (float)( 1 << m ) );
    // per-triplet constants in registers
    float eta[NE];
#pragma unroll
    for ( int e = 0; e < NE; e++ )
        eta[e] = K.eta_u[e];
    const float hpirc = K.hpirc;
    // One batch of up to 32 triplets (slot pairs from get(t), t < cnt):
    // gradients, then their sums on the two neighbours.
    auto batch = [&]( int t0, int cnt, auto get ) {
        const int t = t0 + lane;
        const bool valid = t < cnt;
        int a = 0x7fffffff, c = 0;
        float gjx = 0.f, gjy = 0.f, gjz = 0.f, gkx = 0.f, gky = 0.f, gkz = 0.f;
        if ( valid )
        {
            const unsigned pk = get( t );
            a = (int)( pk & NB::TB_MASK );
            c = (int)( pk >> NB::TB_SHIFT );
            const float4 ga = S.g[a], gc = S.g[c];
            const float4 ha = S.h[a], hc = S.h[c];
            const float ia = ha.x, ib = hc.x;
            const float fa = ha.y, fb = hc.y, dfa = ha.z, dfb = hc.z;
            const float jx = gc.x - ga.x, jy = gc.y - ga.y, jz = gc.z - ga.z;
            const float rjk2 = jx * jx + jy * jy + jz * jz;
            const float irjk = rsqrtf( rjk2 );
            const float rjk = rjk2 * irjk;
            const float inv = ia * ib;
            const float cs = ( ga.x * gc.x + ga.y * gc.y + ga.z * gc.z ) * inv;
            const float R2 = ga.w * ga.w + gc.w * gc.w + rjk2;
            float fjk, dfjk;
            fc_dfc_f32( rjk, hpirc, fjk, dfjk );
            const float pa = fb * fjk, pb = fa * fjk;
            const float F = fa * pa;
            // ladder: pw = b^(2^m), qd = lambda 2^m b^(2^m - 1), both lambda
            // signs at once
            float2 pw[MTOP + 1], qd[MTOP + 1];
            {
                float2 bq = f2( 1.0f - cs, 1.0f + cs );
                float2 pr = f2( 1.0f, 1.0f ); // b^(2^m - 1)
#pragma unroll
                for ( int m = 0; m <= MTOP; m++ )
                {
                    pw[m] = bq;
                    qd[m] = __fmul2_rn( lz[m], pr );
                    if ( m < MTOP )
                    {
                        pr = __fmul2_rn( pr, bq );
                        bq = __fmul2_rn( bq, bq );
                    }
                }
            }
            // dE/dcos (Cc), dE/dR^2 (CR) and dE/dF (CF) of the triplet
            float Cc = 0.f, CR = 0.f, CF = 0.f;
#pragma unroll
            for ( int e = 0; e < NE; e++ )
            {
                const float ex = tri_exp( -eta[e] * R2 );
                float2 sp = f2( 0.f, 0.f ), sd = f2( 0.f, 0.f );
                int z = 0;
#pragma unroll
                for ( int m = 0; m <= MTOP; m++ )
                    if ( ( ZM >> m ) & 1 )
                    {
                        sp = __ffma2_rn( wg[e][z], pw[m], sp );
                        sd = __ffma2_rn( wg[e][z], qd[m], sd );
                        z++;
                    }
                const float spe = ex * ( sp.x + sp.y );
                Cc += ex * ( sd.x + sd.y );
                CF += spe;
                CR -= eta[e] * spe;
            }
            Cc *= F;
            CR *= F;
            // g_j = A_j d_j + U d_k, g_k = U d_j + B_k d_k, from
            // dcos/dd_j = d_k/(r_j r_k) - cos d_j/r_j^2,
            // dR2/dd_j = 2 d_j - 2 (d_k - d_j), dF/dd_j through fc(r_j) and
            // fc(r_jk) (and j <-> k)
            const float dFa = dfa * pa * ia, dFb = dfb * pb * ib;
            const float dFjk = fa * fb * dfjk * irjk;
            const float CR2 = 2.0f * CR;
            const float D = CR2 + CF * dFjk;
            const float Ccs = Cc * cs;
            const float U = Cc * inv - D;
            const float Aj = CR2 + D + CF * dFa - Ccs * ia * ia;
            const float Bk = CR2 + D + CF * dFb - Ccs * ib * ib;
            gjx = Aj * ga.x + U * gc.x;
            gjy = Aj * ga.y + U * gc.y;
            gjz = Aj * ga.z + U * gc.z;
            gkx = U * ga.x + Bk * gc.x;
            gky = U * ga.y + Bk * gc.y;
            gkz = U * ga.z + Bk * gc.z;
            fix += gjx + gkx;
            fiy += gjy + gky;
            fiz += gjz + gkz;
        }
        if constexpr ( !ME )
        {
            // diagonal order: a run of lanes on one diagonal has distinct
            // first slots and distinct second slots; one run at a time,
            // first slots then second slots (in lane order: deterministic)
            const int d = valid ? c - a : -1;
            const int dp = __shfl_up_sync( 0xffffffffu, d, 1 );
            const bool head = valid && ( lane == 0 || dp != d );
            const unsigned heads = __ballot_sync( 0xffffffffu, head );
            const int seg = __popc( heads & ( lt | ( 1u << lane ) ) ) - 1;
            const int nseg = __popc( heads );
            for ( int r = 0; r < nseg; r++ )
            {
                const bool mine = valid && seg == r;
                if ( mine )
                {
                    float4 fa4 = S.f[a];
                    fa4.x -= gjx;
                    fa4.y -= gjy;
                    fa4.z -= gjz;
                    S.f[a] = fa4;
                }
                __syncwarp();
                if ( mine )
                {
                    float4 fc4 = S.f[c];
                    fc4.x -= gkx;
                    fc4.y -= gky;
                    fc4.z -= gkz;
                    S.f[c] = fc4;
                }
                __syncwarp();
            }
        }
        else
        {
        // row order: gradient on the first neighbour summed over the lanes
        // holding the same a (contiguous) with a segmented shuffle reduction
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            const float ox = __shfl_down_sync( 0xffffffffu, gjx, o );
            const float oy = __shfl_down_sync( 0xffffffffu, gjy, o );
            const float oz = __shfl_down_sync( 0xffffffffu, gjz, o );
            const int ok = __shfl_down_sync( 0xffffffffu, a, o );
            if ( lane + o < 32 && ok == a )
            {
                gjx += ox;
                gjy += oy;
                gjz += oz;
            }
        }
        const int ap = __shfl_up_sync( 0xffffffffu, a, 1 );
        const bool head = valid && ( lane == 0 || ap != a );
        const unsigned heads = __ballot_sync( 0xffffffffu, head );
        if ( head )
        {
            float4 fa4 = S.f[a];
            fa4.x -= gjx;
            fa4.y -= gjy;
            fa4.z -= gjz;
            S.f[a] = fa4;
        }
        __syncwarp();
        // gradient on the second neighbour: distinct within a row, so one
        // row segment at a time (in lane order: deterministic)
        const int seg = __popc( heads & ( lt | ( 1u << lane ) ) ) - 1;
        const int nseg = __popc( heads );
        for ( int r = 0; r < nseg; r++ )
        {
            if ( valid && seg == r )
            {
                float4 fc4 = S.f[c];
                fc4.x -= gkx;
                fc4.y -= gky;
                fc4.z -= gkz;
                S.f[c] = fc4;
            }
            __syncwarp();
        }
        }
    };
    const int cached = ( !ME && CAP <= 256 && tc.t ) ? tc.cnt[i] : NNP_TCAP + 1;
    if ( cached <= NNP_TCAP )
    {
        // the triplets the symmetry-function kernel compacted for this atom
        // (each batch's slot pairs are loaded one batch ahead)
        const uint16_t *src = tc.t + (size_t)i * NNP_TCAP;
        unsigned cur = lane < cached ? (unsigned)__ldcs( src + lane ) : 0u;
        for ( int t0 = 0; t0 < cached; t0 += 32 ) // warp-uniform: shuffles inside
        {
            const int tn = t0 + 32 + lane;
            const unsigned nxt = tn < cached ? (unsigned)__ldcs( src + tn ) : 0u;
            batch( t0, cached, [&]( int ) { return cur; } );
            cur = nxt;
        }
    }
    else
    {
        // one pass per channel (one for a one-element potential)
        const int nch = ME ? K.nch : 1; // a compile-time 1 for one element
        for ( int ch = 0; ch < nch; ch++ )
        {
            const int c1 = ME ? K.ch_e1[ch] : 0, c2 = ME ? K.ch_e2[ch] : 0;
            if ( ME )
                load_wg( ch );
            PairWalk<ME> w( S, np, c1, c2 );
            while ( w.active() )
            {
                const int cnt = fill_triplets<ME, CAP>( S, w, rc2 );
                for ( int t0 = 0; t0 < cnt; t0 += 32 ) // warp-uniform: shuffles inside
                    batch( t0, cnt, [&]( int t ) { return (unsigned)S.tb[t]; } );
            }
        }
    }
    // owners: fixed-point sums (order-independent)
    for ( int a = lane; a < np; a += 32 )
    {
        const int j = __float_as_int( S.h[a].w );
        const float4 fa = S.f[a];
        fq_add( &fq[j], fa.x );
        fq_add( &fq[n + j], fa.y );
        fq_add( &fq[2 * n + j], fa.z );
    }
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
    {
        fix += __shfl_xor_sync( 0xffffffffu, fix, o );
        fiy += __shfl_xor_sync( 0xffffffffu, fiy, o );
        fiz += __shfl_xor_sync( 0xffffffffu, fiz, o );
    }
    if ( lane == 0 )
    {
        fq_add( &fq[i], fix );
        fq_add( &fq[n + i], fiy );
        fq_add( &fq[2 * n + i], fiz );
    }
}

template <int NRM, int ZM, int NE, bool ME, int CAP>
__global__ void NNP_F32_BOUNDS( CAP )
    k_nnp_force_f32( const float4 *__restrict__ xr, const uint32_t *__restrict__ nlist,
                     const int *__restrict__ nnum, size_t stride, int n, GbmdGeom g,
                     const NnpParams *__restrict__ Pg, const float *__restrict__ dEdG,
                     unsigned long long *__restrict__ fq, int *__restrict__ flags, ElemAtoms ea,
                     int gstride, NnpTriCache tc )
{
    nnp_force_body<NRM, ZM, NE, ME, CAP>( xr, nlist, nnum, stride, n, g, Pg, dEdG, fq, flags,
                                          ea, gstride, tc, (int)blockIdx.x );
}

// f += conv * fq * 2^-32 (conv = cflength / cfenergy)
__device__ __forceinline__ void fq_add_one( const unsigned long long *__restrict__ fq, int k,
                                            double conv, double *__restrict__ f )
{
    f[k] += conv * ( (double)(long long)fq[k] * FQ_INV );
}

__global__ void k_fq_add( const unsigned long long *__restrict__ fq, int count, double conv,
                          double *__restrict__ f )
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if ( k < count )
        fq_add_one( fq, k, conv, f );
}

// ---------------------------------------------------------------------------
// Launches: one over all atoms (one element), or one per element group (the
// grid covers all atoms; work items past the group's count return at once).
// The neighbour capacity follows the list: the largest list count of the
// last build bounds every atom's count inside rc until the next rebuild.
static bool use_large_capacity( const gbmd_ctx *c ) { return c->nl_maxc > NNP_CAP_SMALL; }

bool gbmd_nnp_f32_cacheable( const gbmd_ctx *c, int nelem )
{
    return nelem == 1 && !use_large_capacity( c );
}

// Dynamic shared memory above 48 KB needs the kernel attribute, set once
// per instantiation and device.
template <class Kern>
static int smem_ready( gbmd_ctx *c, Kern k, size_t bytes, std::atomic<unsigned> &ready )
{
    const unsigned bit = c->device < 32 ? 1u << c->device : 0u;
    if ( !( ready.load( std::memory_order_acquire ) & bit ) )
    {
        GBMD_CUDA( c, cudaFuncSetAttribute( k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)bytes ) );
        ready.fetch_or( bit, std::memory_order_release );
    }
    return GBMD_OK;
}

struct SfLaunch
{
    const NnpParams *Pd;
    float *G;
    int scaled;
    ElemAtoms ea;
    int gstride;
    NnpTriCache tc;
    template <int NRM, int ZM, int NE, bool ME, int CAP> int go( gbmd_ctx *c ) const
    {
        const int n = (int)c->n;
        const int blocks = ( n + NNP_F32_WARPS - 1 ) / NNP_F32_WARPS;
        constexpr size_t smem = nbr_smem_bytes<ME, CAP, false>();
        auto k = k_nnp_sf_f32<NRM, ZM, NE, ME, CAP>;
        static std::atomic<unsigned> ready{ 0 };
        if ( int rc = smem_ready( c, k, smem, ready ) )
            return rc;
        k<<<blocks, NNP_F32_WARPS * 32, smem, c->stream>>>( c->xr.p, c->nlist.p, c->nnum.p,
                                                             c->nl_stride, n, c->geom, Pd, G,
                                                             scaled, c->flags.p, ea, gstride,
                                                             tc );
        GBMD_LAUNCH_CHECK( c, "nnp sf (f32)" );
        return GBMD_OK;
    }
};

struct ForceLaunch
{
    const NnpParams *Pd;
    const float *dEdG;
    unsigned long long *fq;
    ElemAtoms ea;
    int gstride;
    NnpTriCache tc;
    template <int NRM, int ZM, int NE, bool ME, int CAP> int go( gbmd_ctx *c ) const
    {
        const int n = (int)c->n;
        const int blocks = ( n + NNP_F32_WARPS - 1 ) / NNP_F32_WARPS;
        constexpr size_t smem = nbr_smem_bytes<ME, CAP, true>();
        auto k = k_nnp_force_f32<NRM, ZM, NE, ME, CAP>;
        static std::atomic<unsigned> ready{ 0 };
        if ( int rc = smem_ready( c, k, smem, ready ) )
            return rc;
        k<<<blocks, NNP_F32_WARPS * 32, smem, c->stream>>>( c->xr.p, c->nlist.p, c->nnum.p,
                                                             c->nl_stride, n, c->geom, Pd, dEdG,
                                                             fq, c->flags.p, ea, gstride, tc );
        GBMD_LAUNCH_CHECK( c, "nnp force (f32)" );
        return GBMD_OK;
    }
};

// Compiled shapes: up to 8 or 16 radial functions; zeta ladder {1, 2, 4, 16}
// (the reference fixture and the workloads) or every power of two to 32;
// three distinct angular eta (the reference fixture and the workloads) or up
// to four; one element or several; the common or the large neighbour
// capacity.
template <int NRM, int ZM, int NE, class L>
static int dispatch_cap( gbmd_ctx *c, const L &l, bool me )
{
    const bool large = use_large_capacity( c );
    if ( me )
        return large ? l.template go<NRM, ZM, NE, true, NNP_CAP_LARGE>( c )
                     : l.template go<NRM, ZM, NE, true, NNP_CAP_SMALL>( c );
    return large ? l.template go<NRM, ZM, NE, false, NNP_CAP_LARGE>( c )
                 : l.template go<NRM, ZM, NE, false, NNP_CAP_SMALL>( c );
}

template <class L> static int dispatch( gbmd_ctx *c, const NnpParams &p, const L &l, bool me )
{
    const bool narrow = ( p.lad_mask & ~0x17 ) == 0, ne3 = p.neta == 3;
    if ( p.nrad <= 8 )
    {
        if ( narrow )
            return ne3 ? dispatch_cap<8, 0x17, 3>( c, l, me )
                       : dispatch_cap<8, 0x17, NNP_MAXETA>( c, l, me );
        return ne3 ? dispatch_cap<8, 0x3F, 3>( c, l, me )
                   : dispatch_cap<8, 0x3F, NNP_MAXETA>( c, l, me );
    }
    if ( narrow )
        return ne3 ? dispatch_cap<16, 0x17, 3>( c, l, me )
                   : dispatch_cap<16, 0x17, NNP_MAXETA>( c, l, me );
    return ne3 ? dispatch_cap<16, 0x3F, 3>( c, l, me )
               : dispatch_cap<16, 0x3F, NNP_MAXETA>( c, l, me );
}

bool gbmd_nnp_f32_supported( const NnpParams &p )
{
    return p.lad_ok && p.nrad <= 16 && p.neta >= 1 && p.neta <= NNP_MAXETA;
}

int gbmd_nnp_sf_f32_launch( gbmd_ctx *c, const NnpParams &p, const NnpParams *Pd, float *G,
                            int scaled, const ElemAtoms &ea, int gstride, const NnpTriCache &tc )
{
    return dispatch( c, p, SfLaunch{ Pd, G, scaled, ea, gstride, tc }, ea.atoms != nullptr );
}

int gbmd_nnp_force_f32_launch( gbmd_ctx *c, const NnpParams &p, const NnpParams *Pd,
                               const float *dEdG, unsigned long long *fq, const ElemAtoms &ea,
                               int gstride, const NnpTriCache &tc )
{
    return dispatch( c, p, ForceLaunch{ Pd, dEdG, fq, ea, gstride, tc }, ea.atoms != nullptr );
}

// ---------------------------------------------------------------------------
// Serving job tables (gbmd_nnp_step_batch): the common shape only (up to 8
// radial functions, zeta ladder {1, 2, 4, 16}, three angular eta, one
// element, 192 neighbours).  Each block runs the single-system body for the
// job whose block range holds it.
constexpr int JOB_NRM = 8, JOB_ZM = 0x17, JOB_NE = 3, JOB_CAP = NNP_CAP_SMALL;

__global__ void NNP_SF_BOUNDS( JOB_CAP ) k_nnp_sf_f32_jobs( const __grid_constant__ NnpJobTable t )
{
    const int j = nnp_job_of( t.b_sf, t.njobs, (int)blockIdx.x );
    const NnpJobArgs &J = t.job[j];
    nnp_sf_body<JOB_NRM, JOB_ZM, JOB_NE, false, JOB_CAP>(
        J.xr, J.nlist, J.nnum, J.stride, J.n, J.g, J.Pg, J.G, 1, J.flags, ElemAtoms(), J.gstride,
        J.tc, blockIdx.x - (unsigned)t.b_sf[j] );
}

__global__ void NNP_F32_BOUNDS( JOB_CAP )
    k_nnp_force_f32_jobs( const __grid_constant__ NnpJobTable t )
{
    const int j = nnp_job_of( t.b_sf, t.njobs, (int)blockIdx.x );
    const NnpJobArgs &J = t.job[j];
    nnp_force_body<JOB_NRM, JOB_ZM, JOB_NE, false, JOB_CAP>(
        J.xr, J.nlist, J.nnum, J.stride, J.n, J.g, J.Pg, J.dEdG, J.fq, J.flags, ElemAtoms(),
        J.gstride, J.tc, (int)blockIdx.x - t.b_sf[j] );
}

// f = 0 and fq = 0 (the single-system path's memsets), 256 components per block
__global__ void __launch_bounds__( 256 ) k_nnp_zero_jobs( const __grid_constant__ NnpJobTable t )
{
    const int j = nnp_job_of( t.b_fq, t.njobs, (int)blockIdx.x );
    const NnpJobArgs &J = t.job[j];
    const int k = ( (int)blockIdx.x - t.b_fq[j] ) * 256 + (int)threadIdx.x;
    if ( k < 3 * J.n )
    {
        J.f[k] = 0.0;
        J.fq[k] = 0ull;
    }
}

__global__ void __launch_bounds__( 256 ) k_fq_add_jobs( const __grid_constant__ NnpJobTable t )
{
    const int j = nnp_job_of( t.b_fq, t.njobs, (int)blockIdx.x );
    const NnpJobArgs &J = t.job[j];
    const int k = ( (int)blockIdx.x - t.b_fq[j] ) * 256 + (int)threadIdx.x;
    if ( k < 3 * J.n )
        fq_add_one( J.fq, k, J.conv, J.f );
}

static int job_smem_ready( int device )
{
    static std::atomic<unsigned> ready{ 0 };
    const unsigned bit = device < 32 ? 1u << device : 0u;
    if ( ready.load( std::memory_order_acquire ) & bit )
        return GBMD_OK;
    if ( cudaFuncSetAttribute( k_nnp_sf_f32_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbr_smem_bytes<false, JOB_CAP, false>() ) != cudaSuccess ||
         cudaFuncSetAttribute( k_nnp_force_f32_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)nbr_smem_bytes<false, JOB_CAP, true>() ) != cudaSuccess )
        return GBMD_ERR_CUDA;
    ready.fetch_or( bit, std::memory_order_release );
    return GBMD_OK;
}

int gbmd_nnp_sf_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st )
{
    if ( job_smem_ready( device ) )
        return GBMD_ERR_CUDA;
    k_nnp_sf_f32_jobs<<<t.b_sf[t.njobs], NNP_F32_WARPS * 32,
                        nbr_smem_bytes<false, JOB_CAP, false>(),
                        st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

int gbmd_nnp_force_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st )
{
    if ( job_smem_ready( device ) )
        return GBMD_ERR_CUDA;
    k_nnp_force_f32_jobs<<<t.b_sf[t.njobs], NNP_F32_WARPS * 32,
                           nbr_smem_bytes<false, JOB_CAP, true>(),
                           st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

int gbmd_nnp_zero_jobs_launch( const NnpJobTable &t, cudaStream_t st )
{
    k_nnp_zero_jobs<<<t.b_fq[t.njobs], 256, 0, st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

int gbmd_nnp_fq_jobs_launch( const NnpJobTable &t, cudaStream_t st )
{
    k_fq_add_jobs<<<t.b_fq[t.njobs], 256, 0, st>>>( t );
    return cudaGetLastError() == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

// The job-table kernels' shape, checked on the host.
bool gbmd_nnp_f32_job_shape( const NnpParams &p )
{
    return gbmd_nnp_f32_supported( p ) && p.nrad <= JOB_NRM && ( p.lad_mask & ~JOB_ZM ) == 0 &&
           p.neta == JOB_NE;
}

int gbmd_nnp_fq_begin( gbmd_ctx *c, unsigned long long *fq )
{
    GBMD_CUDA( c, cudaMemsetAsync( fq, 0, sizeof( unsigned long long ) * 3 * c->n, c->stream ) );
    return GBMD_OK;
}

int gbmd_nnp_fq_end( gbmd_ctx *c, const NnpParams &p, const unsigned long long *fq )
{
    const int count = (int)( 3 * c->n );
    k_fq_add<<<( count + 255 ) / 256, 256, 0, c->stream>>>( fq, count,
                                                            p.cflength / p.cfenergy, c->f.p );
    GBMD_LAUNCH_CHECK( c, "nnp force fixed-point add" );
    return GBMD_OK;
}
