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
// sit within the FP32 rounding band of the cutoff.  With a half list the
// partner's share of a pair goes out as one vector FP32 reduction
// (red.add.v4.f32 on a float4 per atom) instead of three FP64 atomics, and a
// fold kernel adds those sums into the FP64 forces: half the step time of
// the FP64-atomic version at 4M atoms.
//
// MODE_STEP fuses, for a full list, the force of step n with final_integrate
// of step n, the thermo sums of step n, and initial_integrate of step n+1:
// positions are double-buffered (neighbours read x / xr, the atom's own
// update goes to x_next / xr_next), so the per-step velocity and position
// traffic is paid once.  The update sequence is the reference's, so the FP64
// trajectory stays bit-identical.
#include <cstring>

#include "gbmd_internal.cuh"

#include <cmath>

// atoms per block of the serving job-table kernel; the single-system
// kernels take the block size of the context's tile shape (GBMD_LJ_TPB_*)
constexpr int LJ_THREADS = 128;
constexpr int LJ_BATCH = GBMD_ROW_PAD; // rows per batch == list row padding

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
    size_t lstride; // row stride of the transposed list
    int *flags;     // context flags ([3]: bounded wait timed out)
    // single-type constants (kept in registers by the ONE specialisation)
    float lj1_1, lj2_1, clo1, chi1, esh1;
    float4 *f4; // half lists, mixed: partners' forces (zero between launches)
    int pf;     // mixed: L2 prefetch distance of the list rows (0: none)
};

// The potential energy and sum m v^2 of a warp's 32 atoms go to per-warp
// partial slots (warp w holds atoms 32 w .. 32 w + 31 of the system), so the
// reduction tree, and with it every rounding, is the same whatever the
// block size (the tile shape the autotuner picks).  i is the lane's atom.
template <int MODE>
__device__ __forceinline__ void warp_partials( double pe, double mv2, int i, const LjArgs &a,
                                               double *__restrict__ partials )
{
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
    {
        pe += __shfl_xor_sync( 0xffffffffu, pe, o );
        mv2 += __shfl_xor_sync( 0xffffffffu, mv2, o );
    }
    if ( ( threadIdx.x & 31 ) == 0 && i < a.n )
    {
        partials[a.pstride + ( i >> 5 )] = pe;
        if ( MODE == MODE_STEP )
            partials[i >> 5] = mv2;
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
    // The FP64 path keeps the reference's separately rounded operations;
    // the mixed path lets them fuse (half the FP64-pipe instructions).
    auto madd = [&]( double acc, double m, double q ) {
        return MIXED ? fma( m, q, acc ) : dadd( acc, dmul( m, q ) );
    };
    vx = madd( vx, dtfm, fx );
    vy = madd( vy, dtfm, fy );
    vz = madd( vz, dtfm, fz );
    if ( EFLAG )
        mv2 = dmul( dadd( dadd( dmul( vx, vx ), dmul( vy, vy ) ), dmul( vz, vz ) ), s.mass[t] );
    if ( s.next )
    {
        vx = madd( vx, dtfm, fx );
        vy = madd( vy, dtfm, fy );
        vz = madd( vz, dtfm, fz );
        xi.x = madd( xi.x, s.dtv, vx );
        xi.y = madd( xi.y, s.dtv, vy );
        xi.z = madd( xi.z, s.dtv, vz );
        x_next[i] = xi;
        if ( MIXED )
        {
            const double ox = a.lo[0] + ( unpack_home( hp, 0 ) + 0.5 ) * a.h[0];
            const double oy = a.lo[1] + ( unpack_home( hp, 1 ) + 0.5 ) * a.h[1];
            const double oz = a.lo[2] + ( unpack_home( hp, 2 ) + 0.5 ) * a.h[2];
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
template <bool FORCE, bool EFLAG, bool HALF, int MODE, int TPB>
__global__ void __launch_bounds__( TPB )
    k_lj_fp64( const double4 *__restrict__ x, const int *__restrict__ home,
               const uint32_t *__restrict__ nlist, const int *__restrict__ nnum,
               const GbmdLJ *__restrict__ prm, LjArgs a, double *__restrict__ f,
               double *__restrict__ partials, StepArgs s, double *__restrict__ v,
               double4 *__restrict__ x_next )
{
    __shared__ double s_lj1[GBMD_MAXT * GBMD_MAXT], s_lj2[GBMD_MAXT * GBMD_MAXT],
        s_cut[GBMD_MAXT * GBMD_MAXT], s_esh[GBMD_MAXT * GBMD_MAXT];
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
            const uint32_t e = __ldg( &nlist[(size_t)k * a.lstride + i] );
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
        warp_partials<MODE>( pe, mv2, i, a, partials );
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

__device__ __forceinline__ float rcp_approx( float x )
{
    float r;
    asm( "rcp.approx.ftz.f32 %0, %1;" : "=f"( r ) : "f"( x ) );
    return r;
}

// Per-block tables: stencil shift (o * h) per 27-cell code and, per type
// pair, lj1, lj2, the cutoff band edges and the exact FP64 cutoff.
struct MixTables
{
    float4 sh[27];
    float lj1[GBMD_MAXT * GBMD_MAXT], lj2[GBMD_MAXT * GBMD_MAXT];
    float clo[GBMD_MAXT * GBMD_MAXT], chi[GBMD_MAXT * GBMD_MAXT];
    float esh[GBMD_MAXT * GBMD_MAXT];
    double cut64[GBMD_MAXT * GBMD_MAXT];
};

// Compensated accumulators: each batch of pairs is summed in plain FP32 and
// the batch total enters a Kahan sum (one compensation per batch).
struct MixAcc
{
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float ps = 0.f, pc = 0.f; // potential energy
};

// Rare path: the FP32 squared distance sits within the rounding band of the
// cutoff, so the FP64 path's exact test decides (the LJ force jumps at rc
// and a pair on the wrong side would cost a whole F(rc) of error).
__device__ __forceinline__ bool exact_inside( const double4 *__restrict__ x, int i, uint32_t e,
                                           const int *hc, const LjArgs &a, double cut64 )
{
    const int j = (int)( e & GBMD_JMASK );
    const int sc = (int)( e >> 27 );
    const double4 p = x[i], q = x[j];
    const int s0 = image_shift( hc[0], sc % 3 - 1, a.nc[0] );
    const int s1 = image_shift( hc[1], ( sc / 3 ) % 3 - 1, a.nc[1] );
    const int s2 = image_shift( hc[2], sc / 9 - 1, a.nc[2] );
    const double ex = dsub( p.x, img_coord( q.x, s0, a.L[0] ) );
    const double ey = dsub( p.y, img_coord( q.y, s1, a.L[1] ) );
    const double ez = dsub( p.z, img_coord( q.z, s2, a.L[2] ) );
    const double r64 = dadd( dadd( dmul( ex, ex ), dmul( ey, ey ) ), dmul( ez, ez ) );
    return r64 < cut64;
}

// One pair, mixed precision, branch-free except for the rare exact-band
// test.  Rows past an atom's own count hold the sentinel entry (atom n, far
// away), which falls outside every cutoff and contributes exactly zero.
// f_j -= d: one vector FP32 reduction (16-byte aligned float4) where three
// scalar atomics would go, so a pair costs one L2 transaction
__device__ __forceinline__ void red_sub_v4( float4 *p, float dx, float dy, float dz )
{
    asm volatile( "red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"( p ),
                  "f"( -dx ), "f"( -dy ), "f"( -dz ), "f"( 0.f )
                  : "memory" );
}

template <bool FORCE, bool EFLAG, bool HALF, bool ONE>
__device__ __forceinline__ void lj_pair_mixed( const float4 &xi, const float4 &xj, uint32_t e,
                                               const float4 &sh, int i, int ti, int hp,
                                               const double4 *__restrict__ x,
                                               const MixTables &T, const LjArgs &a, float &bx,
                                               float &by, float &bz, float &bp,
                                               float4 *__restrict__ f4 )
{
    const int sc = (int)( e >> 27 );
    const float dx = ( xi.x - xj.x ) - sh.x;
    const float dy = ( xi.y - xj.y ) - sh.y;
    const float dz = ( xi.z - xj.z ) - sh.z;
    const int tp = ONE ? 0 : ti * GBMD_MAXT + __float_as_int( xj.w );
    const float rsq = dx * dx + dy * dy + dz * dz;
    const float clo = ONE ? a.clo1 : T.clo[tp];
    const float chi = ONE ? a.chi1 : T.chi[tp];
    bool in = rsq < clo;
    if ( rsq >= clo && rsq < chi )
    {
        const int hc[3] = { unpack_home( hp, 0 ), unpack_home( hp, 1 ), unpack_home( hp, 2 ) };
        in = exact_inside( x, i, e, hc, a, T.cut64[tp] );
    }
    const float lj1 = ONE ? a.lj1_1 : T.lj1[tp];
    const float lj2 = ONE ? a.lj2_1 : T.lj2[tp];
    const float r2inv = rcp_approx( rsq );
    const float r6inv = r2inv * r2inv * r2inv;
    if ( FORCE )
    {
        float fpair = r6inv * ( lj1 * r6inv - lj2 ) * r2inv;
        fpair = in ? fpair : 0.f;
        bx += dx * fpair;
        by += dy * fpair;
        bz += dz * fpair;
        if ( HALF && in )
            red_sub_v4( &f4[e & GBMD_JMASK], dx * fpair, dy * fpair, dz * fpair );
    }
    if ( EFLAG )
    {
        float fac = 0.5f;
        if ( HALF )
        {
            const int g0 = image_shift( unpack_home( hp, 0 ), sc % 3 - 1, a.nc[0] );
            const int g1 = image_shift( unpack_home( hp, 1 ), ( sc / 3 ) % 3 - 1, a.nc[1] );
            const int g2 = image_shift( unpack_home( hp, 2 ), sc / 9 - 1, a.nc[2] );
            fac = ( g0 | g1 | g2 ) ? 0.5f : 1.0f;
        }
        const float eij = fac * ( r6inv * ( 0.5f * lj1 * r6inv - lj2 ) * ( 1.0f / 6.0f ) -
                                  ( ONE ? a.esh1 : T.esh[tp] ) );
        bp += in ? eij : 0.f;
    }
}

// Mixed-precision force kernel: one atom per thread.  Each warp walks its
// rows up to the warp's largest count (lists are padded with the sentinel
// entry to that length, so no lane tests its own count), in batches of
// LJ_BATCH rows: the batch's coalesced list loads, then its gathers, then
// the pair math.
// The body takes the block index explicitly: k_lj_mixed runs it for one
// system (bid = blockIdx.x), k_lj_mixed_jobs for the block's job in a batch
// of serving jobs.
template <bool FORCE, bool EFLAG, bool HALF, int MODE, bool ONE>
__device__ __forceinline__ void lj_mixed_body( const float4 *__restrict__ xr,
                                               const double4 *__restrict__ x,
                                               const int *__restrict__ home,
                                               const uint32_t *__restrict__ nlist,
                                               const int *__restrict__ nnum,
                                               const GbmdLJ *__restrict__ prm, const LjArgs &a,
                                               double *__restrict__ f,
                                               double *__restrict__ partials, const StepArgs &s,
                                               double *__restrict__ v,
                                               double4 *__restrict__ x_next,
                                               float4 *__restrict__ xr_next, const int bid )
{
    __shared__ MixTables T;
    for ( int k = threadIdx.x; k < GBMD_MAXT * GBMD_MAXT; k += blockDim.x )
    {
        const float cs = prm->cutsqf[k];
        T.lj1[k] = prm->lj1f[k];
        T.lj2[k] = prm->lj2f[k];
        T.clo[k] = cs * ( 1.0f - a.band );
        T.chi[k] = cs * ( 1.0f + a.band );
        T.esh[k] = prm->eshiftf[k];
        T.cut64[k] = prm->cutsq[k];
    }
    if ( threadIdx.x < 27 )
    {
        const int sc = (int)threadIdx.x; // signed: the offsets are -1, 0, 1
        T.sh[sc] = make_float4( (float)( sc % 3 - 1 ) * a.hf[0],
                                (float)( ( sc / 3 ) % 3 - 1 ) * a.hf[1],
                                (float)( sc / 9 - 1 ) * a.hf[2], 0.f );
    }
    __syncthreads();
    const int i = bid * blockDim.x + threadIdx.x;
    const bool live = i < a.n;
    const int cnt = live ? nnum[i] : 0;
    const int rows = __reduce_max_sync( 0xffffffffu, cnt );
    double pe = 0.0, mv2 = 0.0;
    const float4 xi = live ? xr[i] : make_float4( 0.f, 0.f, 0.f, 0.f );
    const int ti = __float_as_int( xi.w );
    const int hp = live ? home[i] : 0;
    MixAcc acc;
    // stencil shift of the lane's current list entry (cell 13: no shift)
    int sh_sc = 13;
    float4 sh = make_float4( 0.f, 0.f, 0.f, 0.f );
    const uint32_t *row = nlist + i;
    const size_t stride = a.lstride;
    // Software pipeline: the next batch's list entries (an HBM stream) are
    // in flight while this batch's gathers (L1/L2) and math run.
    uint32_t en[LJ_BATCH];
    if ( rows > 0 )
    {
#pragma unroll
        for ( int u = 0; u < LJ_BATCH; u++ )
        {
            en[u] = __ldcs( row ); // streamed once: evict-first
            row += stride;
        }
    }
    for ( int k = 0; k < rows; k += LJ_BATCH )
    {
        uint32_t e[LJ_BATCH];
        float4 xj[LJ_BATCH];
#pragma unroll
        for ( int u = 0; u < LJ_BATCH; u++ )
            e[u] = en[u];
        if ( k + LJ_BATCH < rows ) // warp-uniform
        {
#pragma unroll
            for ( int u = 0; u < LJ_BATCH; u++ )
            {
                en[u] = __ldcs( row ); // streamed once: evict-first
                row += stride;
            }
        }
        // L2 prefetch of the warp's 128-byte row segments a.pf rows ahead
        // (lanes 0..LJ_BATCH-1 one row each): the demand loads above then
        // hit L2 instead of HBM.  Rows past the warp's count are inside the
        // allocation (rows < capacity) or skipped.
        if ( a.pf > 0 && ( threadIdx.x & 31 ) < LJ_BATCH )
        {
            const int kp = k + a.pf + ( threadIdx.x & 31 );
            if ( kp < rows )
                asm volatile( "prefetch.global.L2 [%0];" ::"l"(
                    nlist + (size_t)kp * stride + ( i & ~31 ) ) );
        }
#pragma unroll
        for ( int u = 0; u < LJ_BATCH; u++ )
            xj[u] = __ldg( &xr[e[u] & GBMD_JMASK] );
        float bx = 0.f, by = 0.f, bz = 0.f, bp = 0.f;
#pragma unroll
        for ( int u = 0; u < LJ_BATCH; u++ )
        {
            // A row is sorted by stencil cell, so the shift changes every
            // few entries: reloaded only by the lanes whose cell changed
            // (shared-memory wavefronts count the active lanes' addresses).
            const int sc = (int)( e[u] >> 27 );
            if ( sc != sh_sc )
            {
                sh = T.sh[sc];
                sh_sc = sc;
            }
            lj_pair_mixed<FORCE, EFLAG, HALF, ONE>( xi, xj[u], e[u], sh, i, ti, hp, x, T, a,
                                                    bx, by, bz, bp, a.f4 );
        }
        if ( FORCE )
        {
            kahan_add( acc.sx, acc.cx, bx );
            kahan_add( acc.sy, acc.cy, by );
            kahan_add( acc.sz, acc.cz, bz );
        }
        if ( EFLAG )
            kahan_add( acc.ps, acc.pc, bp );
    }
    if ( live )
    {
        if ( EFLAG )
            pe = (double)acc.ps - (double)acc.pc;
        if ( FORCE )
        {
            // one FP32 -> FP64 conversion per component (the compensation
            // is applied in FP32)
            const double fx = (double)( acc.sx - acc.cx );
            const double fy = (double)( acc.sy - acc.cy );
            const double fz = (double)( acc.sz - acc.cz );
            if ( MODE == MODE_ACC ) // half lists too: partners go to a.f4
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
        warp_partials<MODE>( pe, mv2, i, a, partials );
}

// Register budget: 56 per thread at 64 and 128 atoms per block (9 blocks of
// 128 resident), 64 at 256; measured at 4M atoms the fused step takes 0.607
// ms per launch this way against 0.623 ms at the compiler's own 63 registers.
template <bool FORCE, bool EFLAG, bool HALF, int MODE, bool ONE, int TPB>
__global__ void __launch_bounds__( TPB, 65536 / ( 56 * TPB ) )
    k_lj_mixed( const float4 *__restrict__ xr, const double4 *__restrict__ x,
                const int *__restrict__ home, const uint32_t *__restrict__ nlist,
                const int *__restrict__ nnum, const GbmdLJ *__restrict__ prm, LjArgs a,
                double *__restrict__ f, double *__restrict__ partials, StepArgs s,
                double *__restrict__ v, double4 *__restrict__ x_next,
                float4 *__restrict__ xr_next )
{
    lj_mixed_body<FORCE, EFLAG, HALF, MODE, ONE>( xr, x, home, nlist, nnum, prm, a, f, partials,
                                                  s, v, x_next, xr_next, (int)blockIdx.x );
}

// ---------------------------------------------------------------------------
// Batched fused step over serving jobs: one launch covers every job of the
// batch; job j owns blocks [block0[j], block0[j+1]) and runs exactly the
// single-system kernel's arithmetic on its own arrays, so its result does
// not depend on the batch.  The job table travels in the launch parameters
// (no per-step upload).
struct LjJob
{
    const float4 *xr;
    const double4 *x;
    const int *home;
    const uint32_t *nlist;
    const int *nnum;
    const GbmdLJ *prm;
    double *f, *partials, *v;
    double4 *x_next;
    float4 *xr_next;
    LjArgs a;
    StepArgs s;
};
constexpr int LJ_JOBS_PER_LAUNCH = 48; // ~20 KB of launch parameters
struct LjJobTable
{
    int njobs;
    int block0[LJ_JOBS_PER_LAUNCH + 1];
    LjJob job[LJ_JOBS_PER_LAUNCH];
};

template <bool EFLAG>
__global__ void __launch_bounds__( LJ_THREADS ) k_lj_mixed_jobs( const __grid_constant__ LjJobTable t )
{
    int lo = 0, hi = t.njobs - 1; // the job whose block range holds blockIdx.x
    while ( lo < hi )
    {
        const int mid = ( lo + hi + 1 ) >> 1;
        if ( t.block0[mid] <= (int)blockIdx.x )
            lo = mid;
        else
            hi = mid - 1;
    }
    const LjJob &J = t.job[lo];
    lj_mixed_body<true, EFLAG, false, MODE_STEP, true>(
        J.xr, J.x, J.home, J.nlist, J.nnum, J.prm, J.a, J.f, J.partials, J.s, J.v, J.x_next,
        J.xr_next, (int)blockIdx.x - t.block0[lo] );
}

// ---------------------------------------------------------------------------
static LjArgs make_args( const gbmd_ctx *c, size_t stride )
{
    LjArgs a;
    std::memset( &a, 0, sizeof a ); // padding too: the bytes key md_run's graphs
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
    a.lstride = c->nl_stride;
    a.flags = c->flags.p;
    a.lj1_1 = c->lj.lj1f[0];
    a.lj2_1 = c->lj.lj2f[0];
    a.clo1 = c->lj.cutsqf[0] * ( 1.0f - a.band );
    a.chi1 = c->lj.cutsqf[0] * ( 1.0f + a.band );
    a.esh1 = c->lj.eshiftf[0];
    a.f4 = c->f4.p;
    a.pf = c->tune.lj_pf;
    return a;
}

// f += the partners' contributions gathered in f4, which is left zeroed.
__global__ void k_fold_f4( float4 *__restrict__ f4, int n, double *__restrict__ f )
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n )
        return;
    const float4 q = f4[i];
    f[i] += (double)q.x;
    f[n + i] += (double)q.y;
    f[2 * n + i] += (double)q.z;
    f4[i] = make_float4( 0.f, 0.f, 0.f, 0.f );
}

// The partner buffer of the mixed half-list kernel: n float4, zeroed when
// (re)allocated and by every fold.
static int reserve_f4( gbmd_ctx *c, int n )
{
    if ( c->f4.p && c->f4.cap >= (size_t)n )
        return GBMD_OK;
    gbmd_release( c, c->f4 );
    int rc = gbmd_reserve( c, c->f4, n, "half-list partner forces" );
    if ( rc )
        return rc;
    GBMD_CUDA( c, cudaMemsetAsync( c->f4.p, 0, sizeof( float4 ) * n, c->stream ) );
    return GBMD_OK;
}

StepArgs gbmd_step_args( const gbmd_ctx *c, bool next )
{
    StepArgs s;
    std::memset( &s, 0, sizeof s );
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

template <bool FORCE, bool EFLAG, bool HALF, int MODE, int TPB>
static void launch_tpb( gbmd_ctx *c, GbmdLJ *ljd, const LjArgs &a, const StepArgs &s )
{
    const int blocks = (int)( ( c->n + TPB - 1 ) / TPB );
    if ( c->precision == GBMD_PREC_FP64 )
        k_lj_fp64<FORCE, EFLAG, HALF, MODE, TPB><<<blocks, TPB, 0, c->stream>>>(
            c->x.p, c->home.p, c->nlist.p, c->nnum.p, ljd, a, c->f.p, c->partials.p, s,
            c->v.p, c->x_alt.p );
    else if ( c->ntypes == 1 )
        k_lj_mixed<FORCE, EFLAG, HALF, MODE, true, TPB><<<blocks, TPB, 0, c->stream>>>(
            c->xr.p, c->x.p, c->home.p, c->nlist.p, c->nnum.p, ljd, a, c->f.p,
            c->partials.p, s, c->v.p, c->x_alt.p, c->xr_alt.p );
    else
        k_lj_mixed<FORCE, EFLAG, HALF, MODE, false, TPB><<<blocks, TPB, 0, c->stream>>>(
            c->xr.p, c->x.p, c->home.p, c->nlist.p, c->nnum.p, ljd, a, c->f.p,
            c->partials.p, s, c->v.p, c->x_alt.p, c->xr_alt.p );
}

// The launch for the context's tile shape (atoms per block).
template <bool FORCE, bool EFLAG, bool HALF, int MODE>
static void launch_one( gbmd_ctx *c, GbmdLJ *ljd, const LjArgs &a, const StepArgs &s )
{
    switch ( c->tune.lj_tpb )
    {
    case GBMD_LJ_TPB_SMALL:
        launch_tpb<FORCE, EFLAG, HALF, MODE, GBMD_LJ_TPB_SMALL>( c, ljd, a, s );
        break;
    case GBMD_LJ_TPB_LARGE:
        launch_tpb<FORCE, EFLAG, HALF, MODE, GBMD_LJ_TPB_LARGE>( c, ljd, a, s );
        break;
    default:
        launch_tpb<FORCE, EFLAG, HALF, MODE, GBMD_LJ_TPB_DEFAULT>( c, ljd, a, s );
    }
}

// Per-warp partial sums of a system (warp_partials)
static int lj_warps( const gbmd_ctx *c ) { return (int)( ( c->n + 31 ) / 32 ); }

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
    const bool half = c->half != 0;
    const bool fold = half && c->precision == GBMD_PREC_MIXED;
    if ( fold && ( rc = reserve_f4( c, n ) ) )
        return rc;
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, false );
    if ( half && zero_first )
        GBMD_CUDA( c, cudaMemsetAsync( c->f.p, 0, sizeof( double ) * 3 * n, c->stream ) );
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_FORCE, &t0 );
    if ( half )
    {
        if ( eflag )
            launch_one<true, true, true, MODE_ACC>( c, ljd, a, s );
        else
            launch_one<true, false, true, MODE_ACC>( c, ljd, a, s );
    }
    else if ( zero_first )
    {
        if ( eflag )
            launch_one<true, true, false, MODE_SET>( c, ljd, a, s );
        else
            launch_one<true, false, false, MODE_SET>( c, ljd, a, s );
    }
    else
    {
        if ( eflag )
            launch_one<true, true, false, MODE_ACC>( c, ljd, a, s );
        else
            launch_one<true, false, false, MODE_ACC>( c, ljd, a, s );
    }
    GBMD_LAUNCH_CHECK( c, "lj force" );
    if ( fold )
    {
        k_fold_f4<<<( n + 255 ) / 256, 256, 0, c->stream>>>( c->f4.p, n, c->f.p );
        GBMD_LAUNCH_CHECK( c, "lj fold partner forces" );
    }
    gbmd_ktime_end( c, GBMD_KT_FORCE, t0 );
    if ( eflag )
        return gbmd_reduce_partials( c, lj_warps( c ), 1 );
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
    if ( !c->xr_alt.p || c->xr_alt.cap < (size_t)n + 1 )
        return gbmd_fail( c, GBMD_ERR_ARG, "lj step: shadow buffers not set up (binning)" );
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, next );
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_FORCE, &t0 );
    if ( thermo )
        launch_one<true, true, false, MODE_STEP>( c, ljd, a, s );
    else
        launch_one<true, false, false, MODE_STEP>( c, ljd, a, s );
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
        if ( ( rc = gbmd_reduce_partials( c, lj_warps( c ), 0 ) ) )
            return rc;
        return gbmd_reduce_partials( c, lj_warps( c ), 1 );
    }
    return GBMD_OK;
}

int gbmd_lj_step_key( gbmd_ctx *c, std::string &key )
{
    const int n = (int)c->n;
    size_t stride;
    GbmdLJ *ljd;
    int rc = gbmd_partials_prepare( c, n, &stride, &ljd );
    if ( rc )
        return rc;
    const LjArgs a = make_args( c, stride );
    const StepArgs s = gbmd_step_args( c, true );
    const void *ptrs[] = { c->x.p,  c->x_alt.p,    c->xr.p, c->xr_alt.p, c->home.p, c->nlist.p,
                           c->nnum.p, c->partials.p, c->f.p,  c->v.p,      ljd };
    const int ints[] = { n, (int)c->precision, c->ntypes, c->tune.lj_tpb };
    key.assign( reinterpret_cast<const char *>( ptrs ), sizeof ptrs );
    key.append( reinterpret_cast<const char *>( ints ), sizeof ints );
    key.append( reinterpret_cast<const char *>( &a ), sizeof a );
    key.append( reinterpret_cast<const char *>( &s ), sizeof s );
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
    if ( c->half )
        launch_one<false, true, true, MODE_ACC>( c, ljd, a, s );
    else
        launch_one<false, true, false, MODE_ACC>( c, ljd, a, s );
    GBMD_LAUNCH_CHECK( c, "lj energy" );
    return gbmd_reduce_partials( c, lj_warps( c ), 1 );
}

// Serving: the fused full-list mixed step (force, final integrate, thermo
// sums where thermo[k], next initial integrate unless last[k]) of many
// single-type jobs on one stream, in as few launches as the job table holds
// (two groups: with and without the thermo sums).  Launches issued are added
// to *launches.
int gbmd_lj_step_batch( gbmd_ctx *const *cs, const bool *thermo, const bool *last, int count,
                        int64_t *launches )
{
    if ( count <= 0 )
        return GBMD_OK;
    cudaStream_t st = cs[0]->stream;
    // host staging of the launch parameters (~20 KB): one per host thread, so
    // engines driven from different threads do not share it
    thread_local LjJobTable t;
    int rc;
    for ( int pass = 0; pass < 2; pass++ )
    {
        const bool ef = pass == 1;
        t.njobs = 0;
        int blocks = 0;
        auto flush = [&]() -> int {
            if ( t.njobs == 0 )
                return GBMD_OK;
            t.block0[t.njobs] = blocks;
            if ( ef )
                k_lj_mixed_jobs<true><<<blocks, LJ_THREADS, 0, st>>>( t );
            else
                k_lj_mixed_jobs<false><<<blocks, LJ_THREADS, 0, st>>>( t );
            const cudaError_t e = cudaGetLastError();
            if ( e != cudaSuccess )
                return gbmd_cuda_check( cs[0], e, "lj step batch" );
            ( *launches )++;
            t.njobs = 0;
            blocks = 0;
            return GBMD_OK;
        };
        for ( int k = 0; k < count; k++ )
        {
            gbmd_ctx *c = cs[k];
            if ( thermo[k] != ef || c->n == 0 )
                continue;
            if ( c->precision != GBMD_PREC_MIXED || c->ntypes != 1 || c->md.half ||
                 c->stream != st )
                return gbmd_fail( c, GBMD_ERR_ARG, "lj step batch: job is not batchable" );
            if ( !c->xr_alt.p || c->xr_alt.cap < (size_t)c->n + 1 )
                return gbmd_fail( c, GBMD_ERR_ARG, "lj step batch: shadow buffers not set up" );
            size_t stride;
            GbmdLJ *ljd;
            if ( ( rc = gbmd_partials_prepare( c, c->n, &stride, &ljd ) ) )
                return rc;
            LjJob &J = t.job[t.njobs];
            J.xr = c->xr.p;
            J.x = c->x.p;
            J.home = c->home.p;
            J.nlist = c->nlist.p;
            J.nnum = c->nnum.p;
            J.prm = ljd;
            J.f = c->f.p;
            J.partials = c->partials.p;
            J.v = c->v.p;
            J.x_next = c->x_alt.p;
            J.xr_next = c->xr_alt.p;
            J.a = make_args( c, stride );
            J.s = gbmd_step_args( c, !last[k] );
            t.block0[t.njobs] = blocks;
            blocks += (int)( ( c->n + LJ_THREADS - 1 ) / LJ_THREADS );
            t.njobs++;
            if ( t.njobs == LJ_JOBS_PER_LAUNCH && ( rc = flush() ) )
                return rc;
        }
        if ( ( rc = flush() ) )
            return rc;
    }
    for ( int k = 0; k < count; k++ )
    {
        gbmd_ctx *c = cs[k];
        if ( c->n == 0 )
            continue;
        if ( !last[k] )
        {
            std::swap( c->x, c->x_alt );
            std::swap( c->xr, c->xr_alt );
        }
        if ( thermo[k] )
        {
            if ( ( rc = gbmd_reduce_partials( c, lj_warps( c ), 0 ) ) ||
                 ( rc = gbmd_reduce_partials( c, lj_warps( c ), 1 ) ) )
                return rc;
        }
    }
    return GBMD_OK;
}
