// gbmd_nnp.cuh -- NNP model structures shared by the symmetry-function /
// force kernels (gbmd_nnp.cu) and the tensor-core MLP (gbmd_nnp_mlp_tc.cu).
#pragma once

#include "gbmd_internal.cuh"

#define NNP_MAXSF 64
#define NNP_MAXNODES 64
#define NNP_MAXLAYERS 4
#define NNP_MAXNBR 192 // neighbours inside rc per atom, common capacity
#define NNP_MAXNBR_LARGE 448 // capacity for dense states (flagged if exceeded)
#define NNP_WARPS_F 4 // warps per block, FP32 instantiation
#define NNP_WARPS_D 2 // FP64 (twice the shared memory per warp)
#define NNP_MAXETA 4 // distinct angular eta (grid rows)
#define NNP_MAXLZ 8  // distinct angular (lambda, zeta) (grid columns)
#define NNP_MAXELEM 4 // elements of one potential
#define NNP_MAXCH 10  // angular neighbour-element pairs of one centre element

// Device-side model (one element).
struct NnpParams
{
    int nsf, nrad, nang;
    double rc;
    double eta_r[NNP_MAXSF], rs_r[NNP_MAXSF];
    int ang_eta[NNP_MAXSF], ang_lz[NNP_MAXSF];
    // Several elements: a radial function sums neighbours of element
    // rad_e1 only; angular functions form channels, one per unordered
    // neighbour-element pair {ch_e1, ch_e2}, each with its own grid.  One
    // element: rad_e1 = 0, one channel {0, 0}.
    int elem, nelem;
    int rad_e1[NNP_MAXSF];
    int nch;
    int ch_e1[NNP_MAXCH], ch_e2[NNP_MAXCH];
    // angular function of (channel, eta, (lambda, zeta)) or -1
    int grid_sf[NNP_MAXCH][NNP_MAXETA][NNP_MAXLZ];
    double ang_pre[NNP_MAXSF]; // 2^(1 - zeta)
    int neta, nlz;
    double eta_u[NNP_MAXETA];
    double lam_u[NNP_MAXLZ];
    double zeta_u[NNP_MAXLZ];
    int zeta_int[NNP_MAXLZ]; // >0: integer power by multiplication
    double gmin[NNP_MAXSF], gscale[NNP_MAXSF];
    double smin;
    int nl;                          // weight layers
    int nodes[NNP_MAXLAYERS + 1];    // nodes[0] = nsf
    char act[NNP_MAXLAYERS + 1];     // act[l] for l >= 1
    int woff[NNP_MAXLAYERS + 1], boff[NNP_MAXLAYERS + 1];
    double e_offset;
    double cflength, cfenergy;
    // Power ladder (mixed-precision kernels): when every angular function
    // has lambda = +-1 and zeta = 2^m (m <= 5), (1 + lambda cos)^zeta comes
    // from repeated squaring of 1 +- cos.  lad_sf[eta][lambda > 0][m] is the
    // angular function (index among the angular ones) or -1; lad_mask has
    // bit m set for every zeta = 2^m in use.
    int lad_ok;
    int lad_mask;
    int lad_sf[NNP_MAXCH][NNP_MAXETA][2][6]; // [channel][eta][lambda > 0][m]
};

struct NnpModel
{
    NnpParams p{};             // element 0 (the only one for most potentials)
    std::vector<NnpParams> pe; // every element, in atomic-number order
    int gstride = 0;           // row length of G / dEdG: the largest function count
    DevBuf<int> elem_atoms;    // several elements: atoms grouped by element
    DevBuf<int> elem_aux;      // block counts / offsets, element starts
    std::vector<double> w, b; // host copies (all elements, concatenated)
    double *d_w = nullptr, *d_b = nullptr;
    float *d_wf = nullptr, *d_bf = nullptr;
    DevBuf<double> G, dEdG, E; // per atom
    DevBuf<unsigned long long> fq; // fixed-point force sums (mixed precision)
    DevBuf<uint16_t> tcache;       // compacted triplets (NnpTriCache)
    DevBuf<int> tcount;
    bool g_scaled = false;         // G holds the scaled MLP input (mixed precision)
    std::string dir;
    struct TcModel *d_tc = nullptr; // tensor-core MLP operands (when the shape fits)
    uint64_t gen = 0; // distinct for every loaded model (graph-cache keys)
};

// The atoms a kernel launch covers.  One element: every atom, by index.
// Several elements: one launch per element over that element's atoms
// (atoms[starts[el] .. starts[el + 1]) holds them in index order); type
// gives neighbour elements.
struct ElemAtoms
{
    const int *atoms = nullptr;
    const int *starts = nullptr;
    const int *type = nullptr;
    int el = 0;
    // atom of work item w, or -1 past the end
    __device__ __forceinline__ int atom( int w, int n ) const
    {
        if ( !atoms )
            return w < n ? w : -1;
        const int b = starts[el];
        return w < starts[el + 1] - b ? atoms[b + w] : -1;
    }
};

// Tensor-core MLP (mixed precision): operand images and FP32 constants.
// Each B image is one 32 (N) x 192 (K) BF16 operand in the no-swizzle
// K-major core-matrix layout: element (n, k) at byte
// ((n / 8) * 24 + k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2.  K holds the
// three-way BF16 split of the FP32 matrix, [hi | mid | hi | lo | hi | mid],
// against an A of [hi | hi | mid | hi | lo | mid].
#define TC_B_BYTES ( 4 * 24 * 128 )
struct alignas( 16 ) TcModel // 16-byte multiple: per-element arrays stay TMA-aligned
{
    uint16_t img[4][TC_B_BYTES / 2]; // forward W1, forward W2, backward W2^T, backward W1^T
    float b1[32], b2[32], w3[32], b3;
    float gmin[32], gscale[32], smin;
    int nsf, h1, h2;
    char act1, act2;
};

// Build the tensor-core operands when the network fits (nsf, hidden <= 32,
// two hidden layers, linear output); returns false otherwise.
bool gbmd_tc_model_build( const NnpParams &p, const std::vector<double> &w,
                          const std::vector<double> &b, TcModel &out );
// Compacted triplets of one force evaluation (mixed precision, one element,
// common neighbour capacity): the symmetry-function kernel stores each
// atom's triplets (slot pairs, at most NNP_TCAP) and their count, and the
// force kernel of the same evaluation reads them instead of walking the
// neighbour pairs again; an atom with more falls back to the walk.
#define NNP_TCAP 2048
struct NnpTriCache
{
    uint16_t *t = nullptr; // [n][NNP_TCAP]
    int *cnt = nullptr;    // [n]
};

// Mixed-precision symmetry functions / forces with compacted triplets and
// the power ladder (gbmd_nnp_f32.cu), when the model's angular functions
// allow it.
bool gbmd_nnp_f32_supported( const NnpParams &p );
// The triplet cache applies to this evaluation (one element, common
// neighbour capacity).
bool gbmd_nnp_f32_cacheable( const gbmd_ctx *c, int nelem );
// scaled != 0: the kernel writes smin + (G - Gmin) Gscale (the MLP input).
// ea selects the atoms (one element's group for a potential with several
// elements); G / dEdG rows have gstride entries.
int gbmd_nnp_sf_f32_launch( gbmd_ctx *c, const NnpParams &p, const NnpParams *Pd, float *G,
                            int scaled, const ElemAtoms &ea, int gstride,
                            const NnpTriCache &tc );
// Forces of the atoms ea selects, as fixed-point sums into fq: zero fq with
// gbmd_nnp_fq_begin once, launch per element group, then gbmd_nnp_fq_end
// adds conv * fq into the FP64 forces.
int gbmd_nnp_force_f32_launch( gbmd_ctx *c, const NnpParams &p, const NnpParams *Pd,
                               const float *dEdG, unsigned long long *fq, const ElemAtoms &ea,
                               int gstride, const NnpTriCache &tc );
int gbmd_nnp_fq_begin( gbmd_ctx *c, unsigned long long *fq );
int gbmd_nnp_fq_end( gbmd_ctx *c, const NnpParams &p, const unsigned long long *fq );
// G_scaled != 0: G already holds the scaled input (see gbmd_nnp_sf_f32_launch)
int gbmd_nnp_mlp_tc_launch( gbmd_ctx *c, const TcModel *dev, const float *G, float *dEdG,
                            double *E, int n, double *partials, int G_scaled,
                            const ElemAtoms &ea, int gstride ); // gbmd_nnp_mlp_tc.cu

// ---------------------------------------------------------------------------
// Serving: the mixed-precision step of many NNP jobs in job-table launches.
// A job qualifies when its potential has one element of the compiled common
// shape (up to 8 radial functions, zeta in {1, 2, 4, 16}, three angular
// eta), a tensor-core MLP, and its list fits the common neighbour capacity.
// Every launch runs the single-system kernel bodies on each job's own
// arrays, so a job's result does not depend on the batch.
#define NNP_JOBS_PER_LAUNCH 32
struct NnpJobArgs
{
    // symmetry functions / forces
    const float4 *xr;
    const uint32_t *nlist;
    const int *nnum;
    size_t stride;
    int n, gstride;
    GbmdGeom g;
    const NnpParams *Pg;
    float *G, *dEdG;
    unsigned long long *fq;
    int *flags;
    NnpTriCache tc;
    // tensor-core MLP
    const TcModel *tcm;
    double *E, *pe_part;
    // fixed-point sums -> forces, integrator
    double conv;
    double4 *x;
    float4 *xr_out; // the shadow the integrator refreshes (= xr)
    double *v, *f, *partials;
    const int *type, *home;
    StepArgs s;
    int thermo, last;
};
struct NnpJobTable
{
    int njobs;
    int b_sf[NNP_JOBS_PER_LAUNCH + 1];  // blocks of NNP_F32_WARPS atoms
    int b_mlp[NNP_JOBS_PER_LAUNCH + 1]; // 128-atom tiles
    int b_fq[NNP_JOBS_PER_LAUNCH + 1];  // blocks of 256 of the 3n force components
    int b_nve[NNP_JOBS_PER_LAUNCH + 1]; // blocks of 256 atoms
    NnpJobArgs job[NNP_JOBS_PER_LAUNCH];
};
// The job whose range [b[j], b[j + 1]) holds block `bid`.
__device__ __forceinline__ int nnp_job_of( const int *b, int njobs, int bid )
{
    int lo = 0, hi = njobs - 1;
    while ( lo < hi )
    {
        const int mid = ( lo + hi + 1 ) >> 1;
        if ( b[mid] <= bid )
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
// Qualifies for the job-table step (see above).
bool gbmd_nnp_batchable( const gbmd_ctx *c );
bool gbmd_nnp_f32_job_shape( const NnpParams &p ); // gbmd_nnp_f32.cu
// One step (force, final integrate, next initial integrate unless last,
// thermo sums where thermo) of `count` qualifying jobs sharing a stream:
// gbmd_nnp.cu.  Launches issued are added to *launches.
int gbmd_nnp_step_batch( gbmd_ctx *const *cs, const bool *thermo, const bool *last, int count,
                         int64_t *launches );
// The job-table launches (gbmd_nnp_f32.cu, gbmd_nnp_mlp_tc.cu, gbmd_nve.cu)
int gbmd_nnp_zero_jobs_launch( const NnpJobTable &t, cudaStream_t st );
int gbmd_nnp_sf_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st );
int gbmd_nnp_force_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st );
int gbmd_nnp_fq_jobs_launch( const NnpJobTable &t, cudaStream_t st );
int gbmd_nnp_mlp_tc_jobs_launch( const NnpJobTable &t, int device, cudaStream_t st );
int gbmd_nve_jobs_launch( const NnpJobTable &t, cudaStream_t st );
constexpr int NNP_NVE_THREADS = 256; // = the integrator's block (gbmd_nve.cu)

// ---------------------------------------------------------------------------
// Device helpers shared by the NNP kernels (gbmd_nnp.cu, gbmd_nnp_f32.cu)
template <class T> __device__ __forceinline__ T fc_cos( T r, T rc );
template <> __device__ __forceinline__ double fc_cos( double r, double rc )
{
    return r < rc ? 0.5 * ( cos( M_PI * r / rc ) + 1.0 ) : 0.0;
}
// FP32 cosine cutoff without the hardware approximation: with phi =
// pi r / (2 rc) in [0, pi/2), fc = (cos(pi r / rc) + 1) / 2 = cos^2 phi and
// dfc/dr = -(pi / rc) sin phi cos phi; cos and sin come from their Taylor
// series to degree 12 / 13 (truncation <= 6.4e-9 on [0, pi/2]).  The
// intrinsic cosine's absolute error (~3.6e-7) would enter every term of
// every symmetry function with the same sign tendency.
__device__ __forceinline__ float cutoff_cos2( float phi, float &sphi )
{
    const float u = phi * phi;
    float c = 1.0f / 479001600.0f;
    c = c * u - 1.0f / 3628800.0f;
    c = c * u + 1.0f / 40320.0f;
    c = c * u - 1.0f / 720.0f;
    c = c * u + 1.0f / 24.0f;
    c = c * u - 0.5f;
    c = c * u + 1.0f;
    float sn = 1.0f / 6227020800.0f;
    sn = sn * u - 1.0f / 39916800.0f;
    sn = sn * u + 1.0f / 362880.0f;
    sn = sn * u - 1.0f / 5040.0f;
    sn = sn * u + 1.0f / 120.0f;
    sn = sn * u - 1.0f / 6.0f;
    sn = sn * u + 1.0f;
    sphi = sn * phi;
    return c;
}
__device__ __forceinline__ float fc_f32( float r, float half_pirc )
{
    float s;
    const float c = cutoff_cos2( half_pirc * r, s );
    return c * c;
}
__device__ __forceinline__ void fc_dfc_f32( float r, float half_pirc, float &fc, float &dfc )
{
    float s;
    const float c = cutoff_cos2( half_pirc * r, s );
    fc = c * c;
    dfc = -2.0f * half_pirc * s * c;
}
template <> __device__ __forceinline__ float fc_cos( float r, float rc )
{
    return r < rc ? fc_f32( r, 1.57079632679489662f / rc ) : 0.0f;
}
template <class T> __device__ __forceinline__ T dfc_cos( T r, T rc );
template <> __device__ __forceinline__ double dfc_cos( double r, double rc )
{
    return r < rc ? -0.5 * M_PI / rc * sin( M_PI * r / rc ) : 0.0;
}
template <> __device__ __forceinline__ float dfc_cos( float r, float rc )
{
    float fc, dfc;
    fc_dfc_f32( r, 1.57079632679489662f / rc, fc, dfc );
    return r < rc ? dfc : 0.0f;
}
__device__ __forceinline__ double xexp( double v ) { return exp( v ); }
__device__ __forceinline__ float xexp( float v ) { return expf( v ); }
__device__ __forceinline__ double xsqrt( double v ) { return sqrt( v ); }
__device__ __forceinline__ float xsqrt( float v ) { return sqrtf( v ); }
__device__ __forceinline__ double xpow( double b, double e ) { return pow( b, e ); }
__device__ __forceinline__ float xpow( float b, float e ) { return __powf( b, e ); }

// Integer (or general) power b^z and its derivative z b^(z-1).
template <class T>
__device__ __forceinline__ void power_and_deriv( T b, int zi, T z, T &pw, T &dpw )
{
    if ( zi > 0 )
    {
        T r = 1, q = b;
        T rm1 = 1; // b^(z-1)
        int e = zi - 1;
        while ( e )
        {
            if ( e & 1 )
                rm1 *= q;
            q *= q;
            e >>= 1;
        }
        r = rm1 * b;
        pw = r;
        dpw = (T)zi * rm1;
    }
    else
    {
        pw = xpow( b, z );
        dpw = z * xpow( b, z - (T)1 );
    }
}

// Neighbour geometry of one atom in shared memory (per warp), for up to CAP
// neighbours inside rc.
template <class T, int CAP> struct NbrSmem
{
    T dx[CAP], dy[CAP], dz[CAP], r[CAP];
    T fc[CAP], dfc[CAP];
    int own[CAP];
    T fx[CAP], fy[CAP], fz[CAP];
    int el[CAP]; // neighbour element
};

// Displacement x_img(j) - x_i of list entry e of atom i.
template <class T> struct Disp;
template <> struct Disp<double>
{
    __device__ static void get( const double4 *x, const float4 *, int i, uint32_t e, int hp,
                                const GbmdGeom &g, double cfl, double &dx, double &dy,
                                double &dz )
    {
        const int j = (int)( e & GBMD_JMASK ), sc = (int)( e >> 27 );
        const double4 p = x[i], q = x[j];
        const int s0 = image_shift( unpack_home( hp, 0 ), sc % 3 - 1, g.nc[0] );
        const int s1 = image_shift( unpack_home( hp, 1 ), ( sc / 3 ) % 3 - 1, g.nc[1] );
        const int s2 = image_shift( unpack_home( hp, 2 ), sc / 9 - 1, g.nc[2] );
        dx = ( img_coord( q.x, s0, g.L[0] ) - p.x ) * cfl;
        dy = ( img_coord( q.y, s1, g.L[1] ) - p.y ) * cfl;
        dz = ( img_coord( q.z, s2, g.L[2] ) - p.z ) * cfl;
    }
};
template <> struct Disp<float>
{
    __device__ static void get( const double4 *, const float4 *xr, int i, uint32_t e, int,
                                const GbmdGeom &g, double cfl, float &dx, float &dy, float &dz )
    {
        const int j = (int)( e & GBMD_JMASK ), sc = (int)( e >> 27 );
        const float4 p = xr[i], q = xr[j];
        const float cf = (float)cfl;
        dx = ( q.x + (float)( sc % 3 - 1 ) * g.hf[0] - p.x ) * cf;
        dy = ( q.y + (float)( ( sc / 3 ) % 3 - 1 ) * g.hf[1] - p.y ) * cf;
        dz = ( q.z + (float)( sc / 9 - 1 ) * g.hf[2] - p.z ) * cf;
    }
};

// Gather atom i's neighbours inside rc into the warp's shared arrays; returns
// the count (capped at CAP, overflow flagged).
template <class T, int CAP>
__device__ int gather_nbrs( const double4 *x, const float4 *xr, const uint32_t *nlist,
                            size_t stride, int i, int cnt, int hp, const GbmdGeom &g,
                            const NnpParams &P, NbrSmem<T, CAP> &S, int *flags,
                            const int *type = nullptr )
{
    const int lane = threadIdx.x & 31;
    const T rc = (T)P.rc;
    int base = 0;
    for ( int k0 = 0; k0 < cnt; k0 += 32 )
    {
        const int k = k0 + lane;
        bool in = false;
        T dx = 0, dy = 0, dz = 0, r = 0;
        uint32_t e = 0;
        if ( k < cnt )
        {
            e = nlist[(size_t)k * stride + i];
            Disp<T>::get( x, xr, i, e, hp, g, P.cflength, dx, dy, dz );
            const T r2 = dx * dx + dy * dy + dz * dz;
            r = xsqrt( r2 );
            in = r < rc;
        }
        const unsigned m = __ballot_sync( 0xffffffffu, in );
        const int pos = base + __popc( m & ( ( 1u << lane ) - 1u ) );
        if ( in && pos < CAP )
        {
            S.dx[pos] = dx;
            S.dy[pos] = dy;
            S.dz[pos] = dz;
            S.r[pos] = r;
            S.fc[pos] = fc_cos<T>( r, rc );
            S.dfc[pos] = dfc_cos<T>( r, rc );
            S.own[pos] = (int)( e & GBMD_JMASK );
            S.el[pos] = type ? type[e & GBMD_JMASK] : 0;
            S.fx[pos] = 0;
            S.fy[pos] = 0;
            S.fz[pos] = 0;
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


template <class T> struct NnpWarps
{
    static constexpr int value = sizeof( T ) == 8 ? NNP_WARPS_D : NNP_WARPS_F;
};

template <class T>
__device__ __forceinline__ void copy_params( const NnpParams *Pg, NnpParams &P )
{
    const int *src = reinterpret_cast<const int *>( Pg );
    int *dst = reinterpret_cast<int *>( &P );
    for ( int k = threadIdx.x; k < (int)( sizeof( NnpParams ) / 4 ); k += blockDim.x )
        dst[k] = src[k];
}

// The model constants the inner loops use, converted to the kernel's type
// once per block: in the FP32 kernels a per-use double -> float conversion
// would run on the FP64 pipe (1/64 of the FP32 rate on GB300).
template <class T> struct NnpConst
{
    T eta_r[NNP_MAXSF], rs_r[NNP_MAXSF];
    T eta_u[NNP_MAXETA];
    T lam_u[NNP_MAXLZ], zeta_u[NNP_MAXLZ];
};

template <class T>
__device__ __forceinline__ void load_const( const NnpParams *Pg, NnpConst<T> &C )
{
    for ( int k = threadIdx.x; k < NNP_MAXSF; k += blockDim.x )
    {
        C.eta_r[k] = (T)Pg->eta_r[k];
        C.rs_r[k] = (T)Pg->rs_r[k];
    }
    if ( threadIdx.x < NNP_MAXETA )
        C.eta_u[threadIdx.x] = (T)Pg->eta_u[threadIdx.x];
    if ( threadIdx.x < NNP_MAXLZ )
    {
        C.lam_u[threadIdx.x] = (T)Pg->lam_u[threadIdx.x];
        C.zeta_u[threadIdx.x] = (T)Pg->zeta_u[threadIdx.x];
    }
}
