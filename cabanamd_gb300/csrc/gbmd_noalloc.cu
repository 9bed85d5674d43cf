// gbmd_noalloc.cu -- thermo reduction for callers that cannot allocate GPU
// memory.
//
// Some callers of this library cannot call cudaMalloc: a host application
// that owns all device memory through its own pool and forbids any other
// allocation (an MD engine embedding this backend beside its own solver, for
// example), and hard real-time loops that must not enter the driver's
// allocator, whose calls can block on the device.  For them,
// gbmd_thermo_noalloc computes the same temperature and kinetic energy as
// gbmd_thermo without allocating anything: its per-block partial sums live
// in a fixed file-scope device array.
//
// That array is GBMD_NOALLOC_MAX_BLOCKS doubles (512 KiB) and exists on every
// GPU that loads the library, for as long as the library stays loaded.  One
// partial sum is kept per block of GBMD_NOALLOC_THREADS atoms, so a call
// handles at most GBMD_NOALLOC_MAX_ATOMS atoms; larger calls are rejected.
// All calls share the one array: calls whose kernels overlap on the GPU
// (different streams, or host threads racing) overwrite each other's partial
// sums and give wrong results, so the caller must serialise them.  Every call
// writes each partial slot it reads before reading it, so nothing has to be
// cleared between calls.
#include "gbmd_internal.cuh"

#include <mutex>

#define GBMD_NOALLOC_THREADS 256
#define GBMD_NOALLOC_MAX_BLOCKS 65536
#define GBMD_NOALLOC_MAX_ATOMS ( (int64_t)GBMD_NOALLOC_MAX_BLOCKS * GBMD_NOALLOC_THREADS )
#define GBMD_NOALLOC_MAX_DEVICES 64

// The scratch: one partial sum of m v^2 per block.
static __device__ __align__( 256 ) double g_noalloc_partials[GBMD_NOALLOC_MAX_BLOCKS];

__global__ void __launch_bounds__( GBMD_NOALLOC_THREADS )
    k_noalloc_mv2( const double *__restrict__ v, const int *__restrict__ type,
                   const double *__restrict__ mass, int n, double *__restrict__ partials )
{
    __shared__ double red[GBMD_NOALLOC_THREADS / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if ( i < n )
    {
        const double vx = v[i], vy = v[n + i], vz = v[2 * n + i];
        // property_kine.h:72-78: (vx vx + vy vy + vz vz) m
        s = dmul( dadd( dadd( dmul( vx, vx ), dmul( vy, vy ) ), dmul( vz, vz ) ),
                  mass[type[i]] );
    }
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        s += __shfl_xor_sync( 0xffffffffu, s, o );
    if ( ( threadIdx.x & 31 ) == 0 )
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if ( threadIdx.x == 0 )
    {
        double b = 0.0;
        for ( int k = 0; k < GBMD_NOALLOC_THREADS / 32; k++ )
            b += red[k];
        partials[blockIdx.x] = b;
    }
}

// Fixed-order final sum, then T and KE (property_temperature_impl.h:66-76,
// property_kine_impl.h:66-75).
__global__ void __launch_bounds__( 1024 )
    k_noalloc_finish( const double *__restrict__ partials, int nparts, double t_factor,
                      double ke_factor, double *__restrict__ out )
{
    __shared__ double red[32];
    double s = 0.0;
    for ( int k = threadIdx.x; k < nparts; k += blockDim.x )
        s += partials[k];
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        s += __shfl_xor_sync( 0xffffffffu, s, o );
    if ( ( threadIdx.x & 31 ) == 0 )
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if ( threadIdx.x == 0 )
    {
        double t = 0.0;
        for ( int k = 0; k < (int)( blockDim.x >> 5 ); k++ )
            t += red[k];
        out[0] = t * t_factor;
        out[1] = t * ke_factor;
    }
}

// Device address of the scratch array, looked up once per device (with that
// device current) the first time a call runs on it.
static double *g_scratch_addr[GBMD_NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mutex;

static cudaError_t scratch_for_current_device( double **out )
{
    int dev = 0;
    cudaError_t e = cudaGetDevice( &dev );
    if ( e != cudaSuccess )
        return e;
    if ( dev < 0 || dev >= GBMD_NOALLOC_MAX_DEVICES )
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock( g_scratch_mutex );
    if ( !g_scratch_addr[dev] )
    {
        void *p = nullptr;
        e = cudaGetSymbolAddress( &p, g_noalloc_partials );
        if ( e != cudaSuccess )
            return e;
        g_scratch_addr[dev] = static_cast<double *>( p );
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

extern "C" int gbmd_thermo_noalloc( const double *v_dev, const int32_t *type_dev,
                                    const double *mass_dev, int64_t n, double mvv2e,
                                    double boltz, void *stream, double *out_dev )
{
    if ( !v_dev || !type_dev || !mass_dev || !out_dev )
        return GBMD_ERR_ARG;
    if ( n < 2 )
        return GBMD_ERR_ARG; // temperature needs 3n - 3 > 0 degrees of freedom
    if ( n > GBMD_NOALLOC_MAX_ATOMS )
        return GBMD_ERR_CAPACITY; // scratch holds one partial per 256 atoms
    if ( !( mvv2e > 0 ) || !( boltz > 0 ) )
        return GBMD_ERR_ARG;
    // A launch error is read back with cudaGetLastError, which also returns
    // and clears an error left pending by earlier, unrelated work of the
    // calling thread.  Such an error is not this call's to consume: refuse
    // the call and leave it in place for its owner.
    if ( cudaPeekAtLastError() != cudaSuccess )
        return GBMD_ERR_CUDA;
    double *scratch = nullptr;
    if ( scratch_for_current_device( &scratch ) != cudaSuccess )
        return GBMD_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>( stream );
    const int blocks = (int)( ( n + GBMD_NOALLOC_THREADS - 1 ) / GBMD_NOALLOC_THREADS );
    k_noalloc_mv2<<<blocks, GBMD_NOALLOC_THREADS, 0, s>>>( v_dev, type_dev, mass_dev, (int)n,
                                                           scratch );
    if ( cudaGetLastError() != cudaSuccess )
        return GBMD_ERR_CUDA;
    const int64_t dof = 3 * n - 3;
    const double t_factor = mvv2e / ( 1.0 * dof * boltz );
    const double ke_factor = 0.5 * mvv2e;
    k_noalloc_finish<<<1, 1024, 0, s>>>( scratch, blocks, t_factor, ke_factor, out_dev );
    if ( cudaGetLastError() != cudaSuccess )
        return GBMD_ERR_CUDA;
    return GBMD_OK;
}
