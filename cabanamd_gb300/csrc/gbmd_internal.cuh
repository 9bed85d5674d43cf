// gbmd_internal.cuh -- context, device data layout and shared helpers of the
// GB300 backend for CabanaMD's per-timestep hot path.
//
// Device data layout (one context = one System on one GPU, one CUDA stream):
//   x    double4[n]  position (x, y, z) + (double)type in w; one 32-byte
//                    sector per neighbour gather in the FP64 path
//   xr   float4[n]   mixed-precision shadow: position relative to the centre
//                    of the atom's home cell (fixed at the last rebuild),
//                    type bits in w; one 16-byte gather per neighbour
//   v, f double[3][n] structure-of-arrays (streamed, coalesced)
//   type, id int32[n]
//   home int32[n]    home cell packed as cx | cy << 10 | cz << 20
//   nlist uint32[cap][n]  transposed ("slot-major") Verlet list: entry k of
//                    atom i sits at nlist[k * n + i] so a warp of
//                    consecutive atoms reads one coalesced line per slot.
//                    entry = j | stencil << 27 with stencil the 27-cell
//                    offset code (dx+1) + 3(dy+1) + 9(dz+1) of j's home
//                    cell relative to i's; the periodic image follows from
//                    i's home cell.
//   nnum int32[n]    entries per atom
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/gbmd.h"

#define GBMD_MAXT 8
#define GBMD_RED_RESULTS 8 // reduced scalars at the start of red_out
#define GBMD_RED_WORDS 80  // red_out's doubles: results, block sums, ticket
#define GBMD_JMASK 0x07FFFFFFu
#define GBMD_MAX_ATOMS ( (int64_t)GBMD_JMASK - 1 ) // index n is the sentinel
#define GBMD_MAX_CELLS_PER_DIM 1023
// List rows are padded per warp to a multiple of this (the mixed force
// kernel's batch); the list capacity is kept a multiple of it too.
#ifndef GBMD_ROW_PAD
#define GBMD_ROW_PAD 4
#endif

struct GbmdLJ
{
    double lj1[GBMD_MAXT * GBMD_MAXT];
    double lj2[GBMD_MAXT * GBMD_MAXT];
    double cutsq[GBMD_MAXT * GBMD_MAXT];
    double eshift[GBMD_MAXT * GBMD_MAXT]; // r6c (0.5 lj1 r6c - lj2) / 6 at rc
    float lj1f[GBMD_MAXT * GBMD_MAXT];
    float lj2f[GBMD_MAXT * GBMD_MAXT];
    float cutsqf[GBMD_MAXT * GBMD_MAXT];
    float eshiftf[GBMD_MAXT * GBMD_MAXT];
};

// Per-type integrator constants (integrator_nve_impl.h:49-54), computed on
// the host so no kernel divides in FP64.
struct StepArgs
{
    double dtfm[GBMD_MAXT]; // 0.5 dt / mvv2e / mass[t]
    double mass[GBMD_MAXT];
    double dtv;
    int next; // fused kernels: apply initial_integrate of the next step
};

// Geometry handed to kernels by value.
struct GbmdGeom
{
    double lo[3], hi[3], L[3], h[3];
    double thr_hi[3], thr_lo[3]; // ghost-existence thresholds hi-depth, lo+depth
    float hf[3];
    float hinv_f[3]; // 1 / h rounded to FP32 (cell-index estimate)
    int nc[3];
    int ncell;
};

template <class T> struct DevBuf
{
    T *p = nullptr;
    size_t cap = 0; // elements
};

struct NnpModel; // gbmd_nnp.cu

// Tile shapes (gbmd_tune.cu).  Compiled choices: LJ atoms per block
// GBMD_LJ_TPB_{SMALL, DEFAULT, LARGE}; list build warps (home cells) per
// block and list slots per lane staged in shared memory, the pairs of
// GBMD_NB_SHAPES.  None of them changes a result: each atom's arithmetic and
// every partial sum is the same whichever shape runs.
#define GBMD_LJ_TPB_SMALL 64
#define GBMD_LJ_TPB_DEFAULT 128
#define GBMD_LJ_TPB_LARGE 256
#define GBMD_NB_NSHAPES 4
struct GbmdTune
{
    int lj_tpb = GBMD_LJ_TPB_DEFAULT; // LJ force: atoms (threads) per block
    int lj_pf = 16;                   // LJ mixed force: list-row L2 prefetch distance
    int nb_warps = 12;                // list build: home cells (warps) per block
    int nb_out = 32;                  // list build: slots per lane staged in shared memory
};

struct gbmd_ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool owns_stream = true; // false for serving jobs (engine stream)
    bool owns_host = true;   // h_red / h_flags allocated by this context
    std::string err;
    int sticky_cuda_error = 0;

    // System (system.h:65-136)
    int64_t n = 0;
    double lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
    double boltz = 1.0, mvv2e = 1.0, dt = 0.005;
    int ntypes = 1;
    double mass[GBMD_MAXT] = { 1.0 };
    int precision = GBMD_PREC_FP64;

    DevBuf<double4> x, x_alt;
    DevBuf<float4> xr, xr_alt;
    DevBuf<double> v, v_alt, f;
    // Half lists, mixed precision: the partners' force contributions, summed
    // by vector FP32 reductions and folded into f after the force kernel
    DevBuf<float4> f4;
    DevBuf<int> type, type_alt, id, id_alt, home;
    // Per-atom ghost-existence bits at the last rebuild: bit 2d set when
    // x_d >= hi_d - neigh_cut (an image at -L exists), bit 2d+1 when
    // x_d <= lo_d + neigh_cut (+L image), comm_mpi.h:241-319.
    DevBuf<uint8_t> gflag;
    DevBuf<double> mass_d;

    // Binning
    GbmdGeom geom{};
    double grid_cut = 0.0;
    bool sorted = false;
    DevBuf<int> cell_key, cell_count, cell_start, cell_fill, perm, scan_tmp;

    // Neighbour list
    bool have_list = false;
    int half = 0;
    int no_images = 0; // lists without periodic images (tree-list semantics)
    double neigh_cut = 0.0;
    int max_neigh_guess = 50;
    int nl_cap = 0;       // slots per atom
    int nl_maxc = 0;      // largest per-atom count of the last accepted build
    int nl_attempts = 0;  // builds launched since the last good one
    size_t nl_stride = 0; // row stride of nlist (atoms rounded up to 128)
    DevBuf<uint32_t> nlist;
    DevBuf<int> nnum;

    // Force
    int force_type = GBMD_FORCE_LJ;
    GbmdLJ lj{};
    bool lj_set = false;
    bool lj_dirty = true;
    size_t part_stride = 0;
    NnpModel *nnp = nullptr;

    // Flags / reductions
    DevBuf<int> flags; // [0] list max count, [1] lost atoms, [2] misc, [3] wait timeout,
                       // [4] uploaded atoms with a type out of range
    DevBuf<double> stage;       // gbmd_download_atoms' unpacked [n][3] arrays
    DevBuf<double> partials;    // per-block partial sums
    DevBuf<double> red_out;     // reduced scalars [0, GBMD_RED_RESULTS), then the
                                // reducer's block sums and ticket
    double *h_red = nullptr;    // pinned host mirror of red_out
    int *h_flags = nullptr;     // pinned host mirror of flags
    int *h_flags_dev = nullptr; // its device address (mapped pinned memory), or null

    // MD loop state
    gbmd_md_params md{};
    bool md_ready = false;
    int64_t step = 0;
    int64_t rebuilds = 0;

    // CUDA graphs of runs of fused LJ steps in md_run, cached under the
    // bytes of every launch argument of the run (pointers, LjArgs,
    // StepArgs, step count), so a replay issues exactly the launches it
    // replaces
    bool graphs = true;
    std::vector<std::pair<std::string, cudaGraphExec_t>> graph_cache;
    std::map<std::string, int64_t> graph_launches; // kernels per cached graph
    int64_t graph_replays = 0;

    // Tile shapes: fixed (tune_mode 0) or picked by timing the candidates
    // on the system at gbmd_md_init (tune_mode 1, cached per process by the
    // system's kind and size class)
    GbmdTune tune{};
    int tune_mode = 1;
    bool tuned = false; // tune holds an autotuner's choice

    // Kernel launches issued by this context (every launch site counts)
    int64_t launches = 0;
    double last_run_ms = 0.0;
    int64_t last_run_launches = 0;

    // Kernel timing (CUDA events on this context's stream)
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double ktime_ms[GBMD_KT_COUNT] = { 0 };
    int64_t kcount[GBMD_KT_COUNT] = { 0 };
};

// A context whose work goes to a caller-owned stream and whose pinned host
// mirrors (8 doubles, 8 ints) live in caller-owned memory: the serving
// engine's jobs (gbmd_serve.cu).
int gbmd_create_on_stream( gbmd_ctx **out, int device, cudaStream_t stream, double *h_red,
                           int *h_flags );

// NVTX range for the host side of a phase (md_run's rebuild and step
// launches, the serving engine's admit / chunk / retire).  Header-only NVTX:
// without a profiler attached the calls return at once.
struct NvtxRange
{
    explicit NvtxRange( const char *name ) { nvtxRangePushA( name ); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange( const NvtxRange & ) = delete;
    NvtxRange &operator=( const NvtxRange & ) = delete;
};

// ---------------------------------------------------------------------------
// Error handling
int gbmd_fail( gbmd_ctx *c, int code, const std::string &msg );
int gbmd_cuda_check( gbmd_ctx *c, cudaError_t e, const char *what );
#define GBMD_CUDA( c, call )                                                   \
    do                                                                         \
    {                                                                          \
        cudaError_t _e = ( call );                                             \
        if ( _e != cudaSuccess )                                               \
            return gbmd_cuda_check( c, _e, #call );                            \
    } while ( 0 )
#define GBMD_LAUNCH_CHECK( c, what )                                           \
    do                                                                         \
    {                                                                          \
        ( c )->launches++;                                                     \
        cudaError_t _e = cudaGetLastError();                                   \
        if ( _e != cudaSuccess )                                               \
            return gbmd_cuda_check( c, _e, what );                             \
    } while ( 0 )

// Device buffers are stream-ordered allocations on the context's stream
// (the device's default memory pool, kept resident): growing or freeing a
// buffer never synchronises the device, so one context can retire while
// others sharing the GPU keep running.
template <class T>
int gbmd_reserve( gbmd_ctx *c, DevBuf<T> &b, size_t count, const char *what )
{
    if ( count <= b.cap && b.p )
        return GBMD_OK;
    if ( b.p )
        cudaFreeAsync( b.p, c->stream );
    b.p = nullptr;
    b.cap = 0;
    size_t want = count ? count : 1;
    cudaError_t e = cudaMallocAsync( (void **)&b.p, want * sizeof( T ), c->stream );
    if ( e != cudaSuccess )
    {
        b.p = nullptr;
        return gbmd_cuda_check( c, e, what );
    }
    b.cap = want;
    return GBMD_OK;
}

template <class T> void gbmd_release( gbmd_ctx *c, DevBuf<T> &b )
{
    if ( b.p )
        cudaFreeAsync( b.p, c->stream );
    b.p = nullptr;
    b.cap = 0;
}

template <class T> size_t gbmd_bytes( const DevBuf<T> &b ) { return b.p ? b.cap * sizeof( T ) : 0; }

// Device bytes held by a context (its buffers and NNP model).
size_t gbmd_ctx_device_bytes( const gbmd_ctx *c );

// ---------------------------------------------------------------------------
// Kernel timing helpers (no-ops unless profiling is on)
void gbmd_ktime_begin( gbmd_ctx *c, int which, cudaEvent_t *start );
void gbmd_ktime_end( gbmd_ctx *c, int which, cudaEvent_t start );

// ---------------------------------------------------------------------------
// Strict IEEE FP64 helpers: the FP64 path must perform exactly the
// reference's operation sequence (no fused multiply-add contraction).
// (Macros: the CUDA headers already declare functions named dadd/dsub/dmul
// with a rounding-mode argument.)
#define dmul( a, b ) __dmul_rn( ( a ), ( b ) )
#define dadd( a, b ) __dadd_rn( ( a ), ( b ) )
#define dsub( a, b ) __dsub_rn( ( a ), ( b ) )
#define ddiv( a, b ) __ddiv_rn( ( a ), ( b ) )

// Position of a periodic image: copy then one "x -= L" / "x += L".
__device__ __forceinline__ double img_coord( double xs, int s, double L )
{
    return s < 0 ? dsub( xs, L ) : ( s > 0 ? dadd( xs, L ) : xs );
}

__host__ __device__ __forceinline__ int unpack_home( int packed, int d )
{
    return ( packed >> ( 10 * d ) ) & 1023;
}

// Stencil code -> offset component in {-1,0,1}.
__host__ __device__ __forceinline__ int stencil_d( int code, int d )
{
    return d == 0 ? code % 3 - 1 : ( d == 1 ? ( code / 3 ) % 3 - 1 : code / 9 - 1 );
}

// Periodic shift of the image reached from home cell c by stencil offset o.
__host__ __device__ __forceinline__ int image_shift( int c, int o, int nc )
{
    const int t = c + o;
    return t < 0 ? -1 : ( t >= nc ? 1 : 0 );
}

// ---------------------------------------------------------------------------
// TMA bulk copies and mbarriers (inline PTX, sm_90+ forms valid on sm_103a).
// Every wait is bounded: after GBMD_WAIT_CYCLES the caller gets false and
// reports GBMD_ERR_TIMEOUT through the context flags instead of spinning on.
#define GBMD_WAIT_CYCLES 4000000000LL

__device__ __forceinline__ uint32_t smem_u32( const void *p )
{
    return (uint32_t)__cvta_generic_to_shared( p );
}

__device__ __forceinline__ void mbar_init( uint64_t *bar, uint32_t count )
{
    asm volatile( "mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"( smem_u32( bar ) ),
                  "r"( count )
                  : "memory" );
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile( "fence.mbarrier_init.release.cluster;" ::: "memory" );
}

__device__ __forceinline__ void mbar_arrive_expect_tx( uint64_t *bar, uint32_t bytes )
{
    asm volatile( "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                      smem_u32( bar ) ),
                  "r"( bytes )
                  : "memory" );
}

__device__ __forceinline__ void mbar_arrive( uint64_t *bar )
{
    asm volatile( "mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"( smem_u32( bar ) )
                  : "memory" );
}

__device__ __forceinline__ bool mbar_try_wait( uint64_t *bar, uint32_t parity )
{
    uint32_t ok;
    asm volatile( "{\n\t.reg .pred p;\n\t"
                  "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                  "selp.u32 %0, 1, 0, p;\n\t}"
                  : "=r"( ok )
                  : "r"( smem_u32( bar ) ), "r"( parity )
                  : "memory" );
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded( uint64_t *bar, uint32_t parity,
                                                   long long limit = GBMD_WAIT_CYCLES )
{
    if ( mbar_try_wait( bar, parity ) )
        return true;
    const long long t0 = clock64();
    while ( true )
    {
        if ( mbar_try_wait( bar, parity ) )
            return true;
        if ( clock64() - t0 > limit )
            return false;
    }
}

// 1-D bulk copy global -> shared (16-byte aligned addresses, size % 16 == 0),
// completion signalled on an mbarrier as transaction bytes.
__device__ __forceinline__ void tma_load_1d( void *dst, const void *src, uint32_t bytes,
                                             uint64_t *bar )
{
    asm volatile( "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                  "[%0], [%1], %2, [%3];" ::"r"( smem_u32( dst ) ),
                  "l"( src ), "r"( bytes ), "r"( smem_u32( bar ) )
                  : "memory" );
}

// Relative half-width of the band around rc^2 inside which an FP32 squared
// distance built from home-cell-relative coordinates may disagree with the
// FP64 one (8x the rounding bound for coordinates up to 2 cells + rc).
double gbmd_fp32_band( const GbmdGeom &g, double rc ); // gbmd_neigh.cu

// Internal entry points shared between translation units.
int gbmd_build_list( gbmd_ctx *c );      // gbmd_neigh.cu
bool gbmd_nb_shape_ok( int nw, int nout ); // a compiled list-build shape
void gbmd_nb_shape( int k, int *nw, int *nout ); // k < GBMD_NB_NSHAPES
int gbmd_autotune( gbmd_ctx *c );        // gbmd_tune.cu: pick the tile shapes
// before md_init's first list build: the list-build shape last tuned for the
// system's class, when there is one (gbmd_tune.cu)
void gbmd_pretune( gbmd_ctx *c );
int gbmd_build_list_launch( gbmd_ctx *c );
int gbmd_build_list_finish( gbmd_ctx *c, bool *again );
// Pieces of the two halves for batched rebuilds (gbmd_neigh.cu): sizing and
// buffers only; the builds of sorted, prepared contexts sharing one stream
// in job-table launches; the capacity check without the row padding; the
// row padding of accepted lists in job-table launches.
int gbmd_build_list_prepare( gbmd_ctx *c );
int gbmd_build_list_batch( gbmd_ctx *const *cs, int count, int64_t *launches );
int gbmd_build_list_check( gbmd_ctx *c, bool *again );
int gbmd_pad_lists_batch( gbmd_ctx *const *cs, int count, int64_t *launches );
int gbmd_rebuild( gbmd_ctx *c );         // gbmd_core.cu: wrap + sort + list
// Serving-engine pieces of gbmd_md_run's timestep (gbmd_core.cu)
int gbmd_rebuild_launch( gbmd_ctx *c );
int gbmd_rebuild_finish( gbmd_ctx *c, bool *again );
// Batched rebuilds of contexts sharing one stream (gbmd_core.cu): whether a
// context's rebuild may join a batch; its host half (grid, buffers, list
// sizing); the job-table launches of prepared contexts (wrap, sort, list
// build; the row maxima go to each context's h_flags[0]); and the capacity
// check after the stream passed them, which leaves the row padding of an
// accepted list to gbmd_pad_lists_batch.
bool gbmd_rebuild_batchable( const gbmd_ctx *c );
int gbmd_rebuild_prepare( gbmd_ctx *c );
int gbmd_rebuild_batch_launch( gbmd_ctx *const *cs, int count, int64_t *launches );
int gbmd_rebuild_check( gbmd_ctx *c, bool *again );
int gbmd_job_force_step( gbmd_ctx *c, bool thermo, bool last );
int gbmd_check_flags( gbmd_ctx *c ); // from h_flags[1..3]
void gbmd_thermo_row_from( const gbmd_ctx *c, int64_t step, const double *red, double *row );
int gbmd_lj_launch( gbmd_ctx *c, bool eflag, bool zero_first ); // gbmd_lj.cu
// Fused full-list step: force(n) + final(n) [+ thermo sums] [+ initial(n+1)]
int gbmd_lj_step_launch( gbmd_ctx *c, bool thermo, bool next ); // gbmd_lj.cu
// The launch arguments of the next fused step (no thermo, next step
// follows) as bytes: the graph-cache key of md_run (gbmd_lj.cu)
int gbmd_lj_step_key( gbmd_ctx *c, std::string &key );
StepArgs gbmd_step_args( const gbmd_ctx *c, bool next );        // gbmd_lj.cu
// The fused step of many single-type mixed full-list jobs sharing a stream,
// batched into job-table launches (serving engine).
int gbmd_lj_step_batch( gbmd_ctx *const *cs, const bool *thermo, const bool *last, int count,
                        int64_t *launches ); // gbmd_lj.cu
int gbmd_lj_energy_launch( gbmd_ctx *c ); // gbmd_lj.cu, result in red_out[1]
int gbmd_nve_initial_launch( gbmd_ctx *c );                  // gbmd_nve.cu
// initial_integrate, optionally preceded in the same kernel by the previous
// step's final_integrate (and its sum m v^2 -> red_out[0]).
int gbmd_nve_step_tail_launch( gbmd_ctx *c, bool with_final, bool thermo ); // gbmd_nve.cu
int gbmd_nve_final_launch( gbmd_ctx *c, bool thermo );       // gbmd_nve.cu, sum m v^2 -> red_out[0]
int gbmd_reduce_partials( gbmd_ctx *c, int nparts, int slot ); // gbmd_nve.cu
// Per-block partial-sum slots (slot 0: sum m v^2, slot 1: potential energy)
// sized for n_items, plus the device copy of the LJ table (uploaded when it
// changed).  slot_stride = doubles between slots.
int gbmd_partials_prepare( gbmd_ctx *c, int64_t n_items, size_t *slot_stride,
                           GbmdLJ **lj_dev ); // gbmd_nve.cu
int gbmd_mv2_launch( gbmd_ctx *c ); // gbmd_nve.cu, sum m v^2 -> red_out[0]
int gbmd_update_shadow_launch( gbmd_ctx *c );                  // gbmd_nve.cu
// NNP: symmetry functions, MLP (E_i -> red_out[1] when eflag) and, when
// forces is set, forces accumulated into f.
int gbmd_nnp_launch( gbmd_ctx *c, bool eflag, bool forces ); // gbmd_nnp.cu
void gbmd_nnp_free( gbmd_ctx *c );                             // gbmd_nnp.cu
size_t gbmd_nnp_device_bytes( const gbmd_ctx *c );             // gbmd_nnp.cu
double gbmd_nnp_total_energy( const gbmd_ctx *c, double esum ); // gbmd_nnp.cu
// The NNP model's buffers and values that its launches read, appended to a
// graph-cache key (gbmd_nnp.cu)
void gbmd_nnp_key( const gbmd_ctx *c, std::string &key );

constexpr int GBMD_RED_BLOCK = 256;
