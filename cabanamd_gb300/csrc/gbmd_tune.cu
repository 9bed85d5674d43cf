// gbmd_tune.cu -- tile-shape autotuner.
//
// The kernels of the hot path are compiled for a few tile shapes each:
//   - LJ force: atoms (threads) per block, GBMD_LJ_TPB_{SMALL, DEFAULT,
//     LARGE}, and, in mixed precision, the L2 prefetch distance of the
//     transposed list rows (runtime);
//   - Verlet list build: home cells (warps) per block x list slots per lane
//     staged in shared memory (the pairs gbmd_nb_shape names).
// No shape changes a result: an atom's arithmetic does not depend on the
// block it runs in, partial sums are per warp of 32 atoms, and the list
// build writes the same entries in the same order.  So the fastest shape can
// be picked per system.
//
// With tuning on (the default), gbmd_md_init times every candidate on the
// system itself, after its first list build and before its first force:
// two launches per list-build shape, then one warm-up and three timed
// launches of the plain LJ force per (block size, prefetch) pair; the
// fastest of each wins.  Both kernels only overwrite what they write (the
// list, f), and md_init then builds nothing new and recomputes f.  Choices
// are cached for the process under the system's class -- force, precision,
// list kind, types, image mode, log2 of the atom count and the list's
// largest row in steps of 8 -- so a second system of the same class (a
// serving job of a similar size, a re-run) takes the cached shapes at no
// cost.  The class without the list's largest row is known before the first
// list build, so md_init's first build already runs the list-build shape
// last tuned for it (gbmd_pretune).  NNP systems tune the list build; their
// triplet kernels run one warp per atom and take no tile parameter.
#include "gbmd_internal.cuh"

#include <cmath>
#include <mutex>

namespace
{
std::mutex g_tune_mutex;
std::map<std::string, GbmdTune> g_tune_cache;
std::map<std::string, GbmdTune> g_pretune_cache; // keyed without the row maximum

// The system's class; with_rows adds the list's largest row in steps of 8.
std::string tune_key( const gbmd_ctx *c, bool with_rows = true )
{
    int lg = 0;
    while ( ( (int64_t)1 << ( lg + 1 ) ) <= c->n )
        lg++;
    const int ints[] = { c->device,  c->force_type, c->precision,      c->half,
                         c->ntypes > 1 ? 2 : 1, c->no_images, lg,
                         with_rows ? ( c->nl_maxc + 7 ) / 8 : -1 };
    return std::string( reinterpret_cast<const char *>( ints ), sizeof ints );
}

// Mean device time of `reps` runs of `launch` (CUDA events on the context
// stream), after `warm` untimed runs.
template <class F> int time_runs( gbmd_ctx *c, int warm, int reps, F launch, float *ms )
{
    int rc;
    for ( int k = 0; k < warm; k++ )
        if ( ( rc = launch() ) )
            return rc;
    cudaEvent_t e0, e1;
    GBMD_CUDA( c, cudaEventCreate( &e0 ) );
    if ( cudaEventCreate( &e1 ) != cudaSuccess )
    {
        cudaEventDestroy( e0 );
        return gbmd_fail( c, GBMD_ERR_CUDA, "autotune: event creation failed" );
    }
    rc = GBMD_OK;
    float total = 0.f;
    for ( int k = 0; k < reps && !rc; k++ )
    {
        cudaEventRecord( e0, c->stream );
        rc = launch();
        cudaEventRecord( e1, c->stream );
        if ( !rc && cudaEventSynchronize( e1 ) != cudaSuccess )
            rc = gbmd_fail( c, GBMD_ERR_CUDA, "autotune: timing failed" );
        float t = 0.f;
        if ( !rc )
            cudaEventElapsedTime( &t, e0, e1 );
        total += t;
    }
    cudaEventDestroy( e0 );
    cudaEventDestroy( e1 );
    *ms = total / reps;
    return rc;
}
} // namespace

int gbmd_autotune( gbmd_ctx *c )
{
    if ( c->tune_mode != 1 || c->n == 0 || !c->have_list )
        return GBMD_OK;
    const std::string key = tune_key( c );
    {
        std::lock_guard<std::mutex> lock( g_tune_mutex );
        auto it = g_tune_cache.find( key );
        if ( it != g_tune_cache.end() )
        {
            c->tune = it->second;
            c->tuned = true;
            return GBMD_OK;
        }
    }
    NvtxRange range( "gbmd.autotune" );
    int rc;
    GbmdTune best = c->tune;
    // list build: the list exists at full capacity, so every run is one
    // launch and its padding
    float best_ms = 0.f;
    for ( int k = 0; k < GBMD_NB_NSHAPES; k++ )
    {
        gbmd_nb_shape( k, &c->tune.nb_warps, &c->tune.nb_out );
        float ms = 0.f;
        rc = time_runs( c, 0, 2,
                        [&]() -> int {
                            int r = gbmd_build_list_launch( c );
                            if ( r )
                                return r;
                            GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
                            bool again = false;
                            r = gbmd_build_list_finish( c, &again );
                            if ( !r && again )
                                r = gbmd_fail( c, GBMD_ERR_CAPACITY,
                                               "autotune: list capacity changed while timing" );
                            return r;
                        },
                        &ms );
        if ( rc )
            return rc;
        if ( k == 0 || ms < best_ms )
        {
            best_ms = ms;
            best.nb_warps = c->tune.nb_warps;
            best.nb_out = c->tune.nb_out;
        }
    }
    c->tune.nb_warps = best.nb_warps;
    c->tune.nb_out = best.nb_out;
    if ( c->force_type == GBMD_FORCE_LJ && c->lj_set )
    {
        const int tpbs[] = { GBMD_LJ_TPB_DEFAULT, GBMD_LJ_TPB_SMALL, GBMD_LJ_TPB_LARGE };
        const int pfs_mixed[] = { 16, 0, 8, 32 };
        const int pf_fp64[] = { 16 };
        const bool mixed = c->precision == GBMD_PREC_MIXED;
        const int *pfs = mixed ? pfs_mixed : pf_fp64;
        const int npf = mixed ? 4 : 1;
        bool first = true;
        for ( int tpb : tpbs )
            for ( int q = 0; q < npf; q++ )
            {
                c->tune.lj_tpb = tpb;
                c->tune.lj_pf = pfs[q];
                float ms = 0.f;
                rc = time_runs( c, 1, 3, [&]() { return gbmd_lj_launch( c, false, true ); },
                                &ms );
                if ( rc )
                    return rc;
                if ( first || ms < best_ms )
                {
                    best_ms = ms;
                    best.lj_tpb = tpb;
                    best.lj_pf = pfs[q];
                    first = false;
                }
            }
    }
    c->tune = best;
    c->tuned = true;
    std::lock_guard<std::mutex> lock( g_tune_mutex );
    g_tune_cache[key] = best;
    g_pretune_cache[tune_key( c, false )] = best;
    return GBMD_OK;
}

void gbmd_pretune( gbmd_ctx *c )
{
    if ( c->tune_mode != 1 || c->n == 0 )
        return;
    std::lock_guard<std::mutex> lock( g_tune_mutex );
    auto it = g_pretune_cache.find( tune_key( c, false ) );
    if ( it != g_pretune_cache.end() )
    {
        c->tune.nb_warps = it->second.nb_warps;
        c->tune.nb_out = it->second.nb_out;
    }
}

extern "C" {

int gbmd_set_tuning( gbmd_ctx *c, int mode )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( mode != 0 && mode != 1 )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_tuning: mode is 0 (fixed shapes) or 1 (autotune)" );
    c->tune_mode = mode;
    return GBMD_OK;
}

int gbmd_set_shapes( gbmd_ctx *c, int lj_threads, int lj_prefetch, int nb_warps, int nb_out )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( lj_threads != GBMD_LJ_TPB_SMALL && lj_threads != GBMD_LJ_TPB_DEFAULT &&
         lj_threads != GBMD_LJ_TPB_LARGE )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_shapes: LJ atoms per block must be 64, 128 or 256" );
    if ( lj_prefetch < 0 || lj_prefetch > 64 )
        return gbmd_fail( c, GBMD_ERR_ARG, "set_shapes: prefetch distance must be 0 .. 64 rows" );
    if ( !gbmd_nb_shape_ok( nb_warps, nb_out ) )
        return gbmd_fail( c, GBMD_ERR_ARG,
                          "set_shapes: list-build shape (warps, staged slots) must be one of "
                          "(12, 32), (8, 32), (16, 24), (8, 48)" );
    c->tune.lj_tpb = lj_threads;
    c->tune.lj_pf = lj_prefetch;
    c->tune.nb_warps = nb_warps;
    c->tune.nb_out = nb_out;
    c->tune_mode = 0;
    c->tuned = false;
    return GBMD_OK;
}

int gbmd_get_shapes( const gbmd_ctx *c, int *shapes )
{
    if ( !c || !shapes )
        return GBMD_ERR_ARG;
    shapes[0] = c->tune.lj_tpb;
    shapes[1] = c->tune.lj_pf;
    shapes[2] = c->tune.nb_warps;
    shapes[3] = c->tune.nb_out;
    shapes[4] = c->tuned ? 1 : 0;
    return GBMD_OK;
}

} // extern "C"
