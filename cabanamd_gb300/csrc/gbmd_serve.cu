// gbmd_serve.cu -- serving engine: independent MD jobs resident in HBM,
// admitted by device-memory footprint, advanced in chunks of timesteps with
// the per-phase work of all running jobs batched into shared launches.
//
// Each job is one CbnMD run (src/cabanamd_impl.h:70-432): a context of its
// own (buffers, cell grid, Verlet list, parameters) whose work goes to one of
// the engine's streams (stream 0 for the jobs of the job-table LJ launch,
// streams 1-4 round-robin for mixed-precision NNP jobs, the others
// round-robin over the rest).  A chunk
// advances every running job by up to `chunk`
// timesteps in lock step; per timestep:
//   1. initial integrate of jobs at their first step (later steps get it
//      fused into the previous step's kernel);
//   2. rebuild (wrap, cell sort, list) of the jobs whose rebuild is due: the
//      jobs sharing a stream in job-table launches, one per phase for all of
//      them (gbmd_rebuild_batch_launch), each job then marked by an event on
//      its stream;
//   3. force + final integrate (+ next initial, + thermo sums), first for
//      the jobs without a rebuild this step, so that the GPU works on them
//      while the host waits for the rebuilt jobs' events (that job's list
//      only, not a whole stream or device), checks their list capacities
//      (relaunching where a list overflowed), then for the rebuilt jobs.
//      LJ jobs in mixed precision with full lists go into one job-table
//      launch per group (gbmd_lj_step_batch); mixed-precision NNP jobs of the
//      common potential shape go into six job-table launches per stream
//      (gbmd_nnp_step_batch: zeroing, symmetry functions, the persistent
//      tensor-core MLP over every job's tiles, forces, fixed-point sums,
//      integrator); the others launch per job;
//   4. thermo sums copied to a pinned ring (no synchronisation).
// One synchronisation ends the chunk: thermo rows and error flags are read,
// finished jobs are downloaded and retired, and queued jobs are admitted
// while a slot and the memory budget allow (FIFO).
//
// The per-job arithmetic is the single-system kernels' (shared device
// bodies), so a job's trajectory is bit-identical whether it runs alone, in
// any mix, or through gbmd_md_init + gbmd_md_run on a context -- for every
// path whose force sums are order-deterministic (LJ full lists in either
// precision, the mixed NNP path's fixed-point force accumulation).  Paths
// that sum forces with floating-point atomics (FP64 NNP, half lists) agree
// to rounding.
#include "gbmd_internal.cuh"
#include "gbmd_nnp.cuh"

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>

#include "../../include/gbmd_serve.h"

namespace
{
struct Job
{
    int64_t jid = 0;
    gbmd_job_spec spec{};
    std::string nnp_dir;
    int64_t n = 0;
    std::vector<double> x, v, f; // initial state until admitted, final state when done
    std::vector<int> type, id;
    gbmd_ctx *c = nullptr;
    int slot = -1;
    int state = GBMD_JOB_QUEUED;
    int error = 0;
    std::string err;
    double t_arrival = -1, t_admit = -1, t_finish = -1;
    uint64_t est_bytes = 0, bytes = 0;
    std::vector<double> rows;  // thermo rows, 4 doubles each
    std::vector<int64_t> ring_steps; // thermo steps copied this chunk
    cudaEvent_t built = nullptr;     // marks the end of the job's list build
};
} // namespace

#define GBMD_ENGINE_STREAMS 12
// streams 1 .. GBMD_NNP_STREAMS carry the mixed-precision NNP jobs, one
// job-table batch per stream and step, so that batches overlap on the GPU
#define GBMD_NNP_STREAMS 4

struct gbmd_engine
{
    int device = 0;
    // streams[0] carries the jobs whose timestep is one job-table launch
    // (LJ, mixed precision, full list); the others are spread over the rest
    // so that small jobs' kernels overlap on the device
    std::vector<cudaStream_t> streams;
    int next_stream = 0, next_nnp_stream = 0;
    uint64_t budget = 0, used = 0, peak = 0;
    int max_running = 0, chunk = 10;
    std::chrono::steady_clock::time_point t0;
    std::string err;
    int64_t next_id = 1;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    std::deque<Job *> queue;
    std::vector<Job *> running;
    // pinned host memory per job slot: 8 doubles (h_red), 8 ints (h_flags)
    // and a ring of `chunk` reduction records (4 doubles each)
    double *h_red = nullptr;
    int *h_flags = nullptr;
    double *h_ring = nullptr;
    std::vector<int> free_slots;
    gbmd_engine_stats st{};
};

static double now_s( const gbmd_engine *e )
{
    return std::chrono::duration<double>( std::chrono::steady_clock::now() - e->t0 ).count();
}

static int efail( gbmd_engine *e, int code, const std::string &msg )
{
    e->err = msg;
    return code;
}

static bool sync_all( gbmd_engine *e )
{
    bool ok = true;
    for ( cudaStream_t st : e->streams )
        ok = cudaStreamSynchronize( st ) == cudaSuccess && ok;
    return ok;
}

// Device bytes a job will hold once running (replaced by the measured
// figure after admission): per-atom arrays, the Verlet list at the density
// estimate the list build uses, and the NNP per-atom arrays.
static uint64_t estimate_bytes( const gbmd_job_spec &s, int64_t n )
{
    const double vol = ( s.hi[0] - s.lo[0] ) * ( s.hi[1] - s.lo[1] ) * ( s.hi[2] - s.lo[2] );
    const double rc = s.md.force_cut + s.md.skin;
    double nb = vol > 0 ? n / vol * 4.18879020478639 * rc * rc * rc : 0.0;
    if ( s.md.half )
        nb *= 0.5;
    const double cap = std::max( (double)s.md.max_neigh_guess, nb * 1.4 + 16.0 ) + 4.0;
    double per_atom = 240.0 + 4.0 * cap;
    if ( s.force_type == GBMD_FORCE_NNP )
    {
        per_atom += 2.0 * 64 * 8 + 8; // G and dE/dG (up to 64 functions), E
        if ( s.precision == GBMD_PREC_MIXED )
            per_atom += 24 + 2.0 * NNP_TCAP + 4; // fixed-point forces, triplet cache
    }
    return (uint64_t)( n * per_atom ) + ( 1u << 20 );
}

static void job_fail( gbmd_engine *e, Job *j, int code, const std::string &msg )
{
    j->state = GBMD_JOB_FAILED;
    j->error = code;
    j->err = msg;
    j->t_finish = now_s( e );
    e->st.failed++;
}

static void release_job_device( gbmd_engine *e, Job *j )
{
    if ( j->built )
    {
        cudaEventDestroy( j->built );
        j->built = nullptr;
    }
    if ( j->c )
    {
        gbmd_destroy( j->c );
        j->c = nullptr;
    }
    if ( j->slot >= 0 )
        e->free_slots.push_back( j->slot );
    j->slot = -1;
    e->used -= std::min( e->used, j->bytes );
    j->bytes = 0;
}

#define JOB_CALL( call, what )                                                                 \
    do                                                                                         \
    {                                                                                          \
        int _rc = ( call );                                                                    \
        if ( _rc )                                                                             \
        {                                                                                      \
            job_fail( e, j, _rc, std::string( what ) + ": " + gbmd_last_error( j->c ) );      \
            return _rc;                                                                        \
        }                                                                                      \
    } while ( 0 )

// Create the job's context on the engine stream, upload, set up the force,
// gbmd_md_init (first rebuild, force, step-0 thermo).
static int admit( gbmd_engine *e, Job *j )
{
    const int slot = e->free_slots.back();
    e->free_slots.pop_back();
    j->slot = slot;
    const gbmd_job_spec &sp = j->spec;
    // stream 0: the LJ jobs of the job-table step; streams 1 ..
    // GBMD_NNP_STREAMS: the mixed NNP jobs (job-table step per stream when
    // they qualify, gbmd_nnp_batchable); the rest round-robin over the others
    const bool lj_batched = sp.force_type == GBMD_FORCE_LJ && sp.precision == GBMD_PREC_MIXED &&
                            !sp.md.half;
    const bool nnp_batched = sp.force_type == GBMD_FORCE_NNP && sp.precision == GBMD_PREC_MIXED;
    cudaStream_t st = e->streams[0];
    if ( nnp_batched )
        st = e->streams[1 + ( e->next_nnp_stream++ % GBMD_NNP_STREAMS )];
    else if ( !lj_batched )
        st = e->streams[1 + GBMD_NNP_STREAMS +
                        ( e->next_stream++ %
                          ( (int)e->streams.size() - 1 - GBMD_NNP_STREAMS ) )];
    int rc = gbmd_create_on_stream( &j->c, e->device, st, e->h_red + 8 * slot,
                                    e->h_flags + 8 * slot );
    if ( rc )
    {
        e->free_slots.push_back( slot );
        j->slot = -1;
        job_fail( e, j, rc, "job context creation failed" );
        return rc;
    }
    const gbmd_job_spec &s = j->spec;
    JOB_CALL( gbmd_set_units( j->c, s.boltz, s.mvv2e, s.dt ), "set_units" );
    JOB_CALL( gbmd_set_box( j->c, s.lo, s.hi ), "set_box" );
    JOB_CALL( gbmd_set_types( j->c, 1, &s.mass ), "set_types" );
    JOB_CALL( gbmd_set_precision( j->c, s.precision ), "set_precision" );
    JOB_CALL( gbmd_upload_atoms( j->c, j->n, j->x.data(), j->v.data(), j->type.data(),
                                 j->id.data() ),
              "upload" );
    if ( s.force_type == GBMD_FORCE_LJ )
        JOB_CALL( gbmd_lj_coeff( j->c, 1, 1, s.lj_epsilon, s.lj_sigma, s.lj_cut ), "lj_coeff" );
    else
        JOB_CALL( gbmd_nnp_load( j->c, j->nnp_dir.c_str(), s.nnp_cflength, s.nnp_cfenergy ),
                  "nnp_load" );
    double row0[4];
    JOB_CALL( gbmd_md_init( j->c, &s.md, row0 ), "md_init" );
    if ( s.md.thermo_every > 0 )
        j->rows.insert( j->rows.end(), row0, row0 + 4 );
    // the initial state is no longer needed on the host
    std::vector<double>().swap( j->x );
    std::vector<double>().swap( j->v );
    std::vector<int>().swap( j->type );
    std::vector<int>().swap( j->id );
    j->bytes = gbmd_ctx_device_bytes( j->c );
    e->used += j->bytes;
    e->peak = std::max( e->peak, e->used );
    j->state = GBMD_JOB_RUNNING;
    j->t_admit = now_s( e );
    e->st.admitted++;
    return GBMD_OK;
}

static void admit_queued( gbmd_engine *e )
{
    NvtxRange range( "engine.admit" );
    const double t0 = now_s( e );
    struct Add
    {
        gbmd_engine *e;
        double t0;
        ~Add() { e->st.admit_seconds += now_s( e ) - t0; }
    } add{ e, t0 };
    while ( !e->queue.empty() && (int)e->running.size() < e->max_running &&
            !e->free_slots.empty() )
    {
        Job *j = e->queue.front();
        if ( j->est_bytes > e->budget )
        {
            e->queue.pop_front();
            job_fail( e, j, GBMD_ERR_CAPACITY, "job exceeds the engine's device memory budget" );
            continue;
        }
        if ( e->used + j->est_bytes > e->budget )
            break; // FIFO: wait for memory
        e->queue.pop_front();
        if ( admit( e, j ) == GBMD_OK )
            e->running.push_back( j );
        else
            release_job_device( e, j );
    }
}

// Finished job: final state (sorted by id) to the host, device freed.
static void retire( gbmd_engine *e, Job *j )
{
    NvtxRange range( "engine.retire" );
    const int64_t n = j->n;
    std::vector<double> x( 3 * n ), v( 3 * n ), f( 3 * n );
    std::vector<int> type( n ), id( n );
    int rc = gbmd_download_atoms( j->c, x.data(), v.data(), f.data(), type.data(), id.data() );
    if ( rc )
    {
        job_fail( e, j, rc, std::string( "download: " ) + gbmd_last_error( j->c ) );
        release_job_device( e, j );
        return;
    }
    std::vector<int64_t> ord( n );
    for ( int64_t k = 0; k < n; k++ )
        ord[k] = k;
    std::sort( ord.begin(), ord.end(), [&]( int64_t a, int64_t b ) { return id[a] < id[b]; } );
    j->x.resize( 3 * n );
    j->v.resize( 3 * n );
    j->f.resize( 3 * n );
    j->type.resize( n );
    j->id.resize( n );
    for ( int64_t k = 0; k < n; k++ )
    {
        const int64_t s = ord[k];
        for ( int d = 0; d < 3; d++ )
        {
            j->x[3 * k + d] = x[3 * s + d];
            j->v[3 * k + d] = v[3 * s + d];
            j->f[3 * k + d] = f[3 * s + d];
        }
        j->type[k] = type[s];
        j->id[k] = id[s];
    }
    e->st.launches += j->c->launches;
    release_job_device( e, j );
    j->state = GBMD_JOB_DONE;
    j->t_finish = now_s( e );
    e->st.finished++;
    e->st.atom_steps += n * j->spec.nsteps;
}

static bool lj_batchable( const gbmd_ctx *c )
{
    return c->force_type == GBMD_FORCE_LJ && !c->md.half && c->precision == GBMD_PREC_MIXED &&
           c->ntypes == 1;
}

// Advance the running jobs by up to e->chunk timesteps.
static int run_chunk( gbmd_engine *e )
{
    NvtxRange range( "engine.chunk" );
    std::vector<Job *> act;
    std::vector<gbmd_ctx *> batch, nbatch;
    std::vector<char> bth, blast, nth, nlast;
    for ( Job *j : e->running )
        j->ring_steps.clear();
    // force + integrate (+ thermo sums) of one step for each job: mixed LJ
    // full-list jobs in one job-table launch, batchable NNP jobs in one
    // job-table step per NNP stream, the others per job
    auto forces = [&]( const std::vector<Job *> &jobs ) -> int {
        batch.clear();
        bth.clear();
        blast.clear();
        nbatch.clear();
        nth.clear();
        nlast.clear();
        for ( Job *j : jobs )
        {
            if ( j->state != GBMD_JOB_RUNNING )
                continue;
            gbmd_ctx *c = j->c;
            const int64_t step = ++c->step;
            e->st.atom_steps_run += j->n;
            const bool th = j->spec.md.thermo_every > 0 && step % j->spec.md.thermo_every == 0;
            const bool last = step == j->spec.nsteps;
            if ( lj_batchable( c ) )
            {
                batch.push_back( c );
                bth.push_back( th );
                blast.push_back( last );
            }
            else if ( gbmd_nnp_batchable( c ) )
            {
                nbatch.push_back( c );
                nth.push_back( th );
                nlast.push_back( last );
            }
            else if ( int rc = gbmd_job_force_step( c, th, last ) )
                job_fail( e, j, rc, gbmd_last_error( c ) );
        }
        // one job-table batch per stream
        for ( int sidx = 1; sidx <= GBMD_NNP_STREAMS && !nbatch.empty(); sidx++ )
        {
            std::vector<gbmd_ctx *> grp;
            std::vector<char> g1, g2;
            for ( size_t q = 0; q < nbatch.size(); q++ )
                if ( nbatch[q]->stream == e->streams[sidx] )
                {
                    grp.push_back( nbatch[q] );
                    g1.push_back( nth[q] );
                    g2.push_back( nlast[q] );
                }
            if ( grp.empty() )
                continue;
            std::unique_ptr<bool[]> t1( new bool[grp.size()] ), t2( new bool[grp.size()] );
            for ( size_t q = 0; q < grp.size(); q++ )
            {
                t1[q] = g1[q] != 0;
                t2[q] = g2[q] != 0;
            }
            if ( int rc = gbmd_nnp_step_batch( grp.data(), t1.get(), t2.get(), (int)grp.size(),
                                               &e->st.launches ) )
                return efail( e, rc, std::string( "batched NNP step: " ) +
                                         gbmd_last_error( grp[0] ) );
        }
        if ( batch.empty() )
            return GBMD_OK;
        std::unique_ptr<bool[]> t1( new bool[batch.size()] ), t2( new bool[batch.size()] );
        for ( size_t q = 0; q < batch.size(); q++ )
        {
            t1[q] = bth[q] != 0;
            t2[q] = blast[q] != 0;
        }
        if ( int rc = gbmd_lj_step_batch( batch.data(), t1.get(), t2.get(), (int)batch.size(),
                                          &e->st.launches ) )
            return efail( e, rc, std::string( "batched LJ step: " ) +
                                     gbmd_last_error( batch[0] ) );
        return GBMD_OK;
    };
    // thermo sums of the jobs' current step to the pinned ring (thermo steps)
    auto thermo_copy = [&]( const std::vector<Job *> &jobs ) -> int {
        for ( Job *j : jobs )
        {
            if ( j->state != GBMD_JOB_RUNNING )
                continue;
            const int64_t step = j->c->step;
            if ( j->spec.md.thermo_every > 0 && step % j->spec.md.thermo_every == 0 )
            {
                const size_t r = j->ring_steps.size();
                double *dst = e->h_ring + ( (size_t)j->slot * e->chunk + r ) * 4;
                if ( cudaMemcpyAsync( dst, j->c->red_out.p, 4 * sizeof( double ),
                                      cudaMemcpyDeviceToHost, j->c->stream ) != cudaSuccess )
                    return efail( e, GBMD_ERR_CUDA, "thermo copy failed" );
                j->ring_steps.push_back( step );
            }
        }
        return GBMD_OK;
    };
    // Jobs' contexts grouped by their stream, in first-seen order.
    using StreamGroups = std::vector<std::pair<cudaStream_t, std::vector<gbmd_ctx *>>>;
    auto add_to_group = []( StreamGroups &g, gbmd_ctx *c ) {
        for ( auto &kv : g )
            if ( kv.first == c->stream )
            {
                kv.second.push_back( c );
                return;
            }
        g.push_back( { c->stream, { c } } );
    };
    // Wait for the rebuilt lists of `jobs` (each job's event only), check
    // their capacities and rebuild where a list overflowed (again waiting);
    // the accepted lists' rows are padded in one job-table launch per stream.
    auto finish_rebuilds = [&]( std::vector<Job *> due ) -> int {
        while ( !due.empty() )
        {
            std::vector<Job *> again;
            StreamGroups pads;
            for ( Job *j : due )
            {
                if ( j->state != GBMD_JOB_RUNNING )
                    continue;
                const double tw = now_s( e );
                const cudaError_t ew = cudaEventSynchronize( j->built );
                e->st.wait_seconds += now_s( e ) - tw;
                if ( ew != cudaSuccess )
                    return efail( e, GBMD_ERR_CUDA, "engine stream failed during a rebuild" );
                bool more = false;
                if ( int rc = gbmd_rebuild_check( j->c, &more ) )
                    job_fail( e, j, rc, gbmd_last_error( j->c ) );
                else if ( more )
                {
                    int rc2 = gbmd_build_list_launch( j->c );
                    if ( !rc2 && cudaEventRecord( j->built, j->c->stream ) != cudaSuccess )
                        rc2 = gbmd_fail( j->c, GBMD_ERR_CUDA, "rebuild event record failed" );
                    if ( rc2 )
                        job_fail( e, j, rc2, gbmd_last_error( j->c ) );
                    else
                        again.push_back( j );
                }
                else
                    add_to_group( pads, j->c );
            }
            for ( auto &kv : pads )
                if ( int rc = gbmd_pad_lists_batch( kv.second.data(), (int)kv.second.size(),
                                                    &e->st.launches ) )
                    return efail( e, rc, std::string( "batched list padding: " ) +
                                             gbmd_last_error( kv.second[0] ) );
            due.swap( again );
        }
        return GBMD_OK;
    };
    // Mark a job's launched rebuild with its event and file it for the
    // capacity check (at once when it rebuilds every step, else one
    // iteration later).
    auto mark_rebuild = [&]( Job *j, int rc, std::vector<Job *> &due,
                             std::vector<Job *> &due_now ) {
        if ( !rc && !j->built &&
             cudaEventCreateWithFlags( &j->built, cudaEventDisableTiming ) != cudaSuccess )
            rc = gbmd_fail( j->c, GBMD_ERR_CUDA, "rebuild event creation failed" );
        if ( !rc && cudaEventRecord( j->built, j->c->stream ) != cudaSuccess )
            rc = gbmd_fail( j->c, GBMD_ERR_CUDA, "rebuild event record failed" );
        if ( rc )
            job_fail( e, j, rc, gbmd_last_error( j->c ) );
        else if ( j->spec.md.rebuild_every < 2 )
            due_now.push_back( j );
        else
            due.push_back( j );
    };
    // A job whose rebuild is due at a step launches it and then lags one
    // iteration: its list check (a host wait on that job's event) and its
    // force come after the next step's work of every other job has been
    // issued, so the GPU still has work queued while the host waits, and
    // the job catches up by doing two steps in that iteration.  Each job's
    // launches keep their order on its stream, so results do not change.
    // Jobs rebuilding every step take the check at once.
    std::vector<Job *> lag;
    for ( int k = 0; k < e->chunk; k++ )
    {
        act.clear();
        for ( Job *j : e->running )
            if ( j->state == GBMD_JOB_RUNNING && j->c->step < j->spec.nsteps &&
                 std::find( lag.begin(), lag.end(), j ) == lag.end() )
                act.push_back( j );
        if ( act.empty() && lag.empty() )
            break;
        // 1. first step: initial integrate (later ones are fused)
        for ( Job *j : act )
            if ( j->c->step == 0 && gbmd_nve_initial_launch( j->c ) )
                job_fail( e, j, GBMD_ERR_CUDA, gbmd_last_error( j->c ) );
        // 2. rebuilds due at this step, launched now, each marked by an event:
        //    the jobs sharing a stream in job-table launches (wrap, sort and
        //    list build of all of them, gbmd_rebuild_batch_launch), the
        //    others (profiled contexts, very large grids) one by one
        std::vector<Job *> due, due_now, rest, batched;
        StreamGroups rb;
        for ( Job *j : act )
        {
            if ( j->state != GBMD_JOB_RUNNING )
                continue;
            if ( ( j->c->step + 1 ) % j->spec.md.rebuild_every != 0 )
            {
                rest.push_back( j );
                continue;
            }
            if ( gbmd_rebuild_batchable( j->c ) )
            {
                if ( int rc = gbmd_rebuild_prepare( j->c ) )
                    job_fail( e, j, rc, gbmd_last_error( j->c ) );
                else
                {
                    add_to_group( rb, j->c );
                    batched.push_back( j );
                }
                continue;
            }
            mark_rebuild( j, gbmd_rebuild_launch( j->c ), due, due_now );
        }
        for ( auto &kv : rb )
        {
            if ( int rc = gbmd_rebuild_batch_launch( kv.second.data(), (int)kv.second.size(),
                                                     &e->st.launches ) )
                return efail( e, rc, std::string( "batched rebuild: " ) +
                                         gbmd_last_error( kv.second[0] ) );
            e->st.batched_rebuilds += (int64_t)kv.second.size();
        }
        for ( Job *j : batched )
            mark_rebuild( j, GBMD_OK, due, due_now );
        // 3. force + integrate of the jobs without a rebuild
        if ( int rc = forces( rest ) )
            return rc;
        // 4. the jobs rebuilt one iteration ago: their lists, their delayed
        //    step, then this step
        if ( !lag.empty() )
        {
            if ( int rc = finish_rebuilds( lag ) )
                return rc;
            if ( int rc = forces( lag ) )
                return rc;
            if ( int rc = thermo_copy( lag ) )
                return rc;
            std::vector<Job *> more;
            for ( Job *j : lag )
                if ( j->state == GBMD_JOB_RUNNING && j->c->step < j->spec.nsteps )
                    more.push_back( j );
            if ( int rc = forces( more ) )
                return rc;
            rest.insert( rest.end(), more.begin(), more.end() );
        }
        // 5. jobs rebuilding every step: checked at once
        if ( !due_now.empty() )
        {
            if ( int rc = finish_rebuilds( due_now ) )
                return rc;
            if ( int rc = forces( due_now ) )
                return rc;
            rest.insert( rest.end(), due_now.begin(), due_now.end() );
        }
        // 6. thermo sums to the pinned ring
        if ( int rc = thermo_copy( rest ) )
            return rc;
        lag.swap( due );
    }
    // the jobs rebuilt in the last iteration
    if ( !lag.empty() )
    {
        if ( int rc = finish_rebuilds( lag ) )
            return rc;
        if ( int rc = forces( lag ) )
            return rc;
        if ( int rc = thermo_copy( lag ) )
            return rc;
    }
    // end of chunk: flags, one synchronisation, rows, retirements
    for ( Job *j : e->running )
        if ( j->state == GBMD_JOB_RUNNING &&
             cudaMemcpyAsync( j->c->h_flags, j->c->flags.p, 4 * sizeof( int ),
                              cudaMemcpyDeviceToHost, j->c->stream ) != cudaSuccess )
            return efail( e, GBMD_ERR_CUDA, "flag copy failed" );
    {
        const double tw = now_s( e );
        const bool ok = sync_all( e );
        e->st.wait_seconds += now_s( e ) - tw;
        if ( !ok )
            return efail( e, GBMD_ERR_CUDA, "engine stream failed" );
    }
    const double tr = now_s( e );
    struct AddR
    {
        gbmd_engine *e;
        double t0;
        ~AddR() { e->st.retire_seconds += now_s( e ) - t0; }
    } addr{ e, tr };
    std::vector<Job *> keep;
    for ( Job *j : e->running )
    {
        if ( j->state == GBMD_JOB_RUNNING )
        {
            for ( size_t r = 0; r < j->ring_steps.size(); r++ )
            {
                double row[4];
                gbmd_thermo_row_from( j->c, j->ring_steps[r],
                                      e->h_ring + ( (size_t)j->slot * e->chunk + r ) * 4, row );
                j->rows.insert( j->rows.end(), row, row + 4 );
            }
            if ( int rc = gbmd_check_flags( j->c ) )
                job_fail( e, j, rc, gbmd_last_error( j->c ) );
        }
        if ( j->state == GBMD_JOB_RUNNING && j->c->step >= j->spec.nsteps )
            retire( e, j );
        if ( j->state == GBMD_JOB_RUNNING )
            keep.push_back( j );
        else if ( j->c || j->slot >= 0 )
        {
            if ( j->c )
                e->st.launches += j->c->launches;
            release_job_device( e, j );
        }
    }
    e->running.swap( keep );
    e->st.chunks++;
    return GBMD_OK;
}

extern "C" {

int gbmd_engine_create( gbmd_engine **out, int device, uint64_t budget_bytes, int max_running,
                        int chunk )
{
    if ( !out )
        return GBMD_ERR_ARG;
    *out = nullptr;
    if ( max_running <= 0 || budget_bytes == 0 || chunk < 0 )
        return GBMD_ERR_ARG;
    int ndev = 0;
    if ( cudaGetDeviceCount( &ndev ) != cudaSuccess || ndev <= 0 )
        return GBMD_ERR_NODEVICE;
    if ( device < 0 || device >= ndev || cudaSetDevice( device ) != cudaSuccess )
        return GBMD_ERR_ARG;
    gbmd_engine *e = new gbmd_engine();
    e->device = device;
    e->budget = budget_bytes;
    e->max_running = max_running;
    e->chunk = chunk ? chunk : 10;
    e->t0 = std::chrono::steady_clock::now();
    bool streams_ok = true;
    for ( int k = 0; k < GBMD_ENGINE_STREAMS && streams_ok; k++ )
    {
        cudaStream_t st = nullptr;
        streams_ok = cudaStreamCreateWithFlags( &st, cudaStreamNonBlocking ) == cudaSuccess;
        if ( streams_ok )
            e->streams.push_back( st );
    }
    if ( !streams_ok ||
         cudaMallocHost( (void **)&e->h_red, sizeof( double ) * 8 * max_running ) !=
             cudaSuccess ||
         cudaMallocHost( (void **)&e->h_flags, sizeof( int ) * 8 * max_running ) !=
             cudaSuccess ||
         cudaMallocHost( (void **)&e->h_ring, sizeof( double ) * 4 * e->chunk * max_running ) !=
             cudaSuccess )
    {
        gbmd_engine_destroy( e );
        return GBMD_ERR_CUDA;
    }
    for ( int s = max_running - 1; s >= 0; s-- )
        e->free_slots.push_back( s );
    e->st.budget_bytes = budget_bytes;
    *out = e;
    return GBMD_OK;
}

void gbmd_engine_destroy( gbmd_engine *e )
{
    if ( !e )
        return;
    cudaSetDevice( e->device );
    sync_all( e );
    for ( auto &kv : e->jobs )
    {
        if ( kv.second->built )
            cudaEventDestroy( kv.second->built );
        if ( kv.second->c )
            gbmd_destroy( kv.second->c );
    }
    if ( e->h_red )
        cudaFreeHost( e->h_red );
    if ( e->h_flags )
        cudaFreeHost( e->h_flags );
    if ( e->h_ring )
        cudaFreeHost( e->h_ring );
    sync_all( e );
    for ( cudaStream_t st : e->streams )
        cudaStreamDestroy( st );
    delete e;
}

const char *gbmd_engine_last_error( const gbmd_engine *e )
{
    return e ? e->err.c_str() : "null engine";
}

double gbmd_engine_now( const gbmd_engine *e ) { return e ? now_s( e ) : 0.0; }

int gbmd_job_submit( gbmd_engine *e, const gbmd_job_spec *spec, int64_t n, const double *x,
                     const double *v, const int *type, const int *id, double arrival,
                     int64_t *job_id )
{
    if ( !e || !spec || !job_id )
        return GBMD_ERR_ARG;
    if ( n < 2 || n > GBMD_MAX_ATOMS || !x || !v || !type || !id )
        return efail( e, GBMD_ERR_ARG, "job_submit: need n >= 2 atoms with x, v, type, id" );
    if ( spec->force_type != GBMD_FORCE_LJ && spec->force_type != GBMD_FORCE_NNP )
        return efail( e, GBMD_ERR_ARG, "job_submit: unknown force type" );
    if ( spec->force_type == GBMD_FORCE_NNP && !spec->nnp_dir )
        return efail( e, GBMD_ERR_ARG, "job_submit: NNP job without a potential directory" );
    if ( spec->nsteps < 0 || !( spec->md.force_cut > 0 ) || spec->md.rebuild_every < 1 )
        return efail( e, GBMD_ERR_ARG, "job_submit: bad step count or MD parameters" );
    for ( int64_t k = 0; k < n; k++ )
        if ( type[k] != 0 )
            return efail( e, GBMD_ERR_ARG, "job_submit: jobs have one atom type (0)" );
    std::unique_ptr<Job> j( new Job() );
    j->jid = e->next_id++;
    j->spec = *spec;
    if ( spec->nnp_dir )
        j->nnp_dir = spec->nnp_dir;
    j->spec.nnp_dir = nullptr;
    j->n = n;
    j->x.assign( x, x + 3 * n );
    j->v.assign( v, v + 3 * n );
    j->type.assign( type, type + n );
    j->id.assign( id, id + n );
    const double t = now_s( e );
    j->t_arrival = arrival >= 0 && arrival <= t ? arrival : t;
    j->est_bytes = estimate_bytes( *spec, n );
    *job_id = j->jid;
    e->queue.push_back( j.get() );
    e->jobs[j->jid] = std::move( j );
    e->st.submitted++;
    return GBMD_OK;
}

int gbmd_engine_step( gbmd_engine *e, int *running, int *queued, int *finished )
{
    if ( !e )
        return GBMD_ERR_ARG;
    cudaSetDevice( e->device );
    const double t_begin = now_s( e );
    const int64_t fin0 = e->st.finished + e->st.failed;
    admit_queued( e );
    int rc = GBMD_OK;
    if ( !e->running.empty() )
        rc = run_chunk( e );
    admit_queued( e ); // slots freed by this chunk
    e->st.busy_seconds += now_s( e ) - t_begin;
    if ( running )
        *running = (int)e->running.size();
    if ( queued )
        *queued = (int)e->queue.size();
    if ( finished )
        *finished = (int)( e->st.finished + e->st.failed - fin0 );
    return rc;
}

int gbmd_job_poll( gbmd_engine *e, int64_t job_id, int *state, int *error, double *times )
{
    if ( !e )
        return GBMD_ERR_ARG;
    auto it = e->jobs.find( job_id );
    if ( it == e->jobs.end() )
        return efail( e, GBMD_ERR_ARG, "job_poll: unknown job" );
    const Job &j = *it->second;
    if ( state )
        *state = j.state;
    if ( error )
        *error = j.error;
    if ( times )
    {
        times[0] = j.t_arrival;
        times[1] = j.t_admit;
        times[2] = j.t_finish;
    }
    return GBMD_OK;
}

const char *gbmd_job_error( gbmd_engine *e, int64_t job_id )
{
    if ( !e )
        return "null engine";
    auto it = e->jobs.find( job_id );
    return it == e->jobs.end() ? "unknown job" : it->second->err.c_str();
}

int gbmd_job_result( gbmd_engine *e, int64_t job_id, int64_t *n, double *x, double *v, double *f,
                     int *type, int *id, double *thermo, int max_rows, int *nrows )
{
    if ( !e )
        return GBMD_ERR_ARG;
    auto it = e->jobs.find( job_id );
    if ( it == e->jobs.end() )
        return efail( e, GBMD_ERR_ARG, "job_result: unknown job" );
    const Job &j = *it->second;
    if ( j.state != GBMD_JOB_DONE )
        return efail( e, GBMD_ERR_ARG, "job_result: job is not done" );
    if ( n )
        *n = j.n;
    if ( x )
        std::copy( j.x.begin(), j.x.end(), x );
    if ( v )
        std::copy( j.v.begin(), j.v.end(), v );
    if ( f )
        std::copy( j.f.begin(), j.f.end(), f );
    if ( type )
        std::copy( j.type.begin(), j.type.end(), type );
    if ( id )
        std::copy( j.id.begin(), j.id.end(), id );
    const int have = (int)( j.rows.size() / 4 );
    const int put = thermo ? std::min( have, std::max( max_rows, 0 ) ) : 0;
    if ( put )
        std::copy( j.rows.begin(), j.rows.begin() + 4 * put, thermo );
    if ( nrows )
        *nrows = thermo ? put : have;
    return GBMD_OK;
}

int gbmd_job_cancel( gbmd_engine *e, int64_t job_id )
{
    if ( !e )
        return GBMD_ERR_ARG;
    auto it = e->jobs.find( job_id );
    if ( it == e->jobs.end() )
        return efail( e, GBMD_ERR_ARG, "job_cancel: unknown job" );
    Job *j = it->second.get();
    if ( j->state == GBMD_JOB_QUEUED )
        e->queue.erase( std::remove( e->queue.begin(), e->queue.end(), j ), e->queue.end() );
    else if ( j->state == GBMD_JOB_RUNNING )
    {
        // gbmd_engine_step ends with every stream drained, so nothing of
        // this job is in flight; its memory and slot go back to the pool
        cudaSetDevice( e->device );
        release_job_device( e, j );
        e->running.erase( std::remove( e->running.begin(), e->running.end(), j ),
                          e->running.end() );
    }
    else
        return efail( e, GBMD_ERR_ARG, "job_cancel: job has finished" );
    job_fail( e, j, GBMD_ERR_CANCELLED, "cancelled" );
    e->st.cancelled++;
    return GBMD_OK;
}

int gbmd_job_release( gbmd_engine *e, int64_t job_id )
{
    if ( !e )
        return GBMD_ERR_ARG;
    auto it = e->jobs.find( job_id );
    if ( it == e->jobs.end() )
        return efail( e, GBMD_ERR_ARG, "job_release: unknown job" );
    if ( it->second->state != GBMD_JOB_DONE && it->second->state != GBMD_JOB_FAILED )
        return efail( e, GBMD_ERR_ARG, "job_release: job has not finished" );
    e->jobs.erase( it );
    return GBMD_OK;
}

int gbmd_engine_get_stats( const gbmd_engine *e, gbmd_engine_stats *out )
{
    if ( !e || !out )
        return GBMD_ERR_ARG;
    *out = e->st;
    out->running = (int64_t)e->running.size();
    out->queued = (int64_t)e->queue.size();
    out->used_bytes = e->used;
    out->peak_used_bytes = e->peak;
    out->budget_bytes = e->budget;
    return GBMD_OK;
}

} // extern "C"
