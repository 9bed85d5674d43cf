// gbmd_nnp.cu -- neural-network potential: Behler-Parrinello symmetry
// functions, the per-element MLP, and forces through dE/dG.
//
// Reference call sites (paths inside the CabanaMD project):
//   src/force_types/force_nnp_cabana_neigh_impl.h:41-66   ForceNNP::init_coeff
//     loads <dir>/input.nn, scaling.data, weights.%03zu.data through n2p2
//   :68-99    compute: calculateSymmetryFunctionGroups -> calculate-
//             AtomicNeuralNetworks -> calculateForces (n2p2 v2.0.1)
//   :101-130  compute_energy: ((sum E_i + N_local offset) / convEnergy
//             + N meanEnergy) * 27.211384021355236
// n2p2 itself is not vendored; the arithmetic follows the published
// definitions (symmetry function types 2 and 3, cosine cutoff):
//   fc(r) = 0.5 (cos(pi r / rc) + 1) for r < rc
//   G2_i = sum_j exp(-eta (r_ij - rs)^2) fc(r_ij)
//   G3_i = 2^(1-zeta) sum_{j<k} (1 + lambda cos t)^zeta
//          exp(-eta (r_ij^2 + r_ik^2 + r_jk^2)) fc(r_ij) fc(r_ik) fc(r_jk)
//
// GB300 design.  One warp per atom: the lanes gather the atom's neighbours
// inside rc into shared memory, then split the j<k triplets; per triplet the
// geometry, the distinct exponentials (one per distinct eta) and the
// distinct powers (one per distinct (lambda, zeta)) are computed once and
// shared by all angular functions.  The force pass recomputes the triplet
// geometry and folds the 24 angular dE/dG weights into three scalar
// coefficients (of dcos, dR^2 and dF) before the vector math; per-neighbour
// forces collect in shared memory and reach the owners with one FP64 atomic
// per neighbour.  FP64 and FP32 ("mixed") instantiate the same kernels; in
// mixed precision the MLP runs as BF16 tensor-core tiles (gbmd_nnp_mlp_tc.cu)
// and forces accumulate in FP64.
#include "gbmd_internal.cuh"

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>

#include "gbmd_nnp.cuh"

#include <atomic>

// ---------------------------------------------------------------------------
// host: n2p2 file parsing
static const char *kElements[] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",
    "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn",
    "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh",
    "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd",
    "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re",
    "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi" };

struct SfDef
{
    int type;
    int ec;     // centre element (atomic number)
    int z1, z2; // neighbour elements (atomic numbers; z1 <= z2, z2 = 0 for radial)
    double eta, rs, lam, zeta, rc;
    bool operator<( const SfDef &o ) const
    {
        // n2p2's canonical order (also scaling.data's row order)
        if ( type != o.type ) return type < o.type;
        if ( rc != o.rc ) return rc < o.rc;
        if ( z1 != o.z1 ) return z1 < o.z1;
        if ( z2 != o.z2 ) return z2 < o.z2;
        if ( eta != o.eta ) return eta < o.eta;
        if ( zeta != o.zeta ) return zeta < o.zeta;
        if ( lam != o.lam ) return lam < o.lam;
        return rs < o.rs;
    }
};

static int atomic_number( const std::string &sym )
{
    for ( int k = 0; k < (int)( sizeof( kElements ) / sizeof( kElements[0] ) ); k++ )
        if ( sym == kElements[k] )
            return k + 1;
    return 0;
}

static std::vector<std::string> split_ws( const std::string &s )
{
    std::istringstream is( s.substr( 0, s.find( '#' ) ) );
    std::vector<std::string> t;
    std::string w;
    while ( is >> w )
        t.push_back( w );
    return t;
}

// One element's function set (sorted) -> its parameter block: radial
// functions with their neighbour element, angular functions on per-channel
// (eta, (lambda, zeta)) grids.  zs: the potential's elements (atomic
// numbers, ascending).
static int build_params( gbmd_ctx *c, const std::vector<SfDef> &sfs, const std::vector<int> &zs,
                         int elem, NnpParams &p )
{
    auto index_of = [&]( int z ) {
        return (int)( std::find( zs.begin(), zs.end(), z ) - zs.begin() );
    };
    p.nsf = (int)sfs.size();
    p.elem = elem;
    p.nelem = (int)zs.size();
    p.rc = sfs[0].rc;
    for ( auto &s : sfs )
        if ( s.rc != p.rc )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: all functions must share one cutoff" );
    std::vector<double> etas;
    std::vector<std::pair<double, double>> lzs;
    std::vector<std::pair<int, int>> chs;
    for ( auto &s : sfs )
        if ( s.type == 2 )
        {
            p.eta_r[p.nrad] = s.eta;
            p.rs_r[p.nrad] = s.rs;
            p.rad_e1[p.nrad] = index_of( s.z1 );
            p.nrad++;
        }
    std::vector<int> ang_ch;
    for ( auto &s : sfs )
        if ( s.type == 3 )
        {
            if ( s.rs != 0.0 )
                return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: angular rs must be 0" );
            auto ie = std::find( etas.begin(), etas.end(), s.eta );
            if ( ie == etas.end() )
            {
                etas.push_back( s.eta );
                ie = etas.end() - 1;
            }
            auto lz = std::make_pair( s.lam, s.zeta );
            auto il = std::find( lzs.begin(), lzs.end(), lz );
            if ( il == lzs.end() )
            {
                lzs.push_back( lz );
                il = lzs.end() - 1;
            }
            auto ch = std::make_pair( index_of( s.z1 ), index_of( s.z2 ) );
            auto ic = std::find( chs.begin(), chs.end(), ch );
            if ( ic == chs.end() )
            {
                chs.push_back( ch );
                ic = chs.end() - 1;
            }
            p.ang_eta[p.nang] = (int)( ie - etas.begin() );
            p.ang_lz[p.nang] = (int)( il - lzs.begin() );
            p.ang_pre[p.nang] = std::pow( 2.0, 1.0 - s.zeta );
            ang_ch.push_back( (int)( ic - chs.begin() ) );
            p.nang++;
        }
    if ( (int)etas.size() > NNP_MAXETA || (int)lzs.size() > NNP_MAXLZ )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: too many distinct eta or (lambda, zeta)" );
    if ( (int)chs.size() > NNP_MAXCH )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: too many neighbour-element pairs" );
    if ( p.nrad > 16 )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: at most 16 radial functions" );
    p.neta = (int)etas.size();
    p.nlz = (int)lzs.size();
    p.nch = chs.empty() ? 1 : (int)chs.size();
    for ( int k = 0; k < NNP_MAXCH; k++ )
    {
        p.ch_e1[k] = k < (int)chs.size() ? chs[k].first : 0;
        p.ch_e2[k] = k < (int)chs.size() ? chs[k].second : 0;
    }
    for ( int h = 0; h < NNP_MAXCH; h++ )
        for ( int e = 0; e < NNP_MAXETA; e++ )
            for ( int l = 0; l < NNP_MAXLZ; l++ )
                p.grid_sf[h][e][l] = -1;
    for ( int s2 = 0; s2 < p.nang; s2++ )
    {
        int &slot = p.grid_sf[ang_ch[s2]][p.ang_eta[s2]][p.ang_lz[s2]];
        if ( slot >= 0 )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: duplicate angular function" );
        slot = s2;
    }
    for ( int k = 0; k < p.neta; k++ )
        p.eta_u[k] = etas[k];
    for ( int k = 0; k < p.nlz; k++ )
    {
        p.lam_u[k] = lzs[k].first;
        p.zeta_u[k] = lzs[k].second;
        const double z = lzs[k].second;
        p.zeta_int[k] = ( z >= 1.0 && z <= 64.0 && z == std::floor( z ) ) ? (int)z : 0;
    }
    // power ladder (mixed-precision kernels): lambda = +-1 and zeta a power
    // of two up to 32, mapped per channel
    p.lad_ok = p.nang > 0 ? 1 : 0;
    p.lad_mask = 0;
    for ( int h = 0; h < NNP_MAXCH; h++ )
        for ( int e = 0; e < NNP_MAXETA; e++ )
            for ( int q = 0; q < 2; q++ )
                for ( int mm = 0; mm < 6; mm++ )
                    p.lad_sf[h][e][q][mm] = -1;
    for ( int s2 = 0; s2 < p.nang && p.lad_ok; s2++ )
    {
        const double lam = p.lam_u[p.ang_lz[s2]], z = p.zeta_u[p.ang_lz[s2]];
        int mm = -1;
        for ( int k = 0; k < 6; k++ )
            if ( z == (double)( 1 << k ) )
                mm = k;
        if ( ( lam != 1.0 && lam != -1.0 ) || mm < 0 )
        {
            p.lad_ok = 0;
            break;
        }
        p.lad_sf[ang_ch[s2]][p.ang_eta[s2]][lam > 0 ? 1 : 0][mm] = s2;
        p.lad_mask |= 1 << mm;
    }
    return GBMD_OK;
}

static int load_model( gbmd_ctx *c, const std::string &dir, double cflength, double cfenergy,
                       NnpModel &m )
{
    std::ifstream in( dir + "/input.nn" );
    if ( !in )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: cannot open " + dir + "/input.nn" );
    std::vector<std::string> elements;
    std::map<std::string, double> atom_energy;
    std::vector<SfDef> sfs;
    std::vector<int> hidden;
    std::string acts;
    int cutoff_type = -1;
    double smin = 0.0, smax = 1.0;
    bool scale = false;
    std::string line;
    try
    {
        while ( std::getline( in, line ) )
        {
            auto t = split_ws( line );
            if ( t.empty() )
                continue;
            const std::string &k = t[0];
            if ( k == "elements" )
                elements.assign( t.begin() + 1, t.end() );
            else if ( k == "atom_energy" && t.size() >= 3 )
                atom_energy[t[1]] = std::stod( t[2] );
            else if ( k == "cutoff_type" )
                cutoff_type = std::stoi( t.at( 1 ) );
            else if ( k == "scale_symmetry_functions" )
                scale = true;
            else if ( k == "scale_min_short" )
                smin = std::stod( t.at( 1 ) );
            else if ( k == "scale_max_short" )
                smax = std::stod( t.at( 1 ) );
            else if ( k == "global_nodes_short" )
                for ( size_t q = 1; q < t.size(); q++ )
                    hidden.push_back( std::stoi( t[q] ) );
            else if ( k == "global_activation_short" )
                for ( size_t q = 1; q < t.size(); q++ )
                    acts += t[q];
            else if ( k == "symfunction_short" )
            {
                const int type = std::stoi( t.at( 2 ) );
                SfDef s{};
                s.type = type;
                s.ec = atomic_number( t.at( 1 ) );
                if ( type == 2 )
                {
                    s.z1 = atomic_number( t.at( 3 ) );
                    s.eta = std::stod( t.at( 4 ) );
                    s.rs = std::stod( t.at( 5 ) );
                    s.rc = std::stod( t.at( 6 ) );
                }
                else if ( type == 3 )
                {
                    const int za = atomic_number( t.at( 3 ) ), zb = atomic_number( t.at( 4 ) );
                    s.z1 = std::min( za, zb );
                    s.z2 = std::max( za, zb );
                    s.eta = std::stod( t.at( 5 ) );
                    s.lam = std::stod( t.at( 6 ) );
                    s.zeta = std::stod( t.at( 7 ) );
                    s.rc = std::stod( t.at( 8 ) );
                    s.rs = t.size() > 9 ? std::stod( t[9] ) : 0.0;
                }
                else
                    return gbmd_fail( c, GBMD_ERR_IO,
                                      "nnp_load: only symmetry function types 2 and 3" );
                if ( !s.ec || !s.z1 || ( type == 3 && !s.z2 ) )
                    return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: unknown element in " + line );
                sfs.push_back( s );
            }
        }
    }
    catch ( const std::exception &e )
    {
        return gbmd_fail( c, GBMD_ERR_IO, std::string( "nnp_load: input.nn parse error: " ) +
                                              e.what() );
    }
    // n2p2's element map: elements indexed in order of atomic number
    std::vector<int> zs;
    for ( auto &el : elements )
    {
        const int z = atomic_number( el );
        if ( !z )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: unknown element " + el );
        zs.push_back( z );
    }
    std::sort( zs.begin(), zs.end() );
    if ( zs.empty() || (int)zs.size() > NNP_MAXELEM ||
         std::adjacent_find( zs.begin(), zs.end() ) != zs.end() )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: 1..4 distinct elements" );
    if ( cutoff_type != 1 )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: only cutoff_type 1 (cosine)" );
    if ( !scale )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: scale_symmetry_functions required" );
    if ( hidden.empty() || (int)hidden.size() + 1 > NNP_MAXLAYERS )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: 1..3 hidden layers" );
    if ( acts.size() != hidden.size() + 1 )
        return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: one activation per layer" );
    const int ne = (int)zs.size();
    m.pe.assign( ne, NnpParams{} );
    m.w.clear();
    m.b.clear();
    m.gstride = 0;
    for ( int el = 0; el < ne; el++ )
    {
        std::vector<SfDef> mine;
        for ( auto &s : sfs )
            if ( s.ec == zs[el] )
            {
                if ( std::find( zs.begin(), zs.end(), s.z1 ) == zs.end() ||
                     ( s.type == 3 && std::find( zs.begin(), zs.end(), s.z2 ) == zs.end() ) )
                    return gbmd_fail( c, GBMD_ERR_IO,
                                      "nnp_load: a neighbour element is not in 'elements'" );
                mine.push_back( s );
            }
        if ( mine.empty() || (int)mine.size() > NNP_MAXSF )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: 1..64 symmetry functions per element" );
        std::sort( mine.begin(), mine.end() );
        NnpParams &p = m.pe[el];
        int rc;
        if ( ( rc = build_params( c, mine, zs, el, p ) ) )
            return rc;
        m.gstride = std::max( m.gstride, p.nsf );
        // layers
        p.nl = (int)hidden.size() + 1;
        p.nodes[0] = p.nsf;
        for ( int l = 1; l <= p.nl; l++ )
        {
            p.nodes[l] = l < p.nl ? hidden[l - 1] : 1;
            if ( p.nodes[l] > NNP_MAXNODES )
                return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: at most 64 nodes per layer" );
            p.act[l] = acts[l - 1];
            if ( std::string( "tpsl" ).find( p.act[l] ) == std::string::npos )
                return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: activations t, p, s, l only" );
        }
        // weights.%03d.data (atomic number), appended to the shared arrays
        int wo = (int)m.w.size(), bo = (int)m.b.size();
        const int wbase = wo, bbase = bo;
        for ( int l = 1; l <= p.nl; l++ )
        {
            p.woff[l] = wo;
            p.boff[l] = bo;
            wo += p.nodes[l] * p.nodes[l - 1];
            bo += p.nodes[l];
        }
        m.w.resize( wo, 0.0 );
        m.b.resize( bo, 0.0 );
        char name[32];
        snprintf( name, sizeof( name ), "/weights.%03d.data", zs[el] );
        std::ifstream wf( dir + name );
        if ( !wf )
            return gbmd_fail( c, GBMD_ERR_IO, std::string( "nnp_load: cannot open " ) + dir + name );
        int nread = 0;
        while ( std::getline( wf, line ) )
        {
            auto t = split_ws( line );
            if ( t.size() < 5 )
                continue;
            const double val = std::stod( t[0] );
            if ( t[1] == "a" && t.size() >= 7 )
            {
                const int lf = std::stoi( t[3] ), nf = std::stoi( t[4] ) - 1;
                const int lt = std::stoi( t[5] ), nt = std::stoi( t[6] ) - 1;
                if ( lt != lf + 1 || lt < 1 || lt > p.nl || nf < 0 || nf >= p.nodes[lf] ||
                     nt < 0 || nt >= p.nodes[lt] )
                    return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: weight index out of range" );
                m.w[p.woff[lt] + nt * p.nodes[lf] + nf] = val;
                nread++;
            }
            else if ( t[1] == "b" )
            {
                const int l = std::stoi( t[3] ), nd = std::stoi( t[4] ) - 1;
                if ( l < 1 || l > p.nl || nd < 0 || nd >= p.nodes[l] )
                    return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: bias index out of range" );
                m.b[p.boff[l] + nd] = val;
                nread++;
            }
        }
        if ( nread != ( wo - wbase ) + ( bo - bbase ) )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: weight count does not match the layers" );
        p.e_offset = atom_energy.count( kElements[zs[el] - 1] )
                         ? atom_energy[kElements[zs[el] - 1]]
                         : 0.0;
        p.cflength = cflength;
        p.cfenergy = cfenergy;
        p.smin = smin;
    }
    // scaling.data: element index (atomic-number order, 1-based), function
    // index, Gmin, Gmax, ...
    {
        std::ifstream sc( dir + "/scaling.data" );
        if ( !sc )
            return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: cannot open scaling.data" );
        std::vector<std::vector<int>> seen( ne );
        for ( int el = 0; el < ne; el++ )
            seen[el].assign( m.pe[el].nsf, 0 );
        while ( std::getline( sc, line ) )
        {
            auto t = split_ws( line );
            if ( t.size() < 4 )
                continue;
            const int e = std::stoi( t[0] ) - 1, s = std::stoi( t[1] ) - 1;
            if ( e < 0 || e >= ne || s < 0 || s >= m.pe[e].nsf )
                continue;
            const double gmin = std::stod( t[2] ), gmax = std::stod( t[3] );
            m.pe[e].gmin[s] = gmin;
            m.pe[e].gscale[s] = ( smax - smin ) / ( gmax - gmin );
            seen[e][s] = 1;
        }
        for ( int el = 0; el < ne; el++ )
            for ( int s = 0; s < m.pe[el].nsf; s++ )
                if ( !seen[el][s] )
                    return gbmd_fail( c, GBMD_ERR_IO, "nnp_load: scaling.data misses a function" );
    }
    // the neighbour cutoff must cover every element's functions
    m.p = m.pe[0];
    for ( auto &q : m.pe )
        m.p.rc = std::max( m.p.rc, q.rc );
    m.dir = dir;
    return GBMD_OK;
}

// The warps' neighbour arrays live in dynamic shared memory: the dense-state
// capacity (NNP_MAXNBR_LARGE) needs more than the 48 KB of static shared
// memory.
extern __shared__ double nnp_dyn_smem_d[];

// ---------------------------------------------------------------------------
// symmetry functions.  Angular sums are accumulated on the compile-time grid
// (distinct eta) x (distinct (lambda, zeta)) so every accumulator stays in a
// register; the grid is mapped to n2p2's function order at the store.

template <class T, int NRM, int CAP>
__global__ void __launch_bounds__( NnpWarps<T>::value * 32 )
    k_nnp_sf( const double4 *__restrict__ x, const float4 *__restrict__ xr,
              const int *__restrict__ home, const uint32_t *__restrict__ nlist,
              const int *__restrict__ nnum, size_t stride, int n, GbmdGeom g,
              const NnpParams *__restrict__ Pg, T *__restrict__ Gout, int scaled,
              int *__restrict__ flags, ElemAtoms ea, int gstride )
{
    NbrSmem<T, CAP> *smem = reinterpret_cast<NbrSmem<T, CAP> *>( nnp_dyn_smem_d );
    __shared__ NnpParams P;
    __shared__ NnpConst<T> C;
    copy_params<T>( Pg, P );
    load_const<T>( Pg, C );
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = ea.atom( blockIdx.x * NnpWarps<T>::value + warp, n );
    if ( i < 0 )
        return;
    NbrSmem<T, CAP> &S = smem[warp];
    const int np = gather_nbrs<T, CAP>( x, xr, nlist, stride, i, nnum[i], home[i], g, P, S,
                                        flags, ea.type );
    T accr[NRM];
    T accg[NNP_MAXETA][NNP_MAXLZ];
#pragma unroll
    for ( int s = 0; s < NRM; s++ )
        accr[s] = 0;
#pragma unroll
    for ( int e = 0; e < NNP_MAXETA; e++ )
#pragma unroll
        for ( int l = 0; l < NNP_MAXLZ; l++ )
            accg[e][l] = 0;
    // radial: lanes over neighbours
    for ( int a = lane; a < np; a += 32 )
    {
        const T r = S.r[a], fc = S.fc[a];
        const int el = S.el[a];
#pragma unroll
        for ( int s = 0; s < NRM; s++ )
            if ( s < P.nrad && el == P.rad_e1[s] )
            {
                const T dr = r - C.rs_r[s];
                accr[s] += xexp( -C.eta_r[s] * dr * dr ) * fc;
            }
    }
    // warp reduction (in FP64) and store in n2p2 order; with `scaled` the
    // stored value is the MLP input smin + (G - Gmin) Gscale, formed in FP64
    // (in FP32 the scaling would multiply G's rounding by G / (Gmax - Gmin))
    auto put = [&]( int s, double v ) {
        Gout[(size_t)i * gstride + s] =
            scaled ? (T)( P.smin + ( v - P.gmin[s] ) * P.gscale[s] ) : (T)v;
    };
#pragma unroll
    for ( int s = 0; s < NRM; s++ )
    {
        double v = (double)accr[s];
#pragma unroll
        for ( int o = 16; o; o >>= 1 )
            v += __shfl_xor_sync( 0xffffffffu, v, o );
        if ( lane == 0 && s < P.nrad )
            put( s, v );
    }
    // angular: a warp-uniform over the first neighbour, lanes over the
    // second; one pass per channel (neighbour-element pair; one pass for a
    // one-element potential)
    const T rc = (T)P.rc;
    for ( int ch = 0; ch < P.nch; ch++ )
    {
        const int c1 = P.ch_e1[ch], c2 = P.ch_e2[ch];
        if ( ch > 0 )
        {
#pragma unroll
            for ( int e = 0; e < NNP_MAXETA; e++ )
#pragma unroll
                for ( int l = 0; l < NNP_MAXLZ; l++ )
                    accg[e][l] = 0;
        }
        for ( int a = 0; a < np; a++ )
        {
            const T ax = S.dx[a], ay = S.dy[a], az = S.dz[a], ra = S.r[a], fa = S.fc[a];
            const int ela = S.el[a];
            if ( ela != c1 && ela != c2 ) // warp-uniform
                continue;
            const int want = ela == c1 ? c2 : c1; // the partner element
            for ( int c = a + 1 + lane; c < np; c += 32 )
            {
                if ( S.el[c] != want )
                    continue;
                const T bx = S.dx[c], by = S.dy[c], bz = S.dz[c], rb = S.r[c];
                const T jx = bx - ax, jy = by - ay, jz = bz - az;
                const T rjk2 = jx * jx + jy * jy + jz * jz;
                const T rjk = xsqrt( rjk2 );
                if ( !( rjk < rc ) )
                    continue;
                const T cs = ( ax * bx + ay * by + az * bz ) / ( ra * rb );
                const T R2 = ra * ra + rb * rb + rjk2;
                const T F = fa * S.fc[c] * fc_cos<T>( rjk, rc );
                T pw[NNP_MAXLZ];
#pragma unroll
                for ( int l = 0; l < NNP_MAXLZ; l++ )
                {
                    T d;
                    pw[l] = 0;
                    if ( l < P.nlz )
                        power_and_deriv<T>( (T)1 + C.lam_u[l] * cs, P.zeta_int[l],
                                            C.zeta_u[l], pw[l], d );
                }
#pragma unroll
                for ( int e = 0; e < NNP_MAXETA; e++ )
                    if ( e < P.neta )
                    {
                        const T ex = xexp( -C.eta_u[e] * R2 ) * F;
#pragma unroll
                        for ( int l = 0; l < NNP_MAXLZ; l++ )
                            accg[e][l] += ex * pw[l];
                    }
            }
        }
#pragma unroll
        for ( int e = 0; e < NNP_MAXETA; e++ )
#pragma unroll
            for ( int l = 0; l < NNP_MAXLZ; l++ )
            {
                double v = (double)accg[e][l];
#pragma unroll
                for ( int o = 16; o; o >>= 1 )
                    v += __shfl_xor_sync( 0xffffffffu, v, o );
                const int sf = P.grid_sf[ch][e][l];
                if ( lane == 0 && sf >= 0 )
                    put( P.nrad + sf, sizeof( T ) == 8 ? (double)( (T)P.ang_pre[sf] * (T)v )
                                                       : P.ang_pre[sf] * v );
            }
    }
}

// ---------------------------------------------------------------------------
// MLP (SIMT, one thread per atom): E_i and dE/dG_i (raw G units)
__device__ __forceinline__ double actf( char a, double v )
{
    switch ( a )
    {
    case 't': return tanh( v );
    case 'p': return v > 30.0 ? v : log1p( exp( v ) );
    case 's': return 1.0 / ( 1.0 + exp( -v ) );
    default: return v;
    }
}
__device__ __forceinline__ double dactf( char a, double v )
{
    switch ( a )
    {
    case 't': { const double t = tanh( v ); return 1.0 - t * t; }
    case 'p': return 1.0 / ( 1.0 + exp( -v ) );
    case 's': { const double s = 1.0 / ( 1.0 + exp( -v ) ); return s * ( 1.0 - s ); }
    default: return 1.0;
    }
}

template <class T>
__global__ void __launch_bounds__( 128 )
    k_nnp_mlp_simt( const T *__restrict__ G, int n, const NnpParams *__restrict__ Pg,
                    const double *__restrict__ W, const double *__restrict__ B,
                    T *__restrict__ dEdG, double *__restrict__ E, double *__restrict__ partials,
                    ElemAtoms ea, int gstride )
{
    __shared__ NnpParams P;
    __shared__ double red[4];
    {
        const int *src = reinterpret_cast<const int *>( Pg );
        int *dst = reinterpret_cast<int *>( &P );
        for ( int k = threadIdx.x; k < (int)( sizeof( NnpParams ) / 4 ); k += blockDim.x )
            dst[k] = src[k];
    }
    __syncthreads();
    const int i = ea.atom( blockIdx.x * blockDim.x + threadIdx.x, n );
    double e_out = 0.0;
    if ( i >= 0 )
    {
        double a[NNP_MAXLAYERS + 1][NNP_MAXNODES];
        double z[NNP_MAXLAYERS + 1][NNP_MAXNODES];
        for ( int s = 0; s < P.nsf; s++ )
            a[0][s] = P.smin + ( (double)G[(size_t)i * gstride + s] - P.gmin[s] ) * P.gscale[s];
        for ( int l = 1; l <= P.nl; l++ )
            for ( int jn = 0; jn < P.nodes[l]; jn++ )
            {
                double acc = B[P.boff[l] + jn];
                const double *w = W + P.woff[l] + jn * P.nodes[l - 1];
                for ( int in = 0; in < P.nodes[l - 1]; in++ )
                    acc += w[in] * a[l - 1][in];
                z[l][jn] = acc;
                a[l][jn] = actf( P.act[l], acc );
            }
        e_out = a[P.nl][0];
        E[i] = e_out;
        double gcur[NNP_MAXNODES], gnext[NNP_MAXNODES];
        gcur[0] = dactf( P.act[P.nl], z[P.nl][0] );
        for ( int l = P.nl; l >= 1; l-- )
        {
            for ( int in = 0; in < P.nodes[l - 1]; in++ )
            {
                double acc = 0.0;
                for ( int jn = 0; jn < P.nodes[l]; jn++ )
                    acc += W[P.woff[l] + jn * P.nodes[l - 1] + in] * gcur[jn];
                gnext[in] = l > 1 ? acc * dactf( P.act[l - 1], z[l - 1][in] ) : acc;
            }
            for ( int in = 0; in < P.nodes[l - 1]; in++ )
                gcur[in] = gnext[in];
        }
        for ( int s = 0; s < P.nsf; s++ )
            dEdG[(size_t)i * gstride + s] = (T)( gcur[s] * P.gscale[s] );
    }
    // per-block sum of E_i (potential energy slot)
    double v = e_out;
#pragma unroll
    for ( int o = 16; o; o >>= 1 )
        v += __shfl_xor_sync( 0xffffffffu, v, o );
    if ( ( threadIdx.x & 31 ) == 0 )
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    if ( threadIdx.x == 0 )
        partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
}

// ---------------------------------------------------------------------------
// forces
template <class T, int NRM, int CAP>
__global__ void __launch_bounds__( NnpWarps<T>::value * 32 )
    k_nnp_force( const double4 *__restrict__ x, const float4 *__restrict__ xr,
                 const int *__restrict__ home, const uint32_t *__restrict__ nlist,
                 const int *__restrict__ nnum, size_t stride, int n, GbmdGeom g,
                 const NnpParams *__restrict__ Pg, const T *__restrict__ dEdG,
                 double *__restrict__ f, int *__restrict__ flags, ElemAtoms ea, int gstride )
{
    NbrSmem<T, CAP> *smem = reinterpret_cast<NbrSmem<T, CAP> *>( nnp_dyn_smem_d );
    __shared__ NnpParams P;
    __shared__ NnpConst<T> C;
    copy_params<T>( Pg, P );
    load_const<T>( Pg, C );
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = ea.atom( blockIdx.x * NnpWarps<T>::value + warp, n );
    if ( i < 0 )
        return;
    NbrSmem<T, CAP> &S = smem[warp];
    const int np = gather_nbrs<T, CAP>( x, xr, nlist, stride, i, nnum[i], home[i], g, P, S,
                                        flags, ea.type );
    // dE/dG weights: radial, and angular on the (eta, (lambda, zeta)) grid
    // of the current channel with the 2^(1 - zeta) prefactor folded in
    T wr[NRM];
    T wg[NNP_MAXETA][NNP_MAXLZ];
#pragma unroll
    for ( int s = 0; s < NRM; s++ )
        wr[s] = s < P.nrad ? dEdG[(size_t)i * gstride + s] : (T)0;
    T fix = 0, fiy = 0, fiz = 0;
    const T rc = (T)P.rc;
    // radial
    for ( int a = lane; a < np; a += 32 )
    {
        const T r = S.r[a], fc = S.fc[a], dfc = S.dfc[a];
        const int el = S.el[a];
        T coef = 0;
#pragma unroll
        for ( int s = 0; s < NRM; s++ )
            if ( s < P.nrad && el == P.rad_e1[s] )
            {
                const T eta = C.eta_r[s];
                const T dr = r - C.rs_r[s];
                coef += wr[s] * xexp( -eta * dr * dr ) * ( (T)-2 * eta * dr * fc + dfc );
            }
        const T gx = coef * S.dx[a] / r, gy = coef * S.dy[a] / r, gz = coef * S.dz[a] / r;
        S.fx[a] -= gx; // lane owns neighbour a in this loop
        S.fy[a] -= gy;
        S.fz[a] -= gz;
        fix += gx;
        fiy += gy;
        fiz += gz;
    }
    __syncwarp();
    // angular: one pass per channel (neighbour-element pair; one pass for a
    // one-element potential)
    for ( int ch = 0; ch < P.nch; ch++ )
    {
        const int c1 = P.ch_e1[ch], c2 = P.ch_e2[ch];
#pragma unroll
        for ( int e = 0; e < NNP_MAXETA; e++ )
#pragma unroll
            for ( int l = 0; l < NNP_MAXLZ; l++ )
            {
                const int sf = P.grid_sf[ch][e][l];
                wg[e][l] = sf >= 0 ? dEdG[(size_t)i * gstride + P.nrad + sf] * (T)P.ang_pre[sf]
                                   : (T)0;
            }
        for ( int a = 0; a < np; a++ )
        {
            const T ax = S.dx[a], ay = S.dy[a], az = S.dz[a], ra = S.r[a];
            const T fa = S.fc[a], dfa = S.dfc[a];
            const int ela = S.el[a];
            if ( ela != c1 && ela != c2 ) // warp-uniform
                continue;
            const int want = ela == c1 ? c2 : c1; // the partner element
            T gax = 0, gay = 0, gaz = 0; // gradient on neighbour a from this lane's triplets
            for ( int c = a + 1 + lane; c < np; c += 32 )
            {
                if ( S.el[c] != want )
                    continue;
                const T bx = S.dx[c], by = S.dy[c], bz = S.dz[c], rb = S.r[c];
                const T jx = bx - ax, jy = by - ay, jz = bz - az;
                const T rjk2 = jx * jx + jy * jy + jz * jz;
                const T rjk = xsqrt( rjk2 );
                if ( !( rjk < rc ) )
                    continue;
                const T inv = (T)1 / ( ra * rb );
                const T cs = ( ax * bx + ay * by + az * bz ) * inv;
                const T R2 = ra * ra + rb * rb + rjk2;
                const T fb = S.fc[c], dfb = S.dfc[c];
                const T fjk = fc_cos<T>( rjk, rc ), dfjk = dfc_cos<T>( rjk, rc );
                const T F = fa * fb * fjk;
                T pw[NNP_MAXLZ], dpw[NNP_MAXLZ];
    #pragma unroll
                for ( int l = 0; l < NNP_MAXLZ; l++ )
                {
                    pw[l] = 0;
                    dpw[l] = 0;
                    if ( l < P.nlz )
                    {
                        power_and_deriv<T>( (T)1 + C.lam_u[l] * cs, P.zeta_int[l],
                                            C.zeta_u[l], pw[l], dpw[l] );
                        dpw[l] *= C.lam_u[l];
                    }
                }
                // fold the angular weights into the coefficients of dcos, dR^2, dF
                T Cc = 0, CR = 0, CF = 0;
    #pragma unroll
                for ( int e = 0; e < NNP_MAXETA; e++ )
                    if ( e < P.neta )
                    {
                        const T ex = xexp( -C.eta_u[e] * R2 );
                        T sp = 0, sd = 0;
    #pragma unroll
                        for ( int l = 0; l < NNP_MAXLZ; l++ )
                        {
                            sp += wg[e][l] * pw[l];
                            sd += wg[e][l] * dpw[l];
                        }
                        Cc += ex * sd;
                        CF += ex * sp;
                        CR -= C.eta_u[e] * ex * sp;
                    }
                Cc *= F;
                CR *= F;
                const T ia2 = (T)1 / ( ra * ra ), ib2 = (T)1 / ( rb * rb );
                const T dFa = dfa * fb * fjk / ra, dFb = fa * dfb * fjk / rb,
                        dFjk = fa * fb * dfjk / rjk;
                const T gjx = Cc * ( bx * inv - cs * ax * ia2 ) + CR * ( (T)2 * ax - (T)2 * jx ) +
                              CF * ( dFa * ax - dFjk * jx );
                const T gjy = Cc * ( by * inv - cs * ay * ia2 ) + CR * ( (T)2 * ay - (T)2 * jy ) +
                              CF * ( dFa * ay - dFjk * jy );
                const T gjz = Cc * ( bz * inv - cs * az * ia2 ) + CR * ( (T)2 * az - (T)2 * jz ) +
                              CF * ( dFa * az - dFjk * jz );
                const T gkx = Cc * ( ax * inv - cs * bx * ib2 ) + CR * ( (T)2 * bx + (T)2 * jx ) +
                              CF * ( dFb * bx + dFjk * jx );
                const T gky = Cc * ( ay * inv - cs * by * ib2 ) + CR * ( (T)2 * by + (T)2 * jy ) +
                              CF * ( dFb * by + dFjk * jy );
                const T gkz = Cc * ( az * inv - cs * bz * ib2 ) + CR * ( (T)2 * bz + (T)2 * jz ) +
                              CF * ( dFb * bz + dFjk * jz );
                gax += gjx;
                gay += gjy;
                gaz += gjz;
                // neighbour c is touched by one lane per a (c distinct across lanes)
                S.fx[c] -= gkx;
                S.fy[c] -= gky;
                S.fz[c] -= gkz;
                fix += gjx + gkx;
                fiy += gjy + gky;
                fiz += gjz + gkz;
            }
    #pragma unroll
            for ( int o = 16; o; o >>= 1 )
            {
                gax += __shfl_xor_sync( 0xffffffffu, gax, o );
                gay += __shfl_xor_sync( 0xffffffffu, gay, o );
                gaz += __shfl_xor_sync( 0xffffffffu, gaz, o );
            }
            if ( lane == 0 )
            {
                S.fx[a] -= gax;
                S.fy[a] -= gay;
                S.fz[a] -= gaz;
            }
            __syncwarp();
        }
    }
    // scatter to owners (one FP64 atomic per neighbour and component); the
    // force unit conversion: dE/dx = dE_nn/dx_nn * cflength / cfenergy
    const double conv = P.cflength / P.cfenergy;
    for ( int a = lane; a < np; a += 32 )
    {
        const int j = S.own[a];
        atomicAdd( &f[j], conv * (double)S.fx[a] );
        atomicAdd( &f[n + j], conv * (double)S.fy[a] );
        atomicAdd( &f[2 * n + j], conv * (double)S.fz[a] );
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
        atomicAdd( &f[i], conv * (double)fix );
        atomicAdd( &f[n + i], conv * (double)fiy );
        atomicAdd( &f[2 * n + i], conv * (double)fiz );
    }
}

// ---------------------------------------------------------------------------
// Several elements: atoms grouped by element, in index order within each
// group (a stable partition, so launches are reproducible).  Three passes:
// per-block element counts; group starts and block offsets (one block);
// the scatter.
constexpr int EG_THREADS = 256;

__global__ void k_elem_count( const int *__restrict__ type, int n, int ne, int *__restrict__ cnt )
{
    __shared__ int c[NNP_MAXELEM];
    if ( threadIdx.x < NNP_MAXELEM )
        c[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i < n )
    {
        const int t = type[i];
        if ( t >= 0 && t < ne )
            atomicAdd( &c[t], 1 );
    }
    __syncthreads();
    if ( threadIdx.x < ne )
        cnt[blockIdx.x * ne + threadIdx.x] = c[threadIdx.x];
}

// cnt[b][e] -> offset of block b's first atom of element e; starts[e].
// One block of EG_SCAN threads: per element, an exclusive scan over the
// blocks in chunks of EG_SCAN, carried from chunk to chunk and element to
// element (the offsets of a serial pass over e, then b).
constexpr int EG_SCAN = 1024;
__global__ void __launch_bounds__( EG_SCAN )
    k_elem_offsets( int *__restrict__ cnt, int nb, int ne, int *__restrict__ starts )
{
    __shared__ int wsum[EG_SCAN / 32];
    __shared__ int carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if ( t == 0 )
        carry = 0;
    __syncthreads();
    for ( int e = 0; e < ne; e++ )
    {
        if ( t == 0 )
            starts[e] = carry;
        for ( int b0 = 0; b0 < nb; b0 += EG_SCAN )
        {
            const int b = b0 + t;
            const int v = b < nb ? cnt[b * ne + e] : 0;
            int x = v; // inclusive scan within the warp
#pragma unroll
            for ( int o = 1; o < 32; o <<= 1 )
            {
                const int y = __shfl_up_sync( 0xffffffffu, x, o );
                if ( lane >= o )
                    x += y;
            }
            if ( lane == 31 )
                wsum[w] = x;
            __syncthreads();
            if ( w == 0 )
            {
                int y = wsum[lane]; // EG_SCAN / 32 == 32 warp totals
#pragma unroll
                for ( int o = 1; o < 32; o <<= 1 )
                {
                    const int z = __shfl_up_sync( 0xffffffffu, y, o );
                    if ( lane >= o )
                        y += z;
                }
                wsum[lane] = y;
            }
            __syncthreads();
            const int before = carry + ( w ? wsum[w - 1] : 0 ) + x - v;
            if ( b < nb )
                cnt[b * ne + e] = before;
            __syncthreads(); // every thread has read carry and wsum
            if ( t == EG_SCAN - 1 )
                carry = before + v;
            __syncthreads();
        }
    }
    if ( t == 0 )
        starts[ne] = carry;
}

__global__ void k_elem_scatter( const int *__restrict__ type, int n, int ne,
                                const int *__restrict__ off, int *__restrict__ atoms )
{
    __shared__ int wsum[EG_THREADS / 32][NNP_MAXELEM];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int t = i < n ? type[i] : -1;
    unsigned mine = 0;
    for ( int e = 0; e < ne; e++ )
    {
        const unsigned m = __ballot_sync( 0xffffffffu, t == e );
        if ( t == e )
            mine = __popc( m & ( ( 1u << lane ) - 1u ) );
        if ( lane == 0 )
            wsum[w][e] = __popc( m );
    }
    __syncthreads();
    if ( t >= 0 && t < ne )
    {
        int before = 0;
        for ( int k = 0; k < w; k++ )
            before += wsum[k][t];
        atoms[off[blockIdx.x * ne + t] + before + (int)mine] = i;
    }
}

static int group_by_element( gbmd_ctx *c, NnpModel &m )
{
    const int n = (int)c->n, ne = (int)m.pe.size();
    const int nb = ( n + EG_THREADS - 1 ) / EG_THREADS;
    int rc;
    if ( ( rc = gbmd_reserve( c, m.elem_atoms, n, "nnp element atoms" ) ) ||
         ( rc = gbmd_reserve( c, m.elem_aux, (size_t)nb * ne + NNP_MAXELEM + 1,
                              "nnp element offsets" ) ) )
        return rc;
    int *cnt = m.elem_aux.p + NNP_MAXELEM + 1, *starts = m.elem_aux.p;
    k_elem_count<<<nb, EG_THREADS, 0, c->stream>>>( c->type.p, n, ne, cnt );
    k_elem_offsets<<<1, EG_SCAN, 0, c->stream>>>( cnt, nb, ne, starts );
    k_elem_scatter<<<nb, EG_THREADS, 0, c->stream>>>( c->type.p, n, ne, cnt, m.elem_atoms.p );
    GBMD_LAUNCH_CHECK( c, "nnp element groups" );
    return GBMD_OK;
}

// ---------------------------------------------------------------------------
// host launch
static NnpParams *model_params_dev( gbmd_ctx *c )
{
    // the parameter blocks (one per element) live behind the weights in d_w
    NnpModel &m = *c->nnp;
    return reinterpret_cast<NnpParams *>( m.d_w + m.w.size() );
}

// The generic kernels for a neighbour capacity CAP (dynamic shared memory
// sized for it; the attribute is set once per instantiation and device).
template <class Kern> static int dyn_smem_ready( gbmd_ctx *c, Kern k, size_t bytes,
                                                 std::atomic<unsigned> &ready )
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

template <class T, int NRM, int CAP>
static int launch_generic_sf( gbmd_ctx *c, int blocks, const NnpParams *Pd, T *G, int scaled,
                              const ElemAtoms &ea, int gstride )
{
    constexpr int NW = NnpWarps<T>::value;
    constexpr size_t smem = sizeof( NbrSmem<T, CAP> ) * NW;
    static std::atomic<unsigned> ready{ 0 };
    int rc = dyn_smem_ready( c, k_nnp_sf<T, NRM, CAP>, smem, ready );
    if ( rc )
        return rc;
    k_nnp_sf<T, NRM, CAP><<<blocks, NW * 32, smem, c->stream>>>(
        c->x.p, c->xr.p, c->home.p, c->nlist.p, c->nnum.p, c->nl_stride, (int)c->n, c->geom, Pd,
        G, scaled, c->flags.p, ea, gstride );
    GBMD_LAUNCH_CHECK( c, "nnp sf" );
    return GBMD_OK;
}

template <class T, int NRM, int CAP>
static int launch_generic_force( gbmd_ctx *c, int blocks, const NnpParams *Pd, const T *dEdG,
                                 const ElemAtoms &ea, int gstride )
{
    constexpr int NW = NnpWarps<T>::value;
    constexpr size_t smem = sizeof( NbrSmem<T, CAP> ) * NW;
    static std::atomic<unsigned> ready{ 0 };
    int rc = dyn_smem_ready( c, k_nnp_force<T, NRM, CAP>, smem, ready );
    if ( rc )
        return rc;
    k_nnp_force<T, NRM, CAP><<<blocks, NW * 32, smem, c->stream>>>(
        c->x.p, c->xr.p, c->home.p, c->nlist.p, c->nnum.p, c->nl_stride, (int)c->n, c->geom, Pd,
        dEdG, c->f.p, c->flags.p, ea, gstride );
    GBMD_LAUNCH_CHECK( c, "nnp force" );
    return GBMD_OK;
}

template <class T, int NRM>
static int launch_typed( gbmd_ctx *c, bool eflag, bool forces, size_t stride_partials )
{
    NnpModel &m = *c->nnp;
    const int n = (int)c->n;
    const int ne = (int)m.pe.size();
    int rc;
    if ( ( rc = gbmd_reserve( c, m.G, (size_t)n * m.gstride, "nnp G" ) ) ||
         ( rc = gbmd_reserve( c, m.dEdG, (size_t)n * m.gstride, "nnp dEdG" ) ) ||
         ( rc = gbmd_reserve( c, m.E, n, "nnp E" ) ) )
        return rc;
    T *G = reinterpret_cast<T *>( m.G.p );
    T *dEdG = reinterpret_cast<T *>( m.dEdG.p );
    const NnpParams *Pd = model_params_dev( c );
    constexpr int NW = NnpWarps<T>::value;
    const int blocks = ( n + NW - 1 ) / NW;
    // neighbour capacity: the list's largest count bounds the count inside
    // rc of every atom until the next rebuild
    const bool large = c->nl_maxc > NNP_MAXNBR;
    // Several elements: one launch per element over its atoms (grid sized for
    // all atoms; work items past the element's count return at once).
    ElemAtoms ea;
    if ( ne > 1 )
    {
        if ( ( rc = group_by_element( c, m ) ) )
            return rc;
        ea.atoms = m.elem_atoms.p;
        ea.starts = m.elem_aux.p;
        ea.type = c->type.p;
        // rows of elements with fewer functions than gstride stay zero-padded
        GBMD_CUDA( c, cudaMemsetAsync( m.G.p, 0, sizeof( T ) * n * m.gstride, c->stream ) );
        GBMD_CUDA( c, cudaMemsetAsync( m.dEdG.p, 0, sizeof( T ) * n * m.gstride, c->stream ) );
    }
    // mixed precision, n2p2's usual angular form (every element):
    // compacted-triplet kernels (gbmd_nnp_f32.cu) writing the scaled MLP
    // input when the tensor-core MLP consumes it
    bool f32 = sizeof( T ) == 4;
    for ( auto &q : m.pe )
        f32 = f32 && gbmd_nnp_f32_supported( q );
    NnpTriCache tcache;
    if ( f32 && forces && gbmd_nnp_f32_cacheable( c, ne ) )
    {
        if ( ( rc = gbmd_reserve( c, m.tcache, (size_t)n * NNP_TCAP, "nnp triplet cache" ) ) ||
             ( rc = gbmd_reserve( c, m.tcount, n, "nnp triplet counts" ) ) )
            return rc;
        tcache.t = m.tcache.p;
        tcache.cnt = m.tcount.p;
    }
    const int scaled = sizeof( T ) == 4 && m.d_tc ? 1 : 0;
    cudaEvent_t t0;
    gbmd_ktime_begin( c, GBMD_KT_NNP_SF, &t0 );
    if ( f32 )
    {
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            if ( ( rc = gbmd_nnp_sf_f32_launch( c, m.pe[el], Pd + el,
                                                reinterpret_cast<float *>( G ), scaled, ea,
                                                m.gstride, tcache ) ) )
                return rc;
        }
    }
    else
    {
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            if ( ( rc = large ? launch_generic_sf<T, NRM, NNP_MAXNBR_LARGE>(
                                    c, blocks, Pd + el, G, scaled, ea, m.gstride )
                              : launch_generic_sf<T, NRM, NNP_MAXNBR>( c, blocks, Pd + el, G,
                                                                       scaled, ea,
                                                                       m.gstride ) ) )
                return rc;
        }
    }
    m.g_scaled = scaled != 0;
    gbmd_ktime_end( c, GBMD_KT_NNP_SF, t0 );
    const int mblocks = ( n + 127 ) / 128;
    double *pe_part = c->partials.p + stride_partials; // slot 1: potential energy
    gbmd_ktime_begin( c, GBMD_KT_NNP_MLP, &t0 );
    if ( sizeof( T ) == 4 && m.d_tc )
    {
        // mixed precision: tensor-core tiles (split-BF16 operands, FP32
        // accumulation), one element's model per launch; the tile count
        // equals mblocks, and element el's tiles write partial sums
        // el * mblocks onwards
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            if ( ( rc = gbmd_nnp_mlp_tc_launch( c, m.d_tc + el,
                                                reinterpret_cast<const float *>( G ),
                                                reinterpret_cast<float *>( dEdG ), m.E.p, n,
                                                pe_part + (size_t)el * mblocks, scaled, ea,
                                                m.gstride ) ) )
                return rc;
        }
    }
    else
    {
        // element el's blocks write partial sums el * mblocks onwards
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            k_nnp_mlp_simt<T><<<mblocks, 128, 0, c->stream>>>(
                G, n, Pd + el, m.d_w, m.d_b, dEdG, m.E.p, pe_part + (size_t)el * mblocks, ea,
                m.gstride );
            GBMD_LAUNCH_CHECK( c, "nnp mlp" );
        }
    }
    gbmd_ktime_end( c, GBMD_KT_NNP_MLP, t0 );
    const int nparts = mblocks * ne;
    if ( !forces )
        return eflag ? gbmd_reduce_partials( c, nparts, 1 ) : GBMD_OK;
    gbmd_ktime_begin( c, GBMD_KT_NNP_FORCE, &t0 );
    if ( f32 )
    {
        if ( ( rc = gbmd_reserve( c, m.fq, (size_t)3 * n, "nnp fixed-point forces" ) ) ||
             ( rc = gbmd_nnp_fq_begin( c, m.fq.p ) ) )
            return rc;
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            if ( ( rc = gbmd_nnp_force_f32_launch( c, m.pe[el], Pd + el,
                                                   reinterpret_cast<const float *>( dEdG ),
                                                   m.fq.p, ea, m.gstride, tcache ) ) )
                return rc;
        }
        if ( ( rc = gbmd_nnp_fq_end( c, m.p, m.fq.p ) ) )
            return rc;
    }
    else
    {
        for ( int el = 0; el < ne; el++ )
        {
            ea.el = el;
            if ( ( rc = large ? launch_generic_force<T, NRM, NNP_MAXNBR_LARGE>(
                                    c, blocks, Pd + el, dEdG, ea, m.gstride )
                              : launch_generic_force<T, NRM, NNP_MAXNBR>( c, blocks, Pd + el,
                                                                          dEdG, ea,
                                                                          m.gstride ) ) )
                return rc;
        }
    }
    gbmd_ktime_end( c, GBMD_KT_NNP_FORCE, t0 );
    if ( eflag )
        return gbmd_reduce_partials( c, nparts, 1 );
    return GBMD_OK;
}

// ---------------------------------------------------------------------------
// Serving: one step of many NNP jobs in job-table launches.  The launches
// and their order are those of the single-system step (force_launch with f
// zeroed first, then gbmd_nve_step_tail_launch / gbmd_nve_final_launch),
// each one covering every job of the table: f and the fixed-point sums
// zeroed, symmetry functions (scaled MLP input, compacted triplets kept),
// tensor-core MLP, forces, fixed-point sums into f, integrator; on thermo
// steps the two per-job reductions follow.
bool gbmd_nnp_batchable( const gbmd_ctx *c )
{
    if ( c->force_type != GBMD_FORCE_NNP || !c->nnp || c->precision != GBMD_PREC_MIXED ||
         c->half || !c->sorted || !c->have_list || c->n <= 0 )
        return false;
    const NnpModel &m = *c->nnp;
    return m.pe.size() == 1 && m.d_tc && gbmd_nnp_f32_job_shape( m.pe[0] ) &&
           gbmd_nnp_f32_cacheable( c, 1 ) &&
           c->neigh_cut >= m.p.rc / m.p.cflength;
}

int gbmd_nnp_step_batch( gbmd_ctx *const *cs, const bool *thermo, const bool *last, int count,
                         int64_t *launches )
{
    if ( count <= 0 )
        return GBMD_OK;
    const cudaStream_t st = cs[0]->stream;
    const int device = cs[0]->device;
    // host staging of the launch parameters: one per host thread
    thread_local NnpJobTable t;
    int k0 = 0;
    while ( k0 < count )
    {
        t.njobs = 0;
        t.b_sf[0] = t.b_mlp[0] = t.b_fq[0] = t.b_nve[0] = 0;
        int k = k0;
        for ( ; k < count && t.njobs < NNP_JOBS_PER_LAUNCH; k++ )
        {
            gbmd_ctx *c = cs[k];
            if ( !gbmd_nnp_batchable( c ) || c->stream != st )
                return gbmd_fail( c, GBMD_ERR_ARG, "nnp step batch: job is not batchable" );
            NnpModel &m = *c->nnp;
            const int n = (int)c->n;
            size_t stride;
            int rc;
            if ( ( rc = gbmd_partials_prepare( c, n, &stride, nullptr ) ) ||
                 ( rc = gbmd_reserve( c, m.G, (size_t)n * m.gstride, "nnp G" ) ) ||
                 ( rc = gbmd_reserve( c, m.dEdG, (size_t)n * m.gstride, "nnp dEdG" ) ) ||
                 ( rc = gbmd_reserve( c, m.E, n, "nnp E" ) ) ||
                 ( rc = gbmd_reserve( c, m.fq, (size_t)3 * n, "nnp fixed-point forces" ) ) ||
                 ( rc = gbmd_reserve( c, m.tcache, (size_t)n * NNP_TCAP, "nnp triplet cache" ) ) ||
                 ( rc = gbmd_reserve( c, m.tcount, n, "nnp triplet counts" ) ) )
                return rc;
            NnpJobArgs &J = t.job[t.njobs];
            J.xr = c->xr.p;
            J.nlist = c->nlist.p;
            J.nnum = c->nnum.p;
            J.stride = c->nl_stride;
            J.n = n;
            J.gstride = m.gstride;
            J.g = c->geom;
            J.Pg = model_params_dev( c );
            J.G = reinterpret_cast<float *>( m.G.p );
            J.dEdG = reinterpret_cast<float *>( m.dEdG.p );
            J.fq = m.fq.p;
            J.flags = c->flags.p;
            J.tc.t = m.tcache.p;
            J.tc.cnt = m.tcount.p;
            J.tcm = m.d_tc;
            J.E = m.E.p;
            J.pe_part = c->partials.p + stride; // slot 1: potential energy
            J.conv = m.p.cflength / m.p.cfenergy;
            J.x = c->x.p;
            J.xr_out = c->xr.p;
            J.v = c->v.p;
            J.f = c->f.p;
            J.partials = c->partials.p; // slot 0: sum m v^2
            J.type = c->type.p;
            J.home = c->home.p;
            J.s = gbmd_step_args( c, !last[k] );
            J.thermo = thermo[k] ? 1 : 0;
            J.last = last[k] ? 1 : 0;
            m.g_scaled = true;
            const int j = t.njobs++;
            t.b_sf[j + 1] = t.b_sf[j] + ( n + 3 ) / 4;
            t.b_mlp[j + 1] = t.b_mlp[j] + ( n + 127 ) / 128;
            t.b_fq[j + 1] = t.b_fq[j] + ( 3 * n + 255 ) / 256;
            t.b_nve[j + 1] = t.b_nve[j] + ( n + NNP_NVE_THREADS - 1 ) / NNP_NVE_THREADS;
        }
        gbmd_ctx *c0 = cs[k0];
        if ( gbmd_nnp_zero_jobs_launch( t, st ) || gbmd_nnp_sf_jobs_launch( t, device, st ) ||
             gbmd_nnp_mlp_tc_jobs_launch( t, device, st ) ||
             gbmd_nnp_force_jobs_launch( t, device, st ) || gbmd_nnp_fq_jobs_launch( t, st ) ||
             gbmd_nve_jobs_launch( t, st ) )
            return gbmd_fail( c0, GBMD_ERR_CUDA, "nnp step batch: a job-table launch failed" );
        *launches += 6;
        for ( int q = k0; q < k; q++ )
        {
            gbmd_ctx *c = cs[q];
            if ( !thermo[q] )
                continue;
            const int n = (int)c->n;
            int rc;
            if ( ( rc = gbmd_reduce_partials( c, ( n + 127 ) / 128, 1 ) ) ||
                 ( rc = gbmd_reduce_partials( c, ( n + NNP_NVE_THREADS - 1 ) / NNP_NVE_THREADS,
                                              0 ) ) )
                return rc;
        }
        k0 = k;
    }
    return GBMD_OK;
}

int gbmd_nnp_launch( gbmd_ctx *c, bool eflag, bool forces )
{
    if ( !c->nnp )
        return gbmd_fail( c, GBMD_ERR_ARG, "NNP potential not loaded" );
    if ( c->n == 0 )
        return GBMD_OK;
    if ( c->neigh_cut < c->nnp->p.rc / c->nnp->p.cflength )
        return gbmd_fail( c, GBMD_ERR_ARG, "nnp: neighbour cutoff below the NNP cutoff" );
    size_t stride;
    int rc = gbmd_partials_prepare( c, c->n, &stride, nullptr );
    if ( rc )
        return rc;
    const NnpModel &m = *c->nnp;
    if ( m.pe.size() > 1 && c->ntypes != (int)m.pe.size() )
        return gbmd_fail( c, GBMD_ERR_ARG,
                          "nnp: the system's atom types must be the potential's elements (" +
                              std::to_string( m.pe.size() ) + ")" );
    bool small = true;
    for ( auto &q : m.pe )
        small = small && q.nrad <= 8;
    if ( c->precision == GBMD_PREC_FP64 )
        return small ? launch_typed<double, 8>( c, eflag, forces, stride )
                     : launch_typed<double, 16>( c, eflag, forces, stride );
    return small ? launch_typed<float, 8>( c, eflag, forces, stride )
                 : launch_typed<float, 16>( c, eflag, forces, stride );
}

void gbmd_nnp_free( gbmd_ctx *c )
{
    if ( !c->nnp )
        return;
    NnpModel &m = *c->nnp;
    if ( m.d_w )
        cudaFreeAsync( m.d_w, c->stream );
    if ( m.d_b )
        cudaFreeAsync( m.d_b, c->stream );
    if ( m.d_wf )
        cudaFreeAsync( m.d_wf, c->stream );
    if ( m.d_bf )
        cudaFreeAsync( m.d_bf, c->stream );
    if ( m.d_tc )
        cudaFreeAsync( m.d_tc, c->stream );
    gbmd_release( c, m.G );
    gbmd_release( c, m.dEdG );
    gbmd_release( c, m.E );
    gbmd_release( c, m.fq );
    gbmd_release( c, m.tcache );
    gbmd_release( c, m.tcount );
    delete c->nnp;
    c->nnp = nullptr;
}

size_t gbmd_nnp_device_bytes( const gbmd_ctx *c )
{
    if ( !c->nnp )
        return 0;
    const NnpModel &m = *c->nnp;
    const size_t pwords = ( sizeof( NnpParams ) + 7 ) / 8 * m.pe.size();
    return sizeof( double ) * ( m.w.size() + pwords + m.b.size() ) +
           ( m.d_tc ? sizeof( TcModel ) * m.pe.size() : 0 ) + gbmd_bytes( m.G ) +
           gbmd_bytes( m.dEdG ) +
           gbmd_bytes( m.E ) + gbmd_bytes( m.fq ) + gbmd_bytes( m.tcache ) +
           gbmd_bytes( m.tcount );
}

void gbmd_nnp_key( const gbmd_ctx *c, std::string &key )
{
    const NnpModel &m = *c->nnp;
    const void *ptrs[] = { m.d_w, m.d_b, m.d_tc, m.G.p, m.dEdG.p, m.E.p, m.fq.p,
                           m.tcache.p, m.tcount.p, m.elem_atoms.p, m.elem_aux.p };
    key.append( reinterpret_cast<const char *>( ptrs ), sizeof ptrs );
    const int ints[] = { m.gstride, (int)m.pe.size(), m.g_scaled ? 1 : 0 };
    key.append( reinterpret_cast<const char *>( ints ), sizeof ints );
    // the model's host-side values (kernel shapes, conversion factors) are
    // fixed per load
    key.append( reinterpret_cast<const char *>( &m.gen ), sizeof m.gen );
}

// Reference energy assembly (force_nnp_cabana_neigh_impl.h:112-127) from
// sum E_i: offsets, conversion, mean energy, Hartree -> eV factor.
double gbmd_nnp_total_energy( const gbmd_ctx *c, double esum )
{
    const NnpParams &p = c->nnp->p;
    double e = esum;
    e += (double)c->n * p.e_offset;
    e /= 1.0;                 // convEnergy: n2p2 normalisation is not used
    e += (double)c->n * 0.0;  // meanEnergy
    e *= 27.211384021355236;
    return e;
}

extern "C" int gbmd_nnp_load( gbmd_ctx *c, const char *dir, double cflength, double cfenergy )
{
    if ( !c || !dir )
        return GBMD_ERR_ARG;
    if ( !( cflength > 0 ) || !( cfenergy > 0 ) )
        return gbmd_fail( c, GBMD_ERR_ARG, "nnp_load: conversion factors must be > 0" );
    NnpModel *m = new NnpModel();
    int rc = load_model( c, dir, cflength, cfenergy, *m );
    if ( rc )
    {
        delete m;
        return rc;
    }
    // device copies: weights, then the parameter block right behind them
    const size_t nw = m->w.size(), nb = m->b.size();
    const size_t pwords = ( sizeof( NnpParams ) * m->pe.size() + 7 ) / 8;
    cudaStream_t st = c->stream;
    if ( cudaMallocAsync( (void **)&m->d_w, sizeof( double ) * ( nw + pwords ), st ) !=
             cudaSuccess ||
         cudaMallocAsync( (void **)&m->d_b, sizeof( double ) * nb, st ) != cudaSuccess )
    {
        if ( m->d_w )
            cudaFreeAsync( m->d_w, st );
        delete m;
        return gbmd_fail( c, GBMD_ERR_CUDA, "nnp_load: device allocation failed" );
    }
    // tensor-core operands, one model per element, when every element's
    // network fits; GBMD_NNP_MLP=simt selects the SIMT MLP instead
    const size_t ne = m->pe.size();
    std::vector<TcModel> tc( ne );
    const char *mlp_env = std::getenv( "GBMD_NNP_MLP" );
    bool use_tc = !( mlp_env && std::string( mlp_env ) == "simt" );
    for ( size_t k = 0; k < ne && use_tc; k++ )
        use_tc = gbmd_tc_model_build( m->pe[k], m->w, m->b, tc[k] );
    cudaError_t e = cudaMemcpyAsync( m->d_w, m->w.data(), sizeof( double ) * nw,
                                     cudaMemcpyHostToDevice, st );
    if ( e == cudaSuccess )
        e = cudaMemcpyAsync( m->d_w + nw, m->pe.data(), sizeof( NnpParams ) * m->pe.size(),
                             cudaMemcpyHostToDevice, st );
    if ( e == cudaSuccess )
        e = cudaMemcpyAsync( m->d_b, m->b.data(), sizeof( double ) * nb, cudaMemcpyHostToDevice,
                             st );
    // tensor-core operands for the mixed-precision MLP, when the net fits
    if ( e == cudaSuccess && use_tc )
    {
        e = cudaMallocAsync( (void **)&m->d_tc, sizeof( TcModel ) * ne, st );
        if ( e == cudaSuccess )
            e = cudaMemcpyAsync( m->d_tc, tc.data(), sizeof( TcModel ) * ne,
                                 cudaMemcpyHostToDevice, st );
    }
    if ( e == cudaSuccess )
        e = cudaStreamSynchronize( st ); // host copies (tc, m->w) stay alive until here
    if ( e != cudaSuccess )
    {
        cudaFreeAsync( m->d_w, st );
        cudaFreeAsync( m->d_b, st );
        if ( m->d_tc )
            cudaFreeAsync( m->d_tc, st );
        delete m;
        return gbmd_cuda_check( c, e, "nnp_load: device copies" );
    }
    static std::atomic<uint64_t> loads{ 0 };
    m->gen = ++loads;
    gbmd_nnp_free( c );
    c->nnp = m;
    c->force_type = GBMD_FORCE_NNP;
    return GBMD_OK;
}

extern "C" int gbmd_nnp_download( gbmd_ctx *c, double *G, double *E, int *nsf )
{
    if ( !c )
        return GBMD_ERR_ARG;
    if ( !c->nnp )
        return gbmd_fail( c, GBMD_ERR_ARG, "nnp_download: no NNP loaded" );
    NnpModel &m = *c->nnp;
    if ( nsf )
        *nsf = m.gstride;
    const int64_t n = c->n;
    GBMD_CUDA( c, cudaStreamSynchronize( c->stream ) );
    if ( n == 0 || !m.G.p )
        return GBMD_OK;
    const size_t cnt = (size_t)n * m.gstride;
    if ( G )
    {
        if ( c->precision == GBMD_PREC_FP64 )
            GBMD_CUDA( c, cudaMemcpy( G, m.G.p, sizeof( double ) * cnt, cudaMemcpyDeviceToHost ) );
        else
        {
            std::vector<float> tmp( cnt );
            GBMD_CUDA( c, cudaMemcpy( tmp.data(), m.G.p, sizeof( float ) * cnt,
                                      cudaMemcpyDeviceToHost ) );
            const int nsf = m.gstride;
            for ( size_t k = 0; k < cnt; k++ )
            {
                const int s = (int)( k % nsf );
                // the compacted-triplet kernel may hold the scaled MLP input
                G[k] = m.g_scaled ? m.p.gmin[s] + ( tmp[k] - m.p.smin ) / m.p.gscale[s]
                                  : (double)tmp[k];
            }
        }
    }
    if ( E )
        GBMD_CUDA( c, cudaMemcpy( E, m.E.p, sizeof( double ) * n, cudaMemcpyDeviceToHost ) );
    return GBMD_OK;
}
