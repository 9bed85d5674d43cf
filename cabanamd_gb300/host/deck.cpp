// deck.cpp -- input deck, lattice / velocity creation and LAMMPS data files,
// restating CabanaMD's host-side set-up (paths inside the CabanaMD project):
//   src/inputFile_impl.h:125-534   check_lammps_command (keyword semantics)
//   src/inputFile_impl.h:536-865   create_lattice and the velocity set-up
//   src/inputFile.h:66-148         the LAMMPS geom velocity generator
//   src/read_data.h:99-422         data file header / Masses / Atoms /
//                                  Velocities sections, write_data
// Build with -ffp-contract=off: the lattice coordinates and velocity
// scaling follow the reference's operation order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>

#include "cbnmd.h"

namespace cbnmd
{

static std::vector<std::string> words_of( const std::string &line )
{
    std::istringstream is( line );
    std::vector<std::string> w;
    std::string t;
    while ( is >> t )
        w.push_back( t );
    return w;
}

// Argument i of a deck command as a number: the whole token must parse.
static double num( const std::vector<std::string> &w, size_t i )
{
    if ( i >= w.size() )
        throw Error( "deck: missing argument in '" + w[0] + "'" );
    size_t used = 0;
    double v = 0.0;
    try
    {
        v = std::stod( w[i], &used );
    }
    catch ( const std::exception & )
    {
        used = 0;
    }
    if ( used != w[i].size() )
        throw Error( "deck: bad number '" + w[i] + "' in '" + w[0] + "'" );
    return v;
}

static int inum( const std::vector<std::string> &w, size_t i )
{
    if ( i >= w.size() )
        throw Error( "deck: missing argument in '" + w[0] + "'" );
    size_t used = 0;
    int v = 0;
    try
    {
        v = std::stoi( w[i], &used );
    }
    catch ( const std::exception & )
    {
        used = 0;
    }
    if ( used != w[i].size() )
        throw Error( "deck: bad integer '" + w[i] + "' in '" + w[0] + "'" );
    return v;
}

// One deck line with the reference's keyword semantics.
void apply_deck_line( Deck &d, const std::string &line )
{
    const auto w = words_of( line );
    if ( w.empty() || w[0][0] == '#' )
        return;
    const std::string &k = w[0];
    if ( k == "units" )
    {
        if ( w.size() < 2 )
            throw Error( "deck: units needs a style" );
        if ( w[1] == "metal" )
        {
            d.units = UNITS_METAL;
            d.boltz = 8.617343e-5;
            d.mvv2e = 1.0364269e-4;
            d.dt = 0.001; // set unconditionally, as the reference does
        }
        else if ( w[1] == "real" )
        {
            d.units = UNITS_REAL;
            d.boltz = 0.0019872067;
            d.mvv2e = 48.88821291 * 48.88821291;
            if ( !d.timestep_set )
                d.dt = 1.0;
        }
        else if ( w[1] == "lj" )
        {
            d.units = UNITS_LJ;
            d.boltz = 1.0;
            d.mvv2e = 1.0;
            if ( !d.timestep_set )
                d.dt = 0.005;
        }
        else
            throw Error( "deck: 'units' supports metal, real and lj" );
    }
    else if ( k == "atom_style" )
    {
        if ( w.size() < 2 || w[1] != "atomic" )
            throw Error( "deck: only 'atom_style atomic' is supported" );
    }
    else if ( k == "lattice" )
    {
        if ( w.size() < 3 )
            throw Error( "deck: lattice needs a style and a constant" );
        if ( w[1] == "sc" )
        {
            d.lattice = LATTICE_SC;
            d.lattice_constant = num( w, 2 );
        }
        else if ( w[1] == "fcc" )
        {
            d.lattice = LATTICE_FCC;
            // LJ units give the reduced density (inputFile_impl.h:212-214)
            d.lattice_constant = d.units == UNITS_LJ ? std::pow( 4.0 / num( w, 2 ), 1.0 / 3.0 )
                                                     : num( w, 2 );
        }
        else
            throw Error( "deck: 'lattice' supports sc and fcc" );
        if ( w.size() > 3 )
        {
            if ( w[3] != "origin" )
                throw Error( "deck: 'lattice' supports only the 'origin' option" );
            d.offset[0] = num( w, 4 );
            d.offset[1] = num( w, 5 );
            d.offset[2] = num( w, 6 );
        }
    }
    else if ( k == "region" )
    {
        if ( w.size() < 9 || w[2] != "block" )
            throw Error( "deck: 'region' supports 'block'" );
        Block b{ num( w, 3 ), num( w, 4 ), num( w, 5 ), num( w, 6 ), num( w, 7 ), num( w, 8 ) };
        bool replaced = false;
        for ( auto &r : d.regions )
            if ( r.first == w[1] )
            {
                r.second = b;
                replaced = true;
            }
        if ( !replaced )
            d.regions.push_back( { w[1], b } );
        const double a = d.lattice_constant;
        d.box_lo[0] = std::min( d.box_lo[0], a * b.xlo );
        d.box_lo[1] = std::min( d.box_lo[1], a * b.ylo );
        d.box_lo[2] = std::min( d.box_lo[2], a * b.zlo );
        d.box_hi[0] = std::max( d.box_hi[0], a * b.xhi );
        d.box_hi[1] = std::max( d.box_hi[1], a * b.yhi );
        d.box_hi[2] = std::max( d.box_hi[2], a * b.zhi );
    }
    else if ( k == "create_box" )
        d.ntypes = inum( w, 1 );
    else if ( k == "create_atoms" )
    {
        if ( w.size() >= 4 && w[2] == "region" )
        {
            bool found = false;
            for ( auto &r : d.regions )
                found = found || r.first == w[3];
            if ( !found )
                throw Error( "deck: region '" + w[3] + "' is not defined" );
            d.region_type[w[3]] = inum( w, 1 );
        }
        else if ( w.size() >= 3 && w[2] == "box" )
        {
            if ( d.regions.empty() )
                throw Error( "deck: create_atoms box needs a region" );
            // the reference takes the first region of its (sorted) map
            std::string first = d.regions[0].first;
            for ( auto &r : d.regions )
                first = std::min( first, r.first );
            d.region_type[first] = inum( w, 1 );
        }
        else
            throw Error( "deck: 'create_atoms' supports 'box' and 'region'" );
    }
    else if ( k == "mass" )
        d.mass[inum( w, 1 ) - 1] = num( w, 2 );
    else if ( k == "read_data" )
    {
        d.read_data = true;
        d.data_in = w.at( 1 );
    }
    else if ( k == "write_data" )
    {
        d.write_data = true;
        d.data_out = w.at( 1 );
    }
    else if ( k == "pair_style" )
    {
        if ( w.size() >= 3 && w[1] == "lj/cut" )
        {
            d.force_nnp = false;
            d.force_cutoff = num( w, 2 );
        }
        else if ( w.size() >= 2 && w[1] == "nnp" )
        {
            d.force_nnp = true;
            d.pair_style = w;
        }
        else
            throw Error( "deck: 'pair_style' supports lj/cut and nnp" );
    }
    else if ( k == "pair_coeff" )
    {
        if ( d.force_nnp )
            d.force_cutoff = num( w, 3 );
        else
            d.pair_coeff.push_back( w );
    }
    else if ( k == "velocity" )
    {
        if ( w.size() < 5 || w[2] != "create" )
            throw Error( "deck: 'velocity' supports only 'create'" );
        const int t = w[1] == "all" ? 1 : inum( w, 1 );
        d.velocity[t] = { num( w, 3 ), inum( w, 4 ) };
    }
    else if ( k == "neighbor" )
        d.skin = num( w, 1 );
    else if ( k == "neigh_modify" )
    {
        for ( size_t i = 1; i < w.size(); i += 2 )
        {
            if ( w[i] == "every" )
                d.rebuild_every = inum( w, i + 1 );
            else if ( w[i] == "one" )
                d.max_neigh_guess = inum( w, i + 1 );
            else
                throw Error( "deck: 'neigh_modify' supports 'every' and 'one'" );
        }
    }
    else if ( k == "comm_modify" )
    {
        if ( w.size() < 4 || w[1] != "cutoff" || w[2] != "*" )
            throw Error( "deck: 'comm_modify' supports 'cutoff * <value>'" );
        d.comm_ghost_cutoff = num( w, 3 );
    }
    else if ( k == "fix" )
    {
        if ( w.size() < 4 || w[3] != "nve" )
            throw Error( "deck: 'fix' supports 'nve'" );
    }
    else if ( k == "run" )
        d.nsteps = inum( w, 1 );
    else if ( k == "thermo" )
        d.thermo = inum( w, 1 );
    else if ( k == "timestep" )
    {
        d.dt = num( w, 1 );
        d.timestep_set = true;
    }
    else if ( k == "newton" )
    {
        if ( w.size() < 2 || ( w[1] != "on" && w[1] != "off" ) )
            throw Error( "deck: 'newton' must be followed by on or off" );
        d.half = w[1] == "on";
        d.newton_set = true;
    }
    else if ( k == "group" )
    {
        if ( w.size() < 4 || w[2] != "region" )
            throw Error( "deck: 'group' supports 'region'" );
    }
    else if ( k == "dump" )
    {
        // dump <id> all vtk <N> <file> (inputFile_impl.h:327-357)
        if ( w.size() < 4 || w[3] != "vtk" )
            throw Error( "deck: 'dump' command only supports 'vtk'" );
        if ( w[2] != "all" )
            throw Error( "deck: 'dump' command only supports dumping 'all' types" );
        const int rate = (int)num( w, 4 ); // the reference truncates stod too
        if ( rate < 1 )
            throw Error( "deck: 'dump' needs a rate >= 1" );
        if ( w.size() < 6 )
            throw Error( "deck: missing argument in 'dump'" );
        if ( w[5].find( '*' ) == std::string::npos )
            throw Error( "deck: 'dump' requires '*' in file name, so it can be replaced by "
                         "the time step" );
        if ( w[5].find( '%' ) == std::string::npos )
            throw Error( "deck: 'dump' requires '%' in file name, so it can be replaced by "
                         "the rank" );
        d.vtk_rate = rate;
        d.vtk_file = w[5];
    }
    else if ( k == "variable" )
        throw Error( "deck: 'variable' is not supported" );
    else
        throw Error( "deck: unknown keyword in '" + line + "'" );
}

Deck parse_deck( const std::string &path )
{
    std::ifstream in( path );
    if ( !in )
        throw Error( "deck: cannot open " + path );
    Deck d;
    std::string line;
    while ( std::getline( in, line ) )
        apply_deck_line( d, line );
    return d;
}

// --------------------------------------------------------------------------
// inputFile.h:73-148.  The hash adds the bytes of the seed and of the three
// coordinates as `char`; the reference's CI builds on x86-64, where char is
// signed, so the bytes are taken as signed char here on every host.
void GeomRandom::reset( int seed, const double coord[3] )
{
    unsigned int hash = 0;
    auto mix = [&hash]( const void *p, size_t nb ) {
        const signed char *s = static_cast<const signed char *>( p );
        for ( size_t i = 0; i < nb; i++ )
        {
            hash += (unsigned int)(int)s[i];
            hash += ( hash << 10 );
            hash ^= ( hash >> 6 );
        }
    };
    mix( &seed, sizeof( int ) );
    mix( coord, 3 * sizeof( double ) );
    hash += ( hash << 3 );
    hash ^= ( hash >> 11 );
    hash += ( hash << 15 );
    seed_ = (int)( hash & 0x7ffffff ); // the reference keeps these 27 bits
    if ( !seed_ )
        seed_ = 1;
    for ( int i = 0; i < 5; i++ )
        uniform();
}

// Park-Miller minimal standard generator (Schrage's factorisation).
double GeomRandom::uniform()
{
    const int a = 16807, m = 2147483647, q = 127773, r = 2836;
    const int k = seed_ / q;
    seed_ = a * ( seed_ - k * q ) - r * k;
    if ( seed_ < 0 )
        seed_ += m;
    return ( 1.0 / m ) * seed_;
}

// --------------------------------------------------------------------------
static bool in_block( const Block &b, double a, double x, double y, double z )
{
    // region test in lattice units, as the reference's in_any_region
    return x >= a * b.xlo && x < a * b.xhi && y >= a * b.ylo && y < a * b.yhi &&
           z >= a * b.zlo && z < a * b.zhi;
}

static void init_units( const Deck &d, HostSystem &s )
{
    s.boltz = d.boltz;
    s.mvv2e = d.mvv2e;
    s.dt = d.dt;
    s.ntypes = d.ntypes;
    s.mass.assign( d.ntypes, 1.0 );
    for ( auto &m : d.mass )
        if ( m.first >= 0 && m.first < d.ntypes )
            s.mass[m.first] = m.second;
}

HostSystem create_lattice( const Deck &d )
{
    if ( d.lattice == LATTICE_NONE || d.regions.empty() )
        throw Error( "deck: no lattice / region to create atoms in" );
    HostSystem s;
    init_units( d, s );
    // the domain's high corner grows by the vacuum multiplier; atoms still
    // fill only the deck's box (inputFile_impl.h:553-559, 604-616)
    const double *mx = d.box_hi;
    for ( int q = 0; q < 3; q++ )
    {
        s.lo[q] = d.box_lo[q];
        s.hi[q] = d.box_hi[q] * d.vacuum;
    }
    const double a = d.lattice_constant;
    // one rank: the local mesh is the whole domain (inputFile_impl.h:580-603)
    const int ixs = (int)( s.lo[0] / a - 0.5 ), iys = (int)( s.lo[1] / a - 0.5 ),
              izs = (int)( s.lo[2] / a - 0.5 );
    int ixe = (int)std::max( std::min( mx[0] / a, s.hi[0] / a + 0.5 ), (double)ixs );
    int iye = (int)std::max( std::min( mx[1] / a, s.hi[1] / a + 0.5 ), (double)iys );
    int ize = (int)std::max( std::min( mx[2] / a, s.hi[2] / a + 0.5 ), (double)izs );
    if ( ixs == ixe )
        ixe -= 1;
    if ( iys == iye )
        iye -= 1;
    if ( izs == ize )
        ize -= 1;
    double basis[4][3] = { { 0, 0, 0 }, { 0.5, 0.5, 0 }, { 0.5, 0, 0.5 }, { 0, 0.5, 0.5 } };
    int nb = 4;
    if ( d.lattice == LATTICE_SC )
    {
        nb = 1;
        basis[0][0] = basis[0][1] = basis[0][2] = 0.0;
    }
    for ( int b = 0; b < nb; b++ )
        for ( int q = 0; q < 3; q++ )
            basis[b][q] += d.offset[q];
    // regions in the reference's std::map order (sorted by name)
    std::vector<std::pair<std::string, Block>> regs = d.regions;
    std::sort( regs.begin(), regs.end(),
               []( const auto &p, const auto &q ) { return p.first < q.first; } );
    for ( int iz = izs; iz <= ize; iz++ )
        for ( int iy = iys; iy <= iye; iy++ )
            for ( int ix = ixs; ix <= ixe; ix++ )
                for ( int k = 0; k < nb; k++ )
                {
                    const double xt = a * ( 1.0 * ix + basis[k][0] );
                    const double yt = a * ( 1.0 * iy + basis[k][1] );
                    const double zt = a * ( 1.0 * iz + basis[k][2] );
                    if ( !( xt >= s.lo[0] && yt >= s.lo[1] && zt >= s.lo[2] && xt < s.hi[0] &&
                            yt < s.hi[1] && zt < s.hi[2] && xt < mx[0] && yt < mx[1] &&
                            zt < mx[2] ) )
                        continue;
                    int type = -1;
                    for ( auto &r : regs )
                    {
                        auto it = d.region_type.find( r.first );
                        if ( it != d.region_type.end() && in_block( r.second, a, xt, yt, zt ) )
                        {
                            // several matching regions: the reference draws
                            // one with rand(); the first is taken here
                            type = it->second - 1;
                            break;
                        }
                    }
                    if ( type < 0 )
                        continue;
                    s.x.push_back( xt );
                    s.x.push_back( yt );
                    s.x.push_back( zt );
                    s.type.push_back( type );
                    s.id.push_back( (int)s.id.size() + 1 );
                }
    s.n = (int64_t)s.id.size();
    // velocities: uniform random per atom from the geom generator, divided
    // by sqrt(m), zero total momentum, scaled to the target temperature
    s.v.assign( 3 * s.n, 0.0 );
    double total_mass = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    for ( int64_t i = 0; i < s.n; i++ )
    {
        GeomRandom rnd;
        auto it = d.velocity.find( s.type[i] + 1 );
        const int seed = it != d.velocity.end() ? it->second.second : 0;
        rnd.reset( seed, &s.x[3 * i] );
        const double m = s.mass[s.type[i]];
        const double vx = rnd.uniform() - 0.5;
        const double vy = rnd.uniform() - 0.5;
        const double vz = rnd.uniform() - 0.5;
        s.v[3 * i] = vx / std::sqrt( m );
        s.v[3 * i + 1] = vy / std::sqrt( m );
        s.v[3 * i + 2] = vz / std::sqrt( m );
        total_mass += m;
        px += m * s.v[3 * i];
        py += m * s.v[3 * i + 1];
        pz += m * s.v[3 * i + 2];
    }
    const double svx = px / total_mass, svy = py / total_mass, svz = pz / total_mass;
    double smv2 = 0.0;
    for ( int64_t i = 0; i < s.n; i++ )
    {
        s.v[3 * i] -= svx;
        s.v[3 * i + 1] -= svy;
        s.v[3 * i + 2] -= svz;
        const double m = s.mass[s.type[i]];
        smv2 += ( s.v[3 * i] * s.v[3 * i] + s.v[3 * i + 1] * s.v[3 * i + 1] +
                  s.v[3 * i + 2] * s.v[3 * i + 2] ) *
                m;
    }
    const double T = smv2 * ( s.mvv2e / ( 1.0 * ( 3 * s.n - 3 ) * s.boltz ) );
    for ( int64_t i = 0; i < s.n; i++ )
    {
        auto it = d.velocity.find( s.type[i] + 1 );
        const double target = it != d.velocity.end() ? it->second.first : 0.0;
        const double f = T > 0 ? std::sqrt( target / T ) : 0.0;
        s.v[3 * i] *= f;
        s.v[3 * i + 1] *= f;
        s.v[3 * i + 2] *= f;
    }
    return s;
}

// --------------------------------------------------------------------------
// LAMMPS data files: header lines ("N atoms", "N atom types", "lo hi xlo
// xhi", ...), then the Masses, Atoms (atomic: id type x y z) and Velocities
// (id vx vy vz) sections, read as src/read_data.h:99-380 does for one rank.
// A whole token as a number: "1.0e" or "12abc" are errors, not 1.0 / 12.
static double num_of( const std::string &t, const std::string &path )
{
    size_t used = 0;
    double v = 0.0;
    try
    {
        v = std::stod( t, &used );
    }
    catch ( const std::exception & )
    {
        used = 0;
    }
    if ( used != t.size() || !std::isfinite( v ) )
        throw Error( "read_data: bad number '" + t + "' in " + path );
    return v;
}

static int64_t int_of( const std::string &t, const std::string &path )
{
    size_t used = 0;
    long long v = 0;
    try
    {
        v = std::stoll( t, &used );
    }
    catch ( const std::exception & )
    {
        used = 0;
    }
    if ( used != t.size() )
        throw Error( "read_data: bad integer '" + t + "' in " + path );
    return v;
}

HostSystem read_data( const std::string &path, const Deck &d )
{
    std::ifstream in( path );
    if ( !in )
        throw Error( "read_data: cannot open " + path );
    HostSystem s;
    init_units( d, s );
    std::string line;
    std::getline( in, line ); // title
    int64_t natoms = -1;
    bool box[3] = { false, false, false };
    std::map<int64_t, int64_t> slot; // id -> row
    bool atoms_read = false;
    while ( std::getline( in, line ) )
    {
        const std::string body = line.substr( 0, line.find( '#' ) );
        const auto w = words_of( body );
        if ( w.empty() )
            continue;
        if ( body.find( "atom types" ) != std::string::npos )
        {
            s.ntypes = (int)int_of( w[0], path );
            if ( s.ntypes < 1 )
                throw Error( "read_data: no atom types in " + path );
            s.mass.resize( s.ntypes, 1.0 );
        }
        else if ( body.find( "atoms" ) != std::string::npos )
            natoms = int_of( w[0], path );
        else if ( body.find( "xlo xhi" ) != std::string::npos )
        {
            s.lo[0] = num_of( w[0], path );
            s.hi[0] = num_of( w.at( 1 ), path );
            box[0] = true;
        }
        else if ( body.find( "ylo yhi" ) != std::string::npos )
        {
            s.lo[1] = num_of( w[0], path );
            s.hi[1] = num_of( w.at( 1 ), path );
            box[1] = true;
        }
        else if ( body.find( "zlo zhi" ) != std::string::npos )
        {
            s.lo[2] = num_of( w[0], path );
            s.hi[2] = num_of( w.at( 1 ), path );
            box[2] = true;
        }
        else if ( w[0] == "Masses" )
        {
            int got = 0;
            while ( got < s.ntypes && std::getline( in, line ) )
            {
                const auto m = words_of( line.substr( 0, line.find( '#' ) ) );
                if ( m.size() < 2 )
                    continue;
                const int t = (int)int_of( m[0], path ) - 1;
                if ( t >= 0 && t < s.ntypes )
                    s.mass[t] = num_of( m[1], path );
                got++;
            }
        }
        else if ( w[0] == "Atoms" )
        {
            if ( natoms < 0 )
                throw Error( "read_data: Atoms before the atom count" );
            int64_t got = 0;
            while ( got < natoms && std::getline( in, line ) )
            {
                const auto a = words_of( line.substr( 0, line.find( '#' ) ) );
                if ( a.size() < 5 )
                    continue;
                const double x = num_of( a[2], path ), y = num_of( a[3], path ),
                             z = num_of( a[4], path );
                const int64_t aid = int_of( a[0], path ), atype = int_of( a[1], path );
                if ( atype < 1 || atype > s.ntypes )
                    throw Error( "read_data: atom type out of range in " + path );
                got++;
                // one rank: keep what lies inside the box, as the reference
                if ( !( x >= s.lo[0] && y >= s.lo[1] && z >= s.lo[2] && x < s.hi[0] &&
                        y < s.hi[1] && z < s.hi[2] ) )
                    continue;
                if ( !slot.emplace( aid, (int64_t)s.id.size() ).second )
                    throw Error( "read_data: duplicate atom id in " + path );
                s.id.push_back( (int)aid );
                s.type.push_back( (int)atype - 1 );
                s.x.push_back( x );
                s.x.push_back( y );
                s.x.push_back( z );
            }
            if ( got < natoms )
                throw Error( "read_data: the Atoms section ends before " +
                             std::to_string( natoms ) + " atoms in " + path );
            s.n = (int64_t)s.id.size();
            s.v.assign( 3 * s.n, 0.0 );
            atoms_read = true;
        }
        else if ( w[0] == "Velocities" )
        {
            if ( !atoms_read )
                throw Error( "read_data: Must read Atoms before Velocities" ); // read_data.h:341
            int64_t got = 0;
            while ( got < natoms && std::getline( in, line ) )
            {
                const auto a = words_of( line.substr( 0, line.find( '#' ) ) );
                if ( a.size() < 4 )
                    continue;
                got++;
                double vq[3];
                for ( int q = 0; q < 3; q++ )
                    vq[q] = num_of( a[1 + q], path );
                auto it = slot.find( int_of( a[0], path ) );
                if ( it == slot.end() )
                    continue;
                for ( int q = 0; q < 3; q++ )
                    s.v[3 * it->second + q] = vq[q];
            }
            if ( got < natoms )
                throw Error( "read_data: the Velocities section ends before " +
                             std::to_string( natoms ) + " atoms in " + path );
        }
    }
    if ( !box[0] || !box[1] || !box[2] || natoms < 0 )
        throw Error( "read_data: incomplete header in " + path );
    // one rank keeps the atoms inside its box; all of them must be there
    // (read_data.h:368-374)
    if ( s.n != natoms )
        throw Error( "read_data: Created incorrect # of atoms (" + std::to_string( s.n ) +
                     " of " + std::to_string( natoms ) + ") from " + path );
    for ( auto &m : d.mass ) // deck masses override the file's
        if ( m.first >= 0 && m.first < s.ntypes )
            s.mass[m.first] = m.second;
    return s;
}

void write_data( const std::string &path, const HostSystem &s )
{
    FILE *f = std::fopen( path.c_str(), "w" );
    if ( !f )
        throw Error( "write_data: cannot open " + path );
    std::fprintf( f, "LAMMPS data file from the GB300 CabanaMD backend\n\n" );
    std::fprintf( f, "%lld atoms\n%d atom types\n\n", (long long)s.n, s.ntypes );
    std::fprintf( f, "%.17g %.17g xlo xhi\n%.17g %.17g ylo yhi\n%.17g %.17g zlo zhi\n\n",
                  s.lo[0], s.hi[0], s.lo[1], s.hi[1], s.lo[2], s.hi[2] );
    std::fprintf( f, "Masses\n\n" );
    for ( int t = 0; t < s.ntypes; t++ )
        std::fprintf( f, "%d %.17g\n", t + 1, t < (int)s.mass.size() ? s.mass[t] : 1.0 );
    std::fprintf( f, "\nAtoms # atomic\n\n" );
    for ( int64_t i = 0; i < s.n; i++ )
        std::fprintf( f, "%d %d %.17g %.17g %.17g\n", s.id[i], s.type[i] + 1, s.x[3 * i],
                      s.x[3 * i + 1], s.x[3 * i + 2] );
    std::fprintf( f, "\nVelocities\n\n" );
    for ( int64_t i = 0; i < s.n; i++ )
        std::fprintf( f, "%d %.17g %.17g %.17g\n", s.id[i], s.v[3 * i], s.v[3 * i + 1],
                      s.v[3 * i + 2] );
    std::fclose( f );
}

} // namespace cbnmd
