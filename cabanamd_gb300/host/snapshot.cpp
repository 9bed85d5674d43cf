// snapshot.cpp -- binary configuration snapshots and the correctness diff
// (CabanaMD's --dumpbinary / --correctness, CbnMD::dump_binary and
// CbnMD::check_correctness in src/cabanamd_impl.h:434-642).
//
// One file per dump step and rank, named <dir>/output.<step:%010d>.<rank:%03d>
// (cabanamd_impl.h:448-449), holding one record:
//   int32 n | int32 id[n] | int32 type[n] | float64 q[n] |
//   float64 x[n][3] | float64 v[n][3] | float64 f[n][3]
// The field order and widths are the reference's (T_INT = int, T_FLOAT =
// double, src/types.h).  Two defects of the reference are fixed here:
//  - its writer passes an AoSoA slice's data pointer to fwrite for 3n values,
//    which walks the structure-of-arrays tiles rather than n xyz triples, and
//    its reader indexes a [3][n] view as (atom, dim); here x, v and f are
//    written and read as n contiguous xyz triples, atom-major;
//  - its reader finds an atom whose id differs at the same position by a
//    linear scan per atom (quadratic in n); here ids are matched through a
//    hash map.
// The diff line (step, |dr|, max|dr_k|, |dv|, max|dv_k|, |df|, max|df_k|,
// cabanamd_impl.h:560-640) and the correctness file's header are the
// reference's; the file is truncated at step 0 and appended to after.
#include <cmath>
#include <cstdio>
#include <unordered_map>

#include "cbnmd.h"

namespace cbnmd
{

std::string snapshot_path( const std::string &dir, int64_t step, int rank )
{
    char tail[64];
    std::snprintf( tail, sizeof tail, "/output.%010lld.%03d", (long long)step, rank );
    return dir + tail;
}

Snapshot snapshot_of( const HostSystem &h, const std::vector<double> &f )
{
    if ( h.n > INT32_MAX )
        throw Error( "snapshot: more atoms than an int32 count holds" );
    Snapshot s;
    s.n = h.n;
    s.id = h.id;
    s.type = h.type;
    s.q.assign( h.n, 0.0 ); // atom style atomic: no charges
    s.x = h.x;
    s.v = h.v;
    s.f = f.empty() ? std::vector<double>( 3 * h.n, 0.0 ) : f;
    return s;
}

namespace
{
struct File
{
    FILE *p;
    explicit File( FILE *f ) : p( f ) {}
    ~File()
    {
        if ( p )
            std::fclose( p );
    }
};

template <class T>
void put( FILE *fp, const std::vector<T> &a, size_t count, const std::string &path )
{
    if ( a.size() != count )
        throw Error( "snapshot: array of the wrong length for " + path );
    if ( count && std::fwrite( a.data(), sizeof( T ), count, fp ) != count )
        throw Error( "snapshot: short write to " + path );
}

template <class T>
void get( FILE *fp, std::vector<T> &a, size_t count, const std::string &path )
{
    a.resize( count );
    if ( count && std::fread( a.data(), sizeof( T ), count, fp ) != count )
        throw Error( "Error reading reference data: " + path );
}
} // namespace

void write_snapshot( const std::string &path, const Snapshot &s )
{
    File f( std::fopen( path.c_str(), "wb" ) );
    if ( !f.p )
        throw Error( "Cannot open dump file: " + path );
    const int32_t n = (int32_t)s.n;
    if ( std::fwrite( &n, sizeof n, 1, f.p ) != 1 )
        throw Error( "snapshot: short write to " + path );
    put( f.p, s.id, s.n, path );
    put( f.p, s.type, s.n, path );
    put( f.p, s.q, s.n, path );
    put( f.p, s.x, 3 * s.n, path );
    put( f.p, s.v, 3 * s.n, path );
    put( f.p, s.f, 3 * s.n, path );
}

Snapshot read_snapshot( const std::string &path )
{
    File f( std::fopen( path.c_str(), "rb" ) );
    if ( !f.p )
        throw Error( "Cannot open input file: " + path );
    int32_t n = 0;
    if ( std::fread( &n, sizeof n, 1, f.p ) != 1 || n < 0 )
        throw Error( "Error reading reference data: " + path );
    Snapshot s;
    s.n = n;
    get( f.p, s.id, n, path );
    get( f.p, s.type, n, path );
    get( f.p, s.q, n, path );
    get( f.p, s.x, 3 * (size_t)n, path );
    get( f.p, s.v, 3 * (size_t)n, path );
    get( f.p, s.f, 3 * (size_t)n, path );
    if ( std::fgetc( f.p ) != EOF )
        throw Error( "snapshot: trailing bytes in " + path );
    return s;
}

SnapshotDiff snapshot_diff( const Snapshot &cur, const Snapshot &ref )
{
    if ( cur.n != ref.n )
        throw Error( "Mismatch in current and reference atom counts" );
    std::unordered_map<int, int64_t> where;
    where.reserve( (size_t)cur.n * 2 );
    for ( int64_t i = 0; i < cur.n; i++ )
        if ( !where.emplace( cur.id[i], i ).second )
            throw Error( "snapshot: duplicate atom id " + std::to_string( cur.id[i] ) );
    double s2[3] = { 0, 0, 0 };
    SnapshotDiff d;
    const std::vector<double> *a[3] = { &cur.x, &cur.v, &cur.f };
    const std::vector<double> *b[3] = { &ref.x, &ref.v, &ref.f };
    double *mx[3] = { &d.max_dr, &d.max_dv, &d.max_df };
    for ( int64_t i = 0; i < ref.n; i++ )
    {
        const auto it = where.find( ref.id[i] );
        if ( it == where.end() )
            throw Error( "Unable to find current id matching reference id: " +
                         std::to_string( ref.id[i] ) );
        const int64_t j = it->second;
        for ( int q = 0; q < 3; q++ )
            for ( int k = 0; k < 3; k++ )
            {
                const double del = ( *a[q] )[3 * j + k] - ( *b[q] )[3 * i + k];
                s2[q] += del * del;
                *mx[q] = std::fmax( *mx[q], std::fabs( del ) );
            }
    }
    d.dr_norm = std::sqrt( s2[0] );
    d.dv_norm = std::sqrt( s2[1] );
    d.df_norm = std::sqrt( s2[2] );
    return d;
}

std::string correctness_line( int64_t step, const SnapshotDiff &d )
{
    char buf[256];
    std::snprintf( buf, sizeof buf, "%lld %g %g %g %g %g %g\n", (long long)step, d.dr_norm,
                   d.max_dr, d.dv_norm, d.max_dv, d.df_norm, d.max_df );
    return buf;
}

void write_correctness( const std::string &file, int64_t step, const SnapshotDiff &d )
{
    File f( std::fopen( file.c_str(), step == 0 ? "w" : "a" ) );
    if ( !f.p )
        throw Error( "Cannot open correctness file: " + file );
    if ( step == 0 )
        std::fputs( "# timestep deltarnorm maxdelr deltavnorm maxdelv deltafnorm maxdelf\n", f.p );
    std::fputs( correctness_line( step, d ).c_str(), f.p );
}

} // namespace cbnmd
