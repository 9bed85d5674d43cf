// vtk.cpp -- the particle files of CabanaMD's "dump <id> all vtk N file"
// (VTKWriter::writeParticles, src/vtk_writer.h:206-294; called every N steps
// from CbnMD::run, src/cabanamd_impl.h:388-390).
//
// File name: the first '*' of the pattern becomes the step, zero-padded to
// four digits, and the first '%' becomes "_<rank>" ("dump%_*.vtu" at step 10
// on rank 0: "dump_0_0010.vtu").  Content: one ASCII UnstructuredGrid piece
// holding the local atoms as points with no cells; point data Velocity
// (Float64 x3), Id (Int32) and Type (Int32, the 0-based internal type), then
// the positions, each value printed with %g as the reference does.  The
// reference writes the .pvtu index only on rank 1, so a one-process run has
// the pieces alone; this driver is one process and does the same.
#include <cstdio>
#include <sstream>

#include "cbnmd.h"

namespace cbnmd
{

std::string vtk_particles_path( const std::string &pattern, int64_t step, int rank )
{
    std::string p = pattern;
    const size_t star = p.find( '*' );
    if ( star == std::string::npos )
        throw Error( "VTK output file does not contain required '*'" );
    char digits[32];
    std::snprintf( digits, sizeof digits, "%04lld", (long long)step );
    p.replace( star, 1, digits );
    const size_t pct = p.find( '%' );
    if ( pct == std::string::npos )
        throw Error( "VTK output file does not contain required '%'" );
    p.replace( pct, 1, "_" + std::to_string( rank ) );
    return p;
}

void write_vtk_particles( const std::string &path, const HostSystem &h )
{
    FILE *f = std::fopen( path.c_str(), "w" );
    if ( !f )
        throw Error( "Cannot open VTK output file " + path );
    const int64_t n = h.n;
    std::fprintf( f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" "
                     "byte_order=\"LittleEndian\" header_type=\"UInt32\">\n<UnstructuredGrid>\n"
                     "<Piece NumberOfPoints=\"%lld\" NumberOfCells=\"0\">\n\t<PointData>\n",
                  (long long)n );
    auto triples = [&]( const char *name, const std::vector<double> &a ) {
        std::fprintf( f, "\t\t<DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"3\" "
                         "format=\"ascii\">\n",
                      name );
        for ( int64_t i = 0; i < n; i++ )
            std::fprintf( f, "%g %g %g ", a[3 * i], a[3 * i + 1], a[3 * i + 2] );
        std::fprintf( f, "\n\t\t</DataArray>\n" );
    };
    auto ints = [&]( const char *name, const std::vector<int> &a ) {
        std::fprintf( f, "\t\t<DataArray type=\"Int32\" Name=\"%s\" NumberOfComponents=\"1\" "
                         "format=\"ascii\">\n",
                      name );
        for ( int64_t i = 0; i < n; i++ )
            std::fprintf( f, "%d ", a[i] );
        std::fprintf( f, "\n\t\t</DataArray>\n" );
    };
    triples( "Velocity", h.v );
    ints( "Id", h.id );
    ints( "Type", h.type );
    std::fprintf( f, "\t</PointData>\n\t<CellData>\n\t</CellData>\n\t<Points>\n" );
    triples( "Points", h.x );
    std::fprintf( f, "\t</Points>\n\t<Cells>\n" );
    for ( const char *c : { "Int32\" Name=\"connectivity", "Int32\" Name=\"offsets",
                            "UInt8\" Name=\"types" } )
        std::fprintf( f, "\t\t<DataArray type=\"%s\" NumberOfComponents=\"1\" "
                         "format=\"ascii\">\n\n\t\t</DataArray>\n",
                      c );
    std::fprintf( f, "\t</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n" );
    if ( std::fclose( f ) != 0 )
        throw Error( "Error writing VTK output file " + path );
}

} // namespace cbnmd
