// modules.cpp -- CabanaMD's module interfaces as thin adapters over the C
// ABI (include/gbmd.h).  Each member function is the reference's call of the
// same name (paths inside the CabanaMD project):
//   System          src/system.h:65-272
//   Comm            src/comm_mpi.h:141-353 (one rank: wrap; images in-list)
//   Binning         src/binning_cabana.h:64-66
//   Neighbor        src/neighbor.h:54-75, neighbor_types/neighbor_verlet.h
//   Force           src/force.h:57-74
//   Integrator      src/integrator_nve.h:91-110
//   Temperature / KinE / PotE   src/property_*.h
#include <cstring>
#include <string>

#include "cbnmd.h"

namespace cbnmd
{

void check( gbmd_ctx *c, int rc, const char *what )
{
    if ( rc != GBMD_OK )
        throw Error( std::string( what ) + ": " + ( c ? gbmd_last_error( c ) : "no context" ) +
                     " (code " + std::to_string( rc ) + ")" );
}

System::System( int device )
{
    const int rc = gbmd_create( &c_, device );
    if ( rc != GBMD_OK )
        throw Error( "System: no GB300 context (code " + std::to_string( rc ) +
                     "); this build has no CPU fallback" );
}

System::~System() { gbmd_destroy( c_ ); }

void System::init( const HostSystem &h, int precision )
{
    boltz = h.boltz;
    mvv2e = h.mvv2e;
    dt = h.dt;
    check( c_, gbmd_set_units( c_, h.boltz, h.mvv2e, h.dt ), "set_units" );
    check( c_, gbmd_set_box( c_, h.lo, h.hi ), "set_box" );
    check( c_, gbmd_set_types( c_, h.ntypes, h.mass.data() ), "set_types" );
    check( c_, gbmd_set_precision( c_, precision ), "set_precision" );
    check( c_, gbmd_upload_atoms( c_, h.n, h.x.data(), h.v.data(), h.type.data(), h.id.data() ),
           "upload_atoms" );
}

void System::download( HostSystem &h, std::vector<double> *f ) const
{
    int64_t n = 0;
    check( c_, gbmd_num_atoms( c_, &n ), "num_atoms" );
    h.n = n;
    h.x.resize( 3 * n );
    h.v.resize( 3 * n );
    h.type.resize( n );
    h.id.resize( n );
    if ( f )
        f->resize( 3 * n );
    check( c_, gbmd_download_atoms( c_, h.x.data(), h.v.data(), f ? f->data() : nullptr,
                                    h.type.data(), h.id.data() ),
           "download_atoms" );
}

int64_t System::N() const
{
    int64_t n = 0;
    check( c_, gbmd_num_atoms( c_, &n ), "num_atoms" );
    return n;
}

int Comm::exchange()
{
    check( s_->ctx(), gbmd_exchange( s_->ctx() ), "Comm::exchange" );
    return 0; // one rank: nothing leaves
}

void Binning::create_binning( double dx, double, double, int, bool, bool, bool )
{
    check( s_->ctx(), gbmd_binning( s_->ctx(), dx ), "Binning::create_binning" );
}

void Neighbor::create( System *s )
{
    check( s->ctx(), gbmd_set_list_images( s->ctx(), tree ? 0 : 1 ), "Neighbor::create" );
    check( s->ctx(), gbmd_neigh_build( s->ctx(), neigh_cut, half_neigh ? 1 : 0, max_neigh_guess ),
           "Neighbor::create" );
}

void Force::init_coeff( const std::vector<std::vector<std::string>> &lines )
{
    gbmd_ctx *c = s_->ctx();
    for ( const auto &w : lines )
    {
        if ( w.size() >= 2 && w[0] == "pair_style" && w[1] == "nnp" )
        {
            // pair_style nnp dir <path> ... cflength <x> cfenergy <y>
            std::string dir;
            double cfl = 1.0, cfe = 1.0;
            for ( size_t i = 2; i + 1 < w.size(); i++ )
            {
                if ( w[i] == "dir" )
                    dir = w[i + 1];
                else if ( w[i] == "cflength" )
                    cfl = std::stod( w[i + 1] );
                else if ( w[i] == "cfenergy" )
                    cfe = std::stod( w[i + 1] );
            }
            if ( dir.empty() )
                throw Error( "Force::init_coeff: pair_style nnp without 'dir'" );
            check( c, gbmd_nnp_load( c, dir.c_str(), cfl, cfe ), "Force::init_coeff (nnp)" );
            nnp_ = true;
        }
        else if ( w.size() >= 6 && w[0] == "pair_coeff" )
        {
            // pair_coeff i j eps sigma cut (force_lj_cabana_neigh_impl.h:70-85)
            check( c,
                   gbmd_lj_coeff( c, std::stoi( w[1] ), std::stoi( w[2] ), std::stod( w[3] ),
                                  std::stod( w[4] ), std::stod( w[5] ) ),
                   "Force::init_coeff (lj)" );
            nnp_ = false;
        }
        else
            throw Error( "Force::init_coeff: unsupported line" );
    }
}

void Force::compute( System *s, Neighbor * )
{
    check( s->ctx(), gbmd_force_compute( s->ctx() ), "Force::compute" );
}

double Force::compute_energy( System *s, Neighbor * )
{
    double e = 0.0;
    check( s->ctx(), gbmd_force_energy( s->ctx(), &e ), "Force::compute_energy" );
    return e;
}

void Integrator::initial_integrate( System *s )
{
    check( s->ctx(), gbmd_integrate_initial( s->ctx() ), "Integrator::initial_integrate" );
}

void Integrator::final_integrate( System *s )
{
    check( s->ctx(), gbmd_integrate_final( s->ctx() ), "Integrator::final_integrate" );
}

double temperature( System *s )
{
    double T = 0.0, KE = 0.0;
    check( s->ctx(), gbmd_thermo( s->ctx(), &T, &KE ), "Temperature::compute" );
    return T;
}

double kinetic_energy( System *s )
{
    double T = 0.0, KE = 0.0;
    check( s->ctx(), gbmd_thermo( s->ctx(), &T, &KE ), "KinE::compute" );
    return KE;
}

double potential_energy( System *s, Force *f, Neighbor *n ) { return f->compute_energy( s, n ); }

} // namespace cbnmd
