// cbnmd_gb300.cpp -- CabanaMD's driver (src/CabanaMD.cpp, CbnMD::init / run
// in src/cabanamd_impl.h:70-432) on the GB300 backend.
//
//   cbnmd_gb300 -il <deck> [-o out] [--force-iteration NEIGH_FULL|NEIGH_HALF]
//               [--precision fp64|mixed] [--device N] [--modules]
//               [--init-only <data file>] [--parse-only]
//               [--dumpbinary N DIR] [--correctness N DIR FILE]
//               [--neigh-type VERLET_2D|VERLET_CSR|TREE_2D|TREE_CSR] [--vacuum R]
//   cbnmd_gb300 --snapdiff <current snapshot> <reference snapshot>
//
// The deck's commands, the lattice / velocity set-up, the timestep order and
// the output lines (print_summary, cabanamd_impl.h:645-676, and the final
// performance block, :401-425) are the reference's.  Two loops run it:
//  - default: gbmd_md_run in thermo-interval chunks (fused kernels, one
//    launch per step for LJ full lists);
//  - --modules: the reference's own loop, module call by module call, through
//    the adapter classes (System, Comm, Binning, Neighbor, Force, Integrator).
// --neigh-type TREE_* builds lists without periodic images, as CabanaMD's
// ArborX tree lists over the local atoms do (neighbor_tree.h:43-58); the
// VERLET_* layouts are one transposed list here.  --vacuum R multiplies the
// domain's high corner by R > 1 while the lattice fills the deck's box.
// --init-only writes the initial state as a LAMMPS data file without using
// the GPU; --parse-only prints the parsed deck.  --dumpbinary writes a binary
// snapshot every N steps (and at step 0) and --correctness compares the state
// every N steps with the snapshots in DIR, appending one line per check to
// FILE (CbnMD::dump_binary / check_correctness, cabanamd_impl.h:434-642);
// --snapdiff prints that line for two snapshot files, without a GPU.  Reference command-line
// options that select Kokkos back ends (--device-type, --neigh-parallel,
// --neigh-type) are accepted and have no effect: there is one back end.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <memory>
#include <sstream>

#include "cbnmd.h"

using namespace cbnmd;

namespace
{
struct Args
{
    std::string deck, out, init_only;
    bool parse_only = false, modules = false, tree = false;
    double vacuum = 1.0;
    int dump_rate = 0, corr_rate = 0;
    std::string dump_dir, corr_dir, corr_file, diff_cur, diff_ref;
    int precision = GBMD_PREC_FP64;
    int device = 0;
    int force_iteration = -1; // -1: the deck's newton setting
};

[[noreturn]] void usage( const char *msg )
{
    std::fprintf( stderr,
                  "%s\nusage: cbnmd_gb300 -il <deck> [-o out] [--force-iteration NEIGH_FULL|"
                  "NEIGH_HALF] [--precision fp64|mixed] [--device N] [--modules] "
                  "[--init-only file] [--parse-only] [--dumpbinary N DIR] [--neigh-type T] [--vacuum R] "
                  "[--correctness N DIR FILE]\n       cbnmd_gb300 --snapdiff CUR REF\n",
                  msg );
    std::exit( 2 );
}

Args parse_args( int argc, char **argv )
{
    Args a;
    for ( int i = 1; i < argc; i++ )
    {
        const std::string k = argv[i];
        auto val = [&]() -> std::string {
            if ( i + 1 >= argc )
                usage( ( "missing value after " + k ).c_str() );
            return argv[++i];
        };
        if ( k == "-il" || k == "--input-lammps" )
            a.deck = val();
        else if ( k == "-o" || k == "--output-file" )
            a.out = val();
        else if ( k == "-e" || k == "--error-file" )
            val();
        else if ( k == "--force-iteration" )
        {
            const std::string v = val();
            if ( v == "NEIGH_FULL" )
                a.force_iteration = 0;
            else if ( v == "NEIGH_HALF" )
                a.force_iteration = 1;
            else
                usage( "--force-iteration takes NEIGH_FULL or NEIGH_HALF" );
        }
        else if ( k == "--precision" )
        {
            const std::string v = val();
            if ( v == "fp64" )
                a.precision = GBMD_PREC_FP64;
            else if ( v == "mixed" )
                a.precision = GBMD_PREC_MIXED;
            else
                usage( "--precision takes fp64 or mixed" );
        }
        else if ( k == "--device" )
            a.device = std::stoi( val() );
        else if ( k == "--modules" )
            a.modules = true;
        else if ( k == "--init-only" )
            a.init_only = val();
        else if ( k == "--parse-only" )
            a.parse_only = true;
        else if ( k == "--dumpbinary" )
        {
            a.dump_rate = std::stoi( val() );
            a.dump_dir = val();
            if ( a.dump_rate < 1 )
                usage( "--dumpbinary takes a rate >= 1" );
        }
        else if ( k == "--correctness" )
        {
            a.corr_rate = std::stoi( val() );
            a.corr_dir = val();
            a.corr_file = val();
            if ( a.corr_rate < 1 )
                usage( "--correctness takes a rate >= 1" );
        }
        else if ( k == "--snapdiff" )
        {
            a.diff_cur = val();
            a.diff_ref = val();
        }
        else if ( k == "--neigh-type" )
        {
            const std::string v = val();
            if ( v == "TREE_2D" || v == "TREE_CSR" )
                a.tree = true;
            else if ( v != "VERLET_2D" && v != "VERLET_CSR" )
                usage( ( "Unknown commandline option: --neigh-type " + v ).c_str() );
        }
        else if ( k == "--vacuum" )
        {
            a.vacuum = std::stod( val() );
            if ( !( a.vacuum > 1.0 ) )
                usage( "Vacuum multiplier must be bigger than 1.0" );
        }
        else if ( k == "--device-type" || k == "--neigh-parallel" )
            val();
        else if ( k == "-h" || k == "--help" )
            usage( "" );
        else
            usage( ( "unknown option " + k ).c_str() );
    }
    if ( a.deck.empty() && a.diff_cur.empty() )
        usage( "no input deck (-il)" );
    return a;
}

struct Out
{
    std::ofstream file;
    std::ostream &os() { return file.is_open() ? (std::ostream &)file : std::cout; }
};

void print_header( std::ostream &o )
{
    o << "\n#Timestep Temperature PotE ETot Time Atomsteps/s\n";
}

// print_summary (cabanamd_impl.h:645-676)
void print_row( std::ostream &o, int step, double T, double PE, double KE, double time,
                double rate )
{
    o << step << "\t" << std::fixed << std::setprecision( 6 ) << T << "\t" << PE << "\t"
      << PE + KE << "\t" << std::setprecision( 2 ) << time << "\t" << std::scientific << rate
      << "\n";
    o << std::defaultfloat;
}

void print_json_deck( const Deck &d )
{
    std::printf( "{\"units\": %d, \"lattice\": %d, \"lattice_constant\": %.17g, "
                 "\"box_lo\": [%.17g, %.17g, %.17g], \"box_hi\": [%.17g, %.17g, %.17g], "
                 "\"ntypes\": %d, \"force\": \"%s\", \"force_cutoff\": %.17g, \"skin\": %.17g, "
                 "\"rebuild_every\": %d, \"max_neigh_guess\": %d, \"half\": %d, "
                 "\"nsteps\": %d, \"thermo\": %d, \"dt\": %.17g, \"boltz\": %.17g, "
                 "\"mvv2e\": %.17g, \"pair_coeff_rows\": %d, \"read_data\": \"%s\", "
                 "\"vtk_rate\": %d, \"vtk_file\": \"%s\"}\n",
                 (int)d.units, (int)d.lattice, d.lattice_constant, d.box_lo[0], d.box_lo[1],
                 d.box_lo[2], d.box_hi[0], d.box_hi[1], d.box_hi[2], d.ntypes,
                 d.force_nnp ? "nnp" : "lj/cut", d.force_cutoff, d.skin, d.rebuild_every,
                 d.max_neigh_guess, d.half ? 1 : 0, d.nsteps, d.thermo, d.dt, d.boltz, d.mvv2e,
                 (int)d.pair_coeff.size(), d.data_in.c_str(), d.vtk_rate, d.vtk_file.c_str() );
}

std::vector<std::vector<std::string>> coeff_lines( const Deck &d )
{
    if ( d.force_nnp )
        return { d.pair_style };
    return d.pair_coeff;
}
} // namespace

int main( int argc, char **argv )
{
    const Args a = parse_args( argc, argv );
    try
    {
        if ( !a.diff_cur.empty() )
        {
            const SnapshotDiff df =
                snapshot_diff( read_snapshot( a.diff_cur ), read_snapshot( a.diff_ref ) );
            std::printf( "# deltarnorm maxdelr deltavnorm maxdelv deltafnorm maxdelf\n"
                         "%.17g %.17g %.17g %.17g %.17g %.17g\n",
                         df.dr_norm, df.max_dr, df.dv_norm, df.max_dv, df.df_norm, df.max_df );
            return 0;
        }
        Deck d = parse_deck( a.deck );
        d.vacuum = a.vacuum;
        if ( a.force_iteration >= 0 )
            d.half = a.force_iteration == 1;
        if ( a.parse_only )
        {
            print_json_deck( d );
            return 0;
        }
        HostSystem h = d.read_data ? read_data( d.data_in, d ) : create_lattice( d );
        if ( !a.init_only.empty() )
        {
            write_data( a.init_only, h );
            return 0;
        }
        if ( d.force_nnp && d.half )
            throw Error( "Half neighbor list not implemented for the neural network potential." );
        Out out;
        if ( !a.out.empty() )
            out.file.open( a.out );
        std::ostream &o = out.os();
        const double neigh_cut = d.force_cutoff + d.skin;

        // CbnMD::init (cabanamd_impl.h:70-255)
        System sys( a.device );
        sys.init( h, a.precision );
        Comm comm( &sys, neigh_cut );
        Integrator integrator( &sys );
        Binning binning( &sys );
        Neighbor neighbor( neigh_cut, d.half, d.max_neigh_guess, a.tree );
        Force force( &sys );
        force.init_coeff( coeff_lines( d ) );
        o << "Using: " << force.name() << " " << neighbor.name() << " " << comm.name() << " "
          << binning.name() << " " << integrator.name() << "\n";
        o << "Atoms: " << h.n << " " << h.n << "\n";
        const double N = (double)h.n;
        gbmd_ctx *c = sys.ctx();
        const auto t0 = std::chrono::steady_clock::now();
        auto seconds = [&]() {
            return std::chrono::duration<double>( std::chrono::steady_clock::now() - t0 ).count();
        };
        double last = 0.0;
        // dump_binary / check_correctness after step 0 and after each step
        // (cabanamd_impl.h:245-252, 392-396); the VTK particle files after
        // steps 1..nsteps (:388-390)
        auto snapshots = [&]( int step ) {
            const bool dump = a.dump_rate > 0 && step % a.dump_rate == 0;
            const bool corr = a.corr_rate > 0 && step % a.corr_rate == 0;
            const bool vtk = d.vtk_rate > 0 && step > 0 && step % d.vtk_rate == 0;
            if ( !dump && !corr && !vtk )
                return;
            HostSystem cur;
            std::vector<double> f;
            sys.download( cur, &f );
            if ( vtk )
                write_vtk_particles( vtk_particles_path( d.vtk_file, step, 0 ), cur );
            if ( !dump && !corr )
                return;
            const Snapshot snap = snapshot_of( cur, f );
            if ( dump )
                write_snapshot( snapshot_path( a.dump_dir, step, 0 ), snap );
            if ( corr )
                write_correctness(
                    a.corr_file, step,
                    snapshot_diff( snap, read_snapshot( snapshot_path( a.corr_dir, step, 0 ) ) ) );
        };
        if ( a.modules )
        {
            comm.exchange();
            binning.create_binning( neigh_cut, neigh_cut, neigh_cut, 1, true, false, true );
            comm.exchange_halo();
            neighbor.create( &sys );
            check( c, gbmd_zero_force( c ), "zero force" );
            force.compute( &sys, &neighbor );
            comm.update_force();
            if ( d.thermo > 0 )
            {
                print_header( o );
                print_row( o, 0, temperature( &sys ), potential_energy( &sys, &force, &neighbor ) / N,
                           kinetic_energy( &sys ) / N, 0.0, 0.0 );
            }
            snapshots( 0 );
            for ( int step = 1; step <= d.nsteps; step++ )
            {
                integrator.initial_integrate( &sys );
                if ( step % d.rebuild_every == 0 )
                {
                    comm.exchange();
                    binning.create_binning( neigh_cut, neigh_cut, neigh_cut, 1, true, false,
                                            true );
                    comm.exchange_halo();
                    neighbor.create( &sys );
                }
                else
                    comm.update_halo();
                check( c, gbmd_zero_force( c ), "zero force" );
                force.compute( &sys, &neighbor );
                comm.update_force();
                integrator.final_integrate( &sys );
                if ( d.thermo > 0 && step % d.thermo == 0 )
                {
                    const double T = temperature( &sys );
                    const double PE = potential_energy( &sys, &force, &neighbor ) / N;
                    const double KE = kinetic_energy( &sys ) / N;
                    const double t = seconds();
                    print_row( o, step, T, PE, KE, t, N * d.thermo / ( t - last ) );
                    last = t;
                }
                snapshots( step );
            }
        }
        else
        {
            gbmd_md_params p{ d.force_cutoff, d.skin, d.half ? 1 : 0, d.rebuild_every,
                              d.thermo, d.max_neigh_guess };
            check( c, gbmd_set_list_images( c, a.tree ? 0 : 1 ), "list images" );
            double row0[4];
            check( c, gbmd_md_init( c, &p, row0 ), "md_init" );
            if ( d.thermo > 0 )
            {
                print_header( o );
                print_row( o, 0, row0[1], row0[2], row0[3], 0.0, 0.0 );
            }
            snapshots( 0 );
            // Each gbmd_md_run call ends at the next thermo, dump, VTK or check
            // step.
            auto next_stop = [&]( int done ) {
                int stop = d.nsteps;
                for ( int r : { d.thermo, a.dump_rate, a.corr_rate, d.vtk_rate } )
                    if ( r > 0 )
                        stop = std::min( stop, ( done / r + 1 ) * r );
                return stop;
            };
            const int chunk = d.thermo > 0 ? d.thermo : d.nsteps;
            int done = 0;
            std::vector<double> rows( 4 * ( chunk + 1 ) );
            while ( done < d.nsteps )
            {
                const int k = next_stop( done ) - done;
                int nr = 0;
                check( c, gbmd_md_run( c, k, rows.data(), chunk + 1, &nr ), "md_run" );
                done += k;
                for ( int r = 0; r < nr; r++ )
                {
                    const double t = seconds();
                    print_row( o, (int)rows[4 * r], rows[4 * r + 1], rows[4 * r + 2],
                               rows[4 * r + 3], t, N * d.thermo / ( t - last ) );
                    last = t;
                }
                snapshots( done );
            }
        }
        check( c, gbmd_synchronize( c ), "synchronize" );
        const double time = seconds();
        const double sps = d.nsteps / time;
        // final performance lines (cabanamd_impl.h:401-425; one process)
        o << std::fixed << std::setprecision( 2 ) << "\n#Procs Atoms | Time T_Force T_Neigh "
          << "T_Comm T_Int T_lb T_Other |\n1 " << h.n << " | " << time
          << " - - - - - - | PERFORMANCE\n\n#Steps/s Atomsteps/s Atomsteps/(proc*s)\n"
          << std::scientific << sps << " " << sps * N << " " << sps * N << "\n";
        o << std::defaultfloat;
        if ( d.write_data )
        {
            HostSystem fin;
            sys.download( fin );
            fin.lo[0] = h.lo[0], fin.lo[1] = h.lo[1], fin.lo[2] = h.lo[2];
            fin.hi[0] = h.hi[0], fin.hi[1] = h.hi[1], fin.hi[2] = h.hi[2];
            fin.ntypes = h.ntypes;
            fin.mass = h.mass;
            write_data( d.data_out, fin );
        }
        return 0;
    }
    catch ( const std::exception &e )
    {
        std::fprintf( stderr, "cbnmd_gb300: %s\n", e.what() );
        return 1;
    }
}
