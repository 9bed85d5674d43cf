// cbnmd.h -- host side of the GB300 backend: the input-deck front end and
// the C++ module adapters that CabanaMD's driver talks to.
//
// CabanaMD (paths inside the project) drives one run as
//   InputFile::read_file / check_lammps_command   src/inputFile_impl.h:125-534
//   InputFile::create_lattice (+ velocities)      src/inputFile_impl.h:536-865
//   read_lammps_data_file / write_data            src/read_data.h:99-422
//   CbnMD::init / run                             src/cabanamd_impl.h:70-432
// over the module interfaces Force / Neighbor / Integrator / System /
// Binning / Comm and the Temperature / KinE / PotE properties.  This header
// restates the deck and lattice semantics for the GB300 build and declares
// adapter classes with the same member functions, each forwarding to the C
// ABI in include/gbmd.h, so a caller written against the reference's
// modules calls the same functions here.
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbmd.h"

namespace cbnmd
{

// --------------------------------------------------------------------------
// Errors: the reference's log_err throws (src/output.h:37-54)
struct Error : std::runtime_error
{
    explicit Error( const std::string &m ) : std::runtime_error( m ) {}
};

// --------------------------------------------------------------------------
// Host state of one system (System's host mirror, src/system.h:65-136)
struct HostSystem
{
    int64_t n = 0;
    int ntypes = 1;
    double lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
    std::vector<double> x, v; // [n][3]
    std::vector<int> type;    // 0-based
    std::vector<int> id;
    std::vector<double> mass; // per type
    double boltz = 1.0, mvv2e = 1.0, dt = 0.005;
};

// --------------------------------------------------------------------------
// Input deck (LAMMPS subset, src/inputFile_impl.h:125-534)
enum Units { UNITS_LJ, UNITS_METAL, UNITS_REAL };
enum Lattice { LATTICE_NONE, LATTICE_SC, LATTICE_FCC };

struct Block
{
    double xlo, xhi, ylo, yhi, zlo, zhi;
};

struct Deck
{
    Units units = UNITS_LJ;
    bool timestep_set = false;
    double boltz = 1.0, mvv2e = 1.0, dt = 0.005;
    Lattice lattice = LATTICE_NONE;
    double lattice_constant = 0.0;
    double offset[3] = { 0, 0, 0 };
    std::vector<std::pair<std::string, Block>> regions; // in deck order
    std::map<std::string, int> region_type;             // create_atoms
    double box_lo[3] = { 1e300, 1e300, 1e300 }, box_hi[3] = { -1e300, -1e300, -1e300 };
    int ntypes = 1;
    std::map<int, double> mass; // type (0-based) -> mass
    bool read_data = false, write_data = false;
    std::string data_in, data_out;
    // force
    bool force_nnp = false;
    double force_cutoff = 0.0;
    std::vector<std::vector<std::string>> pair_coeff; // lj/cut rows
    std::vector<std::string> pair_style;              // nnp tokens
    // velocity create: type (1-based, 1 for "all") -> (T, seed)
    std::map<int, std::pair<double, int>> velocity;
    double skin = 0.0;
    int rebuild_every = 20;
    int max_neigh_guess = 50;
    double comm_ghost_cutoff = 0.0;
    bool half = false; // full list unless "newton on" (src/inputCL.cpp:57-64 default)
    bool newton_set = false;
    int nsteps = 100; // src/inputFile.h:238-260 defaults
    int thermo = 10;
    // command line (src/inputCL.cpp): --vacuum multiplier of the box's high
    // corner (the lattice still fills the deck's box, inputFile_impl.h:553-559)
    double vacuum = 1.0;
    // "dump <id> all vtk N file" (inputFile_impl.h:327-357): particle files
    // every N steps; the file name's '*' takes the step and '%' the rank
    int vtk_rate = 0;
    std::string vtk_file;
};

// Parse a deck file; unknown or unsupported commands throw, as the
// reference's check_lammps_command does.
Deck parse_deck( const std::string &path );
void apply_deck_line( Deck &d, const std::string &line );

// Lattice + velocities exactly as InputFile::create_lattice (one rank).
HostSystem create_lattice( const Deck &d );

// LAMMPS data files (src/read_data.h): Atoms (atomic), Masses, Velocities.
HostSystem read_data( const std::string &path, const Deck &d );
void write_data( const std::string &path, const HostSystem &s );

// The LAMMPS "velocity ... loop geom" generator the reference restates
// (src/inputFile.h:66-148): a Park-Miller stream seeded by a hash of the
// seed and the atom's coordinates.
class GeomRandom
{
  public:
    void reset( int seed, const double coord[3] );
    double uniform();

  private:
    int seed_ = 0;
};

// --------------------------------------------------------------------------
// Binary snapshots and the correctness diff (--dumpbinary / --correctness,
// src/cabanamd_impl.h:434-642); the record layout is in snapshot.cpp.
struct Snapshot
{
    int64_t n = 0;
    std::vector<int> id, type;
    std::vector<double> q;       // [n]
    std::vector<double> x, v, f; // [n][3]
};

struct SnapshotDiff
{
    double dr_norm = 0, max_dr = 0, dv_norm = 0, max_dv = 0, df_norm = 0, max_df = 0;
};

std::string snapshot_path( const std::string &dir, int64_t step, int rank );
Snapshot snapshot_of( const HostSystem &h, const std::vector<double> &f );
void write_snapshot( const std::string &path, const Snapshot &s );
Snapshot read_snapshot( const std::string &path );
// Current minus reference, atoms matched by id; throws on a count mismatch
// or a reference id that the current snapshot lacks.
SnapshotDiff snapshot_diff( const Snapshot &cur, const Snapshot &ref );
std::string correctness_line( int64_t step, const SnapshotDiff &d );
void write_correctness( const std::string &file, int64_t step, const SnapshotDiff &d );

// VTK particle files of "dump ... vtk" (src/vtk_writer.h:152-294): an ASCII
// UnstructuredGrid piece with Velocity, Id and Type point data and the
// positions, written at steps N, 2N, ... (cabanamd_impl.h:388-390).
std::string vtk_particles_path( const std::string &pattern, int64_t step, int rank );
void write_vtk_particles( const std::string &path, const HostSystem &h );

// --------------------------------------------------------------------------
// Module adapters over the C ABI (src/system.h, comm_mpi.h, binning_cabana.h,
// neighbor.h, force.h, integrator_nve.h, property_*.h).  They own nothing
// but a pointer to the shared context; the System adapter owns it.
class System
{
  public:
    explicit System( int device = 0 );
    ~System();
    System( const System & ) = delete;
    System &operator=( const System & ) = delete;
    void init( const HostSystem &h, int precision );
    // Current state in device order; f (optional) receives the forces.
    void download( HostSystem &h, std::vector<double> *f = nullptr ) const;
    gbmd_ctx *ctx() const { return c_; }
    int64_t N() const;
    double boltz = 1.0, mvv2e = 1.0, dt = 0.005;

  private:
    gbmd_ctx *c_ = nullptr;
};

void check( gbmd_ctx *c, int rc, const char *what );

class Comm
{
  public:
    Comm( System *s, double neigh_cut ) : s_( s ), cut_( neigh_cut ) {}
    int exchange();          // comm_mpi.h:141-168 (wrap into the box)
    void exchange_halo() {}  // images are resolved inside the list
    void update_halo() {}
    void update_force() {}   // ghost forces are the owners' already
    std::string name() const { return "Comm:GB300-periodic-images"; }

  private:
    System *s_;
    double cut_;
};

class Binning
{
  public:
    explicit Binning( System *s ) : s_( s ) {}
    // binning_cabana.h:64-66 (dx = dy = dz = the neighbour cutoff)
    void create_binning( double dx, double dy, double dz, int halo_depth, bool do_local,
                         bool do_ghost, bool sort );
    std::string name() const { return "Binning:GB300-counting-sort"; }

  private:
    System *s_;
};

class Neighbor
{
  public:
    // neighbor_verlet.h:36-41
    Neighbor( double neigh_cut, bool half_neigh, int max_neigh_guess, bool tree = false )
        : neigh_cut( neigh_cut ), half_neigh( half_neigh ), max_neigh_guess( max_neigh_guess ),
          tree( tree )
    {
    }
    // neighbor_verlet.h:43-62; tree: neighbor_tree.h:43-58 (no periodic images)
    void create( System *s );
    std::string name() const
    {
        return tree ? "Neighbor:GB300-no-image-list" : "Neighbor:GB300-transposed-Verlet";
    }
    double neigh_cut;
    bool half_neigh;
    int max_neigh_guess;
    bool tree;
};

class Force
{
  public:
    explicit Force( System *s ) : s_( s ) {}
    // force.h:57-74: LJ rows "pair_coeff i j eps sigma cut" or the
    // pair_style nnp tokens (dir <path> ... cflength x cfenergy y)
    void init_coeff( const std::vector<std::vector<std::string>> &lines );
    void compute( System *s, Neighbor *n );        // accumulates into zeroed f
    double compute_energy( System *s, Neighbor *n ); // total, not divided by N
    std::string name() const { return nnp_ ? "Force:GB300-NNP" : "Force:GB300-LJ"; }

  private:
    System *s_;
    bool nnp_ = false;
};

class Integrator
{
  public:
    explicit Integrator( System *s ) : s_( s ) {}
    void initial_integrate( System *s ); // integrator_nve.h:91-101
    void final_integrate( System *s );   // integrator_nve.h:102-110
    std::string name() const { return "Integrator:GB300-NVE"; }

  private:
    System *s_;
};

// property_temperature.h / property_kine.h / property_pote.h
double temperature( System *s );
double kinetic_energy( System *s );
double potential_energy( System *s, Force *f, Neighbor *n );

} // namespace cbnmd
