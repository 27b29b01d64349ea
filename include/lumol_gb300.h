/*
 * lumol_gb300.h -- C ABI of the GB300 force / energy / integration engine for Lumol.
 *
 * One engine handle owns the device state of one or more independent systems
 * (a "batch"; a Lumol `System` is a batch of one).  All host arrays are owned
 * by the caller and copied in and out; device memory belongs to the handle
 * until lg_destroy.  Every function returns LG_OK (0) or an LG_ERR_* status;
 * lg_last_error() gives the message.  A handle is not re-entrant: callers
 * serialise access to it (Lumol's SharedEwald does the same with a RwLock,
 * lumol-core/src/energy/global/ewald.rs:847-875).  Distinct handles may be used
 * from different threads.
 *
 * Units are Lumol's internal units (lumol-core/src/units.rs:4-16): Angstrom,
 * femtosecond, unified atomic mass, Kelvin; energies in u A^2 / fs^2, which is
 * 1e4 kJ/mol (units::from(0.544, "kJ/mol") = 5.44e-5; the module comment of
 * units.rs says 1e-4 kJ/mol, its conversions use 1e4).
 *
 * Arrays of vectors are 3*n doubles, x y z per atom, the layout of
 * `&[Vector3D]` (lumol-core/src/types/vectors.rs:59).  A virial is 9 doubles,
 * row-major, the layout of `Matrix3` (lumol-core/src/types/matrix.rs:73).
 */
#ifndef LUMOL_GB300_H
#define LUMOL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LG_ABI_VERSION 1

/* ---- status codes --------------------------------------------------------- */
enum {
    LG_OK = 0,
    LG_ERR_ARGUMENT = 1,  /* invalid argument; the reference panics in the same cases */
    LG_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    LG_ERR_STATE = 3,     /* call out of order (e.g. compute before set_cell) */
    LG_ERR_CAPACITY = 4,  /* a device list overflowed and could not be regrown */
    LG_ERR_NONFINITE = 5, /* a non-finite energy was produced (compute.rs:125) */
    LG_ERR_NO_DEVICE = 6  /* no CUDA device is visible: there is no CPU fallback */
};

/* ---- enumerations mirroring the reference --------------------------------- */
/* Pair potentials (lumol-core/src/energy/functions.rs). */
enum {
    LG_PAIR_ABSENT = 0,     /* no PairInteraction for this kind pair */
    LG_PAIR_NULL = 1,       /* NullPotential (functions.rs:29-50) */
    LG_PAIR_LJ = 2,         /* LennardJones {sigma, epsilon} (functions.rs:71-107) */
    LG_PAIR_BUCKINGHAM = 3, /* Buckingham {a, c, rho} (functions.rs:276-319) */
    LG_PAIR_HARMONIC = 4,   /* Harmonic {k, x0} (functions.rs:127-160) */
    LG_PAIR_BMH = 5,        /* BornMayerHuggins {a, c, d, sigma, rho} (functions.rs:321-386) */
    LG_PAIR_MORSE = 6,      /* Morse {a, x0, depth} (functions.rs:388-437) */
    LG_PAIR_GAUSSIAN = 7,   /* Gaussian {a, b}, b > 0 (functions.rs:439-494) */
    LG_PAIR_MIE = 8         /* Mie {sigma, epsilon, n, m}, m < n (functions.rs:496-592) */
};

/* PairRestriction (lumol-core/src/energy/restrictions.rs:13-33). */
enum {
    LG_RESTRICT_NONE = 0,
    LG_RESTRICT_INTRA = 1,
    LG_RESTRICT_INTER = 2,
    LG_RESTRICT_EXCLUDE12 = 3,
    LG_RESTRICT_EXCLUDE13 = 4,
    LG_RESTRICT_EXCLUDE14 = 5,
    LG_RESTRICT_SCALE14 = 6
};

/* Coulombic potentials (energy/global/ewald.rs, energy/global/wolf.rs). */
enum { LG_COULOMB_NONE = 0, LG_COULOMB_EWALD = 1, LG_COULOMB_WOLF = 2 };

/* Arithmetic of the force path. */
enum {
    LG_PRECISION_FP64 = 0,  /* reference arithmetic in FP64, pair sets bit-exact */
    LG_PRECISION_MIXED = 1  /* FP32 pair / Ewald arithmetic with compensated per-atom
                               force sums; FP64 energies, virials, rho(k) and x/v state */
};

/* Energy / force / virial terms (bit mask). */
enum {
    LG_TERM_PAIRS = 1,          /* EnergyEvaluator::pairs (sys/energy.rs:47-59) */
    LG_TERM_TAIL = 2,           /* EnergyEvaluator::pairs_tail (sys/energy.rs:63-79) */
    LG_TERM_BONDS = 4,          /* bonds (sys/energy.rs:90-100) */
    LG_TERM_ANGLES = 8,         /* angles (sys/energy.rs:110-120) */
    LG_TERM_COUL_REAL = 16,     /* Ewald real space, or the whole Wolf sum */
    LG_TERM_COUL_SELF = 32,     /* Ewald self energy (ewald.rs:619-626) */
    LG_TERM_COUL_KSPACE = 64,   /* Ewald k-space (ewald.rs:677-733) */
    LG_TERM_DIHEDRALS = 128,    /* dihedral angles (sys/energy.rs:130-141) */
    LG_TERM_ALL = 255
};

/* Quantities (bit mask). */
enum { LG_WANT_FORCES = 1, LG_WANT_ENERGY = 2, LG_WANT_VIRIAL = 4 };

/* ---- descriptors ---------------------------------------------------------- */
/* One PairInteraction (lumol-core/src/energy/pairs.rs:57-95). */
typedef struct {
    int32_t type;         /* LG_PAIR_* */
    int32_t shifted;      /* 1: PairInteraction::shifted (energy shifted, force not) */
    int32_t restriction;  /* LG_RESTRICT_* */
    int32_t tail;         /* 1: enable_tail_corrections */
    double p0, p1, p2;    /* LJ: sigma, epsilon; Buckingham: a, c, rho; Harmonic: k, x0;
                             Morse: a, x0, depth; Gaussian: a, b; BMH and Mie: see p3, p4 */
    double cutoff;
    double scale14;       /* factor of LG_RESTRICT_SCALE14 */
    double p3, p4;        /* BMH: {a, c, d, sigma, rho} = p0..p4; Mie: {sigma, epsilon, n, m} = p0..p3 */
    int32_t table_size;   /* > 0: TableComputation::new(potential, table_size, table_max)
                             (energy/computations.rs:63-128): energies and forces interpolated
                             from table_size points on [0, table_max), zero beyond; tail
                             corrections from the potential itself (computations.rs:151-173) */
    int32_t table_pad;
    double table_max;
} lg_pair;

/* Bond, angle and dihedral potentials beyond the pair kinds (functions.rs). */
enum {
    LG_BONDED_COSINE_HARMONIC = 10, /* CosineHarmonic::new(k, x0): k/2 (cos x - cos x0)^2 (functions.rs:162-210) */
    LG_BONDED_TORSION = 11          /* Torsion {k, delta, n}: k (1 + cos(n x - delta)) (functions.rs:212-258) */
};
/* A bond, angle or dihedral potential: bonds LG_PAIR_NULL / LG_PAIR_HARMONIC /
 * LG_PAIR_MORSE; angles also LG_BONDED_COSINE_HARMONIC; dihedrals also
 * LG_BONDED_TORSION (x0 = delta, n = multiplicity).  Morse {a, x0, depth}
 * (functions.rs:405-437, BondPotential / AnglePotential / DihedralPotential)
 * takes k = depth, x0 and a. */
typedef struct {
    int32_t type;  /* LG_PAIR_ABSENT, LG_PAIR_NULL, LG_PAIR_HARMONIC, LG_PAIR_MORSE or LG_BONDED_* */
    int32_t n;     /* Torsion multiplicity */
    double k, x0;
    double a;      /* Morse width */
} lg_bonded;

/* Ewald::new(cutoff, kmax, alpha) (ewald.rs:278-305) or Wolf::new(cutoff) (wolf.rs:68-84). */
typedef struct {
    int32_t kind;         /* LG_COULOMB_* */
    int32_t restriction;  /* CoulombicPotential::set_restriction (global/mod.rs:197-202) */
    int32_t kmax;         /* Ewald only, > 0 */
    int32_t pad;
    double cutoff;
    double alpha;         /* Ewald only; <= 0 selects the default PI / cutoff */
    double scale14;
} lg_coulomb;

/* Engine options. */
typedef struct {
    int32_t device;      /* CUDA device ordinal */
    int32_t precision;   /* LG_PRECISION_* */
    double skin;         /* Verlet-list skin in Angstrom (0: default 1.0) */
    int32_t threads_per_atom;  /* 1, 2, 4, 8, 16 or 32 threads per atom in the pair kernels;
                                  0: chosen by the autotuner.  A fixed value makes every
                                  system's results independent of the rest of the batch. */
    int32_t flags;       /* LG_OPT_* bits */
} lg_options;

/* lg_options.flags.  Batches of mixed-precision systems with pair potentials
   only (no bonds, restrictions or Coulomb) run MD in one persistent launch per
   lg_md_run chunk of up to 256 steps (runs of 4 or more steps, or any run of
   a batch of at most four systems), one thread-block cluster per group of
   systems; this flag keeps them on the per-step kernels instead. */
#define LG_OPT_NO_PERSISTENT 1
/* Every block of the persistent kernel stages its group's positions in shared
   memory for the neighbour gathers (by default they go through L1, which
   keeps more of the neighbour list cached; measured 5 % slower on the batched
   LJ workload, where the copy each step costs more than it saves). */
#define LG_OPT_STAGING 2
/* Bits 4-7 of lg_options.flags fix the cluster size of the persistent kernel
   (the value is log2(size) + 1, so 1, 2, 3, 4 select 1, 2, 4, 8 blocks);
   0 lets the planner choose. */
#define LG_OPT_CLUSTER_SHIFT 4

typedef struct lg_engine lg_engine;

/* ---- lifetime --------------------------------------------------------------- */
int lg_version(void);
/* Message of the last failure on `engine` (or of the last failed lg_create when NULL). */
const char* lg_last_error(const lg_engine* engine);

/* Creates an engine with `n_systems` independent systems (1 for a Lumol System). */
int lg_create(const lg_options* options, int32_t n_systems, lg_engine** engine);
void lg_destroy(lg_engine* engine);

/* ---- system description (per system index `s`) ----------------------------- */
/* CellShape (cells.rs:12-20) of a cell given to lg_set_cell_ex. */
#define LG_CELL_ORTHORHOMBIC 0
#define LG_CELL_TRICLINIC 1

/* UnitCell::ortho / cubic / triclinic (cells.rs:51-94): `matrix` is the 3x3
 * cell, row-major, its columns the cell vectors (UnitCell::matrix).  The shape
 * follows from the matrix: any non-zero off-diagonal entry makes it
 * triclinic (UnitCell::triclinic with any angle; its 90-degree angles leave
 * cos(pi / 2) terms off the diagonal).  Replaces setting `System::cell`. */
int lg_set_cell(lg_engine* e, int32_t s, const double matrix[9]);
/* The same with the shape given: LG_CELL_TRICLINIC for any cell whose
 * volume is positive (a triclinic cell with a diagonal matrix still takes the
 * triclinic branches, as in the reference); LG_CELL_ORTHORHOMBIC for a matrix
 * with a positive diagonal.  An orthorhombic matrix may have off-diagonal
 * terms (UnitCell::scale_mut keeps the shape, cells.rs:201-207, so
 * AnisoBerendsenBarostat leaves them): as in the reference, the minimum
 * image, wrap and volume read its diagonal, the face distances and the
 * k-vectors the whole matrix. */
int lg_set_cell_ex(lg_engine* e, int32_t s, const double matrix[9], int32_t shape);

/* Particles of system `s` (Configuration, sys/config/configuration.rs:42-51):
 * kinds index the pair table, molecules give each atom's molecule index
 * (atoms of a molecule are contiguous, as in Lumol). */
int lg_set_particles(lg_engine* e, int32_t s, int64_t n, const int32_t* kinds,
                     const double* charges, const double* masses, const int32_t* molecules);

/* Bonds (i, j) and angles (i, j, k) of system `s` with their potentials
 * (Molecule::bonds/angles with System::bond_potential / angle_potential,
 * sys/system.rs:185-204).  Bond paths for restrictions are derived from the
 * bonds as Bonding::rebuild does (sys/config/bonding.rs:78-186). */
int lg_set_bonds(lg_engine* e, int32_t s, int64_t n_bonds, const int32_t* bonds,
                 const lg_bonded* potentials);
int lg_set_angles(lg_engine* e, int32_t s, int64_t n_angles, const int32_t* angles,
                  const lg_bonded* potentials);
/* The dihedral angles (i, j, k, m) of system `s` (4 per dihedral, particle
 * indices, in the orientation Bonding::rebuild gives them, bonding.rs:111-157)
 * with their potential (System::dihedral_potential). */
int lg_set_dihedrals(lg_engine* e, int32_t s, int64_t n_dihedrals, const int32_t* dihedrals,
                     const lg_bonded* potentials);

/* Pair table of system `s`: n_kinds^2 entries, symmetric, replacing
 * System::set_pair_potential (sys/system.rs:122-131).  Fails like the
 * reference when a cutoff exceeds half the smallest cell length. */
int lg_set_pairs(lg_engine* e, int32_t s, int32_t n_kinds, const lg_pair* table);

/* Coulomb potential of system `s`, replacing System::set_coulomb_potential
 * (sys/system.rs:159-170) with SharedEwald or Wolf. */
int lg_set_coulomb(lg_engine* e, int32_t s, const lg_coulomb* coulomb);

/* ---- forces, energy, virial ---------------------------------------------- */
/* Computes the requested quantities of system `s` at `positions` (3n, host).
 * forces (3n, host) are ACCUMULATED into, as GlobalPotential::forces does
 * (global/mod.rs:84-105); energy and virial are written.  Any output may be
 * NULL when not requested.  Replaces Forces / PotentialEnergy / AtomicVirial
 * (sys/compute.rs:30-255) and the GlobalPotential methods of Ewald / Wolf. */
int lg_compute(lg_engine* e, int32_t s, const double* positions, uint32_t terms, uint32_t want,
               double* forces, double* energy, double virial[9]);

/* MolecularVirial::compute (sys/compute.rs:278-362) of system `s` at
 * `positions`: pair potentials and real-space Coulomb between molecules with
 * the molecular definition (w_ab (r_ab . r_ij) / r_ab^2, r_ij the image of the
 * centres of mass), the tail correction, and the Ewald k-space atomic virial
 * minus sum_a F_k,a (x) (x_a - com) (ewald.rs:533-571, 736-752; wolf.rs:285-320);
 * bonds, angles and dihedral angles contribute nothing.  `terms` selects among
 * LG_TERM_PAIRS, LG_TERM_TAIL, LG_TERM_COUL_REAL and LG_TERM_COUL_KSPACE.
 * The pair and real-space terms are FP64 on either precision (a mixed engine
 * walks its cell-sorted list, each pair once); the k-space correction takes
 * the engine's own k-space forces. */
int lg_molecular_virial(lg_engine* e, int32_t s, const double* positions, uint32_t terms, double virial[9]);

/* Same for every system of the engine, on device pointers: d_positions and
 * d_forces hold 3*N_total doubles (systems in index order, forces overwritten),
 * d_energy n_systems doubles and d_virial 9*n_systems doubles.  `stream` is a
 * cudaStream_t (NULL: the engine's stream). */
int lg_compute_device(lg_engine* e, const double* d_positions, uint32_t terms, uint32_t want,
                      double* d_forces, double* d_energy, double* d_virial, void* stream);

/* Pair set of family 0 (pair potentials: r < cutoff, not excluded) or 1
 * (real-space Coulomb: r <= cutoff, q_i q_j != 0) at `positions`, as the
 * device kernels see it.  Writes up to `capacity` (i, j), i < j, and the count. */
int lg_pairset(lg_engine* e, int32_t s, const double* positions, int32_t family,
               int32_t* pairs, int64_t capacity, int64_t* count);
/* Test hook: the cell of each atom of system `s` (n entries, atom order) at the
 * last neighbour-list build, as (cz * ny + cy) * nx + cx, and the cells per
 * axis (nx, ny, nz).  Cells are at least half the list radius wide. */
int lg_list_cells(lg_engine* e, int32_t s, int32_t* cells, int32_t ncell[3]);

/* ---- molecular dynamics ------------------------------------------------------ */
/* VelocityVerlet::new + setup (lumol-sim/src/md/integrators.rs:22-42): sets the
 * timestep and zeroes the accelerations.  thermostat_tau > 0 adds a
 * BerendsenThermostat(temperature, tau) (md/thermostats.rs:91-121) applied after
 * every step, as MolecularDynamics::propagate does (md/molecular_dynamics.rs:66-76). */
int lg_md_setup(lg_engine* e, int32_t s, double dt, double thermostat_temperature,
                double thermostat_tau);

/* Integrators (lumol-sim/src/md/integrators.rs). */
enum {
    LG_INTEGRATOR_VELOCITY_VERLET = 0, /* VelocityVerlet (integrators.rs:19-70) */
    LG_INTEGRATOR_VERLET = 1,          /* Verlet (integrators.rs:72-123): keeps the positions at t - dt */
    LG_INTEGRATOR_LEAP_FROG = 2        /* LeapFrog (integrators.rs:125-169) */
};
/* Thermostats, applied after every step (md/thermostats.rs). */
enum {
    LG_THERMOSTAT_NONE = 0,
    LG_THERMOSTAT_BERENDSEN = 1, /* BerendsenThermostat(temperature, tau) (thermostats.rs:77-121) */
    LG_THERMOSTAT_RESCALE = 2,   /* RescaleThermostat::with_tolerance(temperature, tolerance) (thermostats.rs:27-73) */
    LG_THERMOSTAT_CSVR = 3       /* CSVRThermostat(temperature, tau) (thermostats.rs:123-210), noise from `seed` */
};
/* Controls, applied after the thermostat at every step (md/controls.rs). */
#define LG_CONTROL_REMOVE_TRANSLATION 1u /* RemoveTranslation (controls.rs:26-43) */
#define LG_CONTROL_REWRAP 2u             /* Rewrap (controls.rs:73-89): molecules' centres of mass into the cell */
#define LG_CONTROL_REMOVE_ROTATION 4u    /* RemoveRotation (controls.rs:44-71) */

typedef struct lg_md_params {
    int32_t integrator;  /* LG_INTEGRATOR_* */
    int32_t thermostat;  /* LG_THERMOSTAT_* */
    double timestep;
    double temperature;  /* thermostat target (K) */
    double tau;          /* Berendsen / CSVR time scale, in timesteps (>= 1) */
    double tolerance;    /* RescaleThermostat tolerance (K) */
    uint64_t seed;       /* CSVR: the noise of step k is drawn from SplitMix64 streams of (seed, k) */
    uint32_t controls;   /* LG_CONTROL_* bits; applied as RemoveTranslation, RemoveRotation, Rewrap */
    uint32_t reserved;   /* 0 */
} lg_md_params;

/* Barostats (lumol-sim/src/md/integrators.rs). */
enum {
    LG_BAROSTAT_NONE = 0,
    LG_BAROSTAT_BERENDSEN = 1,        /* BerendsenBarostat (integrators.rs:174-250), isotropic */
    LG_BAROSTAT_ANISO_BERENDSEN = 2   /* AnisoBerendsenBarostat (integrators.rs:252-342) */
};
/* BerendsenBarostat::new(timestep, pressure, tau): system `s`, set up with
 * LG_INTEGRATOR_VELOCITY_VERLET by lg_md_setup_ex (whose timestep it uses),
 * integrates with the Velocity-Verlet based Berendsen barostat instead.  Every
 * step scales the positions by eta and the cell matrix by eta^3 (the
 * reference's UnitCell::scale_mut(eta^3 * 1)), evaluates the pressure
 * (N_f k_B T + Tr W) / (3 V) at the new positions with the half-step
 * velocities, takes eta^3 = 1 - 7372 / tau (pressure - P) for the next step,
 * and completes the step with the forces.  The cell change is applied on the
 * device in place; lg_get_cell returns the current cell.  A cell length at or
 * below twice the maximum cutoff fails the run with the reference's panic
 * message.  LG_BAROSTAT_NONE turns it off. */
int lg_md_set_barostat(lg_engine* e, int32_t s, int32_t kind, double pressure, double tau);
/* AnisoBerendsenBarostat::new(timestep, stress, tau) (integrators.rs:268-287;
 * `hydrostatic(timestep, p, tau)` is stress = p * 1): every step scales the
 * positions by the matrix eta (x = eta x) and the cell by it (cell * eta, the
 * shape kept: an orthorhombic cell takes off-diagonal terms that its
 * orthorhombic branches then ignore, as in the reference), evaluates the stress
 * (sum_i m v (x) v + W) / V at the new positions with the half-step velocities,
 * takes eta = 1 - dt 7372 / tau (stress - Stress) made symmetric for the next
 * step, and completes the step with the forces.  `stress` is 9 doubles,
 * row-major.  A face distance at or below twice the maximum cutoff fails the
 * run with the reference's panic message. */
int lg_md_set_aniso_barostat(lg_engine* e, int32_t s, const double stress[9], double tau);
/* The cell matrix of system `s` (9 doubles, row-major). */
int lg_get_cell(lg_engine* e, int32_t s, double matrix[9]);
/* Its CellShape (LG_CELL_*), face distances (UnitCell::lengths, cells.rs:134-146)
 * and volume (cells.rs:185-200), as the engine computed them. */
int lg_cell_info(lg_engine* e, int32_t s, int32_t* shape, double lengths[3], double* volume);

/* Molecular dynamics of system `s` with any integrator, thermostat and
 * controls of the list above, stepped as MolecularDynamics::propagate does
 * (md/molecular_dynamics.rs:66-76: integrate, thermostat, controls).  The
 * integrator's setup runs at the next lg_md_run: VelocityVerlet and LeapFrog
 * zero the accelerations, Verlet takes its positions at t - dt as x - v dt from
 * the state then on the device (integrators.rs:92-104).  For a Verlet system
 * the accelerations of lg_md_get/set_state_all hold those previous positions.
 * Argument checks follow the constructors (thermostats.rs:48-61, 102-109, 151-160). */
int lg_md_setup_ex(lg_engine* e, int32_t s, const lg_md_params* params);
/* Uploads / downloads positions and velocities (3n each) of system `s`. */
int lg_md_set_state(lg_engine* e, int32_t s, const double* positions, const double* velocities);
int lg_md_get_state(lg_engine* e, int32_t s, double* positions, double* velocities);
/* Uploads / downloads the state of every system at once: 3 * N_total doubles
 * each, systems in index order.  `accelerations` (VelocityVerlet's, the
 * a(t) the next half kick uses) may be NULL; on upload NULL keeps the device
 * accelerations (zero after a description change). */
int lg_md_set_state_all(lg_engine* e, const double* positions, const double* velocities,
                        const double* accelerations);
int lg_md_get_state_all(lg_engine* e, double* positions, double* velocities, double* accelerations);
/* The same for system `s` with its accelerations (3n each; VelocityVerlet's
 * a(t), Verlet's positions at t - dt), for a snapshot of a running system and
 * its restore; `accelerations` may be NULL (set: zero after a description
 * change, else kept; get: not read). */
int lg_md_set_state_ex(lg_engine* e, int32_t s, const double* positions, const double* velocities,
                       const double* accelerations);
int lg_md_get_state_ex(lg_engine* e, int32_t s, double* positions, double* velocities, double* accelerations);
/* Runs `nsteps` steps of every system with device-resident state.  A system
 * whose positions or velocities became non-finite is flagged (see
 * lg_system_status); the call still completes every system's steps and then
 * returns LG_ERR_NONFINITE. */
int lg_md_run(lg_engine* e, int64_t nsteps);

/* ---- systems joining and leaving a batch -------------------------------------- */
/* Appends `count` empty systems (indices n_systems .. n_systems + count - 1),
 * to be described with lg_set_* and given a state with lg_md_set_state.  At
 * the next use the batch is lowered again; the systems already there keep
 * their device state (positions, velocities, accelerations, thermostat noise
 * counters, Monte Carlo chains) and continue their trajectories.  Device
 * buffers grow only when the batch exceeds the largest size it has had. */
int lg_add_systems(lg_engine* e, int32_t count);
/* Removes system `s`; the systems after it move down one index and, with the
 * others, keep their device state.  Allocates nothing: buffers keep their
 * capacity.  The last system of an engine cannot be removed (destroy it). */
int lg_remove_system(lg_engine* e, int32_t s);
/* Integrator::integrate for a single-system engine (integrators.rs:44-69): runs
 * `nsteps` steps from the host positions / velocities and copies them back.
 * The same as lg_md_propagate(..., LG_SYNC_DOWNLOAD): the host arrays are
 * uploaded only when they differ from what the engine last exchanged. */
int lg_md_integrate(lg_engine* e, double* positions, double* velocities, int64_t nsteps);

/* Lazy host synchronisation behind Integrator::integrate and
 * Propagator::propagate (lumol-sim/src/md/molecular_dynamics.rs:66-76,
 * lumol-sim/src/simulations.rs:87-92): the engine keeps x and v resident on
 * the device and a page-locked copy of the host arrays it last exchanged.
 * A call uploads `positions` / `velocities` only when the device state is not
 * the one last exchanged (first call, description change, another call wrote
 * the state) or when the host arrays differ from that copy (a host-side
 * thermostat, control or user edit); LG_SYNC_TRUST_HOST skips the comparison
 * (the caller knows the arrays are unchanged).  It then runs `nsteps` steps
 * and, with LG_SYNC_DOWNLOAD, copies the state back (one device
 * synchronisation for the steps and the copy); without it the host arrays are
 * left as they were, e.g. between the steps that outputs read.  Single-system
 * engines only.  Returns LG_ERR_NONFINITE (after completing the steps) when
 * the velocities became non-finite (compute.rs:141, "Kinetic energy is
 * infinite!"). */
#define LG_SYNC_DOWNLOAD 1u
#define LG_SYNC_TRUST_HOST 2u
int lg_md_propagate(lg_engine* e, double* positions, double* velocities, int64_t nsteps, uint32_t flags);

/* Per-system status flags (n_systems entries) of the last runs: LG_SYS_NONFINITE
 * when a system's velocities or its energy became non-finite (the reference
 * panics there, sys/compute.rs:125,141).  lg_md_run completes the steps of
 * every system and returns LG_ERR_NONFINITE; the other systems' results are
 * unaffected.  `clear` resets the flags after reading them. */
#define LG_SYS_NONFINITE 1u
int lg_system_status(lg_engine* e, uint32_t* flags, int32_t clear);

/* ---- Monte Carlo ------------------------------------------------------------- */
/* EnergyCache::init (sys/cache.rs:75-98) at `positions` for system `s`. */
int lg_mc_init(lg_engine* e, int32_t s, const double* positions, double* energy);
/* EnergyCache::move_molecule_cost (sys/cache.rs:145-220) with the Coulomb
 * GlobalCache cost (ewald.rs:572-613, 758-839; wolf.rs:121-165). */
int lg_mc_move_molecule_cost(lg_engine* e, int32_t s, int64_t molecule,
                             const double* new_positions, double* cost);
/* EnergyCache::update (sys/cache.rs:118-127) after the move was applied:
 * `positions` are the molecule's positions after Translate::apply's
 * center-of-mass wrap (lumol-sim/src/mc/moves/translate.rs:114-125), or
 * Rotate::apply's positions; NULL keeps the positions the cost was computed
 * for (GlobalCache::update has no positions, global/mod.rs:183-188; a wrap
 * changes no energy); after lg_mc_move_all_molecules_cost they are not read. */
int lg_mc_update(lg_engine* e, int32_t s, const double* molecule_positions, double* energy);

/* EnergyCache::move_all_molecules_cost (sys/cache.rs:238-292) for the
 * configuration a Resize move prepares (lumol-sim/src/mc/moves/resize.rs:63-107):
 * the new orthorhombic cell (9 doubles, row-major) and the new positions of
 * every atom of system `s` (3n) are installed on the device and the change of
 * the energy against the cache is returned (pairs, tail, Coulomb; the rigid
 * molecules' bonded energies do not change).  Fails with the reference's
 * message when a cell length is at most twice the maximum cutoff.  Then
 * lg_mc_update keeps the new configuration (Resize::apply), or lg_mc_restore
 * puts the previous cell and positions back (Resize::restore, resize.rs:121-124);
 * a pending Resize is restored by the next cost call otherwise. */
int lg_mc_move_all_molecules_cost(lg_engine* e, int32_t s, const double new_cell[9], const double* new_positions,
                                  double* cost);
/* Rejection of the pending move of system `s`: a pending Resize's previous
 * configuration comes back; a single-molecule move has changed nothing. */
int lg_mc_restore(lg_engine* e, int32_t s);

/* Batched Monte Carlo: every system given lg_mc_setup runs its own Metropolis
 * chain of single-particle Translate moves on the device (MonteCarlo::propagate,
 * lumol-sim/src/mc/monte_carlo.rs:289-329, with Translate::new(delta),
 * mc/moves/translate.rs:41-125: a uniform displacement in [-delta/sqrt(3),
 * delta/sqrt(3)) per axis, Metropolis acceptance, centre-of-mass wrap), the
 * cost being EnergyCache::move_molecule_cost (sys/cache.rs:145-220).  Systems
 * with pair potentials and one-particle molecules only; delta <= skin / 2.
 * The random stream is the engine's own (SplitMix64 seeded by `seed`), not the
 * reference's xorshift stream. */
int lg_mc_setup(lg_engine* e, int32_t s, double temperature, double delta, uint64_t seed);
/* The chain of system `s` with MonteCarlo::add(Translate::new(delta), f_t) and
 * MonteCarlo::add(Rotate::new(theta), f_r) (mc/moves/translate.rs,
 * rotate.rs:34-124): molecules of any size move rigidly, a move picked by its
 * cumulative frequency (monte_carlo.rs:190-208, 289-298), a molecule uniformly,
 * then a displacement (as lg_mc_setup) or a rotation about the centre of mass
 * (an axis uniform on the unit sphere, an angle uniform in [-theta, theta),
 * Matrix3::rotation); the cost counts the pair potentials between the moved
 * molecule and the other atoms.  A translated molecule is wrapped by its
 * centre of mass, a rotated one is not (as the reference applies them).  Pair
 * potentials only; a frequency of 0 leaves that move out.  (A chain that
 * lg_mc_setup gives a triclinic system runs this way too: the move draw comes
 * first, then the molecule, the displacement, the Metropolis number.)
 * lg_mc_run checks that the largest rotated displacement stays within half the
 * skin. */
int lg_mc_setup_ex(lg_engine* e, int32_t s, double temperature, double translate_delta, double translate_frequency,
                   double rotate_theta, double rotate_frequency, uint64_t seed);
/* Runs `moves` attempted moves in every chain. */
int lg_mc_run(lg_engine* e, int64_t moves);
/* Cached energy, accepted and attempted moves of chain `s`. */
int lg_mc_stats(lg_engine* e, int32_t s, double* energy, int64_t* accepted, int64_t* attempted);

/* ---- diagnostics (no counterpart in the reference) ----------------------------- */
/* Kernel groups timed by lg_kernel_times, in output order. */
enum {
    LG_KT_NLIST = 0,   /* cell binning + Verlet list build (forced rebuild) */
    LG_KT_PAIR = 1,    /* pair potentials + real-space Coulomb */
    LG_KT_BONDED = 2,  /* bonds and angles */
    LG_KT_EIKR = 3,    /* Ewald e^{ik.r} per atom */
    LG_KT_RHO = 4,     /* Ewald structure factors rho(k) */
    LG_KT_FIELD = 5,   /* Ewald k-space field and forces */
    LG_KT_VV = 6,      /* the two Velocity-Verlet half steps */
    LG_KT_STEP = 7,    /* one whole MD step, launched without a graph */
    LG_KT_COUNT = 8
};
/* The engine's CUDA stream (a cudaStream_t), to time its work with events. */
int lg_get_stream(lg_engine* e, void** stream);
/* Average device time (ms) of each kernel group over `reps` launches, timed
 * with CUDA events on the engine's stream at the current device state. */
int lg_kernel_times(lg_engine* e, int32_t reps, double ms[LG_KT_COUNT]);
/* Number of kernels this engine has launched (graph replays included). */
int lg_launch_count(lg_engine* e, uint64_t* count);
/* The persistent kernel's plan for the current batch: cluster size and number
 * of groups (0 and 0 while MD runs on the per-step kernels or before the first
 * lg_md_run). */
int lg_md_plan(lg_engine* e, int32_t* cluster, int32_t* groups);
/* Test hook: leaves system `s` as an interrupted list build would, with
 * `extra` stale atoms counted in its first cell, and asks for a rebuild.  The
 * next build finds the counts inconsistent, writes nothing out of range, and
 * the engine recounts and rebuilds before using the list. */
int lg_test_stale_cell_counts(lg_engine* e, int32_t s, int32_t extra);
/* Measured FMA throughput of the FP64 (fp64 = 1) or FP32 pipe of the current
 * device, in TFLOP/s (2 flops per FMA). */
int lg_fma_peak(int32_t fp64, double* tflops);

/* ---- Ewald k-space without device allocation ----------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc --
 * code running inside a host framework whose device memory belongs to its own
 * pool allocator, and per-step or per-move loops where cudaMalloc / cudaFree
 * would synchronise the device -- this computes what
 * lg_compute(LG_TERM_COUL_KSPACE) computes for one orthorhombic system, on
 * device pointers the caller owns, and allocates nothing: its scratch is one
 * fixed __device__ array of about 2 MB that every GPU loading the library holds
 * until exit.  Limits: n <= LG_NOALLOC_MAX_ATOMS, 1 <= kmax <= LG_NOALLOC_MAX_KMAX;
 * larger sizes are rejected with LG_ERR_ARGUMENT (message in lg_last_error(NULL)).
 * d_positions: 3n, d_charges: n; d_forces (3n) is ACCUMULATED into; d_energy (1)
 * and d_virial (9) are written (either may be NULL).  `stream` is a
 * cudaStream_t (NULL: the default stream).  Calls share the scratch array:
 * calls whose work overlaps on the GPU race.  The first call on a device sets
 * the scratch address up for that device and should come before any stream
 * capture.  The address it keeps belongs to the device's primary context, so
 * the entry point must not be used again after cudaDeviceReset. */
#define LG_NOALLOC_MAX_ATOMS 4096
#define LG_NOALLOC_MAX_KMAX 8
int lg_ewald_kspace_noalloc(const double* d_positions, const double* d_charges, int64_t n,
                            const double cell_lengths[3], double alpha, int32_t kmax,
                            double* d_forces, double* d_energy, double* d_virial, void* stream);

#ifdef __cplusplus
}
#endif
#endif
