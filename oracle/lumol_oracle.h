/*
 * lumol_oracle.h -- CPU oracle for the lumol-gb300 parity tests.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++17 restatement of lumol-core's
 * CPU arithmetic for the force / energy / virial / integration path.  It is the
 * checker the GPU engine is compared against; the product never links, loads or
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may use it.
 *
 * Parity pin: the restatement is checked against the reference's own unit-test
 * literals (energy/functions.rs, energy/pairs.rs, sys/energy.rs,
 * energy/global/ewald.rs, energy/global/wolf.rs) and against the NIST LJ and
 * SPC/E reference data shipped with the reference (tests/nist-lj.rs,
 * tests/nist-spce.rs).  erf/erfc come from the C library, the reference takes
 * them from the `special` 0.10 crate (lumol-core/src/math.rs:10-18), so values
 * that depend on erfc are pinned only to the tolerance of those tests.
 */
#ifndef LUMOL_ORACLE_H
#define LUMOL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pair potential kinds (lumol-core/src/energy/functions.rs). */
enum {
    ORC_PAIR_ABSENT = 0,     /* no PairInteraction registered for the kind pair */
    ORC_PAIR_NULL = 1,       /* NullPotential */
    ORC_PAIR_LJ = 2,         /* LennardJones {sigma, epsilon} */
    ORC_PAIR_BUCKINGHAM = 3, /* Buckingham {a, c, rho} */
    ORC_PAIR_HARMONIC = 4,   /* Harmonic {k, x0} */
    ORC_PAIR_BMH = 5,        /* BornMayerHuggins {a, c, d, sigma, rho} */
    ORC_PAIR_MORSE = 6,      /* Morse {a, x0, depth} */
    ORC_PAIR_GAUSSIAN = 7,   /* Gaussian {a, b} */
    ORC_PAIR_MIE = 8         /* Mie {sigma, epsilon, n, m} */
};

/* PairRestriction (lumol-core/src/energy/restrictions.rs:13-33). */
enum {
    ORC_RESTRICT_NONE = 0,
    ORC_RESTRICT_INTRA = 1,
    ORC_RESTRICT_INTER = 2,
    ORC_RESTRICT_EXCLUDE12 = 3,
    ORC_RESTRICT_EXCLUDE13 = 4,
    ORC_RESTRICT_EXCLUDE14 = 5,
    ORC_RESTRICT_SCALE14 = 6
};

enum { ORC_COULOMB_NONE = 0, ORC_COULOMB_EWALD = 1, ORC_COULOMB_WOLF = 2 };
/* CellShape (cells.rs:12-20) */
enum { ORC_CELL_ORTHORHOMBIC = 0, ORC_CELL_TRICLINIC = 1 };

/* Energy / force / virial terms, combinable as a bit mask. */
enum {
    ORC_TERM_PAIRS = 1,
    ORC_TERM_TAIL = 2,
    ORC_TERM_BONDS = 4,
    ORC_TERM_ANGLES = 8,
    ORC_TERM_COUL_REAL = 16,  /* Ewald real space, or the whole Wolf sum */
    ORC_TERM_COUL_SELF = 32,  /* Ewald self energy (Wolf self is part of COUL_REAL) */
    ORC_TERM_COUL_KSPACE = 64,
    ORC_TERM_DIHEDRALS = 128,
    ORC_TERM_ALL = 255
};

/* PairInteraction (lumol-core/src/energy/pairs.rs:57-95). */
typedef struct {
    int32_t type;        /* ORC_PAIR_* */
    int32_t shifted;     /* PairInteraction::shifted */
    int32_t restriction; /* ORC_RESTRICT_* */
    int32_t tail;        /* enable_tail_corrections */
    double p0, p1, p2;   /* LJ: sigma, epsilon; Buckingham: a, c, rho; Harmonic: k, x0 */
    double cutoff;
    double scale14;      /* Scale14 factor */
    double p3, p4;       /* further parameters: BMH {a, c, d, sigma, rho} = p0..p4;
                            Morse {a, x0, depth} = p0..p2; Gaussian {a, b} = p0, p1;
                            Mie {sigma, epsilon, n, m} = p0..p3 */
    int32_t table_size;  /* > 0: TableComputation of the potential (energy/computations.rs:63-173) */
    int32_t table_pad;
    double table_max;
} orc_pair;

/* Bond, angle and dihedral potentials: ORC_PAIR_NULL, ORC_PAIR_HARMONIC {k, x0},
 * ORC_BONDED_COSINE_HARMONIC {k, x0} (CosineHarmonic::new, functions.rs:162-210),
 * ORC_BONDED_TORSION {k, delta = x0, n} (functions.rs:212-258),
 * ORC_PAIR_MORSE {depth = k, x0, a} (functions.rs:405-437). */
enum { ORC_BONDED_COSINE_HARMONIC = 10, ORC_BONDED_TORSION = 11 };
typedef struct {
    int32_t type;        /* 0: absent, ORC_PAIR_NULL, ORC_PAIR_HARMONIC or ORC_BONDED_* */
    int32_t n;           /* Torsion multiplicity */
    double k, x0;
    double a;            /* Morse width */
} orc_bonded;

typedef struct {
    int32_t kind;        /* ORC_COULOMB_* */
    int32_t restriction; /* ORC_RESTRICT_* */
    int32_t kmax;        /* Ewald */
    int32_t pad;
    double cutoff;
    double alpha;        /* Ewald alpha; <= 0 means PI / cutoff (ewald.rs:278-279) */
    double scale14;
} orc_coulomb;

typedef struct {
    int64_t n;
    const double* positions;  /* 3n, unwrapped */
    const int32_t* kinds;     /* n, kind index 0..n_kinds-1 */
    const double* charges;    /* n */
    const double* masses;     /* n */
    const int32_t* molecules; /* n, molecule index; atoms of a molecule are contiguous */
    int64_t n_bonds;
    const int32_t* bonds;     /* 2 * n_bonds */
    int32_t n_kinds;
    const orc_pair* pairs;         /* n_kinds^2, symmetric */
    const orc_bonded* bond_pots;   /* n_kinds^2, symmetric */
    const orc_bonded* angle_pots;  /* n_kinds^3, symmetric in first/last */
    orc_coulomb coulomb;
    double cell[3];           /* orthorhombic cell lengths */
    const orc_bonded* dihedral_pots;  /* n_kinds^4, symmetric under reversal; may be NULL */
    int32_t cell_shape;       /* ORC_CELL_*; a triclinic cell is given by cell_matrix */
    int32_t cell_pad;
    double cell_matrix[9];    /* row-major, columns the cell vectors (UnitCell::matrix) */
} orc_desc;

typedef struct orc_system orc_system;

orc_system* orc_create(const orc_desc* desc);
void orc_destroy(orc_system* s);
int orc_num_threads(void);
void orc_set_threads(int n);

void orc_set_positions(orc_system* s, const double* positions);
void orc_get_positions(const orc_system* s, double* positions);
int64_t orc_n_angles(const orc_system* s);
void orc_angles(const orc_system* s, int32_t* out); /* 3 * n_angles, sorted */

/* Energies (internal units).  `terms` is a mask of ORC_TERM_*. */
double orc_energy(orc_system* s, int terms);
/* forces (3n) are ACCUMULATED into `forces`. */
void orc_forces(orc_system* s, int terms, double* forces);
void orc_virial(orc_system* s, int terms, double* virial9);
/* MolecularVirial (sys/compute.rs:278-362) with the terms PAIRS, TAIL,
 * COUL_REAL and COUL_KSPACE (bonds, angles and dihedral angles give none). */
void orc_molecular_virial(orc_system* s, int terms, double* virial9);

/* Pair set of a family: 0 = pair potentials (r < cutoff and not excluded),
 * 1 = real-space Coulomb (r <= cutoff, q_i q_j != 0).  Returns the count and
 * writes up to `cap` (i, j) with i < j into out. */
int64_t orc_pairset(orc_system* s, int family, int32_t* out, int64_t cap);

/* Velocity-Verlet (lumol-sim/src/md/integrators.rs:22-70), with an optional
 * Berendsen thermostat (md/thermostats.rs:112-121) when tau > 0.
 * positions / velocities / accelerations: 3n in/out. */
void orc_velocity_verlet(orc_system* s, double* positions, double* velocities,
                         double* accelerations, double dt, int64_t nsteps,
                         double thermostat_temperature, double thermostat_tau);
double orc_temperature(const orc_system* s, const double* velocities);

/* MolecularDynamics::propagate (lumol-sim/src/md/molecular_dynamics.rs:66-76)
 * for `nsteps` steps: integrator 0 VelocityVerlet, 1 Verlet, 2 LeapFrog
 * (md/integrators.rs); thermostat 0 none, 1 Berendsen(T0, tau), 2
 * Rescale(T0, tol), 3 CSVR(T0, tau) (md/thermostats.rs) with the noise of
 * SplitMix64 streams of (seed, count) (*count: thermostat applications so far,
 * in / out); controls bit 1 RemoveTranslation, bit 4 RemoveRotation, bit 2
 * Rewrap (md/controls.rs), applied in that order.
 * `state` (3n) is the integrator's: accelerations, or Verlet's positions at
 * t - dt (orc_verlet_setup). */
void orc_md_run(orc_system* s, double* positions, double* velocities, double* state, int integrator, double dt,
                int thermostat, double T0, double tau, double tol, uint64_t seed, uint64_t* count,
                uint32_t controls, int64_t nsteps);
/* Verlet::setup (md/integrators.rs:92-104): prev = x - v dt. */
void orc_verlet_setup(const orc_system* s, const double* positions, const double* velocities, double dt,
                      double* prev);
double orc_kinetic_energy(const orc_system* s, const double* velocities);

/* One bonded potential evaluated at x: energy and force (functions.rs). */
void orc_bonded_eval(const orc_bonded* p, double x, double* energy, double* force);
/* UnitCell::dihedral_and_derivatives (cells.rs:379-411) of four points in a cell
 * of lengths `cell`: the angle and the derivatives d1..d4 (12 doubles). */
void orc_dihedral_geometry(const double cell[3], const double* r1, const double* r2, const double* r3,
                           const double* r4, double* phi, double* derivatives);
int64_t orc_n_dihedrals(const orc_system* s);
void orc_dihedrals(const orc_system* s, int32_t* out); /* 4 * n_dihedrals, sorted */

/* One PairInteraction evaluated at distance r: energy, force, tail energy,
 * tail virial (energy/pairs.rs:185-296). */
void orc_pair_eval(const orc_pair* p, double r, double* energy, double* force,
                   double* tail_energy, double* tail_virial);

/* UnitCell::scale_mut (cells.rs:201-207) to new orthorhombic lengths, and the
 * current lengths (3 doubles). */
void orc_set_cell(orc_system* s, double a, double b, double c);
void orc_get_cell(const orc_system* s, double* lengths);
void orc_set_cell_matrix(orc_system* s, const double* matrix, int32_t shape);
void orc_get_cell_matrix(const orc_system* s, double* matrix);
void orc_cell_info(const orc_system* s, double* lengths, double* volume);
void orc_cell_apply(const orc_system* s, double* v, int32_t wrap);
int orc_aniso_barostat_run(orc_system* s, double* x, double* v, double* a, double* eta, double dt,
                           const double* stress0, double tau, int64_t nsteps);
/* Interactions::maximum_cutoff (interactions.rs:173-190). */
double orc_maximum_cutoff(const orc_system* s);
/* BerendsenBarostat::integrate (lumol-sim/src/md/integrators.rs:213-250) and an
 * optional Berendsen thermostat (tau_thermostat > 0), nsteps times; `eta` is
 * the barostat's scaling factor (1 after setup, in / out).  Returns 1 where
 * the reference panics (a cell length at or below twice the maximum cutoff). */
int orc_berendsen_barostat_run(orc_system* s, double* positions, double* velocities, double* accelerations,
                               double* eta, double dt, double pressure, double tau, double T0,
                               double tau_thermostat, int64_t nsteps);

/* EnergyCache (lumol-core/src/sys/cache.rs). */
void orc_cache_init(orc_system* s);
double orc_cache_energy(const orc_system* s);
double orc_move_molecule_cost(orc_system* s, int64_t molecule, const double* new_positions);
void orc_cache_update(orc_system* s);
/* EnergyCache::move_all_molecules_cost (cache.rs:238-292) of a Resize move's
 * configuration: new cell lengths (3) and positions (3n), installed in the
 * system; orc_cache_update keeps them, orc_cache_restore puts the previous
 * configuration back (Resize::restore, mc/moves/resize.rs:121-124). */
double orc_move_all_molecules_cost(orc_system* s, const double* cell_matrix, const double* new_positions);
void orc_cache_restore(orc_system* s);

#ifdef __cplusplus
}
#endif
#endif
