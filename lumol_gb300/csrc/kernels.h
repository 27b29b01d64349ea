// kernels.h -- device buffers of one engine (a batch of systems) and the
// launch functions of every kernel.
#pragma once

#include <string>

#include "device_common.cuh"

namespace lg {

// Raw device pointers of a batch.  Atoms of all systems are concatenated in
// system order; per-atom arrays have n entries.
struct Batch {
    int n = 0;           // atoms in the batch
    int nsys = 0;        // systems
    int precision = 0;   // LG_PRECISION_*
    // state
    double4_32a* posq = nullptr;      // x, y, z (unwrapped, FP64) and charge
    double4_32a* vel = nullptr;       // vx, vy, vz and mass
    double4_32a* acc = nullptr;       // accelerations (VelocityVerlet / LeapFrog), or Verlet's positions at t - dt
    double* force = nullptr;      // 3n, Vector3D layout
    int* kind = nullptr;          // kind index within the system's pair table
    int* mol = nullptr;           // global molecule index
    int* sysid = nullptr;         // system of each atom
    SysDev* sys = nullptr;
    PairDev* ptab = nullptr;
    // bond paths: same-molecule partners closer than four bonds
    int* spec_off = nullptr;      // n + 1
    int* spec_j = nullptr;
    int8_t* spec_path = nullptr;
    // bonded terms gathered per atom
    int* bt_off = nullptr;        // n + 1
    int4* bt = nullptr;           // (type | m << 2, a, b, c): type 0 bond, 1 angle, 2 dihedral (a, b, c, m)
    int* bt_role = nullptr;
    double4_32a* bt_par = nullptr; // (k, x0, extra, kind): see bonded_par in the engine
    // neighbour list
    int maxnb = 0;
    int ncells = 0;
    int* nbr = nullptr;           // n * maxnb
    int* nnb = nullptr;           // n
    int* atom_cell = nullptr;
    int* cell_count = nullptr;    // ncells
    int* cell_start = nullptr;    // ncells + nsys: per system, its cells then an end sentinel
    int* plan = nullptr;          // 3 + 3 nsys: the systems that rebuild and their atom / cell prefix sums
    int sms = 152;                // multiprocessors of the device (grid sizes of the list-build kernels)
    int* perm = nullptr;          // n: cell-sorted position of each atom (mixed path; null for FP64)
    int2* km = nullptr;           // n: (kind, molecule) in cell-sorted order (mixed path)
    int* cell_atoms = nullptr;    // n: atoms in cell order, per system at [begin, end)
    float4* wpos = nullptr;       // wrapped FP32 positions at build, charge
    double4_32a* pos_build = nullptr; // positions at the last build
    uint32_t* status = nullptr;   // ST_* bits
    uint32_t* sys_rebuild = nullptr;  // nsys: 1 when that system's list must be rebuilt
    uint32_t* sys_status = nullptr;   // nsys: SYS_* bits of each system (non-finite state or energy)
    // Ewald k-space
    int nkvec = 0;
    int kdim = 0;                 // max kmax + 1 (eikr stores k = 0..kmax per axis)
    int kchunk = 32;              // k-vectors per chunk of the field kernel
    int nkchunks = 0;
    KVecDev* kvec = nullptr;
    double2* eikr = nullptr;      // [(kk * 3 + axis) * n + i]
    double2* rho = nullptr;       // nkvec
    double* fpart = nullptr;      // [chunk][3 n] partial k-space fields
    double* kred = nullptr;       // [k][7]: energy, virial xx xy xz yy yz zz
    // reductions
    double* red = nullptr;        // [n][RED_STRIDE] per-atom partial energies / virials
    double* host_const = nullptr; // [nsys][RED_STRIDE]: tail energy/virial, Ewald self energy
    // per-atom MD kernels run on tiles of VV_TILE atoms that never straddle two systems
    int ntiles = 0;
    int2* tiles = nullptr;        // ntiles: (system, first atom)
    double* kepart = nullptr;     // n: kinetic energies after md_second (mixed: per atom at its sorted position; plain: per chunk of 32 / tpa atoms, at begin + chunk)
    double* mom = nullptr;        // 3n: momentum of each chunk (RemoveTranslation), at 3 (begin + chunk)
    unsigned long long* md_count = nullptr;  // nsys: thermostat applications so far (the CSVR noise stream)
    double* adj = nullptr;        // 4 nsys: each system's pending thermostat factor and centre-of-mass velocity
    int nmol = 0;                 // molecules of the batch (Rewrap)
    int* mol_start = nullptr;     // nmol + 1: first atom of each molecule
    // mixed precision
    int tpa = 32;                 // threads per atom of the pair kernels (autotuned)
    int pair_general = 1;         // 0: pair potentials only, no restriction and no Coulomb in the batch
    int lj1 = 0;                  // 1: every system has one kind and a Lennard-Jones pair (a specialised force loop)
    int norestr = 0;              // 1: no pair or Coulomb restriction in the batch (a specialised general kernel)
    uint4* posfx = nullptr;       // wrapped positions as 32-bit fractions of L, charge bits (cell order)
    uint4* pfx_build = nullptr;   // n: fixed-point positions at the last list build (atom order, mixed path)
    // plain path: half-list evaluation.  Rows are sorted by neighbour index;
    // row i's pairs with j > i are evaluated once and their forces stored, the
    // j < i entries read them back through the reverse index.
    int* nlo = nullptr;           // n: entries j < i at the head of each row
    int* rev = nullptr;           // n * maxnb: for j < i, the slot of i in row j
    double4_32a* pf = nullptr;    // n * maxnb: force on i from pair (i, j > i)
    float* inv_mass = nullptr;    // n: 1 / m in FP32 (mixed path)
    PairDevF* ptabf = nullptr;
    KVecF* kvecf = nullptr;
    float2* eikrf = nullptr;
    float2* rhof = nullptr;
    float* qf = nullptr;          // n: FP32 charges of the Ewald systems (written with e^{ik.r}, mixed path)
};

// persist.cu: batched MD of pairs-only systems, one persistent launch per run of steps
constexpr int PK_MAXG = 64;       // systems per group
struct PkArgs {
    int ngroups;
    const int* group_off;         // ngroups + 1: each group's range in group_sys
    const int* group_sys;         // system indices, group by group
    int* group_flag;              // ngroups: a list overflow stopped the group (zero before a launch)
    double* ke;                   // n: kinetic energy of each force-phase chunk of a system, at begin + chunk
    int nsteps;
    int thermo;                   // some system has a thermostat
    int stage;                    // > 0: every block stages this many atoms' positions in shared memory
    // the state before the launch, written by its first step (a replay after a
    // list overflow restores it); the kernel also clears its group flags
    double4_32a* cp_pos;
    double4_32a* cp_vel;
    double4_32a* cp_acc;
};
constexpr int PK_STAGE_MAX = 9216;  // atoms a group may stage (20 bytes each)
// one-kind Lennard-Jones batches stage positions only (16 bytes each) in the
// same shared-memory limit
constexpr int PK_STAGE_MAX_LJ1 = 11264;
cudaError_t launch_md_persist(const Batch& b, const PkArgs& a, int cluster, cudaStream_t st);
int persist_max_clusters(int tpa, int cluster, int stage_atoms);
size_t persist_smem_bytes(int stage_atoms);

// nlist.cu
void launch_nlist_build(const Batch& b, cudaStream_t st);
// forces.cu
void launch_pair_forces(const Batch& b, uint32_t terms, bool ev, cudaStream_t st);
void launch_bonded(const Batch& b, uint32_t terms, bool ev, cudaStream_t st);
void launch_kspace(const Batch& b, bool forces, bool ev, cudaStream_t st);
void launch_kspace_part(const Batch& b, int part, bool ev, cudaStream_t st);
void launch_field_reduce(const Batch& b, cudaStream_t st);
// mixed.cu
void launch_pair_mixed(const Batch& b, uint32_t terms, bool ev, cudaStream_t st);
void launch_split_positions(const Batch& b, cudaStream_t st);
void launch_kspace_mixed_part(const Batch& b, int part, bool ev, cudaStream_t st);
void launch_reduce(const Batch& b, uint32_t terms, bool kspace, double* out, cudaStream_t st);
// MolecularVirial's pair / real-space part minus the Ewald k-space correction
// (kforce: the k-space forces, or null) into the per-atom virial slots of red.
void launch_molecular_virial(const Batch& b, uint32_t terms, double4_32a* com, const double* kforce,
                             cudaStream_t st);
void launch_pairset(const Batch& b, int family, int s_begin, int s_end, int* out, long long cap,
                    unsigned long long* count, cudaStream_t st);
// md.cu
void launch_pack_positions(const Batch& b, const double* pos3, cudaStream_t st);
void launch_pack_vectors(int n, const double* src3, double4_32a* dst, cudaStream_t st);
void launch_unpack_vectors(int n, const double4_32a* src, double* dst3, cudaStream_t st);
void launch_unpack_positions(const Batch& b, double* pos3, cudaStream_t st);
void launch_pack_velocities(const Batch& b, const double* vel3, cudaStream_t st);
void launch_unpack_velocities(const Batch& b, double* vel3, cudaStream_t st);
// Positions and velocities of atoms [0, b.n) into 3n arrays, in one launch.
void launch_unpack_state(const Batch& b, double* pos3, double* vel3, cudaStream_t st);
// *status into page-locked host memory (dst: its device address)
void launch_status_copy(const uint32_t* status, uint32_t* dst, cudaStream_t st);
constexpr int VV_TILE = 256;
void launch_md_first(const Batch& b, bool adjust, cudaStream_t st);
void launch_md_second(const Batch& b, cudaStream_t st);
void launch_md_adjust(const Batch& b, cudaStream_t st);
void launch_md_finalize(const Batch& b, cudaStream_t st);
void launch_rewrap(const Batch& b, cudaStream_t st);
void launch_verlet_setup(const Batch& b, int s, int begin, int end, cudaStream_t st);
void launch_request_rebuild(const Batch& b, cudaStream_t st);
// cell_atoms and perm set to the identity order (after an interrupted build).
void launch_identity_order(const Batch& b, cudaStream_t st);
// Sets ST_REBUILD only (the systems to rebuild are already flagged in sys_rebuild).
void launch_request_rebuild_flag(const Batch& b, cudaStream_t st);
// Kinetic energy of every system (nsys doubles) at the current velocities.
void launch_kinetic(const Batch& b, double* out, cudaStream_t st);
void launch_kinetic_tensor(const Batch& b, double* out, cudaStream_t st);
void launch_carry_vectors(const double4_32a* src, double4_32a* dst, int n, bool keep_w, cudaStream_t st);
void launch_check_displacement(const Batch& b, cudaStream_t st);

// mc.cu
void launch_mc_cost(const Batch& b, int s, const SysDev& sd, int mbeg, int msize, const double* d_newpos,
                    double2* d_new_eikr, double2* d_drho, double* d_partial, double* d_dk, double* d_out,
                    cudaStream_t st);
void launch_mc_accept(const Batch& b, const SysDev& sd, int mbeg, int msize, const double* d_newpos,
                      const SysDev* d_sys, const double2* d_drho, cudaStream_t st);
void launch_mc_chains(const Batch& b, McState* mc, bool fp64, bool molecular, cudaStream_t st);
// diag.cu
int measure_fma_peak(int fp64, double* tflops);
// runtime.cu: the message lg_last_error(NULL) returns
void set_global_error(const std::string& msg);

}  // namespace lg
