// engine.h -- the engine object behind the C ABI of include/lumol_gb300.h,
// shared by the host translation units of the engine:
//
//   lower.cu    the description of every system (particles, topology, pair
//               table, Coulomb potential, cell) lowered into the flat device
//               layout of kernels.h, and the host restatements of the
//               reference's scalar arithmetic that feed it;
//   runtime.cu  status words, list regrowth, force passes, state transfers,
//               the autotuner, MD step graphs and the persistent-kernel plan;
//   capi.cu     the C entry points of description, forces, MD, diagnostics;
//   capi_mc.cu  the C entry points of Monte Carlo.
//
// Host arithmetic that feeds results (potential shifts, Ewald k-vector
// factors, tail corrections, self energy) restates the reference operation by
// operation; these files are compiled with -ffp-contract=off so the host
// compiler does not fuse it either.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <functional>
#include <vector>

#include "../../include/lumol_gb300.h"
#include "kernels.h"

namespace lg {

constexpr int MIN_KCHUNK = 8;

// Message of the last failed call that has no engine (lg_create, the
// allocation-free entry point), per thread.
extern thread_local std::string g_create_error;

// Tuned launch parameters per workload shape: (device, precision, atoms,
// list capacity, k-vectors, persistent batch) -> (threads per atom,
// k-vectors per field chunk).
extern std::mutex g_tune_mutex;
extern std::map<std::tuple<int, int, int, int, int, bool>, std::pair<int, int>> g_tune_cache;

// A device buffer that keeps its memory when asked for no more than it holds:
// a batch that shrinks (a system leaves) or is re-lowered at the same size
// allocates nothing; only growth calls cudaMalloc.  The contents are kept when
// the memory is kept.
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;    // elements in use
    size_t cap = 0;  // elements allocated
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cap = 0;
    }
    cudaError_t alloc(size_t count) {
        if (count == 0) count = 1;
        if (p && count <= cap) {
            n = count;
            return cudaSuccess;
        }
        release();
        cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
        if (e == cudaSuccess) n = cap = count;
        return e;
    }
};

static_assert(MD_VELOCITY_VERLET == LG_INTEGRATOR_VELOCITY_VERLET && MD_VERLET == LG_INTEGRATOR_VERLET &&
                  MD_LEAP_FROG == LG_INTEGRATOR_LEAP_FROG,
              "integrator values");
static_assert(TH_NONE == LG_THERMOSTAT_NONE && TH_BERENDSEN == LG_THERMOSTAT_BERENDSEN &&
                  TH_RESCALE == LG_THERMOSTAT_RESCALE && TH_CSVR == LG_THERMOSTAT_CSVR,
              "thermostat values");
static_assert(SYS_NONFINITE == LG_SYS_NONFINITE, "system status values");
static_assert(CTL_REMOVE_TRANSLATION == LG_CONTROL_REMOVE_TRANSLATION && CTL_REWRAP == LG_CONTROL_REWRAP &&
                  CTL_REMOVE_ROTATION == LG_CONTROL_REMOVE_ROTATION,
              "control values");

// UnitCell (lumol-core/src/sys/config/cells.rs): its shape and matrix, and
// what the engine derives from them with the reference's operations.
struct HostCell {
    int shape = LG_CELL_ORTHORHOMBIC;
    double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};    // UnitCell::matrix, row-major (columns: cell vectors)
    double inv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // Matrix3::inverse (types/matrix.rs:212-227)
    double len[3] = {0, 0, 0};                    // lengths(): distances between opposite faces (cells.rs:134-146)
    double volume = 0.0;                          // volume() (cells.rs:185-200)
};
// Fills c from a cell matrix and its shape; false for a singular matrix.
bool cell_init(HostCell& c, const double m[9], int shape);

struct HostSystem {
    bool has_cell = false;
    HostCell cell;
    double L[3] = {0, 0, 0};  // cell.len (the orthorhombic lengths a, b, c)
    int64_t n = 0;
    std::vector<int32_t> kinds, mols;
    std::vector<double> charges, masses;
    std::vector<int32_t> bonds;
    std::vector<lg_bonded> bond_pots;
    std::vector<int32_t> angles;
    std::vector<lg_bonded> angle_pots;
    std::vector<int32_t> dihedrals;
    std::vector<lg_bonded> dihedral_pots;
    int32_t nk = 0;
    std::vector<lg_pair> pairs;
    lg_coulomb coul{};
    // molecular dynamics
    double dt = 0.0, T0 = 0.0, tau = 0.0, tol = 0.0;
    int32_t integrator = LG_INTEGRATOR_VELOCITY_VERLET, thermostat = LG_THERMOSTAT_NONE;
    uint32_t controls = 0;
    uint64_t seed = 0;
    bool md_ready = false;
    bool verlet_setup = false;  // Verlet::setup runs at the next lg_md_run
    bool reset_acc = false;     // VelocityVerlet / LeapFrog::setup zeroes the accelerations at the next commit
    // BerendsenBarostat (lumol-sim/src/md/integrators.rs:174-250)
    int32_t barostat = LG_BAROSTAT_NONE;
    double baro_pressure = 0.0, baro_tau = 0.0, baro_eta = 1.0;
    double baro_stress[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // AnisoBerendsenBarostat: target stress
    double baro_m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};       // and its eta (Matrix3::one() at setup)
    // derived
    std::vector<int64_t> mol_begin;  // first atom of each molecule (local index), plus the end
    double tail_energy = 0.0, tail_virial = 0.0, ewald_self = 0.0;
    double alpha = 0.0;
};

}  // namespace lg

using namespace lg;

struct lg_engine {
    lg_options opt{};
    int nsys = 0;
    std::vector<HostSystem> sys;
    std::string err;
    cudaStream_t stream = nullptr;
    bool dirty = true;
    std::vector<int64_t> begin;  // atom offsets (nsys + 1)
    // Systems that join or leave keep the others' device state: carry_from[s]
    // is the index system s had at the last commit (-1: new or re-described
    // particles, its state comes from the next lg_md_set_state).
    std::vector<int> carry_from;
    double skin = 1.0;

    Batch b;
    // device storage
    DBuf<double4_32a> posq, vel, acc, pos_build;
    DBuf<double> force, pos3, vel3, red, host_const, kepart, mom, out, fpart, kred, mc_part, kin, kten;
    DBuf<unsigned long long> md_count, cp_count;
    DBuf<double> adj;
    DBuf<int> mol_start;
    DBuf<int2> tiles;
    DBuf<double4_32a> cp_pos, cp_vel, cp_acc;  // MD checkpoint: a chunk whose list overflowed is replayed
    DBuf<int> kind, mol, sysid, spec_off, spec_j, bt_off, bt_role, nbr, nnb, atom_cell, cell_count, cell_start,
        cell_atoms, plan, perm;
    DBuf<int2> km;
    DBuf<int8_t> spec_path;
    DBuf<int4> bt;
    DBuf<double4_32a> bt_par;
    DBuf<double2> eikr, rho;
    DBuf<float4> wpos;
    DBuf<uint4> posfx, pfx_build;
    DBuf<float> inv_mass;
    DBuf<int> nlo, rev;
    DBuf<double4_32a> pf;
    DBuf<double4_32a> molcom;  // per-atom centre of mass of its molecule (molecular virial)
    DBuf<PairDevF> ptabf;
    DBuf<double2> table;  // TableComputation tables (plain path)
    DBuf<float2> tablef;  // the same in FP32 (mixed path)
    DBuf<KVecF> kvecf;
    DBuf<float2> eikrf, rhof;
    DBuf<float> qf;
    DBuf<SysDev> sysdev;
    DBuf<PairDev> ptab;
    DBuf<KVecDev> kvec;
    DBuf<uint32_t> status, sys_rebuild, sys_status;
    DBuf<int> pairs_out;
    DBuf<unsigned long long> pairs_count;
    uint32_t* h_status = nullptr;  // pinned
    uint32_t* d_h_status = nullptr;  // h_status as kernels address it
    double* h_out = nullptr;       // pinned, nsys * RED_STRIDE
    size_t h_out_cap = 0;          // systems h_out holds
    std::vector<SysDev> h_sysdev;
    std::vector<int> h_kvec_sys;

    bool tuned = false;
    bool nonfinite = false;  // a system's state became non-finite during the current lg_md_run
    // Lazy host synchronisation (lg_md_propagate): the positions and velocities
    // the host and the engine last exchanged (pinned, 3n + 3n doubles), valid
    // while no other call has written the device state since.
    double* h_shadow = nullptr;
    double* d_shadow = nullptr;  // h_shadow as kernels address it
    size_t shadow_n3 = 0;
    bool shadow_valid = false;
    uint64_t state_gen = 0;  // completed lg_md_run calls (a generation counter of the device state)
    int max_nk = 0;
    // kernels launched so far (graph replays counted by their kernel nodes)
    uint64_t launches = 0;
    size_t graph_kernels = 0;

    // persistent batched MD (mixed batches of pair-potential systems)
    int pk_cluster = 0;  // cluster size of the plan; 0: not planned, -1: not eligible
    int pk_groups = 0;
    int pk_stage = 0;    // atoms each block stages in shared memory (0: gathers from global memory)
    DBuf<int> pk_group_off, pk_group_sys, pk_group_flag;
    DBuf<double> pk_ke;
    // one graph per (steps, thermostat): checkpoint copies, flag reset, the launch
    // (a graph replay avoids the per-launch cost of a cluster launch)
    std::map<int, cudaGraphExec_t> pk_graphs;

    // MD graphs, one per chunk length
    std::map<int, cudaGraphExec_t> graphs;
    std::map<int, size_t> graph_nodes;
    int graph_mode = -1;  // md_mode() of the captured graphs

    // batched Monte Carlo chains
    DBuf<McState> mc_chains;
    std::vector<McState> h_mc;
    bool mc_energies_ready = false;

    // MC (single molecule moves)
    DBuf<double> mc_newpos, mc_partial, mc_dk, mc_out;
    DBuf<double2> mc_eikr, mc_drho;
    double mc_energy = 0.0;
    double mc_pending_cost = 0.0;
    bool mc_pending = false;
    int mc_sys = -1;
    int64_t mc_mol_begin = 0, mc_mol_size = 0;
    // a pending move_all_molecules_cost: the configuration before the move
    bool mc_resize = false;
    HostCell mc_old_cell;
    DBuf<double4_32a> mc_saved_pos;

    void drop_graphs() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
        graph_nodes.clear();
        for (auto& g : pk_graphs) cudaGraphExecDestroy(g.second);
        pk_graphs.clear();
    }

    ~lg_engine() {
        drop_graphs();
        if (h_shadow) cudaFreeHost(h_shadow);
        if (h_status) cudaFreeHost(h_status);
        if (h_out) cudaFreeHost(h_out);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace lg {

int fail(lg_engine* e, int code, const std::string& msg);

#define CUDA_TRY(e, call)                                                                          \
    do {                                                                                           \
        cudaError_t _err = (call);                                                                 \
        if (_err != cudaSuccess)                                                                   \
            return fail((e), LG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_err)); \
    } while (0)

bool valid_sys(lg_engine* e, int32_t s);
void invalidate(lg_engine* e);

// ---- lower.cu -------------------------------------------------------------------
void fill_md(SysDev& d, const HostSystem& h);
double max_cutoff(const HostSystem& h);
int check_pair_cutoffs(lg_engine* e, const HostSystem& h);
// System::set_pair_potential / set_coulomb_potential's check (sys/system.rs:122-131,
// 159-170) of the potentials of h against the cell lengths L.
int check_cell_cutoffs(lg_engine* e, const HostSystem& h, const double len[3]);
// Lowers the description into device memory when it changed (e->dirty).
int commit(lg_engine* e);
// A new orthorhombic cell for system s of a lowered batch, in place: the
// cell-dependent fields of its device record, Ewald k-vector factors and tail
// constants, and a list rebuild; the device state is kept.  Returns -1 (and
// changes nothing) when the cell grid or the k-vector set would change: the
// caller then lowers the batch again (invalidate); LG_OK or an LG_ERR_* else.
int set_cell_fast(lg_engine* e, int s, const HostCell& cell);
// Installs `cell` as system s's cell on the host (no device work).
void set_host_cell(HostSystem& h, const HostCell& cell);
// commit() for a batch whose systems all keep their device state (systems
// left, or were re-described without new particles); LG_ERR_STATE otherwise.
int commit_carried(lg_engine* e);

// ---- runtime.cu -----------------------------------------------------------------
int regrow(lg_engine* e);
// After ST_CELL_OVF: zeroes every cell count and asks every system for a rebuild.
int recount_cells(lg_engine* e);
// Which systems have SYS_NONFINITE set, as "k, l, ..." (the flags stay set).
std::string nonfinite_systems(lg_engine* e);
int read_status(lg_engine* e, uint32_t* out);
int clear_status_bits(lg_engine* e, uint32_t bits);
int nlist_launches(const Batch& b);
void enqueue_forces(lg_engine* e, uint32_t terms, bool ev, cudaStream_t st, bool fixed_written = false);
int compute_batch(lg_engine* e, uint32_t terms, uint32_t want, double* d_force_out, double* d_out);
const void* mapped_host(const void* p);
int put_state(lg_engine* e, int64_t base, int64_t n, const double* positions, const double* velocities);
int get_state(lg_engine* e, int64_t base, int64_t n, double* positions, double* velocities);
// get_state into page-locked host buffers given by their device addresses
int get_state_mapped(lg_engine* e, int64_t base, int64_t n, double* dp, double* dv);
int upload_positions(lg_engine* e, int32_t s, const double* positions);
int autotune(lg_engine* e);
// What the MD steps of a batch need besides the integrators (md_mode bits).
constexpr int MD_ADJUST = 1, MD_REWRAP = 2, MD_VERLET_SYS = 4;
int md_mode(const lg_engine* e);
void enqueue_md_step(lg_engine* e, int mode, bool apply_previous, cudaStream_t st);
void enqueue_md_finish(lg_engine* e, int mode, cudaStream_t st);
bool persist_batch(const lg_engine* e);
bool persist_eligible(const lg_engine* e);
int persist_plan(lg_engine* e);
int md_run_persistent(lg_engine* e, int64_t nsteps, bool thermo, const std::function<int()>& tail);
// lg_md_run of a batch with a barostat system: one step at a time, the cell
// of every barostat system changed between steps from the pressure of the
// previous one (one host synchronisation per step).
int md_run_barostat(lg_engine* e, int64_t nsteps);
int build_md_graph(lg_engine* e, int steps, int mode);

}  // namespace lg
