// capi.cu -- the engine object behind the C ABI of include/lumol_gb300.h.
//
// The host side keeps the description of every system (particles, topology,
// pair table, Coulomb potential, cell) as Lumol's System holds it, lowers it
// into the flat device layout of kernels.h on first use after a change, and
// drives the kernels.  Host arithmetic that feeds results (potential shifts,
// Ewald k-vector factors, tail corrections, self energy) restates the
// reference operation by operation; the file is compiled with
// -ffp-contract=off so the host compiler does not fuse it either.
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
#include <vector>

#include "../../include/lumol_gb300.h"
#include "kernels.h"

using namespace lg;

namespace {

thread_local std::string g_create_error;
constexpr int MIN_KCHUNK = 8;

// Tuned launch parameters per workload shape: (device, precision, atoms,
// list capacity, k-vectors) -> (threads per atom, k-vectors per field chunk).
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int, int, bool>, std::pair<int, int>> g_tune_cache;

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
};

static_assert(MD_VELOCITY_VERLET == LG_INTEGRATOR_VELOCITY_VERLET && MD_VERLET == LG_INTEGRATOR_VERLET &&
                  MD_LEAP_FROG == LG_INTEGRATOR_LEAP_FROG,
              "integrator values");
static_assert(TH_NONE == LG_THERMOSTAT_NONE && TH_BERENDSEN == LG_THERMOSTAT_BERENDSEN &&
                  TH_RESCALE == LG_THERMOSTAT_RESCALE && TH_CSVR == LG_THERMOSTAT_CSVR,
              "thermostat values");
static_assert(CTL_REMOVE_TRANSLATION == LG_CONTROL_REMOVE_TRANSLATION && CTL_REWRAP == LG_CONTROL_REWRAP &&
                  CTL_REMOVE_ROTATION == LG_CONTROL_REMOVE_ROTATION,
              "control values");

struct HostSystem {
    bool has_cell = false;
    double L[3] = {0, 0, 0};
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
    // derived
    std::vector<int64_t> mol_begin;  // first atom of each molecule (local index), plus the end
    double tail_energy = 0.0, tail_virial = 0.0, ewald_self = 0.0;
    double alpha = 0.0;
};

// The MD fields of a system's device record.
void fill_md(SysDev& d, const HostSystem& h) {
    d.dt = h.dt;
    d.hdt = 0.5 * h.dt;
    d.dt2 = h.dt * h.dt;  // integrators.rs:107, 149
    d.hdt2 = 0.5 * d.dt2;
    d.inv_2dt = h.dt > 0.0 ? 1.0 / (2.0 * h.dt) : 0.0;
    d.thermo_T = h.T0;
    d.thermo_tau = h.tau;
    d.thermo_tol = h.tol;
    d.seed = h.seed;
    d.integrator = h.integrator;
    d.thermostat = h.thermostat;
    d.controls = h.controls;
    d.dof = (double)(3 * h.n);
    double total = 0.0;  // RemoveTranslation: masses summed in atom order (controls.rs:31)
    for (double w : h.masses) total += w;
    d.total_mass = total;
}

// A bonded potential as the bonded kernel reads it: (k, x0, extra, kind) with
// k NaN for NullPotential; kind 0 Harmonic, 1 CosineHarmonic (extra = cos x0,
// CosineHarmonic::new, functions.rs:190-195), 2 Torsion (x0 = delta, extra = n).
double4_32a bonded_par(const lg_bonded& p) {
    double k = p.type == LG_PAIR_NULL ? NAN : p.k;
    if (p.type == LG_BONDED_COSINE_HARMONIC) return make_double4_32a(k, p.x0, std::cos(p.x0), 1.0);
    if (p.type == LG_BONDED_TORSION) return make_double4_32a(k, p.x0, (double)p.n, 2.0);
    if (p.type == LG_PAIR_MORSE) return make_double4_32a(k, p.x0, p.a, 3.0);
    return make_double4_32a(k, p.x0, 0.0, 0.0);
}

// ---- host restatement of the reference's scalar functions -----------------
double powi6(double x) {
    double x2 = x * x;
    double x4 = x2 * x2;
    return x2 * x4;
}
// Mie::new's energy prefactor n / (n - m) (n / m)^(m / (n - m)) epsilon (functions.rs:540-549)
double mie_prefactor(const lg_pair& p) {
    double n = p.p2, mm = p.p3;
    return n / (n - mm) * std::pow(n / mm, mm / (n - mm)) * p.p1;
}
// Potential::energy (functions.rs:85-88, 287-292, 135-139, 354-359, 415-418, 475-477, 553-558)
double pot_energy(const lg_pair& p, double r) {
    switch (p.type) {
        case LG_PAIR_LJ: {
            double s6 = powi6(p.p0 / r);
            return 4.0 * p.p1 * (s6 * s6 - s6);
        }
        case LG_PAIR_BUCKINGHAM: {
            double r3 = r * r * r;
            double r6 = r3 * r3;
            double e = std::exp(-r / p.p2);
            return p.p0 * e - p.p1 / r6;
        }
        case LG_PAIR_HARMONIC: {
            double dx = r - p.p1;
            return 0.5 * p.p0 * dx * dx;
        }
        case LG_PAIR_BMH: {  // functions.rs:354-359
            double r2 = r * r;
            double r6 = r2 * r2 * r2;
            double ex = std::exp((p.p3 - r) / p.p4);
            return p.p0 * ex - p.p1 / r6 + p.p2 / (r6 * r2);
        }
        case LG_PAIR_MORSE: {  // functions.rs:415-418
            double rc = 1.0 - std::exp((p.p1 - r) * p.p0);
            return p.p2 * rc * rc;
        }
        case LG_PAIR_GAUSSIAN:  // functions.rs:475-477
            return -p.p0 * std::exp(-p.p1 * r * r);
        case LG_PAIR_MIE: {  // functions.rs:553-558
            double sr = p.p0 / r;
            return mie_prefactor(p) * (std::pow(sr, p.p2) - std::pow(sr, p.p3));
        }
        default:
            return 0.0;
    }
}
// Potential::force (functions.rs:90-93, 294-299, 141-143, 361-366, 420-423, 479-481, 560-565)
double pot_force(const lg_pair& p, double r) {
    switch (p.type) {
        case LG_PAIR_LJ: {
            double s6 = powi6(p.p0 / r);
            return -24.0 * p.p1 * (s6 - 2.0 * (s6 * s6)) / r;
        }
        case LG_PAIR_BUCKINGHAM: {
            double r3 = r * r * r;
            double r7 = r3 * r3 * r;
            double e = std::exp(-r / p.p2);
            return p.p0 / p.p2 * e - 6.0 * p.p1 / r7;
        }
        case LG_PAIR_HARMONIC:
            return p.p0 * (p.p1 - r);
        case LG_PAIR_BMH: {
            double r2 = r * r;
            double r7 = r2 * r2 * r2 * r;
            double e = std::exp((p.p3 - r) / p.p4);
            return p.p0 / p.p4 * e - 6.0 * p.p1 / r7 + 8.0 * p.p2 / (r7 * r2);
        }
        case LG_PAIR_MORSE: {  // as written there: 2 depth (1 - e^2) a
            double e = std::exp((p.p1 - r) * p.p0);
            return 2.0 * p.p2 * (1.0 - e * e) * p.p0;
        }
        case LG_PAIR_GAUSSIAN:
            return 2.0 * p.p1 * r * pot_energy(p, r);
        case LG_PAIR_MIE: {
            double sr = p.p0 / r;
            double rep = std::pow(sr, p.p2), att = std::pow(sr, p.p3);
            return mie_prefactor(p) * (p.p2 * rep - p.p3 * att) / r;
        }
        default:
            return 0.0;
    }
}

// TableComputation::new (energy/computations.rs:101-121): (energy, force) at
// r = i delta, delta = max / size.
void build_table(const lg_pair& p, std::vector<double2>& out) {
    double delta = p.table_max / (double)p.table_size;
    for (int32_t i = 0; i < p.table_size; i++) {
        double r = (double)i * delta;
        out.push_back(make_double2(pot_energy(p, r), pot_force(p, r)));
    }
}
// Computation::compute_energy (computations.rs:123-133) on a table built above
double table_energy(const lg_pair& p, const double2* t, double r) {
    double delta = p.table_max / (double)p.table_size;
    double binf = std::floor(r / delta);
    if (binf < (double)(p.table_size - 1)) {
        size_t bin = (size_t)binf;
        double dx = r - (double)bin * delta;
        double slope = (t[bin + 1].x - t[bin].x) / delta;
        return t[bin].x + dx * slope;
    }
    return 0.0;
}

// PairPotential::tail_energy / tail_virial (functions.rs:97-111, 303-318)
double pot_tail_energy(const lg_pair& p, double rc) {
    if (p.type == LG_PAIR_LJ) {
        double s3 = p.p0 * p.p0 * p.p0;
        double rc3 = rc * rc * rc;
        double s9 = s3 * s3 * s3;
        double rc9 = rc3 * rc3 * rc3;
        return 4.0 / 3.0 * p.p1 * s3 * (1.0 / 3.0 * s9 / rc9 - s3 / rc3);
    }
    if (p.type == LG_PAIR_BUCKINGHAM) {
        double rc2 = rc * rc;
        double rc3 = rc2 * rc;
        double e = std::exp(-rc / p.p2);
        double factor = rc2 - 2.0 * rc * p.p2 + 2.0 * p.p2 * p.p2;
        return p.p0 * p.p2 * e * factor - p.p1 / (3.0 * rc3);
    }
    if (p.type == LG_PAIR_BMH) {  // functions.rs:370-376
        double rc2 = rc * rc;
        double rc3 = rc2 * rc;
        double e = std::exp((p.p3 - rc) / p.p4);
        double factor = rc2 - 2.0 * rc * p.p4 + 2.0 * p.p4 * p.p4;
        return p.p0 * p.p4 * e * factor - p.p1 / (3.0 * rc3) + p.p2 / (5.0 * rc2 * rc3);
    }
    if (p.type == LG_PAIR_GAUSSIAN) {  // functions.rs:485-488
        double b = p.p1;
        return pot_energy(p, rc) * rc / (2.0 * b) -
               p.p0 * std::sqrt(PI) * std::erfc(std::sqrt(b) * rc) / (4.0 * std::pow(b, 1.5));
    }
    if (p.type == LG_PAIR_MIE) {  // functions.rs:569-579
        if (p.p3 <= 3.0) return 0.0;
        double src = p.p0 / rc;
        double n3 = p.p2 - 3.0, m3 = p.p3 - 3.0;
        return mie_prefactor(p) * (p.p0 * p.p0 * p.p0) * (std::pow(src, n3) / n3 - std::pow(src, m3) / m3);
    }
    return 0.0;
}
double pot_tail_virial(const lg_pair& p, double rc) {
    if (p.type == LG_PAIR_LJ) {
        double s3 = p.p0 * p.p0 * p.p0;
        double rc3 = rc * rc * rc;
        double s9 = s3 * s3 * s3;
        double rc9 = rc3 * rc3 * rc3;
        return 8.0 * p.p1 * s3 * (2.0 / 3.0 * s9 / rc9 - s3 / rc3);
    }
    if (p.type == LG_PAIR_BUCKINGHAM) {
        double rc2 = rc * rc;
        double rc3 = rc2 * rc;
        double e = std::exp(-rc / p.p2);
        double factor = rc3 + 3.0 * rc2 * p.p2 + 6.0 * rc * p.p2 * p.p2 + 6.0 * p.p2 * p.p2 * p.p2;
        return p.p0 * e * factor - 20.0 * p.p1 / rc3 + 8.0;
    }
    if (p.type == LG_PAIR_BMH) {  // functions.rs:378-385
        double rc2 = rc * rc;
        double rc3 = rc2 * rc;
        double e = std::exp((p.p3 - rc) / p.p4);
        double factor = rc3 + 3.0 * rc2 * p.p4 + 6.0 * rc * p.p4 * p.p4 + 6.0 * p.p4 * p.p4 * p.p4;
        return p.p0 * e * factor - 20.0 * p.p1 / rc3 + 8.0 * p.p2 / (5.0 * rc2 * rc3);
    }
    if (p.type == LG_PAIR_GAUSSIAN) {  // functions.rs:490-493
        double b = p.p1;
        return 3.0 * std::sqrt(PI) * p.p0 * std::erfc(std::sqrt(b) * rc) / (4.0 * std::pow(b, 1.5)) -
               pot_energy(p, rc) * rc * (2.0 * b * rc * rc + 3.0) / (2.0 * b);
    }
    if (p.type == LG_PAIR_MIE) {  // functions.rs:581-591
        if (p.p3 <= 3.0) return 0.0;
        double src = p.p0 / rc;
        double n3 = p.p2 - 3.0, m3 = p.p3 - 3.0;
        return mie_prefactor(p) * (p.p0 * p.p0 * p.p0) *
               (std::pow(src, n3) * p.p2 / n3 - std::pow(src, m3) * p.p3 / m3);
    }
    return 0.0;
}

// Matrix3::inverse of diag(a, b, c) (types/matrix.rs:212-227), diagonal only
void ortho_inverse_diag(const double L[3], double out[3]) {
    double a = L[0], b = L[1], c = L[2];
    double m[3][3] = {{a, 0.0, 0.0}, {0.0, b, 0.0}, {0.0, 0.0, c}};
    double det = m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) -
                 m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                 m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    double id = 1.0 / det;
    out[0] = (m[1][1] * m[2][2] - m[2][1] * m[1][2]) * id;
    out[1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    out[2] = (m[0][0] * m[1][1] - m[1][0] * m[0][1]) * id;
}

// Ewald::prepare + compute_ewald_factors_triclinic (ewald.rs:130-183, 353-379)
void ewald_factors(const double L[3], double alpha, int kmax, int sys, std::vector<KVecDev>& out) {
    double inv[3];
    ortho_inverse_diag(L, inv);
    double s[3] = {(2.0 * PI) * inv[0], (2.0 * PI) * inv[1], (2.0 * PI) * inv[2]};
    // k_vector([1, 1, 1]).max() * kmax; off-diagonal products are zero
    double mx = std::max(std::max(s[0], s[1]), s[2]) * (double)kmax;
    double kmax2 = 1.0001 * mx * mx;
    double alpha_sq_inv_fourth = 0.25 / (alpha * alpha);
    double four_pi_v = 4.0 * PI / (L[0] * L[1] * L[2]);
    auto push = [&](int ikx, int iky, int ikz) {
        double k[3] = {s[0] * (double)ikx, s[1] * (double)iky, s[2] * (double)ikz};
        double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (k2 > kmax2) return;
        KVecDev f;
        std::memset(&f, 0, sizeof(f));
        f.ikx = ikx;
        f.iky = iky;
        f.ikz = ikz;
        f.sys = sys;
        f.energy = four_pi_v * std::exp(-k2 * alpha_sq_inv_fourth) / k2;
        for (int d = 0; d < 3; d++) f.field[d] = (2.0 * f.energy) * k[d];
        double vf = -2.0 * (1.0 / k2 + alpha_sq_inv_fourth);
        const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
        for (int c = 0; c < 6; c++) {
            double v = (ia[c] == ib[c] ? 1.0 : 0.0) + vf * (k[ia[c]] * k[ib[c]]);
            f.virial[c] = f.energy * v;
        }
        out.push_back(f);
    };
    for (int ikx = 1; ikx < kmax; ikx++)
        for (int iky = -kmax; iky < kmax; iky++)
            for (int ikz = -kmax; ikz < kmax; ikz++) push(ikx, iky, ikz);
    for (int iky = 1; iky < kmax; iky++)
        for (int ikz = -kmax; ikz < kmax; ikz++) push(0, iky, ikz);
    for (int ikz = 1; ikz < kmax; ikz++) push(0, 0, ikz);
}

}  // namespace

namespace lg {
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace lg

struct lg_engine {
    lg_options opt{};
    int nsys = 0;
    std::vector<HostSystem> sys;
    std::string err;
    cudaStream_t stream = nullptr;
    bool dirty = true;
    std::vector<int64_t> begin;  // atom offsets (nsys + 1)
    double skin = 1.0;

    Batch b;
    // device storage
    DBuf<double4_32a> posq, vel, acc, pos_build;
    DBuf<double> force, pos3, vel3, red, host_const, kepart, mom, out, fpart, kred, mc_part;
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
    DBuf<SysDev> sysdev;
    DBuf<PairDev> ptab;
    DBuf<KVecDev> kvec;
    DBuf<uint32_t> status, sys_rebuild;
    DBuf<int> pairs_out;
    DBuf<unsigned long long> pairs_count;
    uint32_t* h_status = nullptr;  // pinned
    double* h_out = nullptr;       // pinned, nsys * RED_STRIDE
    std::vector<SysDev> h_sysdev;
    std::vector<int> h_kvec_sys;

    bool tuned = false;
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

    void drop_graphs() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
        graph_nodes.clear();
        for (auto& g : pk_graphs) cudaGraphExecDestroy(g.second);
        pk_graphs.clear();
    }

    ~lg_engine() {
        drop_graphs();
        if (h_status) cudaFreeHost(h_status);
        if (h_out) cudaFreeHost(h_out);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int fail(lg_engine* e, int code, const std::string& msg) {
    if (e) e->err = msg;
    else g_create_error = msg;
    return code;
}

#define CUDA_TRY(e, call)                                                                          \
    do {                                                                                           \
        cudaError_t _err = (call);                                                                 \
        if (_err != cudaSuccess)                                                                   \
            return fail((e), LG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_err)); \
    } while (0)

bool valid_sys(lg_engine* e, int32_t s) { return e && s >= 0 && s < e->nsys; }

void invalidate(lg_engine* e) {
    e->dirty = true;
    e->drop_graphs();
}

double max_cutoff(const HostSystem& h) {
    double rc = 0.0;
    for (const lg_pair& p : h.pairs)
        if (p.type != LG_PAIR_ABSENT) rc = std::max(rc, p.cutoff);
    if (h.coul.kind != LG_COULOMB_NONE) rc = std::max(rc, h.coul.cutoff);
    return rc;
}

// Bond paths from the bond graph: the shortest path, when it has at most three
// bonds, is the BondPath Bonding::rebuild_connections records for the pair
// (bonds give ONE, angle ends TWO, dihedral ends THREE; bonding.rs:159-186).
void bond_paths(const HostSystem& h, int64_t base, std::vector<std::vector<std::pair<int, int8_t>>>& spec) {
    std::vector<std::vector<int>> adj(h.n);
    for (size_t b = 0; b + 1 < h.bonds.size(); b += 2) {
        int i = h.bonds[b], j = h.bonds[b + 1];
        adj[i].push_back(j);
        adj[j].push_back(i);
    }
    for (int64_t i = 0; i < h.n; i++) {
        if (adj[i].empty()) continue;
        std::vector<std::pair<int, int>> frontier{{(int)i, 0}};
        std::vector<int> seen{(int)i};
        for (size_t f = 0; f < frontier.size(); f++) {
            auto [a, depth] = frontier[f];
            if (depth == 3) continue;
            for (int nb : adj[a]) {
                if (std::find(seen.begin(), seen.end(), nb) != seen.end()) continue;
                seen.push_back(nb);
                frontier.push_back({nb, depth + 1});
                spec[base + i].push_back({(int)(base + nb), (int8_t)(depth + 2)});
            }
        }
    }
}

int commit(lg_engine* e) {
    if (!e->dirty) return LG_OK;
    int nsys = e->nsys;
    e->begin.assign(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
        const HostSystem& h = e->sys[s];
        if (!h.has_cell) return fail(e, LG_ERR_STATE, "system " + std::to_string(s) + " has no cell");
        if (h.nk == 0 && h.n > 0)
            return fail(e, LG_ERR_STATE, "system " + std::to_string(s) + " has no pair table");
        e->begin[s + 1] = e->begin[s] + h.n;
    }
    int64_t n = e->begin[nsys];
    if (n > (int64_t)0x7fffffff / 64) return fail(e, LG_ERR_ARGUMENT, "too many atoms");

    std::vector<double4_32a> h_posq(n), h_vel(n);
    std::vector<int> h_kind(n), h_mol(n), h_sysid(n);
    std::vector<PairDev> h_ptab;
    std::vector<PairDevF> h_ptabf;
    std::vector<double2> h_table;  // TableComputation tables of the pair entries
    std::vector<KVecDev> h_kvec;
    std::vector<std::vector<std::pair<int, int8_t>>> spec(n);
    struct Term {
        int4 t;  // (type | fourth atom << 2, atoms...): 0 bond, 1 angle, 2 dihedral
        int role;
        double4_32a par;
    };
    std::vector<std::vector<Term>> terms(n);
    e->h_sysdev.assign(nsys, SysDev{});
    std::vector<double> h_const((size_t)nsys * RED_STRIDE, 0.0);
    int mol_base = 0, cell_total = 0, kdim = 1;
    std::vector<int2> h_tiles;
    std::vector<int> h_mol_start;  // first atom of each molecule of the batch, then n
    double max_expected = 0.0;
    int64_t max_n = 1;

    for (int s = 0; s < nsys; s++) {
        HostSystem& h = e->sys[s];
        SysDev& d = e->h_sysdev[s];
        std::memset(&d, 0, sizeof(d));
        int64_t base = e->begin[s];
        max_n = std::max(max_n, h.n);
        int max_mol = -1;
        for (int64_t i = 0; i < h.n; i++) {
            h_posq[base + i] = make_double4_32a(0.0, 0.0, 0.0, h.charges[i]);
            h_vel[base + i] = make_double4_32a(0.0, 0.0, 0.0, h.masses[i]);
            h_kind[base + i] = h.kinds[i];
            h_mol[base + i] = mol_base + h.mols[i];
            h_sysid[base + i] = s;
            max_mol = std::max(max_mol, h.mols[i]);
        }
        mol_base += max_mol + 1;
        h.mol_begin.assign(max_mol + 2, h.n);
        for (int64_t i = h.n - 1; i >= 0; i--) h.mol_begin[h.mols[i]] = i;
        bond_paths(h, base, spec);
        for (size_t b = 0; b * 2 < h.bonds.size(); b++) {
            const lg_bonded& p = h.bond_pots[b];
            if (p.type == LG_PAIR_ABSENT) continue;
            double4_32a par = bonded_par(p);
            int i = (int)(base + h.bonds[2 * b]), j = (int)(base + h.bonds[2 * b + 1]);
            int a = std::min(i, j), c = std::max(i, j);  // Bond::new orders i < j (connect.rs:21-26)
            int4 t = make_int4(0, a, c, -1);
            terms[a].push_back({t, 0, par});
            terms[c].push_back({t, 1, par});
        }
        for (size_t a = 0; a * 3 < h.angles.size(); a++) {
            const lg_bonded& p = h.angle_pots[a];
            if (p.type == LG_PAIR_ABSENT) continue;
            double4_32a par = bonded_par(p);
            int i = (int)(base + h.angles[3 * a]), j = (int)(base + h.angles[3 * a + 1]),
                m = (int)(base + h.angles[3 * a + 2]);
            int lo = std::min(i, m), hi = std::max(i, m);  // Angle::new (connect.rs:54-65)
            int4 t = make_int4(1, lo, j, hi);
            terms[lo].push_back({t, 0, par});
            terms[j].push_back({t, 1, par});
            terms[hi].push_back({t, 2, par});
        }
        for (size_t d = 0; d * 4 < h.dihedrals.size(); d++) {
            const lg_bonded& p = h.dihedral_pots[d];
            if (p.type == LG_PAIR_ABSENT) continue;
            double4_32a par = bonded_par(p);
            int q[4];
            for (int k = 0; k < 4; k++) q[k] = (int)(base + h.dihedrals[4 * d + k]);
            int4 t = make_int4(2 | (q[3] << 2), q[0], q[1], q[2]);  // the fourth atom in the type word
            for (int k = 0; k < 4; k++) terms[q[k]].push_back({t, k, par});
        }

        // pair table
        d.ptab = (int)h_ptab.size();
        d.nk = h.nk;
        bool needs_path = false;
        for (const lg_pair& p : h.pairs) {
            PairDev q;
            std::memset(&q, 0, sizeof(q));
            q.type = p.type;
            q.shifted = p.shifted;
            q.restriction = p.restriction;
            q.tail = p.tail;
            q.p0 = p.p0;
            q.p1 = p.p1;
            q.p2 = p.p2;
            q.p3 = p.p3;
            q.p4 = p.p4;
            if (p.type == LG_PAIR_MIE) q.aux = mie_prefactor(p);
            q.cutoff = p.cutoff;
            q.shift = p.shifted ? pot_energy(p, p.cutoff) : 0.0;  // pairs.rs:86-95
            const bool tab = p.type != LG_PAIR_ABSENT && p.table_size > 0;
            size_t toff = h_table.size();
            if (tab) {  // the table replaces the potential (its tails stay the potential's)
                build_table(p, h_table);
                q.type = PAIR_TABLE;
                q.tsize = p.table_size;
                q.tdelta = p.table_max / (double)p.table_size;
                q.table = reinterpret_cast<const double2*>(toff);  // an offset until the upload
                q.shift = p.shifted ? table_energy(p, h_table.data() + toff, p.cutoff) : 0.0;
            }
            q.scale14 = p.scale14;
            q.cutoff2_f = (float)(p.cutoff * p.cutoff);
            if (p.type == LG_PAIR_LJ) {
                double s2 = p.p0 * p.p0, s6 = s2 * s2 * s2;
                q.c6 = 4.0 * p.p1 * s6;
                q.c12 = 4.0 * p.p1 * s6 * s6;
            }
            if (p.type != LG_PAIR_ABSENT && p.restriction > LG_RESTRICT_INTER) needs_path = true;
            h_ptab.push_back(q);
            PairDevF qf;
            std::memset(&qf, 0, sizeof(qf));
            qf.type = p.type;
            qf.restriction = p.restriction;
            if (p.type == LG_PAIR_LJ) {
                double s6 = std::pow(p.p0, 6.0);
                qf.a = (float)(4.0 * p.p1 * s6 * s6);
                qf.b = (float)(4.0 * p.p1 * s6);
            } else if (p.type == LG_PAIR_BUCKINGHAM) {
                qf.a = (float)p.p0;
                qf.b = (float)p.p1;
                qf.c = (float)(1.0 / p.p2);
            } else if (p.type == LG_PAIR_HARMONIC) {
                qf.a = (float)p.p0;
                qf.b = (float)p.p1;
            } else if (p.type == LG_PAIR_BMH) {  // a exp((sigma - r) / rho) - c / r^6 + d / r^8
                qf.a = (float)p.p0;
                qf.b = (float)p.p1;
                qf.c = (float)(1.0 / p.p4);
                qf.d = (float)p.p2;
                qf.e = (float)p.p3;
            } else if (p.type == LG_PAIR_MORSE) {  // depth (1 - exp(a (x0 - r)))^2
                qf.a = (float)p.p2;
                qf.b = (float)p.p0;
                qf.c = (float)p.p1;
            } else if (p.type == LG_PAIR_GAUSSIAN) {  // -a exp(-b r^2)
                qf.a = (float)p.p0;
                qf.b = (float)p.p1;
            } else if (p.type == LG_PAIR_MIE) {  // prefactor ((sigma / r)^n - (sigma / r)^m)
                qf.a = (float)mie_prefactor(p);
                qf.b = (float)p.p0;
                qf.c = (float)p.p2;
                qf.d = (float)p.p3;
            }
            if (tab) {
                qf.type = PAIR_TABLE;
                qf.a = (float)(1.0 / q.tdelta);
                qf.b = (float)q.tdelta;
                qf.c = (float)(p.table_size - 1);
                qf.table = reinterpret_cast<const float2*>(toff);
            }
            qf.rc2 = (float)(p.cutoff * p.cutoff);
            qf.shift = (float)q.shift;
            qf.scale14 = (float)p.scale14;
            h_ptabf.push_back(qf);
        }
        if (h.coul.kind != LG_COULOMB_NONE && h.coul.restriction > LG_RESTRICT_INTER) needs_path = true;
        d.needs_path = needs_path;

        // cell and neighbour list geometry
        for (int k = 0; k < 3; k++) {
            d.L[k] = h.L[k];
            d.invL[k] = 1.0 / h.L[k];
            d.Lf[k] = (float)h.L[k];
            d.invLf[k] = (float)(1.0 / h.L[k]);
            d.Lq[k] = (float)(h.L[k] / 4294967296.0);
            d.fxscale[k] = d.invL[k] * 4294967296.0;
        }
        double rc = max_cutoff(h);
        d.rlist = rc + e->skin;
        d.half_skin2 = 0.25 * e->skin * e->skin;
        d.rebuild2_f = 0.99f * (float)d.half_skin2;
        double margin = 1e-5 * std::max(std::max(h.L[0], h.L[1]), h.L[2]) + 1e-4;
        d.rlist2_f = (float)((d.rlist + margin) * (d.rlist + margin));
        // cells at least half the list radius wide: the list builds look two cells around
        int cells = 1;
        for (int k = 0; k < 3; k++) {
            int nc = (int)std::floor(h.L[k] / (0.5 * (d.rlist + margin)));
            nc = std::max(1, std::min(nc, 128));
            d.ncell[k] = nc;
            cells *= nc;
        }
        d.cell_begin = cell_total;
        cell_total += cells;
        d.tile_begin = (int)h_tiles.size();
        for (int64_t a = 0; a < h.n; a += VV_TILE) h_tiles.push_back(make_int2(s, (int)(base + a)));
        d.tile_end = (int)h_tiles.size();
        double volume = h.L[0] * h.L[1] * h.L[2];
        if (h.n > 0) {
            double expected = (double)h.n / volume * 4.0 / 3.0 * PI * d.rlist * d.rlist * d.rlist;
            max_expected = std::max(max_expected, expected);
        }

        // Coulomb
        d.coul = h.coul.kind;
        d.coul_restr = h.coul.restriction;
        d.coul_rc = h.coul.cutoff;
        d.coul_scale14 = h.coul.scale14;
        d.coul_rc2_f = (float)(h.coul.cutoff * h.coul.cutoff);
        h.ewald_self = 0.0;
        if (h.coul.kind == LG_COULOMB_EWALD) {
            h.alpha = h.coul.alpha > 0.0 ? h.coul.alpha : PI / h.coul.cutoff;  // ewald.rs:278-279
            d.alpha = h.alpha;
            d.kmax = h.coul.kmax;
            kdim = std::max(kdim, h.coul.kmax + 1);
            double inv[3];
            ortho_inverse_diag(h.L, inv);
            for (int k = 0; k < 3; k++) d.k1[k] = (2.0 * PI) * inv[k];
            d.kbegin = (int)h_kvec.size();
            ewald_factors(h.L, h.alpha, h.coul.kmax, s, h_kvec);
            d.kend = (int)h_kvec.size();
            // Ewald::self_energy (ewald.rs:619-626)
            double q2 = 0.0;
            for (double q : h.charges) q2 += q * q;
            h.ewald_self = -h.alpha / std::sqrt(PI) * q2 / FOUR_PI_EPSILON_0;
        } else if (h.coul.kind == LG_COULOMB_WOLF) {
            // Wolf::new (wolf.rs:68-84)
            double cutoff = h.coul.cutoff;
            double alpha = PI / cutoff;
            double ac = alpha * cutoff;
            double ac2 = ac * ac;
            d.alpha = alpha;
            d.wolf_ec = std::erfc(ac) / cutoff;
            d.wolf_fc = std::erfc(ac) / (cutoff * cutoff) + FRAC_2_SQRT_PI * alpha * std::exp(-ac2) / cutoff;
        }
        d.kbegin = h.coul.kind == LG_COULOMB_EWALD ? d.kbegin : (int)h_kvec.size();
        d.kend = h.coul.kind == LG_COULOMB_EWALD ? d.kend : (int)h_kvec.size();

        // Tail corrections (sys/energy.rs:63-79, compute.rs:219-229), kinds in index order
        std::vector<int64_t> counts(h.nk, 0);
        for (int32_t k : h.kinds) counts[k]++;
        double te = 0.0, tv = 0.0;
        for (int a = 0; a < h.nk; a++) {
            if (!counts[a]) continue;
            for (int c = 0; c < h.nk; c++) {
                if (!counts[c]) continue;
                double two_pi_density = 2.0 * PI * (double)counts[a] * (double)counts[c] / volume;
                const lg_pair& p = h.pairs[(size_t)a * h.nk + c];
                if (p.type == LG_PAIR_ABSENT || !p.tail) continue;
                te += two_pi_density * pot_tail_energy(p, p.cutoff);
                tv += two_pi_density * (pot_tail_virial(p, p.cutoff) * (1.0 / 3.0));
            }
        }
        h.tail_energy = te;
        h.tail_virial = tv;
        double* hc = &h_const[(size_t)s * RED_STRIDE];
        hc[0] = te;
        hc[1] = tv;
        hc[2] = h.ewald_self;

        d.begin = (int)base;
        d.end = (int)(base + h.n);
        fill_md(d, h);
        // the system's molecules in the batch molecule table (contiguous atoms each)
        d.mol_first = (int)(h_mol_start.size());
        for (size_t k = 0; k + 1 < h.mol_begin.size(); k++)
            if (h.mol_begin[k + 1] > h.mol_begin[k]) h_mol_start.push_back((int)(base + h.mol_begin[k]));
        d.mol_end = (int)h_mol_start.size();
    }
    h_mol_start.push_back((int)n);

    // per-atom CSR tables
    std::vector<int> h_spec_off(n + 1, 0), h_spec_j;
    std::vector<int8_t> h_spec_path;
    for (int64_t i = 0; i < n; i++) {
        h_spec_off[i] = (int)h_spec_j.size();
        for (auto& pr : spec[i]) {
            h_spec_j.push_back(pr.first);
            h_spec_path.push_back(pr.second);
        }
    }
    h_spec_off[n] = (int)h_spec_j.size();
    std::vector<int> h_bt_off(n + 1, 0), h_bt_role;
    std::vector<int4> h_bt;
    std::vector<double4_32a> h_bt_par;
    for (int64_t i = 0; i < n; i++) {
        h_bt_off[i] = (int)h_bt.size();
        for (auto& t : terms[i]) {
            h_bt.push_back(t.t);
            h_bt_role.push_back(t.role);
            h_bt_par.push_back(t.par);
        }
    }
    h_bt_off[n] = (int)h_bt.size();

    // neighbour capacity: 1.6x the mean count plus a margin, never above the largest system
    int maxnb = (int)std::ceil(1.6 * max_expected + 64.0);
    maxnb = std::min(maxnb, (int)max_n);
    maxnb = std::max(32, (maxnb + 31) / 32 * 32);
    if (e->b.maxnb > maxnb && e->b.n == n) maxnb = e->b.maxnb;  // keep a capacity that was regrown

    // allocate
    CUDA_TRY(e, e->posq.alloc(n));
    CUDA_TRY(e, e->vel.alloc(n));
    CUDA_TRY(e, e->acc.alloc(n));
    CUDA_TRY(e, e->pos_build.alloc(n));
    CUDA_TRY(e, e->force.alloc(3 * n));
    CUDA_TRY(e, e->pos3.alloc(3 * n));
    CUDA_TRY(e, e->vel3.alloc(3 * n));
    CUDA_TRY(e, e->red.alloc((size_t)n * RED_STRIDE));
    CUDA_TRY(e, e->host_const.alloc((size_t)nsys * RED_STRIDE));
    CUDA_TRY(e, e->tiles.alloc(std::max<size_t>(h_tiles.size(), 1)));
    CUDA_TRY(e, e->kepart.alloc(std::max<size_t>(n, 1)));  // chunk kinetic energies: at most one per atom
    CUDA_TRY(e, e->mom.alloc(std::max<size_t>(3 * n, 1)));
    CUDA_TRY(e, e->md_count.alloc(std::max(nsys, 1)));
    CUDA_TRY(e, e->cp_count.alloc(std::max(nsys, 1)));
    CUDA_TRY(e, e->adj.alloc(4 * (size_t)std::max(nsys, 1)));
    CUDA_TRY(e, e->mol_start.alloc(h_mol_start.size()));
    CUDA_TRY(e, e->cp_pos.alloc(n));
    CUDA_TRY(e, e->cp_vel.alloc(n));
    CUDA_TRY(e, e->cp_acc.alloc(n));
    CUDA_TRY(e, e->out.alloc((size_t)nsys * RED_STRIDE));
    CUDA_TRY(e, e->kind.alloc(n));
    CUDA_TRY(e, e->mol.alloc(n));
    CUDA_TRY(e, e->sysid.alloc(n));
    CUDA_TRY(e, e->spec_off.alloc(n + 1));
    CUDA_TRY(e, e->spec_j.alloc(h_spec_j.size()));
    CUDA_TRY(e, e->spec_path.alloc(h_spec_path.size()));
    CUDA_TRY(e, e->bt_off.alloc(n + 1));
    CUDA_TRY(e, e->bt.alloc(h_bt.size()));
    CUDA_TRY(e, e->bt_role.alloc(h_bt_role.size()));
    CUDA_TRY(e, e->bt_par.alloc(h_bt_par.size()));
    CUDA_TRY(e, e->nbr.alloc((size_t)n * maxnb));
    CUDA_TRY(e, e->nnb.alloc(n));
    CUDA_TRY(e, e->atom_cell.alloc(n));
    CUDA_TRY(e, e->cell_count.alloc(cell_total));
    CUDA_TRY(e, e->cell_start.alloc(cell_total + nsys));  // one end sentinel per system
    CUDA_TRY(e, e->cell_atoms.alloc(n));
    CUDA_TRY(e, e->plan.alloc(3 + 3 * (size_t)nsys));
    CUDA_TRY(e, e->wpos.alloc(n));
    CUDA_TRY(e, e->sysdev.alloc(nsys));
    CUDA_TRY(e, e->ptab.alloc(h_ptab.size()));
    CUDA_TRY(e, e->status.alloc(1));
    CUDA_TRY(e, e->sys_rebuild.alloc(nsys));
    int nkv = (int)h_kvec.size();
    int kchunk = 32;
    int nkchunks = 0, max_chunks = 0;
    int max_nk = 0;
    for (int s = 0; s < nsys; s++) max_nk = std::max(max_nk, e->h_sysdev[s].kend - e->h_sysdev[s].kbegin);
    nkchunks = (max_nk + kchunk - 1) / kchunk;
    max_chunks = (max_nk + MIN_KCHUNK - 1) / MIN_KCHUNK;  // room for the smallest chunk the tuner tries
    e->max_nk = max_nk;
    bool mixed = e->opt.precision == LG_PRECISION_MIXED;
    std::vector<KVecF> h_kvecf(nkv);
    for (int k = 0; k < nkv; k++) {
        const KVecDev& v = h_kvec[k];
        h_kvecf[k] = KVecF{v.ikx, v.iky, v.ikz, v.sys, (float)v.field[0], (float)v.field[1], (float)v.field[2],
                           (float)v.energy};
    }
    CUDA_TRY(e, e->ptabf.alloc(h_ptabf.size()));
    // TableComputation tables: FP64 for the plain path, FP32 for the mixed path;
    // the pair entries get their table's device address
    CUDA_TRY(e, e->table.alloc(std::max<size_t>(h_table.size(), 1)));
    CUDA_TRY(e, e->tablef.alloc(std::max<size_t>(h_table.size(), 1)));
    std::vector<float2> h_tablef(h_table.size());
    for (size_t k = 0; k < h_table.size(); k++) h_tablef[k] = make_float2((float)h_table[k].x, (float)h_table[k].y);
    for (PairDev& q : h_ptab)
        if (q.type == PAIR_TABLE) q.table = e->table.p + reinterpret_cast<size_t>(q.table);
    for (PairDevF& q : h_ptabf)
        if (q.type == PAIR_TABLE) q.table = e->tablef.p + reinterpret_cast<size_t>(q.table);
    CUDA_TRY(e, e->posfx.alloc(n));  // fixed-point copy: the mixed path's positions, the plain path's classification
    CUDA_TRY(e, e->nlo.alloc(mixed ? 1 : n));
    CUDA_TRY(e, e->rev.alloc(mixed ? 1 : (size_t)n * maxnb));
    CUDA_TRY(e, e->pf.alloc(mixed ? 1 : (size_t)n * maxnb));
    CUDA_TRY(e, e->perm.alloc(mixed ? n : 1));
    CUDA_TRY(e, e->pfx_build.alloc(mixed ? n : 1));
    CUDA_TRY(e, e->inv_mass.alloc(mixed ? n : 1));
    CUDA_TRY(e, e->km.alloc(mixed ? n : 1));
    CUDA_TRY(e, e->kvecf.alloc(nkv));
    CUDA_TRY(e, e->eikrf.alloc(mixed && nkv ? (size_t)kdim * 3 * n : 1));
    CUDA_TRY(e, e->rhof.alloc(nkv));
    CUDA_TRY(e, e->kvec.alloc(nkv));
    CUDA_TRY(e, e->eikr.alloc(nkv ? (size_t)kdim * 3 * n : 1));
    CUDA_TRY(e, e->rho.alloc(nkv));
    CUDA_TRY(e, e->kred.alloc((size_t)nkv * 7));
    CUDA_TRY(e, e->fpart.alloc(nkv ? (size_t)max_chunks * 3 * n : 1));

    cudaStream_t st = e->stream;
    CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, h_posq.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, h_vel.data(), n * sizeof(double4_32a), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemsetAsync(e->acc.p, 0, n * sizeof(double4_32a), st));
    CUDA_TRY(e, cudaMemsetAsync(e->pos_build.p, 0, n * sizeof(double4_32a), st));
    CUDA_TRY(e, cudaMemcpyAsync(e->kind.p, h_kind.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->mol.p, h_mol.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->sysid.p, h_sysid.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->spec_off.p, h_spec_off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!h_spec_j.empty()) {
        CUDA_TRY(e, cudaMemcpyAsync(e->spec_j.p, h_spec_j.data(), h_spec_j.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->spec_path.p, h_spec_path.data(), h_spec_path.size(),
                                    cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(e, cudaMemcpyAsync(e->bt_off.p, h_bt_off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!h_bt.empty()) {
        CUDA_TRY(e, cudaMemcpyAsync(e->bt.p, h_bt.data(), h_bt.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->bt_role.p, h_bt_role.data(), h_bt_role.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->bt_par.p, h_bt_par.data(), h_bt_par.size() * sizeof(double4_32a),
                                    cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(e, cudaMemsetAsync(e->cell_count.p, 0, cell_total * sizeof(int), st));
    // the cell order starts as the identity (every system rebuilds before its first use)
    std::vector<int> h_iota(n);
    for (int64_t i = 0; i < (int64_t)n; i++) h_iota[i] = (int)i;
    CUDA_TRY(e, cudaMemcpyAsync(e->cell_atoms.p, h_iota.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemsetAsync(e->plan.p, 0, (3 + 3 * (size_t)nsys) * sizeof(int), st));
    std::vector<float> h_inv_mass;
    if (mixed) {
        CUDA_TRY(e, cudaMemcpyAsync(e->perm.p, h_iota.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemsetAsync(e->pfx_build.p, 0, n * sizeof(uint4), st));
        h_inv_mass.resize(n);
        for (int64_t i = 0; i < (int64_t)n; i++) h_inv_mass[i] = (float)(1.0 / h_vel[i].w);
        CUDA_TRY(e, cudaMemcpyAsync(e->inv_mass.p, h_inv_mass.data(), n * sizeof(float), cudaMemcpyHostToDevice,
                                    st));
    }
    CUDA_TRY(e, cudaMemsetAsync(e->nnb.p, 0, n * sizeof(int), st));
    if (!mixed) CUDA_TRY(e, cudaMemsetAsync(e->nlo.p, 0, n * sizeof(int), st));
    CUDA_TRY(e, cudaMemcpyAsync(e->sysdev.p, e->h_sysdev.data(), nsys * sizeof(SysDev), cudaMemcpyHostToDevice, st));
    if (!h_tiles.empty())
        CUDA_TRY(e, cudaMemcpyAsync(e->tiles.p, h_tiles.data(), h_tiles.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                    st));
    CUDA_TRY(e, cudaMemsetAsync(e->kepart.p, 0, std::max<size_t>(n, 1) * sizeof(double), st));
    CUDA_TRY(e, cudaMemsetAsync(e->mom.p, 0, std::max<size_t>(3 * n, 1) * sizeof(double), st));
    CUDA_TRY(e, cudaMemsetAsync(e->md_count.p, 0, std::max(nsys, 1) * sizeof(unsigned long long), st));
    CUDA_TRY(e, cudaMemcpyAsync(e->mol_start.p, h_mol_start.data(), h_mol_start.size() * sizeof(int),
                                cudaMemcpyHostToDevice, st));
    if (!h_table.empty()) {
        CUDA_TRY(e, cudaMemcpyAsync(e->table.p, h_table.data(), h_table.size() * sizeof(double2),
                                    cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->tablef.p, h_tablef.data(), h_tablef.size() * sizeof(float2),
                                    cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(e, cudaMemcpyAsync(e->ptab.p, h_ptab.data(), h_ptab.size() * sizeof(PairDev), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->ptabf.p, h_ptabf.data(), h_ptabf.size() * sizeof(PairDevF), cudaMemcpyHostToDevice,
                                st));
    if (nkv)
        CUDA_TRY(e, cudaMemcpyAsync(e->kvecf.p, h_kvecf.data(), nkv * sizeof(KVecF), cudaMemcpyHostToDevice, st));
    if (nkv)
        CUDA_TRY(e, cudaMemcpyAsync(e->kvec.p, h_kvec.data(), nkv * sizeof(KVecDev), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->host_const.p, h_const.data(), h_const.size() * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    uint32_t st_init = ST_REBUILD;
    CUDA_TRY(e, cudaMemcpyAsync(e->status.p, &st_init, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    std::vector<uint32_t> all_rebuild(nsys, 1u);
    CUDA_TRY(e, cudaMemcpyAsync(e->sys_rebuild.p, all_rebuild.data(), nsys * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                st));
    CUDA_TRY(e, cudaStreamSynchronize(st));

    if (e->h_out) cudaFreeHost(e->h_out);
    e->h_out = nullptr;
    CUDA_TRY(e, cudaMallocHost((void**)&e->h_out, (size_t)nsys * RED_STRIDE * sizeof(double)));

    Batch& b = e->b;
    b = Batch{};
    b.n = (int)n;
    b.nsys = nsys;
    b.precision = e->opt.precision;
    b.posq = e->posq.p;
    b.vel = e->vel.p;
    b.acc = e->acc.p;
    b.force = e->force.p;
    b.kind = e->kind.p;
    b.mol = e->mol.p;
    b.sysid = e->sysid.p;
    b.sys = e->sysdev.p;
    b.ptab = e->ptab.p;
    b.spec_off = e->spec_off.p;
    b.spec_j = e->spec_j.p;
    b.spec_path = e->spec_path.p;
    b.bt_off = h_bt.empty() ? nullptr : e->bt_off.p;
    b.bt = e->bt.p;
    b.bt_role = e->bt_role.p;
    b.bt_par = e->bt_par.p;
    b.maxnb = maxnb;
    b.ncells = cell_total;
    b.nbr = e->nbr.p;
    b.nnb = e->nnb.p;
    b.atom_cell = e->atom_cell.p;
    b.cell_count = e->cell_count.p;
    b.cell_start = e->cell_start.p;
    b.cell_atoms = e->cell_atoms.p;
    b.plan = e->plan.p;
    CUDA_TRY(e, cudaDeviceGetAttribute(&b.sms, cudaDevAttrMultiProcessorCount, e->opt.device));
    b.perm = mixed ? e->perm.p : nullptr;
    b.km = mixed ? e->km.p : nullptr;
    b.wpos = e->wpos.p;
    b.pos_build = e->pos_build.p;
    b.status = e->status.p;
    b.sys_rebuild = e->sys_rebuild.p;
    b.nkvec = nkv;
    b.kdim = kdim;
    b.kchunk = kchunk;
    b.nkchunks = nkchunks;
    b.kvec = e->kvec.p;
    b.eikr = e->eikr.p;
    b.rho = e->rho.p;
    b.fpart = e->fpart.p;
    b.kred = e->kred.p;
    b.red = e->red.p;
    b.host_const = e->host_const.p;
    b.ntiles = (int)h_tiles.size();
    b.tiles = e->tiles.p;
    b.kepart = e->kepart.p;
    b.mom = e->mom.p;
    b.md_count = e->md_count.p;
    b.adj = e->adj.p;
    b.nmol = (int)h_mol_start.size() - 1;
    b.mol_start = e->mol_start.p;
    if (e->h_mc.size() != (size_t)nsys) e->h_mc.assign(nsys, McState{});
    CUDA_TRY(e, e->mc_chains.alloc(nsys));
    CUDA_TRY(e, cudaMemcpy(e->mc_chains.p, e->h_mc.data(), nsys * sizeof(McState), cudaMemcpyHostToDevice));
    e->mc_energies_ready = false;
    b.tpa = e->opt.threads_per_atom ? e->opt.threads_per_atom : (mixed ? 8 : 32);
    b.posfx = e->posfx.p;
    b.nlo = mixed ? nullptr : e->nlo.p;
    b.rev = mixed ? nullptr : e->rev.p;
    b.pf = mixed ? nullptr : e->pf.p;
    b.pfx_build = mixed ? e->pfx_build.p : nullptr;
    b.inv_mass = mixed ? e->inv_mass.p : nullptr;
    b.ptabf = e->ptabf.p;
    // the pairs-only variant of the mixed pair kernel when nothing needs restrictions or Coulomb
    b.pair_general = 0;
    for (const PairDevF& q : h_ptabf) b.pair_general |= (q.type != 0 && q.restriction != 0) ? 1 : 0;
    for (int s = 0; s < nsys; s++) b.pair_general |= e->h_sysdev[s].coul != 0 ? 1 : 0;
    b.kvecf = e->kvecf.p;
    b.eikrf = e->eikrf.p;
    b.rhof = e->rhof.p;
    e->dirty = false;
    e->tuned = false;
    e->pk_cluster = 0;
    return LG_OK;
}

// Regrows the neighbour list after an overflow.
int regrow(lg_engine* e) {
    int maxnb = e->b.maxnb * 3 / 2;
    maxnb = (maxnb + 31) / 32 * 32;
    CUDA_TRY(e, e->nbr.alloc((size_t)e->b.n * maxnb));
    e->b.maxnb = maxnb;
    e->b.nbr = e->nbr.p;
    if (e->b.pf) {
        CUDA_TRY(e, e->rev.alloc((size_t)e->b.n * maxnb));
        CUDA_TRY(e, e->pf.alloc((size_t)e->b.n * maxnb));
        e->b.rev = e->rev.p;
        e->b.pf = e->pf.p;
    }
    launch_request_rebuild(e->b, e->stream);
    e->drop_graphs();
    return LG_OK;
}

int read_status(lg_engine* e, uint32_t* out) {
    CUDA_TRY(e, cudaMemcpyAsync(e->h_status, e->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    *out = *e->h_status;
    return LG_OK;
}

int clear_status_bits(lg_engine* e, uint32_t bits) {
    uint32_t v = *e->h_status & ~bits;
    *e->h_status = v;
    CUDA_TRY(e, cudaMemcpyAsync(e->status.p, e->h_status, sizeof(uint32_t), cudaMemcpyHostToDevice, e->stream));
    return LG_OK;
}

// Kernels launch_nlist_build enqueues.
int nlist_launches(const Batch& b) { return b.n ? (b.perm ? 8 : 9) : 0; }

// Forces (and energies / virials) of the whole batch at the positions in posq.
// The pair kernel assigns the forces, the other force kernels add to them.
// In an MD step vv_first has already written the mixed path's fixed-point
// positions (fixed_written).
void enqueue_forces(lg_engine* e, uint32_t terms, bool ev, cudaStream_t st, bool fixed_written = false) {
    const Batch& b = e->b;
    if (b.n == 0) return;
    launch_nlist_build(b, st);
    e->launches += nlist_launches(b);
    if (!fixed_written) {  // fixed-point copy (mixed: in the order of the list)
        launch_split_positions(b, st);
        e->launches += 1;
    }
    if (terms & (LG_TERM_PAIRS | LG_TERM_COUL_REAL)) {
        launch_pair_forces(b, terms, ev, st);
        e->launches += b.precision == LG_PRECISION_MIXED ? 1 : 2;
    } else {
        cudaMemsetAsync(e->force.p, 0, 3 * (size_t)b.n * sizeof(double), st);
    }
    if ((terms & (LG_TERM_BONDS | LG_TERM_ANGLES | LG_TERM_DIHEDRALS)) && b.bt_off) {
        launch_bonded(b, terms, ev, st);
        e->launches += 1;
    }
    if ((terms & LG_TERM_COUL_KSPACE) && b.nkvec) {
        launch_kspace(b, true, ev, st);
        e->launches += 4;
    }
}

int compute_batch(lg_engine* e, uint32_t terms, uint32_t want, double* d_force_out, double* d_out) {
    bool ev = (want & (LG_WANT_ENERGY | LG_WANT_VIRIAL)) != 0;
    cudaStream_t st = e->stream;
    for (int attempt = 0; attempt < 4; attempt++) {
        launch_check_displacement(e->b, st);
        e->launches += e->b.n ? 1 : 0;
        if (ev) CUDA_TRY(e, cudaMemsetAsync(e->red.p, 0, (size_t)e->b.n * RED_STRIDE * sizeof(double), st));
        enqueue_forces(e, terms, ev, st);
        if (ev) {
            launch_reduce(e->b, terms, (terms & LG_TERM_COUL_KSPACE) && e->b.nkvec, e->out.p, st);
            e->launches += 1;
        }
        CUDA_TRY(e, cudaGetLastError());
        uint32_t status;
        int rc = read_status(e, &status);
        if (rc) return rc;
        if (status & ST_OVERFLOW) {
            rc = clear_status_bits(e, ST_OVERFLOW);
            if (rc) return rc;
            rc = regrow(e);
            if (rc) return rc;
            continue;
        }
        if (status & ST_NONFINITE) {
            clear_status_bits(e, ST_NONFINITE);
            return fail(e, LG_ERR_NONFINITE, "Potential energy is infinite!");
        }
        if (d_force_out)
            CUDA_TRY(e, cudaMemcpyAsync(d_force_out, e->force.p, 3 * (size_t)e->b.n * sizeof(double),
                                        cudaMemcpyDeviceToDevice, st));
        (void)d_out;
        return LG_OK;
    }
    return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
}

// The device address of a page-locked host buffer (cudaHostAlloc /
// cudaHostRegister memory is mapped into the device's address space under
// unified addressing), or null for pageable memory.  The pack / unpack kernels
// read and write such buffers over the host link directly, which fuses the
// host <-> device transfer with the change of layout.
const void* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Host positions and velocities (3 n doubles each) of atoms [base, base + n)
// into the packed device state: read in place from page-locked buffers, else
// staged through pos3 / vel3.
int put_state(lg_engine* e, int64_t base, int64_t n, const double* positions, const double* velocities) {
    cudaStream_t st = e->stream;
    Batch sub = e->b;
    sub.n = (int)n;
    sub.posq = e->posq.p + base;
    sub.vel = e->vel.p + base;
    const double* dp = (const double*)mapped_host(positions);
    const double* dv = (const double*)mapped_host(velocities);
    if (!dp) {
        CUDA_TRY(e, cudaMemcpyAsync(e->pos3.p + 3 * base, positions, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
        dp = e->pos3.p + 3 * base;
    }
    if (!dv) {
        CUDA_TRY(e, cudaMemcpyAsync(e->vel3.p + 3 * base, velocities, 3 * n * sizeof(double), cudaMemcpyHostToDevice,
                                    st));
        dv = e->vel3.p + 3 * base;
    }
    launch_pack_positions(sub, dp, st);
    launch_pack_velocities(sub, dv, st);
    e->launches += 2;
    return LG_OK;
}

// The packed device state of atoms [base, base + n) into host positions and
// velocities (either may be null): written in place into page-locked buffers,
// else staged through pos3 / vel3.
int get_state(lg_engine* e, int64_t base, int64_t n, double* positions, double* velocities) {
    cudaStream_t st = e->stream;
    Batch sub = e->b;
    sub.n = (int)n;
    sub.posq = e->posq.p + base;
    sub.vel = e->vel.p + base;
    if (positions) {
        double* dp = (double*)mapped_host(positions);
        launch_unpack_positions(sub, dp ? dp : e->pos3.p + 3 * base, st);
        e->launches += 1;
        if (!dp)
            CUDA_TRY(e, cudaMemcpyAsync(positions, e->pos3.p + 3 * base, 3 * n * sizeof(double),
                                        cudaMemcpyDeviceToHost, st));
    }
    if (velocities) {
        double* dv = (double*)mapped_host(velocities);
        launch_unpack_velocities(sub, dv ? dv : e->vel3.p + 3 * base, st);
        e->launches += 1;
        if (!dv)
            CUDA_TRY(e, cudaMemcpyAsync(velocities, e->vel3.p + 3 * base, 3 * n * sizeof(double),
                                        cudaMemcpyDeviceToHost, st));
    }
    return LG_OK;
}

// Copies the host positions of system s into its slice of the device state;
// the other systems keep theirs.
int upload_positions(lg_engine* e, int32_t s, const double* positions) {
    const HostSystem& h = e->sys[s];
    if (h.n == 0) return LG_OK;
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    CUDA_TRY(e, cudaMemcpyAsync(e->pos3.p + 3 * base, positions, 3 * h.n * sizeof(double), cudaMemcpyHostToDevice,
                                st));
    Batch sub = e->b;
    sub.n = (int)h.n;
    sub.posq = e->posq.p + base;
    launch_pack_positions(sub, e->pos3.p + 3 * base, st);
    e->launches += 1;
    return LG_OK;
}

int check_pair_cutoffs(lg_engine* e, const HostSystem& h) {
    if (!h.has_cell) return LG_OK;
    double half = 0.5 * std::min(std::min(h.L[0], h.L[1]), h.L[2]);
    for (const lg_pair& p : h.pairs)
        if (p.type != LG_PAIR_ABSENT && half < p.cutoff)
            return fail(e, LG_ERR_ARGUMENT,
                        "Can not add a potential with a cutoff bigger than half of the smallest cell length. "
                        "Try increasing the cell size or decreasing the cutoff.");
    if (h.coul.kind != LG_COULOMB_NONE && half < h.coul.cutoff)
        return fail(e, LG_ERR_ARGUMENT,
                    "Can not add a potential with a cutoff bigger than half of the smallest cell length. "
                    "Try increasing the cell size or decreasing the cutoff.");
    return LG_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int lg_version(void) { return LG_ABI_VERSION; }

const char* lg_last_error(const lg_engine* e) { return e ? e->err.c_str() : g_create_error.c_str(); }

int lg_create(const lg_options* options, int32_t n_systems, lg_engine** out) {
    if (!out) return fail(nullptr, LG_ERR_ARGUMENT, "null engine pointer");
    *out = nullptr;
    if (n_systems <= 0) return fail(nullptr, LG_ERR_ARGUMENT, "n_systems must be positive");
    lg_options opt{0, LG_PRECISION_FP64, 1.0, 0, 0};
    if (options) opt = *options;
    int t = opt.threads_per_atom;
    if (t != 0 && t != 1 && t != 2 && t != 4 && t != 8 && t != 16 && t != 32)
        return fail(nullptr, LG_ERR_ARGUMENT, "threads_per_atom must be 0, 1, 2, 4, 8, 16 or 32");
    if (opt.precision != LG_PRECISION_FP64 && opt.precision != LG_PRECISION_MIXED)
        return fail(nullptr, LG_ERR_ARGUMENT, "unknown precision");
    if (opt.skin <= 0.0) opt.skin = 1.0;
    int count = 0;
    cudaError_t ce = cudaGetDeviceCount(&count);
    if (ce != cudaSuccess || count == 0)
        return fail(nullptr, LG_ERR_NO_DEVICE,
                    std::string("no CUDA device is visible (") + cudaGetErrorString(ce) +
                        "); the engine has no CPU fallback");
    if (opt.device < 0 || opt.device >= count) return fail(nullptr, LG_ERR_ARGUMENT, "invalid device ordinal");
    ce = cudaSetDevice(opt.device);
    if (ce != cudaSuccess) return fail(nullptr, LG_ERR_CUDA, cudaGetErrorString(ce));
    lg_engine* e = new lg_engine();
    e->opt = opt;
    e->skin = opt.skin;
    e->nsys = n_systems;
    e->sys.resize(n_systems);
    ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&e->h_status, sizeof(uint32_t));
    if (ce != cudaSuccess) {
        delete e;
        return fail(nullptr, LG_ERR_CUDA, cudaGetErrorString(ce));
    }
    *out = e;
    return LG_OK;
}

void lg_destroy(lg_engine* e) {
    if (!e) return;
    cudaSetDevice(e->opt.device);
    cudaStreamSynchronize(e->stream);
    delete e;
}

int lg_set_cell(lg_engine* e, int32_t s, const double m[9]) {
    if (!valid_sys(e, s) || !m) return fail(e, LG_ERR_ARGUMENT, "invalid system index or cell");
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
            if (a != c && m[3 * a + c] != 0.0)
                return fail(e, LG_ERR_ARGUMENT, "only orthorhombic cells are supported");
    if (!(m[0] > 0.0 && m[4] > 0.0 && m[8] > 0.0)) return fail(e, LG_ERR_ARGUMENT, "Cell lengths must be positive");
    HostSystem& h = e->sys[s];
    h.L[0] = m[0];
    h.L[1] = m[4];
    h.L[2] = m[8];
    h.has_cell = true;
    invalidate(e);
    return check_pair_cutoffs(e, h);
}

int lg_set_particles(lg_engine* e, int32_t s, int64_t n, const int32_t* kinds, const double* charges,
                     const double* masses, const int32_t* molecules) {
    if (!valid_sys(e, s) || n < 0 || (n > 0 && (!kinds || !charges || !masses || !molecules)))
        return fail(e, LG_ERR_ARGUMENT, "invalid particles");
    HostSystem& h = e->sys[s];
    h.n = n;
    h.kinds.assign(kinds, kinds + n);
    h.charges.assign(charges, charges + n);
    h.masses.assign(masses, masses + n);
    h.mols.assign(molecules, molecules + n);
    for (int64_t i = 0; i < n; i++) {
        if (h.kinds[i] < 0) return fail(e, LG_ERR_ARGUMENT, "negative kind");
        if (h.mols[i] < 0) return fail(e, LG_ERR_ARGUMENT, "negative molecule index");
        if (!(h.masses[i] > 0.0)) return fail(e, LG_ERR_ARGUMENT, "masses must be positive");
        if (i > 0 && h.mols[i] != h.mols[i - 1] && h.mols[i] != h.mols[i - 1] + 1)
            return fail(e, LG_ERR_ARGUMENT, "molecules must be numbered contiguously in atom order");
    }
    h.md_ready = false;
    invalidate(e);
    return LG_OK;
}

int lg_set_bonds(lg_engine* e, int32_t s, int64_t nb, const int32_t* bonds, const lg_bonded* pots) {
    if (!valid_sys(e, s) || nb < 0 || (nb > 0 && (!bonds || !pots))) return fail(e, LG_ERR_ARGUMENT, "invalid bonds");
    HostSystem& h = e->sys[s];
    for (int64_t b = 0; b < 2 * nb; b++)
        if (bonds[b] < 0 || bonds[b] >= h.n) return fail(e, LG_ERR_ARGUMENT, "bond index out of range");
    for (int64_t b = 0; b < nb; b++) {  // BondPotential: Harmonic, Morse, Null
        int t = pots[b].type;
        if (t != LG_PAIR_ABSENT && t != LG_PAIR_NULL && t != LG_PAIR_HARMONIC && t != LG_PAIR_MORSE)
            return fail(e, LG_ERR_ARGUMENT, "unknown bond potential");
        if (bonds[2 * b] == bonds[2 * b + 1]) return fail(e, LG_ERR_ARGUMENT, "a bond needs two particles");
        if (h.mols[bonds[2 * b]] != h.mols[bonds[2 * b + 1]])
            return fail(e, LG_ERR_ARGUMENT, "bonded particles must be in the same molecule");
    }
    h.bonds.assign(bonds, bonds + 2 * nb);
    h.bond_pots.assign(pots, pots + nb);
    invalidate(e);
    return LG_OK;
}

int lg_set_angles(lg_engine* e, int32_t s, int64_t na, const int32_t* angles, const lg_bonded* pots) {
    if (!valid_sys(e, s) || na < 0 || (na > 0 && (!angles || !pots)))
        return fail(e, LG_ERR_ARGUMENT, "invalid angles");
    HostSystem& h = e->sys[s];
    for (int64_t a = 0; a < 3 * na; a++)
        if (angles[a] < 0 || angles[a] >= h.n) return fail(e, LG_ERR_ARGUMENT, "angle index out of range");
    for (int64_t a = 0; a < na; a++)  // AnglePotential: Harmonic, CosineHarmonic, Morse, Null
        if (pots[a].type != LG_PAIR_ABSENT && pots[a].type != LG_PAIR_NULL && pots[a].type != LG_PAIR_HARMONIC &&
            pots[a].type != LG_BONDED_COSINE_HARMONIC && pots[a].type != LG_PAIR_MORSE)
            return fail(e, LG_ERR_ARGUMENT, "unknown angle potential");
    h.angles.assign(angles, angles + 3 * na);
    h.angle_pots.assign(pots, pots + na);
    invalidate(e);
    return LG_OK;
}

int lg_set_dihedrals(lg_engine* e, int32_t s, int64_t nd, const int32_t* dihedrals, const lg_bonded* pots) {
    if (!valid_sys(e, s) || nd < 0 || (nd > 0 && (!dihedrals || !pots)))
        return fail(e, LG_ERR_ARGUMENT, "invalid dihedrals");
    HostSystem& h = e->sys[s];
    for (int64_t a = 0; a < 4 * nd; a++)
        if (dihedrals[a] < 0 || dihedrals[a] >= h.n)
            return fail(e, LG_ERR_ARGUMENT, "dihedral index out of range");
    for (int64_t a = 0; a < nd; a++) {  // DihedralPotential: Harmonic, CosineHarmonic, Torsion, Morse, Null
        int t = pots[a].type;
        if (t != LG_PAIR_ABSENT && t != LG_PAIR_NULL && t != LG_PAIR_HARMONIC && t != LG_BONDED_COSINE_HARMONIC &&
            t != LG_BONDED_TORSION && t != LG_PAIR_MORSE)
            return fail(e, LG_ERR_ARGUMENT, "unknown dihedral potential");
    }
    h.dihedrals.assign(dihedrals, dihedrals + 4 * nd);
    h.dihedral_pots.assign(pots, pots + nd);
    invalidate(e);
    return LG_OK;
}

int lg_set_pairs(lg_engine* e, int32_t s, int32_t nk, const lg_pair* table) {
    if (!valid_sys(e, s) || nk <= 0 || !table) return fail(e, LG_ERR_ARGUMENT, "invalid pair table");
    HostSystem& h = e->sys[s];
    for (int32_t k : h.kinds)
        if (k >= nk) return fail(e, LG_ERR_ARGUMENT, "a particle kind is outside the pair table");
    for (int a = 0; a < nk; a++)
        for (int c = 0; c < nk; c++) {
            const lg_pair& p = table[a * nk + c];
            const lg_pair& q = table[c * nk + a];
            if (p.type != q.type || p.cutoff != q.cutoff || p.p0 != q.p0 || p.p1 != q.p1 || p.p2 != q.p2 ||
                p.p3 != q.p3 || p.p4 != q.p4 || p.restriction != q.restriction || p.shifted != q.shifted ||
                p.tail != q.tail || p.table_size != q.table_size || p.table_max != q.table_max)
                return fail(e, LG_ERR_ARGUMENT, "the pair table must be symmetric");
            if (p.type != LG_PAIR_ABSENT && (p.table_size < 0 || (p.table_size > 0 && !(p.table_max > 0.0))))
                return fail(e, LG_ERR_ARGUMENT, "a TableComputation needs a positive size and maximum");
            if (p.type < LG_PAIR_ABSENT || p.type > LG_PAIR_MIE)
                return fail(e, LG_ERR_ARGUMENT, "unknown pair potential");
            // the reference's constructors panic on these (functions.rs:468-469, 540-541)
            if (p.type == LG_PAIR_GAUSSIAN && !(p.p1 > 0.0))
                return fail(e, LG_ERR_ARGUMENT, "\"b\" has to be positive in Gaussian potential");
            if (p.type == LG_PAIR_MIE && !(p.p3 < p.p2))
                return fail(e, LG_ERR_ARGUMENT,
                            "The repulsive exponent n has to be larger than the attractive exponent m");
            if (p.type != LG_PAIR_ABSENT && !(p.cutoff >= 0.0))
                return fail(e, LG_ERR_ARGUMENT, "invalid pair cutoff");
        }
    h.nk = nk;
    h.pairs.assign(table, table + (size_t)nk * nk);
    invalidate(e);
    return check_pair_cutoffs(e, h);
}

int lg_set_coulomb(lg_engine* e, int32_t s, const lg_coulomb* c) {
    if (!valid_sys(e, s) || !c) return fail(e, LG_ERR_ARGUMENT, "invalid coulomb descriptor");
    if (c->kind == LG_COULOMB_EWALD) {
        // Ewald::new panics (ewald.rs:281-287)
        if (c->cutoff < 0.0) return fail(e, LG_ERR_ARGUMENT, "the cutoff can not be negative in Ewald");
        if (c->alpha < 0.0) return fail(e, LG_ERR_ARGUMENT, "alpha can not be negative in Ewald");
        if (c->kmax <= 0) return fail(e, LG_ERR_ARGUMENT, "kmax can not be 0 in Ewald");
        if (c->restriction == LG_RESTRICT_SCALE14)
            return fail(e, LG_ERR_ARGUMENT, "Scaling restriction scheme using Ewald are not implemented");
    } else if (c->kind == LG_COULOMB_WOLF) {
        if (!(c->cutoff > 0.0)) return fail(e, LG_ERR_ARGUMENT, "Got a negative cutoff in Wolf summation");
    } else if (c->kind != LG_COULOMB_NONE) {
        return fail(e, LG_ERR_ARGUMENT, "unknown coulomb potential");
    }
    HostSystem& h = e->sys[s];
    h.coul = *c;
    invalidate(e);
    return check_pair_cutoffs(e, h);
}

int lg_compute(lg_engine* e, int32_t s, const double* positions, uint32_t terms, uint32_t want, double* forces,
               double* energy, double virial[9]) {
    if (!valid_sys(e, s) || !positions) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = commit(e);
    if (rc) return rc;
    const HostSystem& h = e->sys[s];
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    rc = upload_positions(e, s, positions);
    if (rc) return rc;
    bool ev = (want & (LG_WANT_ENERGY | LG_WANT_VIRIAL)) != 0;
    rc = compute_batch(e, terms, want, nullptr, nullptr);
    if (rc) return rc;
    std::vector<double> f;
    if ((want & LG_WANT_FORCES) && forces && h.n) {
        f.resize(3 * h.n);
        CUDA_TRY(e, cudaMemcpyAsync(f.data(), e->force.p + 3 * base, 3 * h.n * sizeof(double),
                                    cudaMemcpyDeviceToHost, st));
    }
    if (ev)
        CUDA_TRY(e, cudaMemcpyAsync(e->h_out, e->out.p + (size_t)s * RED_STRIDE, RED_STRIDE * sizeof(double),
                                    cudaMemcpyDeviceToHost, st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    if ((want & LG_WANT_FORCES) && forces)
        for (int64_t i = 0; i < 3 * h.n; i++) forces[i] += f[i];
    if ((want & LG_WANT_ENERGY) && energy) *energy = e->h_out[0];
    if ((want & LG_WANT_VIRIAL) && virial)
        for (int c = 0; c < 9; c++) virial[c] = e->h_out[1 + c];
    return LG_OK;
}

int lg_molecular_virial(lg_engine* e, int32_t s, const double* positions, uint32_t terms, double virial[9]) {
    if (!valid_sys(e, s) || !positions || !virial) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->opt.precision != LG_PRECISION_FP64)
        return fail(e, LG_ERR_ARGUMENT, "the molecular virial is computed by fp64 engines");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = commit(e);
    if (rc) return rc;
    cudaStream_t st = e->stream;
    rc = upload_positions(e, s, positions);
    if (rc) return rc;
    // the k-space forces (and the list for the current positions)
    bool kspace = (terms & LG_TERM_COUL_KSPACE) && e->b.nkvec;
    rc = compute_batch(e, terms & LG_TERM_COUL_KSPACE, LG_WANT_FORCES | LG_WANT_VIRIAL, nullptr, nullptr);
    if (rc) return rc;
    if (e->molcom.n < (size_t)e->b.n) CUDA_TRY(e, e->molcom.alloc(e->b.n));
    CUDA_TRY(e, cudaMemsetAsync(e->red.p, 0, (size_t)e->b.n * RED_STRIDE * sizeof(double), st));
    launch_molecular_virial(e->b, terms & (LG_TERM_PAIRS | LG_TERM_COUL_REAL), e->molcom.p,
                            kspace ? e->force.p : nullptr, st);
    launch_reduce(e->b, terms & (LG_TERM_PAIRS | LG_TERM_TAIL | LG_TERM_COUL_REAL | LG_TERM_COUL_KSPACE), kspace,
                  e->out.p, st);
    e->launches += 3;
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaMemcpyAsync(e->h_out, e->out.p + (size_t)s * RED_STRIDE, RED_STRIDE * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    for (int c = 0; c < 9; c++) virial[c] = e->h_out[1 + c];
    return LG_OK;
}

int lg_compute_device(lg_engine* e, const double* d_positions, uint32_t terms, uint32_t want, double* d_forces,
                      double* d_energy, double* d_virial, void* stream) {
    if (!e || !d_positions) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = commit(e);
    if (rc) return rc;
    cudaStream_t user = stream ? (cudaStream_t)stream : e->stream;
    cudaStream_t st = e->stream;
    if (user != st) {
        cudaEvent_t ev;
        CUDA_TRY(e, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaEventRecord(ev, user);
        cudaStreamWaitEvent(st, ev, 0);
        cudaEventDestroy(ev);
    }
    launch_pack_positions(e->b, d_positions, st);
    rc = compute_batch(e, terms, want, (want & LG_WANT_FORCES) ? d_forces : nullptr, nullptr);
    if (rc) return rc;
    bool ev = (want & (LG_WANT_ENERGY | LG_WANT_VIRIAL)) != 0;
    if (ev) {
        for (int s = 0; s < e->nsys; s++) {
            if (d_energy && (want & LG_WANT_ENERGY))
                CUDA_TRY(e, cudaMemcpyAsync(d_energy + s, e->out.p + (size_t)s * RED_STRIDE, sizeof(double),
                                            cudaMemcpyDeviceToDevice, st));
            if (d_virial && (want & LG_WANT_VIRIAL))
                CUDA_TRY(e, cudaMemcpyAsync(d_virial + 9 * s, e->out.p + (size_t)s * RED_STRIDE + 1,
                                            9 * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
    }
    if (user != st) {
        cudaEvent_t ev2;
        CUDA_TRY(e, cudaEventCreateWithFlags(&ev2, cudaEventDisableTiming));
        cudaEventRecord(ev2, st);
        cudaStreamWaitEvent(user, ev2, 0);
        cudaEventDestroy(ev2);
    }
    return LG_OK;
}

int lg_pairset(lg_engine* e, int32_t s, const double* positions, int32_t family, int32_t* pairs, int64_t capacity,
               int64_t* count) {
    if (!valid_sys(e, s) || !positions || !count || (family != 0 && family != 1) || capacity < 0)
        return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = commit(e);
    if (rc) return rc;
    const HostSystem& h = e->sys[s];
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    rc = upload_positions(e, s, positions);
    if (rc) return rc;
    // make sure the list is current (and large enough) for these positions
    rc = compute_batch(e, LG_TERM_PAIRS | LG_TERM_COUL_REAL, LG_WANT_FORCES, nullptr, nullptr);
    if (rc) return rc;
    size_t cap = (size_t)std::max<int64_t>(capacity, 1);
    CUDA_TRY(e, e->pairs_out.alloc(2 * cap));
    CUDA_TRY(e, e->pairs_count.alloc(1));
    CUDA_TRY(e, cudaMemsetAsync(e->pairs_count.p, 0, sizeof(unsigned long long), st));
    launch_pairset(e->b, family, (int)base, (int)(base + h.n), e->pairs_out.p, capacity, e->pairs_count.p, st);
    CUDA_TRY(e, cudaGetLastError());
    unsigned long long total = 0;
    CUDA_TRY(e, cudaMemcpyAsync(&total, e->pairs_count.p, sizeof(total), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    size_t got = std::min<size_t>(total, (size_t)capacity);
    if (got && pairs) {
        std::vector<int32_t> tmp(2 * got);
        CUDA_TRY(e, cudaMemcpy(tmp.data(), e->pairs_out.p, 2 * got * sizeof(int32_t), cudaMemcpyDeviceToHost));
        std::vector<std::pair<int32_t, int32_t>> v(got);
        for (size_t k = 0; k < got; k++) v[k] = {tmp[2 * k], tmp[2 * k + 1]};
        std::sort(v.begin(), v.end());
        for (size_t k = 0; k < got; k++) {
            pairs[2 * k] = v[k].first;
            pairs[2 * k + 1] = v[k].second;
        }
    }
    *count = (int64_t)total;
    return LG_OK;
}

// ---- molecular dynamics -----------------------------------------------------
int lg_md_setup(lg_engine* e, int32_t s, double dt, double T0, double tau) {
    lg_md_params p{};
    p.integrator = LG_INTEGRATOR_VELOCITY_VERLET;
    p.thermostat = tau > 0.0 ? LG_THERMOSTAT_BERENDSEN : LG_THERMOSTAT_NONE;
    p.timestep = dt;
    p.temperature = T0;
    p.tau = tau;
    return lg_md_setup_ex(e, s, &p);
}

int lg_md_setup_ex(lg_engine* e, int32_t s, const lg_md_params* p) {
    if (!valid_sys(e, s) || !p) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (!(p->timestep > 0.0)) return fail(e, LG_ERR_ARGUMENT, "invalid timestep");
    if (p->integrator < LG_INTEGRATOR_VELOCITY_VERLET || p->integrator > LG_INTEGRATOR_LEAP_FROG)
        return fail(e, LG_ERR_ARGUMENT, "unknown integrator");
    if (p->thermostat < LG_THERMOSTAT_NONE || p->thermostat > LG_THERMOSTAT_CSVR)
        return fail(e, LG_ERR_ARGUMENT, "unknown thermostat");
    if (p->controls & ~(LG_CONTROL_REMOVE_TRANSLATION | LG_CONTROL_REWRAP | LG_CONTROL_REMOVE_ROTATION))
        return fail(e, LG_ERR_ARGUMENT, "unknown control");
    // the constructors' checks: RescaleThermostat::new, BerendsenThermostat::new,
    // CSVRThermostat::from_rng (thermostats.rs:48-53, 102-109, 151-160)
    if (p->thermostat != LG_THERMOSTAT_NONE && p->temperature < 0.0)
        return fail(e, LG_ERR_ARGUMENT, "The temperature must be positive in thermostats.");
    if (p->thermostat == LG_THERMOSTAT_BERENDSEN && !(p->tau >= 1.0))
        return fail(e, LG_ERR_ARGUMENT, "The timestep must be larger than 1 in berendsen thermostat.");
    if (p->thermostat == LG_THERMOSTAT_CSVR && !(p->tau >= 1.0))
        return fail(e, LG_ERR_ARGUMENT, "The timestep must be larger than 1 in CSVR thermostat.");
    HostSystem& h = e->sys[s];
    h.dt = p->timestep;
    h.integrator = p->integrator;
    h.thermostat = p->thermostat;
    h.T0 = p->temperature;
    h.tau = (p->thermostat == LG_THERMOSTAT_BERENDSEN || p->thermostat == LG_THERMOSTAT_CSVR) ? p->tau : 0.0;
    h.tol = p->tolerance;
    h.seed = p->seed;
    h.controls = p->controls;
    h.md_ready = true;
    h.verlet_setup = p->integrator == LG_INTEGRATOR_VERLET;
    if (!e->dirty) {
        SysDev& d = e->h_sysdev[s];
        fill_md(d, h);
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        CUDA_TRY(e, cudaMemcpyAsync(e->sysdev.p + s, &d, sizeof(SysDev), cudaMemcpyHostToDevice, e->stream));
        // VelocityVerlet / LeapFrog::setup: accelerations := 0 (integrators.rs:40-42, 146-148);
        // Verlet's previous positions are taken at the next run
        if (p->integrator != LG_INTEGRATOR_VERLET)
            CUDA_TRY(e, cudaMemsetAsync(e->acc.p + e->begin[s], 0, h.n * sizeof(double4_32a), e->stream));
        CUDA_TRY(e, cudaMemsetAsync(e->md_count.p + s, 0, sizeof(unsigned long long), e->stream));
        CUDA_TRY(e, cudaStreamSynchronize(e->stream));
        e->drop_graphs();
    }
    return LG_OK;
}

int lg_md_set_state(lg_engine* e, int32_t s, const double* positions, const double* velocities) {
    if (!valid_sys(e, s) || !positions || !velocities) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    bool was_dirty = e->dirty;
    int rc = commit(e);
    if (rc) return rc;
    const HostSystem& h = e->sys[s];
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    if (h.n == 0) return LG_OK;
    rc = put_state(e, base, h.n, positions, velocities);  // this system's atoms only
    if (rc) return rc;
    if (was_dirty) CUDA_TRY(e, cudaMemsetAsync(e->acc.p, 0, e->b.n * sizeof(double4_32a), st));
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_md_get_state(lg_engine* e, int32_t s, double* positions, double* velocities) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state: call lg_md_set_state first");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    const HostSystem& h = e->sys[s];
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    if (h.n == 0) return LG_OK;
    int rc = get_state(e, base, h.n, positions, velocities);
    if (rc) return rc;
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

}  // extern "C"

namespace {

bool persist_batch(const lg_engine* e);

// The autotuner: times the pair kernel at every threads-per-atom width (2, 4
// and 8 for a batch the persistent kernel runs) and the
// Ewald field kernel at several chunk lengths on the current batch and list,
// keeps the fastest, and caches the choice for this workload shape.
int autotune(lg_engine* e) {
    if (e->tuned || e->b.n == 0) return LG_OK;
    if (e->opt.threads_per_atom) {  // fixed by the caller
        e->tuned = true;
        return LG_OK;
    }
    Batch& b = e->b;
    auto key = std::make_tuple(e->opt.device, b.precision, b.n, b.maxnb, b.nkvec, persist_batch(e));
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            b.tpa = it->second.first;
            b.kchunk = it->second.second;
            b.nkchunks = (e->max_nk + b.kchunk - 1) / b.kchunk;
            e->tuned = true;
            return LG_OK;
        }
    }
    cudaStream_t st = e->stream;
    cudaEvent_t e0, e1;
    CUDA_TRY(e, cudaEventCreate(&e0));
    CUDA_TRY(e, cudaEventCreate(&e1));
    // a current list for the timing
    launch_check_displacement(b, st);
    launch_nlist_build(b, st);
    launch_split_positions(b, st);
    auto time_it = [&](auto&& launch) -> float {
        launch();  // warm
        float best = 1e30f;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0, st);
            launch();
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::min(best, ms);
        }
        return best;
    };
    // (a batch for the persistent kernel: the group sizes it runs)
    const int tpas_all[6] = {1, 2, 4, 8, 16, 32}, tpas_persist[3] = {2, 4, 8};
    const bool pb = std::get<5>(key);
    const int* tpas = pb ? tpas_persist : tpas_all;
    const int ntpas = pb ? 3 : 6;
    int best_tpa = b.tpa;
    float best_t = 1e30f;
    for (int k = 0; k < ntpas; k++) {
        int t = tpas[k];
        b.tpa = t;
        float ms = time_it([&] { launch_pair_forces(b, LG_TERM_ALL, false, st); });
        if (ms < best_t) {
            best_t = ms;
            best_tpa = t;
        }
    }
    b.tpa = best_tpa;
    if (b.nkvec) {
        launch_kspace_part(b, 0, false, st);
        launch_kspace_part(b, 1, false, st);
        const int chunks[4] = {MIN_KCHUNK, 16, 32, 64};
        int best_c = b.kchunk;
        best_t = 1e30f;
        for (int kc : chunks) {
            b.kchunk = kc;
            b.nkchunks = (e->max_nk + kc - 1) / kc;
            float ms = time_it([&] { launch_kspace_part(b, 2, false, st); });
            if (ms < best_t) {
                best_t = ms;
                best_c = kc;
            }
        }
        b.kchunk = best_c;
        b.nkchunks = (e->max_nk + best_c - 1) / best_c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = {b.tpa, b.kchunk};
    }
    e->tuned = true;
    e->drop_graphs();
    return LG_OK;
}

// What the MD steps of a batch need besides the integrators: a thermostat or
// control (MD_ADJUST), Rewrap (MD_REWRAP), a Verlet system (MD_VERLET_SYS:
// its positions move after the forces, so the fixed-point copies are taken
// before each force evaluation).
constexpr int MD_ADJUST = 1, MD_REWRAP = 2, MD_VERLET_SYS = 4;
int md_mode(const lg_engine* e) {
    int mode = 0;
    for (int s = 0; s < e->nsys; s++) {
        const HostSystem& h = e->sys[s];
        if (h.thermostat != LG_THERMOSTAT_NONE || h.controls) mode |= MD_ADJUST;
        if (h.controls & LG_CONTROL_REWRAP) mode |= MD_REWRAP;
        if (h.integrator == LG_INTEGRATOR_VERLET) mode |= MD_VERLET_SYS;
    }
    return mode;
}

// One MD step of every system.  The thermostat and controls of the previous
// step are applied by this step's md_first (apply_previous; Rewrap by a kernel
// before it), and the last step of a run is followed by launch_md_finalize.
void enqueue_md_step(lg_engine* e, int mode, bool apply_previous, cudaStream_t st) {
    bool adjust = (mode & MD_ADJUST) && apply_previous;
    if (adjust && (mode & MD_REWRAP)) {
        launch_rewrap(e->b, st);
        e->launches += e->b.nmol ? 1 : 0;
    }
    launch_md_first(e->b, adjust, st);
    enqueue_forces(e, LG_TERM_ALL, false, st, !(mode & MD_VERLET_SYS));
    launch_md_second(e->b, st);
    e->launches += e->b.ntiles ? 2 : 0;
    if (mode & MD_ADJUST) {  // this step's thermostat factor and controls, per system
        launch_md_adjust(e->b, st);
        e->launches += 1;
    }
}

// The pending thermostat and controls at the end of a run.
void enqueue_md_finish(lg_engine* e, int mode, cudaStream_t st) {
    if (!(mode & MD_ADJUST)) return;
    launch_md_finalize(e->b, st);
    e->launches += e->b.ntiles ? 1 : 0;
    if (mode & MD_REWRAP) {
        launch_rewrap(e->b, st);
        e->launches += e->b.nmol ? 1 : 0;
    }
}

// ---- persistent batched MD -------------------------------------------------------
// A batch the persistent kernel can run: mixed precision, pair potentials
// only, Velocity-Verlet with at most a Berendsen thermostat.  It also needs a group size of 2, 4 or 8 threads per atom (the
// per-step kernel's, so both paths sum every force in the same order).
bool persist_batch(const lg_engine* e) {
    const Batch& b = e->b;
    if ((e->opt.flags & LG_OPT_NO_PERSISTENT) || b.precision != LG_PRECISION_MIXED || b.pair_general || b.bt_off ||
        b.nkvec != 0 || b.n == 0)
        return false;
    for (int s = 0; s < e->nsys; s++) {  // VelocityVerlet, no thermostat or Berendsen, no control
        const HostSystem& h = e->sys[s];
        if (h.integrator != LG_INTEGRATOR_VELOCITY_VERLET || h.controls ||
            (h.thermostat != LG_THERMOSTAT_NONE && h.thermostat != LG_THERMOSTAT_BERENDSEN))
            return false;
    }
    return true;
}
bool persist_eligible(const lg_engine* e) {
    int t = e->b.tpa;
    return persist_batch(e) && (t == 2 || t == 4 || t == 8);
}

// Packs the systems into groups of about equal work (atoms times the expected
// neighbour count; longest first, each to the least loaded group) for each
// cluster size the device can hold, and keeps the size whose largest group
// per block is smallest.  A system's arithmetic does not depend on its group.
int persist_plan(lg_engine* e) {
    e->pk_cluster = -1;
    const Batch& b = e->b;
    int nsys = e->nsys;
    // work of a system: its neighbour-list entries (measured when the lists
    // exist, else estimated from the density) plus a per-atom share
    std::vector<int> h_nnb(b.n);
    CUDA_TRY(e, cudaMemcpy(h_nnb.data(), e->nnb.p, (size_t)b.n * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<double> work(nsys);
    for (int s = 0; s < nsys; s++) {
        const HostSystem& h = e->sys[s];
        double V = h.L[0] * h.L[1] * h.L[2];
        double rl = e->h_sysdev[s].rlist;
        double entries = 0.0;
        for (int64_t i = e->begin[s]; i < e->begin[s + 1]; i++) entries += h_nnb[i];
        if (entries == 0.0) entries = (double)h.n * (double)h.n / V * 4.0 / 3.0 * PI * rl * rl * rl;
        work[s] = entries + 8.0 * (double)h.n;
    }
    std::vector<int> order(nsys);
    for (int s = 0; s < nsys; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
    double best_t = 0.0;
    int best_c = 0;
    std::vector<std::vector<int>> best_bins;
    int forced = (e->opt.flags >> LG_OPT_CLUSTER_SHIFT) & 0xf;
    for (int C : {1, 2, 4, 8}) {
        if (forced && C != (1 << (forced - 1))) continue;
        int gmax = persist_max_clusters(b.tpa, C, PK_STAGE_MAX);
        if (gmax <= 0) continue;
        int G = std::max(std::min(gmax, nsys), (nsys + PK_MAXG - 1) / PK_MAXG);
        std::vector<std::vector<int>> bins(G);
        std::vector<double> load(G, 0.0);
        for (int s : order) {
            int pick = -1;
            for (int g = 0; g < G; g++)
                if ((int)bins[g].size() < PK_MAXG && (pick < 0 || load[g] < load[pick])) pick = g;
            bins[pick].push_back(s);
            load[pick] += work[s];
        }
        double waves = std::ceil((double)G / (double)gmax);
        double t = *std::max_element(load.begin(), load.end()) / C * waves;
        if (best_c == 0 || t < 0.97 * best_t) {
            best_t = t;
            best_c = C;
            best_bins = bins;
        }
    }
    if (best_c == 0) return LG_OK;  // no cluster fits: the per-step kernels run
    std::vector<int> off(1, 0), sys;
    for (auto& bin : best_bins) {
        if (bin.empty()) continue;
        std::sort(bin.begin(), bin.end());
        sys.insert(sys.end(), bin.begin(), bin.end());
        off.push_back((int)sys.size());
    }
    int G = (int)off.size() - 1;
    // the largest group's atoms, staged in shared memory when they fit
    int stage = 0;
    for (int g = 0; g < G; g++) {
        int atoms = 0;
        for (int k = off[g]; k < off[g + 1]; k++) atoms += (int)e->sys[sys[k]].n;
        stage = std::max(stage, atoms);
    }
    e->pk_stage = (stage <= PK_STAGE_MAX && (e->opt.flags & LG_OPT_STAGING)) ? stage : 0;
    cudaStream_t st = e->stream;
    CUDA_TRY(e, e->pk_group_off.alloc(off.size()));
    CUDA_TRY(e, e->pk_group_sys.alloc(sys.size()));
    CUDA_TRY(e, e->pk_group_flag.alloc(G));
    CUDA_TRY(e, e->pk_ke.alloc(b.n));
    CUDA_TRY(e, cudaMemcpyAsync(e->pk_group_off.p, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->pk_group_sys.p, sys.data(), sys.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    e->pk_groups = G;
    e->pk_cluster = best_c;
    return LG_OK;
}

// lg_md_run on the persistent kernel: one launch per chunk, with the same
// checkpoint / regrow / replay on a list overflow as the per-step path.
int md_run_persistent(lg_engine* e, int64_t nsteps, bool thermo) {
    const int chunk = 32;
    cudaStream_t st = e->stream;
    int64_t done = 0;
    int retries = 0;
    size_t bytes = e->b.n * sizeof(double4_32a);
    while (done < nsteps) {
        int steps = (int)std::min<int64_t>(chunk, nsteps - done);
        int key = 2 * steps + (thermo ? 1 : 0);
        auto it = e->pk_graphs.find(key);
        if (it == e->pk_graphs.end()) {
            cudaGraph_t g;
            CUDA_TRY(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            cudaMemcpyAsync(e->cp_pos.p, e->posq.p, bytes, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(e->cp_vel.p, e->vel.p, bytes, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(e->cp_acc.p, e->acc.p, bytes, cudaMemcpyDeviceToDevice, st);
            cudaMemsetAsync(e->pk_group_flag.p, 0, e->pk_groups * sizeof(int), st);
            PkArgs a{e->pk_groups, e->pk_group_off.p, e->pk_group_sys.p, e->pk_group_flag.p, e->pk_ke.p, steps,
                     thermo ? 1 : 0, e->pk_stage};
            cudaError_t le = launch_md_persist(e->b, a, e->pk_cluster, st);
            cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (le != cudaSuccess) return fail(e, LG_ERR_CUDA, std::string("persistent launch: ") + cudaGetErrorString(le));
            if (ce != cudaSuccess) return fail(e, LG_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ce));
            cudaGraphExec_t exec = nullptr;
            ce = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess)
                return fail(e, LG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
            it = e->pk_graphs.emplace(key, exec).first;
        }
        CUDA_TRY(e, cudaGraphLaunch(it->second, st));
        e->launches += 1;
        uint32_t status;
        int rc = read_status(e, &status);
        if (rc) return rc;
        if (status & ST_OVERFLOW) {
            if (++retries > 4) return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
            CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, e->cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, e->cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, e->cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
            rc = clear_status_bits(e, ST_OVERFLOW);
            if (rc) return rc;
            rc = regrow(e);
            if (rc) return rc;
            continue;
        }
        done += steps;
    }
    return LG_OK;
}

int build_md_graph(lg_engine* e, int steps, int mode) {
    if (e->graph_mode != mode) e->drop_graphs();
    cudaGraph_t g;
    uint64_t before = e->launches;
    CUDA_TRY(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; k++) enqueue_md_step(e, mode, k > 0, e->stream);
    enqueue_md_finish(e, mode, e->stream);
    e->launches = before;  // captured launches run (and are counted) at replay
    CUDA_TRY(e, cudaStreamEndCapture(e->stream, &g));
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    cudaGraphExec_t exec = nullptr;
    cudaError_t ce = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(e, LG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
    e->graphs[steps] = exec;
    e->graph_nodes[steps] = nodes;
    e->graph_mode = mode;
    return LG_OK;
}

}  // namespace

extern "C" {

int lg_md_run(lg_engine* e, int64_t nsteps) {
    if (!e || nsteps < 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state: call lg_md_set_state first");
    for (int s = 0; s < e->nsys; s++)
        if (!e->sys[s].md_ready) return fail(e, LG_ERR_STATE, "lg_md_setup was not called for every system");
    const int mode = md_mode(e);
    const bool thermo = (mode & MD_ADJUST) != 0;
    const int chunk = 16;
    cudaStream_t st = e->stream;
    int64_t done = 0;
    int retries = 0;
    // Verlet::setup of the systems set up since the last run, from their current state
    for (int s = 0; s < e->nsys; s++) {
        HostSystem& h = e->sys[s];
        if (!h.verlet_setup) continue;
        launch_verlet_setup(e->b, s, (int)e->begin[s], (int)e->begin[s + 1], st);
        e->launches += h.n ? 1 : 0;
        h.verlet_setup = false;
    }
    CUDA_TRY(e, cudaGetLastError());
    if (!e->tuned) {
        int rc = autotune(e);
        if (rc) return rc;
    }
    // the persistent kernel for runs of several steps: a launch pays for the
    // slowest group's list rebuild, which short runs do not amortize (a
    // 1-step launch measured 193 us against 178 us for the per-step kernels
    // on the 128-replica batch)
    if (persist_eligible(e) && nsteps >= 8) {
        if (e->pk_cluster == 0) {
            int rc = persist_plan(e);
            if (rc) return rc;
        }
        if (e->pk_cluster > 0) return md_run_persistent(e, nsteps, thermo);
    }
    DBuf<double4_32a>& cp_pos = e->cp_pos;
    DBuf<double4_32a>& cp_vel = e->cp_vel;
    DBuf<double4_32a>& cp_acc = e->cp_acc;
    while (done < nsteps) {
        int steps = (int)std::min<int64_t>(chunk, nsteps - done);
        if (e->graph_mode != mode || !e->graphs.count(steps)) {
            int rc = build_md_graph(e, steps, mode);
            if (rc) return rc;
        }
        size_t bytes = e->b.n * sizeof(double4_32a);
        CUDA_TRY(e, cudaMemcpyAsync(cp_pos.p, e->posq.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(cp_vel.p, e->vel.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(cp_acc.p, e->acc.p, bytes, cudaMemcpyDeviceToDevice, st));
        const size_t cbytes = (size_t)e->nsys * sizeof(unsigned long long);  // CSVR noise counters
        if (thermo) CUDA_TRY(e, cudaMemcpyAsync(e->cp_count.p, e->md_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaGraphLaunch(e->graphs[steps], st));
        e->launches += e->graph_nodes[steps];
        uint32_t status;
        int rc = read_status(e, &status);
        if (rc) return rc;
        if (status & ST_OVERFLOW) {
            if (++retries > 4) return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
            CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
            if (thermo)
                CUDA_TRY(e, cudaMemcpyAsync(e->md_count.p, e->cp_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
            rc = clear_status_bits(e, ST_OVERFLOW);
            if (rc) return rc;
            rc = regrow(e);
            if (rc) return rc;
            continue;
        }
        done += steps;
    }
    return LG_OK;
}

int lg_md_set_state_all(lg_engine* e, const double* positions, const double* velocities,
                        const double* accelerations) {
    if (!e || !positions || !velocities) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    bool was_dirty = e->dirty;
    int rc = commit(e);
    if (rc) return rc;
    cudaStream_t st = e->stream;
    size_t n = (size_t)e->b.n;
    if (n == 0) return LG_OK;
    rc = put_state(e, 0, (int64_t)n, positions, velocities);
    if (rc) return rc;
    if (accelerations) {
        CUDA_TRY(e, cudaMemcpyAsync(e->force.p, accelerations, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
        launch_pack_vectors(e->b.n, e->force.p, e->acc.p, st);
        e->launches += 1;
    } else if (was_dirty) {
        CUDA_TRY(e, cudaMemsetAsync(e->acc.p, 0, n * sizeof(double4_32a), st));
    }
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_md_get_state_all(lg_engine* e, double* positions, double* velocities, double* accelerations) {
    if (!e) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state: call lg_md_set_state first");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    cudaStream_t st = e->stream;
    size_t n = (size_t)e->b.n;
    if (n == 0) return LG_OK;
    int rc = get_state(e, 0, (int64_t)n, positions, velocities);
    if (rc) return rc;
    if (accelerations) {
        launch_unpack_vectors(e->b.n, e->acc.p, e->force.p, st);
        e->launches += 1;
        CUDA_TRY(e, cudaMemcpyAsync(accelerations, e->force.p, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_md_integrate(lg_engine* e, double* positions, double* velocities, int64_t nsteps) {
    if (!e || e->nsys != 1) return fail(e, LG_ERR_ARGUMENT, "lg_md_integrate needs a single-system engine");
    int rc = lg_md_set_state(e, 0, positions, velocities);
    if (rc) return rc;
    rc = lg_md_run(e, nsteps);
    if (rc) return rc;
    return lg_md_get_state(e, 0, positions, velocities);
}

// ---- diagnostics ---------------------------------------------------------------
int lg_get_stream(lg_engine* e, void** stream) {
    if (!e || !stream) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    *stream = (void*)e->stream;
    return LG_OK;
}

int lg_md_plan(lg_engine* e, int32_t* cluster, int32_t* groups) {
    if (!e || !cluster || !groups) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    *cluster = e->pk_cluster > 0 ? e->pk_cluster : 0;
    *groups = e->pk_cluster > 0 ? e->pk_groups : 0;
    return LG_OK;
}

int lg_launch_count(lg_engine* e, uint64_t* count) {
    if (!e || !count) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    *count = e->launches;
    return LG_OK;
}

int lg_fma_peak(int32_t fp64, double* tflops) {
    if (!tflops) return fail(nullptr, LG_ERR_ARGUMENT, "invalid arguments");
    int rc = measure_fma_peak(fp64 ? 1 : 0, tflops);
    return rc ? fail(nullptr, LG_ERR_CUDA, "FMA probe failed") : LG_OK;
}

int lg_list_cells(lg_engine* e, int32_t s, int32_t* cells, int32_t ncell[3]) {
    if (!valid_sys(e, s) || !cells || !ncell) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    const SysDev& d = e->h_sysdev[s];
    size_t n = (size_t)e->sys[s].n;
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    CUDA_TRY(e, cudaMemcpy(cells, e->atom_cell.p + e->begin[s], n * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) cells[i] -= d.cell_begin;
    for (int k = 0; k < 3; k++) ncell[k] = d.ncell[k];
    return LG_OK;
}

int lg_kernel_times(lg_engine* e, int32_t reps, double* ms) {
    if (!e || !ms || reps <= 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    cudaStream_t st = e->stream;
    const Batch& b = e->b;
    cudaEvent_t e0, e1;
    CUDA_TRY(e, cudaEventCreate(&e0));
    CUDA_TRY(e, cudaEventCreate(&e1));
    const int mode = md_mode(e);
    // save the state: timing must not advance the trajectory (nor the CSVR noise counters)
    DBuf<double4_32a> sp, sv, sa;
    CUDA_TRY(e, sp.alloc(b.n));
    CUDA_TRY(e, sv.alloc(b.n));
    CUDA_TRY(e, sa.alloc(b.n));
    size_t bytes = (size_t)b.n * sizeof(double4_32a);
    const size_t cbytes = (size_t)e->nsys * sizeof(unsigned long long);
    CUDA_TRY(e, cudaMemcpyAsync(sp.p, e->posq.p, bytes, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(sv.p, e->vel.p, bytes, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(sa.p, e->acc.p, bytes, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->cp_count.p, e->md_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
    for (int g = 0; g < LG_KT_COUNT; g++) {
        float total = 0.f;
        for (int r = 0; r < reps; r++) {
            if (g == LG_KT_NLIST) launch_request_rebuild(b, st);
            CUDA_TRY(e, cudaEventRecord(e0, st));
            switch (g) {
                case LG_KT_NLIST: launch_nlist_build(b, st); break;
                case LG_KT_PAIR: launch_pair_forces(b, LG_TERM_ALL, false, st); break;
                case LG_KT_BONDED: launch_bonded(b, LG_TERM_ALL, false, st); break;
                case LG_KT_EIKR: launch_kspace_part(b, 0, false, st); break;
                case LG_KT_RHO: launch_kspace_part(b, 1, false, st); break;
                case LG_KT_FIELD: launch_kspace_part(b, 2, false, st); break;
                case LG_KT_VV:  // (the chunk sums may not be current: no thermostat here)
                    launch_md_first(b, false, st);
                    launch_md_second(b, st);
                    break;
                case LG_KT_STEP: enqueue_md_step(e, mode, false, st); break;
            }
            CUDA_TRY(e, cudaEventRecord(e1, st));
            CUDA_TRY(e, cudaEventSynchronize(e1));
            float t = 0.f;
            CUDA_TRY(e, cudaEventElapsedTime(&t, e0, e1));
            total += t;
            if (g == LG_KT_VV || g == LG_KT_STEP) {
                CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, sp.p, bytes, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, sv.p, bytes, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, sa.p, bytes, cudaMemcpyDeviceToDevice, st));
            }
        }
        ms[g] = total / reps;
    }
    CUDA_TRY(e, cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CUDA_TRY(e, cudaMemcpyAsync(e->md_count.p, e->cp_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
    // the forces buffer was overwritten by the timing runs: recompute it at the saved state
    launch_request_rebuild(b, st);
    enqueue_forces(e, LG_TERM_ALL, false, st);
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

// ---- Monte Carlo ---------------------------------------------------------------
int lg_mc_init(lg_engine* e, int32_t s, const double* positions, double* energy) {
    if (!valid_sys(e, s) || !positions) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = commit(e);
    if (rc) return rc;
    cudaStream_t st = e->stream;
    rc = upload_positions(e, s, positions);
    if (rc) return rc;
    rc = compute_batch(e, LG_TERM_ALL, LG_WANT_ENERGY, nullptr, nullptr);
    if (rc) return rc;
    // FP64 e^{ik.r} and rho(k) at these positions: the state the move costs update
    Batch fb = e->b;
    fb.precision = LG_PRECISION_FP64;
    launch_kspace_part(fb, 0, false, st);
    launch_kspace_part(fb, 1, false, st);
    CUDA_TRY(e, cudaMemcpyAsync(e->h_out, e->out.p + (size_t)s * RED_STRIDE, sizeof(double), cudaMemcpyDeviceToHost,
                                st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    CUDA_TRY(e, cudaGetLastError());
    e->mc_energy = e->h_out[0];
    e->mc_sys = s;
    e->mc_pending = false;
    if (energy) *energy = e->mc_energy;
    return LG_OK;
}

int lg_mc_move_molecule_cost(lg_engine* e, int32_t s, int64_t molecule, const double* new_positions, double* cost) {
    if (!valid_sys(e, s) || !new_positions || !cost) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty || e->mc_sys != s) return fail(e, LG_ERR_STATE, "lg_mc_init was not called for this system");
    const HostSystem& h = e->sys[s];
    if (molecule < 0 || molecule + 1 >= (int64_t)h.mol_begin.size())
        return fail(e, LG_ERR_ARGUMENT, "molecule index out of range");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int64_t mb = h.mol_begin[molecule], me = h.mol_begin[molecule + 1];
    int msize = (int)(me - mb);
    const SysDev& sd = e->h_sysdev[s];
    cudaStream_t st = e->stream;
    size_t need_pos = (size_t)std::max(msize, 1) * 3;
    if (e->mc_newpos.n < need_pos) CUDA_TRY(e, e->mc_newpos.alloc(need_pos));
    int nblocks = (int)((h.n + 255) / 256);
    if (e->mc_partial.n < (size_t)std::max(2 * nblocks, 2)) CUDA_TRY(e, e->mc_partial.alloc(std::max(2 * nblocks, 2)));
    int nk = sd.coul == LG_COULOMB_EWALD ? sd.kend - sd.kbegin : 0;
    if (e->mc_dk.n < (size_t)std::max(nk, 1)) CUDA_TRY(e, e->mc_dk.alloc(std::max(nk, 1)));
    if (e->mc_drho.n < (size_t)std::max(nk, 1)) CUDA_TRY(e, e->mc_drho.alloc(std::max(nk, 1)));
    size_t need_eikr = (size_t)(sd.kmax + 1) * 3 * std::max(msize, 1);
    if (e->mc_eikr.n < need_eikr) CUDA_TRY(e, e->mc_eikr.alloc(need_eikr));
    if (e->mc_out.n < 3) CUDA_TRY(e, e->mc_out.alloc(3));
    CUDA_TRY(e, cudaMemcpyAsync(e->mc_newpos.p, new_positions, 3 * msize * sizeof(double), cudaMemcpyHostToDevice,
                                st));
    launch_mc_cost(e->b, s, sd, (int)(e->begin[s] + mb), msize, e->mc_newpos.p, e->mc_eikr.p, e->mc_drho.p,
                   e->mc_partial.p, e->mc_dk.p, e->mc_out.p, st);
    e->launches += 2 + (nk > 0 ? 2 : 0);
    double out[3];
    CUDA_TRY(e, cudaMemcpyAsync(out, e->mc_out.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    CUDA_TRY(e, cudaGetLastError());
    e->mc_pending_cost = out[0] + out[1] + out[2];
    e->mc_pending = true;
    e->mc_mol_begin = e->begin[s] + mb;
    e->mc_mol_size = msize;
    *cost = e->mc_pending_cost;
    return LG_OK;
}

int lg_mc_update(lg_engine* e, int32_t s, const double* molecule_positions, double* energy) {
    if (!valid_sys(e, s) || !molecule_positions) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (!e->mc_pending || e->mc_sys != s)
        return fail(e, LG_ERR_STATE, "called EnergyCache::update without call a `*_cost` function first");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    cudaStream_t st = e->stream;
    int msize = (int)e->mc_mol_size;
    const SysDev& sd = e->h_sysdev[s];
    CUDA_TRY(e, cudaMemcpyAsync(e->mc_newpos.p, molecule_positions, 3 * msize * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    const double* d_k1 = (const double*)((const char*)(e->sysdev.p + s) + offsetof(SysDev, k1));
    launch_mc_accept(e->b, sd, (int)e->mc_mol_begin, msize, e->mc_newpos.p, d_k1, e->mc_drho.p, st);
    e->launches += 2;
    CUDA_TRY(e, cudaStreamSynchronize(st));
    CUDA_TRY(e, cudaGetLastError());
    e->mc_energy += e->mc_pending_cost;
    e->mc_pending = false;
    if (energy) *energy = e->mc_energy;
    return LG_OK;
}

int lg_mc_setup(lg_engine* e, int32_t s, double temperature, double delta, uint64_t seed) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    // MonteCarlo::new (mc/monte_carlo.rs) and Translate::new (translate.rs:41-52)
    if (!(temperature > 0.0)) return fail(e, LG_ERR_ARGUMENT, "the temperature must be positive in Monte Carlo");
    if (!(delta > 0.0)) return fail(e, LG_ERR_ARGUMENT, "delta must be positive in Translate move");
    const HostSystem& h = e->sys[s];
    if (h.coul.kind != LG_COULOMB_NONE)
        return fail(e, LG_ERR_ARGUMENT,
                    "batched Monte Carlo chains evaluate pair potentials only; use lg_mc_move_molecule_cost "
                    "for systems with Coulomb interactions");
    for (size_t i = 1; i < h.mols.size(); i++)
        if (h.mols[i] == h.mols[i - 1])
            return fail(e, LG_ERR_ARGUMENT, "batched Monte Carlo chains move single-particle molecules only");
    double half = delta / std::sqrt(3.0);
    if (std::sqrt(3.0) * half > 0.5 * e->skin)
        return fail(e, LG_ERR_ARGUMENT, "the Translate amplitude must not exceed half the neighbour-list skin");
    if (e->h_mc.size() != (size_t)e->nsys) e->h_mc.assign(e->nsys, McState{});
    McState& m = e->h_mc[s];
    m.beta = 1.0 / (K_BOLTZMANN * temperature);
    m.delta = half;
    m.rng = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    m.enabled = 1;
    m.moves_left = 0;
    m.need_rebuild = 0;
    m.accepted = m.attempted = 0;
    if (!e->dirty) {
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        CUDA_TRY(e, cudaMemcpy(e->mc_chains.p + s, &m, sizeof(McState), cudaMemcpyHostToDevice));
    }
    return LG_OK;
}

int lg_mc_run(lg_engine* e, int64_t moves) {
    if (!e || moves < 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state: call lg_md_set_state first");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    cudaStream_t st = e->stream;
    int nsys = e->nsys;
    CUDA_TRY(e, cudaMemcpy(e->h_mc.data(), e->mc_chains.p, nsys * sizeof(McState), cudaMemcpyDeviceToHost));
    if (!e->mc_energies_ready) {
        // EnergyCache::init: the chains start from the full energy of every system
        int rc = compute_batch(e, LG_TERM_ALL, LG_WANT_ENERGY, nullptr, nullptr);
        if (rc) return rc;
        std::vector<double> out((size_t)nsys * RED_STRIDE);
        CUDA_TRY(e, cudaMemcpy(out.data(), e->out.p, out.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (int s = 0; s < nsys; s++) e->h_mc[s].energy = out[(size_t)s * RED_STRIDE];
        e->mc_energies_ready = true;
    }
    bool any = false;
    bool fp64 = e->opt.precision == LG_PRECISION_FP64;
    for (int s = 0; s < nsys; s++)
        if (e->h_mc[s].enabled) {
            e->h_mc[s].moves_left = moves;
            e->h_mc[s].need_rebuild = 0;
            any = true;
        }
    if (!any) return fail(e, LG_ERR_STATE, "lg_mc_setup was not called for any system");
    CUDA_TRY(e, cudaMemcpyAsync(e->mc_chains.p, e->h_mc.data(), nsys * sizeof(McState), cudaMemcpyHostToDevice, st));
    // the list must be current for the positions the chains start from, and so
    // must the fixed-point copies the mixed chains read
    launch_check_displacement(e->b, st);
    launch_nlist_build(e->b, st);
    e->launches += 1 + nlist_launches(e->b);
    if (!fp64) {
        launch_split_positions(e->b, st);
        e->launches += 1;
    }
    for (int64_t launch = 0; launch < moves + 64; launch++) {
        launch_mc_chains(e->b, e->mc_chains.p, fp64, st);
        e->launches += 1;
        CUDA_TRY(e, cudaMemcpyAsync(e->h_mc.data(), e->mc_chains.p, nsys * sizeof(McState), cudaMemcpyDeviceToHost,
                                    st));
        CUDA_TRY(e, cudaStreamSynchronize(st));
        CUDA_TRY(e, cudaGetLastError());
        bool rebuild = false, pending = false;
        for (int s = 0; s < nsys; s++) {
            if (!e->h_mc[s].enabled) continue;
            rebuild = rebuild || e->h_mc[s].need_rebuild;
            pending = pending || e->h_mc[s].moves_left > 0;
        }
        if (!pending) return LG_OK;
        if (rebuild) {
            // rebuild the lists of the stopped chains' systems only
            std::vector<uint32_t> flags(nsys, 0u);
            for (int s = 0; s < nsys; s++) {
                flags[s] = e->h_mc[s].need_rebuild ? 1u : 0u;
                e->h_mc[s].need_rebuild = 0;
            }
            CUDA_TRY(e, cudaMemcpyAsync(e->mc_chains.p, e->h_mc.data(), nsys * sizeof(McState),
                                        cudaMemcpyHostToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->sys_rebuild.p, flags.data(), nsys * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                        st));
            uint32_t rebuild_bit = ST_REBUILD;
            CUDA_TRY(e, cudaMemcpyAsync(e->h_status, e->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            CUDA_TRY(e, cudaStreamSynchronize(st));
            *e->h_status |= rebuild_bit;
            CUDA_TRY(e, cudaMemcpyAsync(e->status.p, e->h_status, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            launch_nlist_build(e->b, st);
            e->launches += nlist_launches(e->b);
            uint32_t status;
            int rc = read_status(e, &status);
            if (rc) return rc;
            if (status & ST_OVERFLOW) {
                rc = clear_status_bits(e, ST_OVERFLOW);
                if (rc) return rc;
                rc = regrow(e);
                if (rc) return rc;
                launch_nlist_build(e->b, st);
            }
        }
    }
    return fail(e, LG_ERR_STATE, "Monte Carlo chains did not finish");
}

int lg_mc_stats(lg_engine* e, int32_t s, double* energy, int64_t* accepted, int64_t* attempted) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    McState m;
    CUDA_TRY(e, cudaMemcpy(&m, e->mc_chains.p + s, sizeof(McState), cudaMemcpyDeviceToHost));
    if (energy) *energy = m.energy;
    if (accepted) *accepted = m.accepted;
    if (attempted) *attempted = m.attempted;
    return LG_OK;
}

}  // extern "C"
