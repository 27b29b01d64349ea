// capi.cu -- the C entry points of include/lumol_gb300.h for the system
// description, forces / energies / virials, molecular dynamics and
// diagnostics (the Monte Carlo entry points are in capi_mc.cu).  The engine
// object and its helpers are in engine.h.
#include "engine.h"

#include <functional>

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
    e->carry_from.assign(n_systems, -1);
    ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&e->h_status, sizeof(uint32_t));
    if (ce == cudaSuccess) ce = cudaHostGetDevicePointer((void**)&e->d_h_status, e->h_status, 0);
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

int lg_set_cell_ex(lg_engine* e, int32_t s, const double m[9], int32_t shape) {
    if (!valid_sys(e, s) || !m) return fail(e, LG_ERR_ARGUMENT, "invalid system index or cell");
    if (shape != LG_CELL_ORTHORHOMBIC && shape != LG_CELL_TRICLINIC) return fail(e, LG_ERR_ARGUMENT, "invalid cell shape");
    for (int k = 0; k < 9; k++)
        if (!std::isfinite(m[k])) return fail(e, LG_ERR_ARGUMENT, "non-finite cell matrix");
    if (shape == LG_CELL_ORTHORHOMBIC && !(m[0] > 0.0 && m[4] > 0.0 && m[8] > 0.0))
        return fail(e, LG_ERR_ARGUMENT, "Cell lengths must be positive");
    HostCell cell;
    if (!cell_init(cell, m, shape)) return fail(e, LG_ERR_ARGUMENT, "the cell matrix is not invertible or its volume is not positive");
    HostSystem& h = e->sys[s];
    int rc = check_cell_cutoffs(e, h, cell.len);
    if (rc) return rc;
    // a cell's shape decides the list grid and the kernels' branches: lower again when it changes
    if (!e->dirty && h.has_cell && h.cell.shape == shape) {  // in place, keeping the state
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        rc = set_cell_fast(e, s, cell);
        if (rc != -1) return rc;
    }
    set_host_cell(h, cell);
    invalidate(e);
    return LG_OK;
}

int lg_set_cell(lg_engine* e, int32_t s, const double m[9]) {
    if (!valid_sys(e, s) || !m) return fail(e, LG_ERR_ARGUMENT, "invalid system index or cell");
    bool diagonal = m[1] == 0.0 && m[2] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[6] == 0.0 && m[7] == 0.0;
    return lg_set_cell_ex(e, s, m, diagonal ? LG_CELL_ORTHORHOMBIC : LG_CELL_TRICLINIC);
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
    if (s < (int)e->carry_from.size()) e->carry_from[s] = -1;  // new particles: no state to carry
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
    e->shadow_valid = false;
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
    h.reset_acc = e->dirty && p->integrator != LG_INTEGRATOR_VERLET;  // a carried system's, at the commit
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

int lg_md_set_barostat(lg_engine* e, int32_t s, int32_t kind, double pressure, double tau) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    if (kind != LG_BAROSTAT_NONE && kind != LG_BAROSTAT_BERENDSEN) return fail(e, LG_ERR_ARGUMENT, "unknown barostat");
    HostSystem& h = e->sys[s];
    if (kind == LG_BAROSTAT_BERENDSEN) {
        if (!h.md_ready || h.integrator != LG_INTEGRATOR_VELOCITY_VERLET)
            return fail(e, LG_ERR_STATE,
                        "the Berendsen barostat needs lg_md_setup_ex with LG_INTEGRATOR_VELOCITY_VERLET first");
        if (!(tau > 0.0)) return fail(e, LG_ERR_ARGUMENT, "the barostat time scale must be positive");
    }
    h.barostat = kind;
    h.baro_pressure = pressure;
    h.baro_tau = tau;
    h.baro_eta = 1.0;  // BerendsenBarostat::new
    if (!e->dirty) {
        SysDev& d = e->h_sysdev[s];
        fill_md(d, h);
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        CUDA_TRY(e, cudaMemcpyAsync(e->sysdev.p + s, &d, sizeof(SysDev), cudaMemcpyHostToDevice, e->stream));
        CUDA_TRY(e, cudaStreamSynchronize(e->stream));
        e->drop_graphs();
        e->pk_cluster = 0;
    }
    return LG_OK;
}

int lg_md_set_aniso_barostat(lg_engine* e, int32_t s, const double stress[9], double tau) {
    if (!valid_sys(e, s) || !stress) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    int rc = lg_md_set_barostat(e, s, LG_BAROSTAT_BERENDSEN, 0.0, tau);  // the same checks
    if (rc) return rc;
    HostSystem& h = e->sys[s];
    h.barostat = LG_BAROSTAT_ANISO_BERENDSEN;
    for (int k = 0; k < 9; k++) {
        h.baro_stress[k] = stress[k];
        h.baro_m[k] = (k % 4 == 0) ? 1.0 : 0.0;  // AnisoBerendsenBarostat::new: eta = Matrix3::one()
    }
    if (!e->dirty) {
        SysDev& d = e->h_sysdev[s];
        fill_md(d, h);
        CUDA_TRY(e, cudaMemcpyAsync(e->sysdev.p + s, &d, sizeof(SysDev), cudaMemcpyHostToDevice, e->stream));
        CUDA_TRY(e, cudaStreamSynchronize(e->stream));
        e->drop_graphs();
    }
    return LG_OK;
}

int lg_get_cell(lg_engine* e, int32_t s, double m[9]) {
    if (!valid_sys(e, s) || !m) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    const HostSystem& h = e->sys[s];
    for (int k = 0; k < 9; k++) m[k] = h.cell.m[k];
    return LG_OK;
}

int lg_cell_info(lg_engine* e, int32_t s, int32_t* shape, double lengths[3], double* volume) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    const HostSystem& h = e->sys[s];
    if (!h.has_cell) return fail(e, LG_ERR_STATE, "system " + std::to_string(s) + " has no cell");
    if (shape) *shape = h.cell.shape;
    if (lengths)
        for (int k = 0; k < 3; k++) lengths[k] = h.cell.len[k];
    if (volume) *volume = h.cell.volume;
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
    // a new state after a description change starts from zero accelerations
    // (systems carried through the change keep theirs)
    if (was_dirty) CUDA_TRY(e, cudaMemsetAsync(e->acc.p + base, 0, h.n * sizeof(double4_32a), st));
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_md_get_state(lg_engine* e, int32_t s, double* positions, double* velocities) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    {
        int rc0 = commit_carried(e);
        if (rc0) return rc0;
    }
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

int lg_md_set_state_ex(lg_engine* e, int32_t s, const double* positions, const double* velocities,
                       const double* accelerations) {
    int rc = lg_md_set_state(e, s, positions, velocities);
    if (rc || !accelerations) return rc;
    const HostSystem& h = e->sys[s];
    if (h.n == 0) return LG_OK;
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    CUDA_TRY(e, cudaMemcpyAsync(e->pos3.p + 3 * base, accelerations, 3 * h.n * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    launch_pack_vectors((int)h.n, e->pos3.p + 3 * base, e->acc.p + base, st);
    e->launches += 1;
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_md_get_state_ex(lg_engine* e, int32_t s, double* positions, double* velocities, double* accelerations) {
    int rc = lg_md_get_state(e, s, positions, velocities);
    if (rc || !accelerations) return rc;
    const HostSystem& h = e->sys[s];
    if (h.n == 0) return LG_OK;
    int64_t base = e->begin[s];
    cudaStream_t st = e->stream;
    launch_unpack_vectors((int)h.n, e->acc.p + base, e->pos3.p + 3 * base, st);
    e->launches += 1;
    CUDA_TRY(e, cudaMemcpyAsync(accelerations, e->pos3.p + 3 * base, 3 * h.n * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));
    return LG_OK;
}

int lg_add_systems(lg_engine* e, int32_t count) {
    if (!e || count <= 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->carry_from.size() != (size_t)e->nsys) e->carry_from.assign(e->nsys, -1);
    e->sys.resize(e->nsys + count);
    e->carry_from.resize(e->nsys + count, -1);
    if (e->h_mc.size() == (size_t)e->nsys) e->h_mc.resize(e->nsys + count, McState{});
    e->nsys += count;
    invalidate(e);
    return LG_OK;
}

int lg_remove_system(lg_engine* e, int32_t s) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    if (e->nsys == 1) return fail(e, LG_ERR_ARGUMENT, "an engine keeps at least one system");
    if (e->carry_from.size() != (size_t)e->nsys) e->carry_from.assign(e->nsys, -1);
    e->sys.erase(e->sys.begin() + s);
    e->carry_from.erase(e->carry_from.begin() + s);
    if (e->h_mc.size() == (size_t)e->nsys) e->h_mc.erase(e->h_mc.begin() + s);
    if (e->mc_sys == s) {
        e->mc_sys = -1;
        e->mc_pending = false;
    } else if (e->mc_sys > s) {
        e->mc_sys -= 1;
    }
    e->nsys -= 1;
    invalidate(e);
    return LG_OK;
}

}  // extern "C"

namespace {

// The steps of lg_md_run.  `tail` (may be empty) is enqueued after the last
// chunk, before the status read that ends it, so a caller that copies the state
// back pays for one synchronisation only; it is enqueued again if that chunk is
// replayed.
int md_run_steps(lg_engine* e, int64_t nsteps, const std::function<int()>& tail) {
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
    // slowest group's list rebuild, which short runs do not amortize (on the
    // 128-replica batch, per step: 218 / 159 / 122 us for runs of 1 / 2 / 4
    // steps against 176 / 149 / 134 us on the per-step graph); a batch of a
    // few systems has no such spread, and one launch per step beats a graph
    // of a dozen kernels
    for (int s = 0; s < e->nsys; s++)
        if (e->sys[s].barostat != LG_BAROSTAT_NONE) {
            int rc = md_run_barostat(e, nsteps);
            if (rc == LG_OK && tail) rc = tail();
            if (rc == LG_OK && tail) CUDA_TRY(e, cudaStreamSynchronize(st));
            return rc;
        }
    if (persist_eligible(e) && (nsteps >= 4 || e->nsys <= 4)) {
        if (e->pk_cluster == 0) {
            int rc = persist_plan(e);
            if (rc) return rc;
        }
        if (e->pk_cluster > 0) return md_run_persistent(e, nsteps, thermo, tail);
    }
    DBuf<double4_32a>& cp_pos = e->cp_pos;
    DBuf<double4_32a>& cp_vel = e->cp_vel;
    DBuf<double4_32a>& cp_acc = e->cp_acc;
    if (nsteps == 0 && tail) {
        int rc = tail();
        if (rc) return rc;
        CUDA_TRY(e, cudaStreamSynchronize(st));
    }
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
        if (done + steps == nsteps && tail) {
            int rc = tail();
            if (rc) return rc;
        }
        uint32_t status;
        int rc = read_status(e, &status);
        if (rc) return rc;
        if (status & (ST_OVERFLOW | ST_CELL_OVF)) {
            if (++retries > 4) return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
            CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
            if (thermo)
                CUDA_TRY(e, cudaMemcpyAsync(e->md_count.p, e->cp_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
            if (status & ST_CELL_OVF) {
                rc = recount_cells(e);
                if (rc) return rc;
            }
            if (status & ST_OVERFLOW) {
                rc = clear_status_bits(e, ST_OVERFLOW);
                if (rc) return rc;
                rc = regrow(e);
                if (rc) return rc;
            }
            continue;
        }
        if (status & ST_NONFINITE) {  // reported after the run; the other systems are unaffected
            e->nonfinite = true;
            rc = clear_status_bits(e, ST_NONFINITE);
            if (rc) return rc;
        }
        done += steps;
    }
    return LG_OK;
}

int md_run_checked(lg_engine* e, int64_t nsteps, const std::function<int()>& tail) {
    if (!e || nsteps < 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    {
        int rc = commit_carried(e);  // systems that left or were re-described keep their state
        if (rc) return rc;
    }
    for (int s = 0; s < e->nsys; s++)
        if (!e->sys[s].md_ready) return fail(e, LG_ERR_STATE, "lg_md_setup was not called for every system");
    e->nonfinite = false;
    int rc = md_run_steps(e, nsteps, tail);
    if (rc) return rc;
    e->state_gen += 1;
    if (e->nonfinite)
        return fail(e, LG_ERR_NONFINITE,
                    "Kinetic energy is infinite! (non-finite velocities in system " + nonfinite_systems(e) +
                        "; every other system completed its steps)");
    return LG_OK;
}

}  // namespace

extern "C" {

int lg_md_run(lg_engine* e, int64_t nsteps) { return md_run_checked(e, nsteps, {}); }

int lg_system_status(lg_engine* e, uint32_t* flags, int32_t clear) {
    if (!e || !flags) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) {
        for (int s = 0; s < e->nsys; s++) flags[s] = 0u;
        return LG_OK;
    }
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    CUDA_TRY(e, cudaMemcpy(flags, e->sys_status.p, e->nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (clear) CUDA_TRY(e, cudaMemset(e->sys_status.p, 0, e->nsys * sizeof(uint32_t)));
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
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    {
        int rc0 = commit_carried(e);
        if (rc0) return rc0;
    }
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

int lg_md_propagate(lg_engine* e, double* positions, double* velocities, int64_t nsteps, uint32_t flags) {
    if (!e || e->nsys != 1) return fail(e, LG_ERR_ARGUMENT, "lg_md_propagate needs a single-system engine");
    if (!positions || !velocities || (flags & ~(LG_SYNC_DOWNLOAD | LG_SYNC_TRUST_HOST)))
        return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    const bool was_dirty = e->dirty;
    int rc = commit(e);
    if (rc) return rc;
    const int64_t n = e->sys[0].n;
    const size_t n3 = 3 * (size_t)n;
    if (e->shadow_n3 != n3 || !e->h_shadow) {
        if (e->h_shadow) cudaFreeHost(e->h_shadow);
        e->h_shadow = nullptr;
        e->shadow_n3 = 0;
        e->shadow_valid = false;
        CUDA_TRY(e, cudaMallocHost((void**)&e->h_shadow, std::max<size_t>(2 * n3, 1) * sizeof(double)));
        CUDA_TRY(e, cudaHostGetDevicePointer((void**)&e->d_shadow, e->h_shadow, 0));
        e->shadow_n3 = n3;
    }
    double* sp = e->h_shadow;
    double* sv = e->h_shadow + n3;
    // the host copy changed (or the device state is not the one last exchanged): upload
    bool upload = !e->shadow_valid;
    if (!upload && !(flags & LG_SYNC_TRUST_HOST))
        upload = std::memcmp(positions, sp, n3 * sizeof(double)) != 0 ||
                 std::memcmp(velocities, sv, n3 * sizeof(double)) != 0;
    if (upload && n > 0) {
        std::memcpy(sp, positions, n3 * sizeof(double));
        std::memcpy(sv, velocities, n3 * sizeof(double));
        rc = put_state(e, 0, n, sp, sv);  // read in place from the page-locked copy
        if (rc) return rc;
        if (was_dirty) CUDA_TRY(e, cudaMemsetAsync(e->acc.p, 0, n * sizeof(double4_32a), e->stream));
    }
    e->shadow_valid = true;
    const bool download = (flags & LG_SYNC_DOWNLOAD) && n > 0;
    std::function<int()> tail;
    double* dsp = e->d_shadow;  // (mapped once: no pointer query per call)
    if (download) tail = [e, n, dsp, n3]() { return get_state_mapped(e, 0, n, dsp, dsp + n3); };
    rc = md_run_checked(e, nsteps, tail);
    if (rc != LG_OK && rc != LG_ERR_NONFINITE) {
        e->shadow_valid = false;
        return rc;
    }
    e->shadow_valid = true;
    if (download) {
        std::memcpy(positions, sp, n3 * sizeof(double));
        std::memcpy(velocities, sv, n3 * sizeof(double));
    }
    return rc;
}

int lg_md_integrate(lg_engine* e, double* positions, double* velocities, int64_t nsteps) {
    if (!e || e->nsys != 1) return fail(e, LG_ERR_ARGUMENT, "lg_md_integrate needs a single-system engine");
    return lg_md_propagate(e, positions, velocities, nsteps, LG_SYNC_DOWNLOAD);
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

int lg_test_stale_cell_counts(lg_engine* e, int32_t s, int32_t extra) {
    if (!valid_sys(e, s) || extra < 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty) return fail(e, LG_ERR_STATE, "no device state");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    // what an interrupted build leaves: counts of binned atoms that were never
    // sorted back to zero, and a rebuild request for the system
    int* first = e->cell_count.p + e->h_sysdev[s].cell_begin;
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    int c = 0;
    CUDA_TRY(e, cudaMemcpy(&c, first, sizeof(int), cudaMemcpyDeviceToHost));
    c += extra;
    CUDA_TRY(e, cudaMemcpy(first, &c, sizeof(int), cudaMemcpyHostToDevice));
    launch_request_rebuild(e->b, e->stream);
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
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

}  // extern "C"
