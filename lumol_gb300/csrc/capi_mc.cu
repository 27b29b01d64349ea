// capi_mc.cu -- the Monte Carlo entry points of include/lumol_gb300.h: the
// EnergyCache move cost / update of one molecule, and the batched device
// Metropolis chains.
#include "engine.h"

namespace {
int mc_restore_resize(lg_engine* e);
}  // namespace

extern "C" {

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
    if (e->mc_resize) {  // a Resize that was neither accepted nor restored: restored now
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        int rc0 = mc_restore_resize(e);
        if (rc0) return rc0;
    }
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

}  // extern "C"

namespace {

// The FP64 e^{ik.r} tables and rho(k) of the Monte Carlo system at the device
// positions (what lg_mc_init computes; the single-molecule costs update them).
void mc_refresh_kspace(lg_engine* e) {
    Batch fb = e->b;
    fb.precision = LG_PRECISION_FP64;
    launch_kspace_part(fb, 0, false, e->stream);
    launch_kspace_part(fb, 1, false, e->stream);
    e->launches += 2;
}

// Installs a cell for system s, in place when the cell grid and the k-vector
// set allow it, else by lowering the batch again (state kept).
int mc_set_cell(lg_engine* e, int s, const HostCell& cell) {
    int rc = set_cell_fast(e, s, cell);
    if (rc != -1) return rc;
    set_host_cell(e->sys[s], cell);
    invalidate(e);
    return commit_carried(e);
}

// Resize::restore (mc/moves/resize.rs:121-124) of a pending
// move_all_molecules_cost: the previous cell and positions come back.
int mc_restore_resize(lg_engine* e) {
    if (!e->mc_resize) return LG_OK;
    int s = e->mc_sys;
    e->mc_resize = false;
    e->mc_pending = false;
    int rc = mc_set_cell(e, s, e->mc_old_cell);
    if (rc) return rc;
    const HostSystem& h = e->sys[s];
    CUDA_TRY(e, cudaMemcpyAsync(e->posq.p + e->begin[s], e->mc_saved_pos.p, h.n * sizeof(double4_32a),
                                cudaMemcpyDeviceToDevice, e->stream));
    launch_request_rebuild(e->b, e->stream);
    e->shadow_valid = false;
    mc_refresh_kspace(e);
    CUDA_TRY(e, cudaStreamSynchronize(e->stream));
    CUDA_TRY(e, cudaGetLastError());
    return LG_OK;
}

}  // namespace

extern "C" {

int lg_mc_move_all_molecules_cost(lg_engine* e, int32_t s, const double new_cell[9], const double* new_positions,
                                  double* cost) {
    if (!valid_sys(e, s) || !new_cell || !new_positions || !cost) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->dirty || e->mc_sys != s) return fail(e, LG_ERR_STATE, "lg_mc_init was not called for this system");
    // the shape is kept (UnitCell::scale_mut, cells.rs:201-207)
    HostCell cell;
    const int shape = e->sys[s].cell.shape;
    if (shape == LG_CELL_ORTHORHOMBIC)
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++)
                if (a != c && new_cell[3 * a + c] != 0.0)
                    return fail(e, LG_ERR_ARGUMENT, "an orthorhombic cell has a diagonal matrix");
    if (!cell_init(cell, new_cell, shape)) return fail(e, LG_ERR_ARGUMENT, "the new cell is singular");
    const double* L = cell.len;
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = mc_restore_resize(e);  // a previous Resize that was neither accepted nor restored
    if (rc) return rc;
    HostSystem& h = e->sys[s];
    double rcut = max_cutoff(h);
    if (0.5 * L[0] <= rcut || 0.5 * L[1] <= rcut || 0.5 * L[2] <= rcut)  // resize.rs:76-86
        return fail(e, LG_ERR_ARGUMENT,
                    "Tried to decrease the cell size in Monte Carlo Resize move but the new size is smaller than "
                    "the interactions cut off radius. You can try to increase the cell size or the number of "
                    "particles.");
    cudaStream_t st = e->stream;
    CUDA_TRY(e, e->mc_saved_pos.alloc(std::max<int64_t>(h.n, 1)));
    CUDA_TRY(e, cudaMemcpyAsync(e->mc_saved_pos.p, e->posq.p + e->begin[s], h.n * sizeof(double4_32a),
                                cudaMemcpyDeviceToDevice, st));
    e->mc_old_cell = h.cell;
    rc = mc_set_cell(e, s, cell);
    if (rc) return rc;
    rc = upload_positions(e, s, new_positions);
    if (rc) return rc;
    rc = compute_batch(e, LG_TERM_ALL, LG_WANT_ENERGY, nullptr, nullptr);
    if (rc) return rc;
    CUDA_TRY(e, cudaMemcpyAsync(e->h_out, e->out.p + (size_t)s * RED_STRIDE, sizeof(double), cudaMemcpyDeviceToHost,
                                st));
    CUDA_TRY(e, cudaStreamSynchronize(st));
    // the rigid molecules keep their bonded energies: the change of the total
    // is the change of the pairs, tails and Coulomb terms
    e->mc_pending_cost = e->h_out[0] - e->mc_energy;
    e->mc_pending = true;
    e->mc_resize = true;
    *cost = e->mc_pending_cost;
    return LG_OK;
}

int lg_mc_restore(lg_engine* e, int32_t s) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (e->mc_sys != s) return fail(e, LG_ERR_STATE, "lg_mc_init was not called for this system");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    int rc = mc_restore_resize(e);
    e->mc_pending = false;
    return rc;
}

int lg_mc_update(lg_engine* e, int32_t s, const double* molecule_positions, double* energy) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    if (!e->mc_pending || e->mc_sys != s)
        return fail(e, LG_ERR_STATE, "called EnergyCache::update without call a `*_cost` function first");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    cudaStream_t st = e->stream;
    if (e->mc_resize) {  // the new cell and positions stay
        e->mc_resize = false;
        mc_refresh_kspace(e);
        CUDA_TRY(e, cudaStreamSynchronize(st));
        CUDA_TRY(e, cudaGetLastError());
        e->mc_energy += e->mc_pending_cost;
        e->mc_pending = false;
        if (energy) *energy = e->mc_energy;
        return LG_OK;
    }
    int msize = (int)e->mc_mol_size;
    const SysDev& sd = e->h_sysdev[s];
    // NULL: the positions the cost was computed for (already on the device)
    if (molecule_positions)
        CUDA_TRY(e, cudaMemcpyAsync(e->mc_newpos.p, molecule_positions, 3 * msize * sizeof(double),
                                    cudaMemcpyHostToDevice, st));
    e->shadow_valid = false;
    launch_mc_accept(e->b, sd, (int)e->mc_mol_begin, msize, e->mc_newpos.p, e->sysdev.p + s, e->mc_drho.p, st);
    e->launches += 2;
    CUDA_TRY(e, cudaStreamSynchronize(st));
    CUDA_TRY(e, cudaGetLastError());
    e->mc_energy += e->mc_pending_cost;
    e->mc_pending = false;
    if (energy) *energy = e->mc_energy;
    return LG_OK;
}

// MonteCarlo::new (mc/monte_carlo.rs) with Translate::new (translate.rs:41-52):
// the chain of system s (molecules: whether molecules of several atoms are allowed)
static int mc_setup_chain(lg_engine* e, int32_t s, double temperature, double delta, uint64_t seed,
                          bool molecules) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    // MonteCarlo::new (mc/monte_carlo.rs) and Translate::new (translate.rs:41-52)
    if (!(temperature > 0.0)) return fail(e, LG_ERR_ARGUMENT, "the temperature must be positive in Monte Carlo");
    if (!(delta > 0.0)) return fail(e, LG_ERR_ARGUMENT, "delta must be positive in Translate move");
    const HostSystem& h = e->sys[s];
    if (!molecules)
        for (size_t i = 1; i < h.mols.size(); i++)
            if (h.mols[i] == h.mols[i - 1])
                return fail(e, LG_ERR_ARGUMENT,
                            "batched Monte Carlo chains of lg_mc_setup move single-particle molecules; "
                            "lg_mc_setup_ex moves whole molecules");
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
    // (lg_mc_setup_ex sets the molecular moves afterwards; the chain of a
    // triclinic cell or of a system with Coulomb interactions runs in the
    // molecular chains' kernel, whose geometry and energy terms are general)
    m.molecular = (h.cell.shape == LG_CELL_ORTHORHOMBIC && h.coul.kind == LG_COULOMB_NONE) ? 0 : 1;
    m.theta = 0.0;
    m.cum_translate = 1.0;
    if (!e->dirty) {
        CUDA_TRY(e, cudaSetDevice(e->opt.device));
        CUDA_TRY(e, cudaMemcpy(e->mc_chains.p + s, &m, sizeof(McState), cudaMemcpyHostToDevice));
    }
    return LG_OK;
}

int lg_mc_setup(lg_engine* e, int32_t s, double temperature, double delta, uint64_t seed) {
    return mc_setup_chain(e, s, temperature, delta, seed, false);
}

int lg_mc_setup_ex(lg_engine* e, int32_t s, double temperature, double translate_delta, double translate_frequency,
                   double rotate_theta, double rotate_frequency, uint64_t seed) {
    if (!valid_sys(e, s)) return fail(e, LG_ERR_ARGUMENT, "invalid system index");
    if (!(temperature > 0.0)) return fail(e, LG_ERR_ARGUMENT, "the temperature must be positive in Monte Carlo");
    if (!(translate_frequency >= 0.0) || !(rotate_frequency >= 0.0) || !(translate_frequency + rotate_frequency > 0.0))
        return fail(e, LG_ERR_ARGUMENT, "move frequencies must be non-negative with a positive sum");
    if (translate_frequency > 0.0 && !(translate_delta > 0.0))
        return fail(e, LG_ERR_ARGUMENT, "delta must be positive in Translate move");
    if (rotate_frequency > 0.0 && !(rotate_theta > 0.0))
        return fail(e, LG_ERR_ARGUMENT, "theta must be positive in Rotate move");
    double half = translate_frequency > 0.0 ? translate_delta / std::sqrt(3.0) : 0.0;
    if (std::sqrt(3.0) * half > 0.5 * e->skin)
        return fail(e, LG_ERR_ARGUMENT, "the Translate amplitude must not exceed half the neighbour-list skin");
    int rc = mc_setup_chain(e, s, temperature, translate_frequency > 0.0 ? translate_delta : 1.0, seed, true);
    if (rc) return rc;
    McState& m = e->h_mc[s];
    m.molecular = 1;
    m.theta = rotate_theta;
    // MonteCarlo::normalize_frequencies (monte_carlo.rs:190-208): the last cumulative frequency is 1
    double sum = translate_frequency + rotate_frequency;
    m.cum_translate = rotate_frequency > 0.0 ? translate_frequency / sum : 1.0;
    m.delta = half;
    if (!e->dirty) CUDA_TRY(e, cudaMemcpy(e->mc_chains.p + s, &m, sizeof(McState), cudaMemcpyHostToDevice));
    return LG_OK;
}

int lg_mc_run(lg_engine* e, int64_t moves) {
    if (!e || moves < 0) return fail(e, LG_ERR_ARGUMENT, "invalid arguments");
    CUDA_TRY(e, cudaSetDevice(e->opt.device));
    {
        int rc0 = commit_carried(e);
        if (rc0) return rc0;
    }
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
    bool molecular = false;  // chains of lg_mc_setup_ex: the molecular chains' kernel runs too
    bool kspace = false;     // ... with Ewald: they read and update the FP64 rho(k)
    for (int s = 0; s < nsys; s++) {
        const McState& m = e->h_mc[s];
        if (!m.enabled || !m.molecular) continue;
        molecular = true;
        kspace = kspace || e->sys[s].coul.kind == LG_COULOMB_EWALD;
        if (m.cum_translate >= 1.0) continue;
        // a rotated atom moves by at most 2 r sin(theta / 2), r its distance from
        // the molecule's centre of mass: it must stay within skin / 2, else no
        // rotation could ever be attempted between two list builds
        const HostSystem& h = e->sys[s];
        std::vector<double4_32a> x(h.n), v(h.n);
        CUDA_TRY(e, cudaMemcpy(x.data(), e->posq.p + e->begin[s], h.n * sizeof(double4_32a), cudaMemcpyDeviceToHost));
        CUDA_TRY(e, cudaMemcpy(v.data(), e->vel.p + e->begin[s], h.n * sizeof(double4_32a), cudaMemcpyDeviceToHost));
        double rmax = 0.0;
        for (size_t mi = 0; mi + 1 < h.mol_begin.size(); mi++) {
            int64_t lo = h.mol_begin[mi], hi = h.mol_begin[mi + 1];
            double total = 0.0, c[3] = {0, 0, 0};
            for (int64_t a = lo; a < hi; a++) {
                total += v[a].w;
                c[0] += v[a].w * x[a].x;
                c[1] += v[a].w * x[a].y;
                c[2] += v[a].w * x[a].z;
            }
            for (int64_t a = lo; a < hi; a++) {
                double dx = x[a].x - c[0] / total, dy = x[a].y - c[1] / total, dz = x[a].z - c[2] / total;
                rmax = std::max(rmax, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
        }
        if (2.0 * rmax * std::sin(0.5 * std::min(m.theta, PI)) > 0.5 * e->skin)
            return fail(e, LG_ERR_ARGUMENT,
                        "the Rotate amplitude must not move an atom farther than half the neighbour-list skin "
                        "(system " + std::to_string(s) + ")");
    }
    e->shadow_valid = false;
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
    if (kspace) {  // the FP64 rho(k) of the current positions
        mc_refresh_kspace(e);
    }
    for (int64_t launch = 0; launch < moves + 64; launch++) {
        launch_mc_chains(e->b, e->mc_chains.p, fp64, molecular, st);
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
        if (!pending) {
            // (the chains updated rho(k) themselves; the e^{ik.r} tables follow the
            // moved atoms for the single-molecule costs that may come next)
            if (kspace) {
                mc_refresh_kspace(e);
                CUDA_TRY(e, cudaStreamSynchronize(st));
            }
            return LG_OK;
        }
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
            if (status & (ST_OVERFLOW | ST_CELL_OVF)) {
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
