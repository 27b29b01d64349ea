// runtime.cu -- what the engine does with a lowered batch: status words,
// list regrowth, force passes, host <-> device state transfers, the
// autotuner, MD step graphs, and the persistent-kernel plan and launches.
#include "engine.h"

namespace lg {

thread_local std::string g_create_error;
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int, int, bool>, std::pair<int, int>> g_tune_cache;

void set_global_error(const std::string& msg) { g_create_error = msg; }

int fail(lg_engine* e, int code, const std::string& msg) {
    if (e) e->err = msg;
    else g_create_error = msg;
    return code;
}

bool valid_sys(lg_engine* e, int32_t s) { return e && s >= 0 && s < e->nsys; }

void invalidate(lg_engine* e) {
    e->dirty = true;
    e->drop_graphs();
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

int recount_cells(lg_engine* e) {
    int rc = clear_status_bits(e, ST_CELL_OVF);
    if (rc) return rc;
    CUDA_TRY(e, cudaMemsetAsync(e->cell_count.p, 0, (size_t)e->b.ncells * sizeof(int), e->stream));
    // The interrupted build may have left the cell order (cell_atoms) and its
    // inverse (perm) incomplete: both go back to the identity, a consistent
    // order that the rebuild replaces (the fixed-point copies are written
    // through perm before the cells are binned from them).
    launch_identity_order(e->b, e->stream);
    launch_request_rebuild(e->b, e->stream);
    return LG_OK;
}

std::string nonfinite_systems(lg_engine* e) {
    std::vector<uint32_t> flags(e->nsys, 0u);
    if (cudaMemcpy(flags.data(), e->sys_status.p, e->nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return "?";
    std::string out;
    for (int s = 0; s < e->nsys; s++)
        if (flags[s] & SYS_NONFINITE) out += (out.empty() ? "" : ", ") + std::to_string(s);
    return out;
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
void enqueue_forces(lg_engine* e, uint32_t terms, bool ev, cudaStream_t st, bool fixed_written) {
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
        if (status & ST_CELL_OVF) {
            rc = recount_cells(e);
            if (rc) return rc;
            continue;
        }
        if (status & ST_OVERFLOW) {
            rc = clear_status_bits(e, ST_OVERFLOW);
            if (rc) return rc;
            rc = regrow(e);
            if (rc) return rc;
            continue;
        }
        if (status & ST_NONFINITE) {
            rc = clear_status_bits(e, ST_NONFINITE);
            if (rc) return rc;
            if (want & LG_WANT_ENERGY)
                return fail(e, LG_ERR_NONFINITE, "Potential energy is infinite! (system " + nonfinite_systems(e) + ")");
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
    e->shadow_valid = false;
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
int get_state_mapped(lg_engine* e, int64_t base, int64_t n, double* dp, double* dv) {
    Batch sub = e->b;
    sub.n = (int)n;
    sub.posq = e->posq.p + base;
    sub.vel = e->vel.p + base;
    launch_unpack_state(sub, dp, dv, e->stream);
    e->launches += n ? 1 : 0;
    return LG_OK;
}

int get_state(lg_engine* e, int64_t base, int64_t n, double* positions, double* velocities) {
    cudaStream_t st = e->stream;
    Batch sub = e->b;
    sub.n = (int)n;
    sub.posq = e->posq.p + base;
    sub.vel = e->vel.p + base;
    if (positions && velocities) {  // one launch for both when the host arrays are page-locked
        double* dp = (double*)mapped_host(positions);
        double* dv = (double*)mapped_host(velocities);
        if (dp && dv) {
            launch_unpack_state(sub, dp, dv, st);
            e->launches += 1;
            return LG_OK;
        }
    }
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
    e->shadow_valid = false;
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

// Threads per atom for a batch the persistent kernel runs, from launches of the
// persistent kernel itself (the per-step pair kernel ranks the widths
// differently: the persistent force phase pays a tail of one chunk and an
// epilogue per chunk, and 2 and 4 threads per atom timed alike there while the
// persistent kernel ran 16 % faster at 2).  Each width runs a warm-up and a
// timed launch of 16 steps from the current state, which every launch's own
// checkpoint restores afterwards; the lists the trials built stay valid for
// the restored positions (the rebuild test is relative to each list's build
// positions).
// *planned: whether some width got a persistent plan (else the batch runs on the
// per-step kernels, which the caller then tunes).
static int tune_persistent(lg_engine* e, cudaEvent_t e0, cudaEvent_t e1, bool* planned) {
    *planned = false;
    cudaStream_t st = e->stream;
    const bool thermo = (md_mode(e) & MD_ADJUST) != 0;
    const size_t bytes = (size_t)e->b.n * sizeof(double4_32a);
    const int tpas[4] = {1, 2, 4, 8};
    int best_tpa = e->b.tpa;
    float best_t = 1e30f;
    for (int t : tpas) {
        e->b.tpa = t;
        int rc = persist_plan(e);
        if (rc) return rc;
        if (e->pk_cluster <= 0) continue;
        float ms = 0.f;
        for (int r = 0; r < 2; r++) {
            CUDA_TRY(e, cudaEventRecord(e0, st));
            rc = md_run_persistent(e, 16, thermo, {});
            CUDA_TRY(e, cudaEventRecord(e1, st));
            CUDA_TRY(e, cudaEventSynchronize(e1));
            CUDA_TRY(e, cudaEventElapsedTime(&ms, e0, e1));
            // (the launch's first step wrote the checkpoint)
            CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, e->cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, e->cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, e->cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
            if (rc) return rc;
        }
        if (ms < best_t) {
            best_t = ms;
            best_tpa = t;
        }
    }
    CUDA_TRY(e, cudaStreamSynchronize(st));
    e->nonfinite = false;
    e->b.tpa = best_tpa;
    e->pk_cluster = 0;  // planned again for the chosen width at the next run
    *planned = best_t < 1e30f;
    return LG_OK;
}

// The autotuner: times the pair kernel at every threads-per-atom width (for a
// batch the persistent kernel runs: the persistent kernel's launches) and the
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
    const bool pb = std::get<5>(key);
    bool planned = false;
    if (pb) {
        int rc = tune_persistent(e, e0, e1, &planned);
        if (rc) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }
    }
    if (!planned) {
        const int tpas[6] = {1, 2, 4, 8, 16, 32};
        int best_tpa = b.tpa;
        float best_t = 1e30f;
        for (int t : tpas) {
            b.tpa = t;
            float ms = time_it([&] { launch_pair_forces(b, LG_TERM_ALL, false, st); });
            if (ms < best_t) {
                best_t = ms;
                best_tpa = t;
            }
        }
        b.tpa = best_tpa;
    }
    float best_t = 1e30f;
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
// only, Velocity-Verlet with at most a Berendsen thermostat.  It also needs a group size of 1, 2, 4 or 8 threads per atom (the
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
    return persist_batch(e) && (t == 1 || t == 2 || t == 4 || t == 8);
}

// Lowers the most loaded group while a move of one of its systems to another
// group, or a swap with a lighter system of another group, makes both loads
// smaller than its load (the best such change first).
static void refine_bins(std::vector<std::vector<int>>& bins, std::vector<double>& load,
                        const std::vector<double>& work) {
    const int G = (int)bins.size();
    for (int iter = 0; iter < 512; iter++) {
        int gm = (int)(std::max_element(load.begin(), load.end()) - load.begin());
        double best = load[gm];
        int bg = -1, ba = -1, bb = -1;  // group, index in gm, index in group (-1: a move)
        for (int g = 0; g < G; g++) {
            if (g == gm) continue;
            for (int x = 0; x < (int)bins[gm].size(); x++) {
                double wa = work[bins[gm][x]];
                if ((int)bins[g].size() < PK_MAXG) {
                    double m = std::max(load[gm] - wa, load[g] + wa);
                    if (m < best * (1.0 - 1e-9)) best = m, bg = g, ba = x, bb = -1;
                }
                for (int y = 0; y < (int)bins[g].size(); y++) {
                    double d = wa - work[bins[g][y]];
                    if (d <= 0.0) continue;
                    double m = std::max(load[gm] - d, load[g] + d);
                    if (m < best * (1.0 - 1e-9)) best = m, bg = g, ba = x, bb = y;
                }
            }
        }
        if (bg < 0) return;
        int a = bins[gm][ba];
        bins[gm].erase(bins[gm].begin() + ba);
        load[gm] -= work[a];
        if (bb >= 0) {
            int c = bins[bg][bb];
            bins[bg].erase(bins[bg].begin() + bb);
            load[bg] -= work[c];
            bins[gm].push_back(c);
            load[gm] += work[c];
        }
        bins[bg].push_back(a);
        load[bg] += work[a];
    }
}

// Packs the systems into groups of about equal work for each cluster size the
// device can hold (longest first, each to the least loaded group, then single
// moves and pairwise swaps out of the most loaded group while they lower it),
// and keeps the size whose largest group per block is smallest.  A system's
// arithmetic does not depend on its group.
int persist_plan(lg_engine* e) {
    e->pk_cluster = -1;
    for (auto& g : e->pk_graphs) cudaGraphExecDestroy(g.second);  // (they hold the old groups)
    e->pk_graphs.clear();
    const Batch& b = e->b;
    int nsys = e->nsys;
    // work of a system: its neighbour-list entries (measured when the lists
    // exist, else estimated from the density) plus a per-atom share.  The
    // share is fitted to the per-cluster times of the first-half and force
    // phases on batched LJ replicas: an atom costs about as much as 32 list
    // entries (its FP64 integration, its chunk's epilogue and lane padding)
    std::vector<int> h_nnb(b.n);
    CUDA_TRY(e, cudaMemcpy(h_nnb.data(), e->nnb.p, (size_t)b.n * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<double> work(nsys);
    for (int s = 0; s < nsys; s++) {
        const HostSystem& h = e->sys[s];
        double V = h.cell.volume;
        double rl = e->h_sysdev[s].rlist;
        double entries = 0.0;
        for (int64_t i = e->begin[s]; i < e->begin[s + 1]; i++) entries += h_nnb[i];
        if (entries == 0.0) entries = (double)h.n * (double)h.n / V * 4.0 / 3.0 * PI * rl * rl * rl;
        work[s] = entries + 32.0 * (double)h.n;
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
        refine_bins(bins, load, work);
        double waves = std::ceil((double)G / (double)gmax);
        double t = *std::max_element(load.begin(), load.end()) / C * waves;
        if (best_c == 0 || t < 0.97 * best_t) {
            best_t = t;
            best_c = C;
            best_bins = bins;
        }
    }
    if (best_c == 0) return LG_OK;  // no cluster fits: the per-step kernels run
    // One cluster owns a group for the whole launch, so a group much larger
    // than an even share of the device (a large system among few) would run
    // on a few SMs while the per-step kernels spread it over all of them: the
    // per-step kernels run instead, unless the batch is small enough that
    // launch latency, not throughput, sets the time.
    {
        double total = 0.0;
        for (double w : work) total += w;
        int sms = std::max(1, b.sms);
        double persistent_t = best_t;             // largest group per block (times waves)
        double spread_t = total / (double)sms;    // an even spread over every SM
        if (b.n > 32768 && persistent_t > 2.0 * spread_t) return LG_OK;
    }
    std::vector<int> off(1, 0), sys;
    for (auto& bin : best_bins) {
        if (bin.empty()) continue;
        // the force phase hands out chunks in group order: the systems with the
        // most work per atom first, so the last chunks, whose length sets the
        // wait at the closing barrier, are the cheapest (a system's results do
        // not depend on its place in the group)
        std::stable_sort(bin.begin(), bin.end(), [&](int x, int y) {
            double wx = work[x] / (double)std::max<int64_t>(1, e->sys[x].n);
            double wy = work[y] / (double)std::max<int64_t>(1, e->sys[y].n);
            return wx > wy;
        });
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
    const int stage_max = e->b.lj1 ? PK_STAGE_MAX_LJ1 : PK_STAGE_MAX;
    e->pk_stage = (stage <= stage_max && (e->opt.flags & LG_OPT_STAGING)) ? stage : 0;
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
// Steps per persistent launch at most.  A launch ends when its slowest cluster
// does, and a cluster's list rebuilds (about 130 us each on the 128-replica
// batch) fall on random steps, so longer launches average them out: 32, 64,
// 128 and 256 steps a launch measured 98.5, 94.9, 93.3 and 92.6 us a step.
// An overflowing list replays the launch from its checkpoint.
constexpr int PK_MAX_STEPS = 256;

int md_run_persistent(lg_engine* e, int64_t nsteps, bool thermo, const std::function<int()>& tail) {
    const int chunk = PK_MAX_STEPS;
    cudaStream_t st = e->stream;
    int64_t done = 0;
    int retries = 0;
    size_t bytes = e->b.n * sizeof(double4_32a);
    if (nsteps == 0 && tail) {
        int rc = tail();
        if (rc) return rc;
        CUDA_TRY(e, cudaStreamSynchronize(st));
    }
    while (done < nsteps) {
        int steps = (int)std::min<int64_t>(chunk, nsteps - done);
        int key = 2 * steps + (thermo ? 1 : 0);
        auto it = e->pk_graphs.find(key);
        if (it == e->pk_graphs.end()) {
            cudaGraph_t g;
            CUDA_TRY(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            // (the kernel's first step writes the checkpoint and clears the group flags)
            PkArgs a{e->pk_groups, e->pk_group_off.p, e->pk_group_sys.p, e->pk_group_flag.p, e->pk_ke.p, steps,
                     thermo ? 1 : 0, e->pk_stage, e->cp_pos.p, e->cp_vel.p, e->cp_acc.p};
            cudaError_t le = launch_md_persist(e->b, a, e->pk_cluster, st);
            // the status word reaches the host inside the graph (no copy call per launch)
            if (le == cudaSuccess) {
                launch_status_copy(e->status.p, e->d_h_status, st);
                le = cudaGetLastError();
            }
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
        e->launches += 2;
        // the caller's download of the last chunk goes before the wait, so one
        // wait covers the launch, its status word and the download (a replayed
        // chunk enqueues the download again)
        if (done + steps == nsteps && tail) {
            int rc = tail();
            if (rc) return rc;
        }
        CUDA_TRY(e, cudaStreamSynchronize(st));
        uint32_t status = *(volatile const uint32_t*)e->h_status;
        int rc = LG_OK;
        if (status & (ST_OVERFLOW | ST_CELL_OVF)) {
            if (++retries > 4) return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
            CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, e->cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, e->cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
            CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, e->cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
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

// ---- Berendsen barostat -----------------------------------------------------------
int md_run_barostat(lg_engine* e, int64_t nsteps) {
    const double WATER_COMPRESSIBILITY = 7372.0;  // integrators.rs:171 (from DL_POLY)
    const int mode = md_mode(e);
    const bool thermo = (mode & MD_ADJUST) != 0;
    cudaStream_t st = e->stream;
    const int nsys = e->nsys;
    CUDA_TRY(e, e->kin.alloc(nsys));
    CUDA_TRY(e, e->kten.alloc(9 * (size_t)nsys));
    std::vector<double> kin(nsys), kten(9 * (size_t)nsys), out((size_t)nsys * RED_STRIDE);
    bool aniso = false;
    for (int s = 0; s < nsys; s++) aniso = aniso || e->sys[s].barostat == LG_BAROSTAT_ANISO_BERENDSEN;
    const size_t bytes = (size_t)e->b.n * sizeof(double4_32a);
    const size_t cbytes = (size_t)nsys * sizeof(unsigned long long);
    for (int64_t step = 0; step < nsteps; step++) {
        // UnitCell::scale_mut(eta^3 * 1) of every barostat system (integrators.rs:227-236)
        for (int s = 0; s < nsys; s++) {
            HostSystem& h = e->sys[s];
            if (h.barostat == LG_BAROSTAT_NONE) continue;
            const bool an = h.barostat == LG_BAROSTAT_ANISO_BERENDSEN;
            double eta = h.baro_eta;
            double e3 = eta * eta * eta;
            // cell * (e3 * 1), or cell * eta of the anisotropic barostat
            // (integrators.rs:309), with Matrix3's product (matrix.rs:342-388)
            const double fi[9] = {e3, 0.0 * e3, 0.0 * e3, 0.0 * e3, e3, 0.0 * e3, 0.0 * e3, 0.0 * e3, e3};
            const double* f = an ? h.baro_m : fi;
            double m[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    m[3 * i + j] = h.cell.m[3 * i] * f[j] + h.cell.m[3 * i + 1] * f[3 + j] + h.cell.m[3 * i + 2] * f[6 + j];
            HostCell cell;
            // (a factor eta <= 0 inverts or collapses the cell: the reference panics as well)
            bool valid = (an || eta > 0.0) && cell_init(cell, m, h.cell.shape);
            const double* L = cell.len;
            double rc = max_cutoff(h);
            if (!valid || 0.5 * L[0] <= rc || 0.5 * L[1] <= rc || 0.5 * L[2] <= rc)
                return fail(e, LG_ERR_ARGUMENT,
                            std::string(an ? "Tried to decrease the cell size in anisotropic Berendesen barostat "
                                           : "Tried to decrease the cell size in Berendesen barostat ") +
                                "but the new size is smaller than the interactions cut off radius. You can try to "
                                "increase the cell size or the number of particles. (system " + std::to_string(s) + ")");
            e->h_sysdev[s].baro_eta = eta;
            for (int k = 0; k < 9; k++) e->h_sysdev[s].baro_m[k] = h.baro_m[k];
            int rc2 = set_cell_fast(e, s, cell);
            if (rc2 != LG_OK && rc2 != -1) return rc2;
            if (rc2 == -1) {  // another cell grid or k-vector set: lower the batch again, keeping the state
                set_host_cell(h, cell);
                invalidate(e);
                int rc3 = commit_carried(e);
                if (rc3) return rc3;
                CUDA_TRY(e, e->kin.alloc(nsys));
                CUDA_TRY(e, e->kten.alloc(9 * (size_t)nsys));
            }
        }
        CUDA_TRY(e, cudaMemcpyAsync(e->cp_pos.p, e->posq.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->cp_vel.p, e->vel.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->cp_acc.p, e->acc.p, bytes, cudaMemcpyDeviceToDevice, st));
        if (thermo) CUDA_TRY(e, cudaMemcpyAsync(e->cp_count.p, e->md_count.p, cbytes, cudaMemcpyDeviceToDevice, st));
        for (int attempt = 0;; attempt++) {
            // the step: the first half (with the previous step's thermostat and
            // controls), the forces with the virial, the kinetic energy of the
            // half-step velocities, the second half
            bool adjust = thermo && step > 0;
            if (adjust && (mode & MD_REWRAP)) {
                launch_rewrap(e->b, st);
                e->launches += e->b.nmol ? 1 : 0;
            }
            launch_md_first(e->b, adjust, st);
            CUDA_TRY(e, cudaMemsetAsync(e->red.p, 0, (size_t)e->b.n * RED_STRIDE * sizeof(double), st));
            enqueue_forces(e, LG_TERM_ALL, true, st, !(mode & MD_VERLET_SYS));
            launch_reduce(e->b, LG_TERM_ALL, e->b.nkvec != 0, e->out.p, st);
            launch_kinetic(e->b, e->kin.p, st);
            if (aniso) {
                launch_kinetic_tensor(e->b, e->kten.p, st);
                e->launches += 1;
            }
            launch_md_second(e->b, st);
            e->launches += (e->b.ntiles ? 2 : 0) + 2;
            if (mode & MD_ADJUST) {
                launch_md_adjust(e->b, st);
                e->launches += 1;
            }
            CUDA_TRY(e, cudaGetLastError());
            CUDA_TRY(e, cudaMemcpyAsync(kin.data(), e->kin.p, nsys * sizeof(double), cudaMemcpyDeviceToHost, st));
            if (aniso)
                CUDA_TRY(e, cudaMemcpyAsync(kten.data(), e->kten.p, 9 * nsys * sizeof(double), cudaMemcpyDeviceToHost,
                                            st));
            CUDA_TRY(e, cudaMemcpyAsync(out.data(), e->out.p, out.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        st));
            uint32_t status;
            int rc = read_status(e, &status);
            if (rc) return rc;
            if (status & (ST_OVERFLOW | ST_CELL_OVF)) {
                if (attempt >= 4) return fail(e, LG_ERR_CAPACITY, "neighbour list overflow persisted after regrowing");
                CUDA_TRY(e, cudaMemcpyAsync(e->posq.p, e->cp_pos.p, bytes, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(e, cudaMemcpyAsync(e->vel.p, e->cp_vel.p, bytes, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(e, cudaMemcpyAsync(e->acc.p, e->cp_acc.p, bytes, cudaMemcpyDeviceToDevice, st));
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
            if (status & ST_NONFINITE) {
                e->nonfinite = true;
                rc = clear_status_bits(e, ST_NONFINITE);
                if (rc) return rc;
            }
            break;
        }
        // System::pressure at the new positions with the half-step velocities
        // (Pressure, sys/compute.rs:399-431), and the next step's factor
        for (int s = 0; s < nsys; s++) {
            HostSystem& h = e->sys[s];
            if (h.barostat == LG_BAROSTAT_NONE) continue;
            const double* w = &out[(size_t)s * RED_STRIDE + 1];
            if (h.barostat == LG_BAROSTAT_ANISO_BERENDSEN) {
                // Stress (compute.rs:466-480): (sum m v (x) v + W) / V; then
                // eta = 1 - dt 7372 / tau (stress0 - stress), made symmetric
                // (integrators.rs:322-331)
                const double factor = h.dt * WATER_COMPRESSIBILITY / h.baro_tau;
                double eta[9];
                for (int k = 0; k < 9; k++) {
                    double stress = (kten[9 * (size_t)s + k] + w[k]) / h.cell.volume;
                    eta[k] = (k % 4 == 0 ? 1.0 : 0.0) - factor * (h.baro_stress[k] - stress);
                }
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < i; j++) {
                        eta[3 * i + j] = 0.5 * (eta[3 * i + j] + eta[3 * j + i]);
                        eta[3 * j + i] = eta[3 * i + j];
                    }
                for (int k = 0; k < 9; k++) h.baro_m[k] = eta[k];
                continue;
            }
            double dof = (double)(3 * h.n);
            double T = 2.0 * kin[s] / (dof * K_BOLTZMANN);  // Temperature (compute.rs:164-172)
            double volume = h.cell.volume;
            double P = (dof * K_BOLTZMANN * T + (w[0] + w[4] + w[8])) / (3.0 * volume);
            double eta3 = 1.0 - WATER_COMPRESSIBILITY / h.baro_tau * (h.baro_pressure - P);
            h.baro_eta = std::cbrt(eta3);
        }
    }
    enqueue_md_finish(e, mode, st);
    CUDA_TRY(e, cudaGetLastError());
    return LG_OK;
}

}  // namespace lg
