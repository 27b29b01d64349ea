// persist.cu -- batched MD of pair-potential systems in one persistent launch.
//
// Independent replicas (Lumol systems with pair potentials only: no bonds, no
// restrictions, no Coulomb) are packed into groups of about equal work, and
// one thread-block cluster owns a group for a whole run of steps.  A step of
// a group is a sequence of phases over its atoms, separated by cluster
// barriers: the first Velocity-Verlet half (integrators.rs:45-53) with the
// previous step's Berendsen factor (thermostats.rs:113-120), the neighbour
// list rebuild of the group's systems that moved more than skin / 2, the
// forces (the mixed path's compensated FP32 pair sums) fused with the second
// half (integrators.rs:55-68) and the kinetic energy of each chunk of atoms;
// every block derives the Berendsen factors from those at the next step.  Groups never wait for one another, so a rebuild in
// one replica delays only its own cluster, and a step costs no kernel launch.
//
// The arithmetic is the per-step mixed path's (same list, same order of the
// force sums, same fixed-point positions); results agree with it to rounding
// (the thermostat's kinetic energy is summed per chunk instead of per tile).
#include <cooperative_groups.h>

#include "kernels.h"
#include "mixed_common.cuh"

namespace cg = cooperative_groups;

namespace lg {

constexpr int PK_THREADS = 1024;
constexpr int PK_WARPS = PK_THREADS / 32;
constexpr int PK_SORT = 128;  // per-warp buffer of the cell sort

// last r in [0, R) with pre[r] <= v
__device__ __forceinline__ int pk_find(const int* pre, int R, int v) {
    int a = 0, b = R - 1;
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (pre[mid] <= v) a = mid;
        else b = mid - 1;
    }
    return a;
}

// This block's share [lo, hi) of n items split evenly over the C blocks of a
// cluster: contiguous (coalesced) and within one item of the others, so no
// block of a phase that ends at a cluster barrier carries more than its share.
__device__ __forceinline__ int2 pk_share(int n, int rank, int C) {
    return make_int2((int)((long long)n * rank / C), (int)((long long)n * (rank + 1) / C));
}

// Cluster-wide barrier.  barrier.cluster.arrive has release and
// barrier.cluster.wait acquire semantics at cluster scope, so every global
// write made before the barrier is visible to every block of the cluster
// after it.
__device__ __forceinline__ void pk_sync(cg::cluster_group& cluster) { cluster.sync(); }

// Berendsen factor sqrt(1 + (T0 / T - 1) / tau) (thermostats.rs:113-120) of
// each system of the group, T = 2 K / (dof kB) (compute.rs:133-144), K summed
// over the system's force-phase chunks in a fixed order (lane-strided, then a
// fixed shuffle tree), so every block of the cluster computes the same factors
// without another barrier.  Warp w of the block handles systems w, w + 32, ...
__device__ __forceinline__ void pk_lambdas(const Batch& b, const PkArgs& a, const int* s_sys, int G, int wib,
                                           int lane, int gpw, double* s_lambda) {
    for (int r = wib; r < G; r += PK_WARPS) {
        const SysDev& sd = b.sys[s_sys[r]];
        // (a persistent batch has Berendsen thermostats or none: thermostat_factor's arithmetic)
        double k = chunk_ke_sum(sd, a.ke, gpw, lane);
        double f = sd.thermostat == TH_BERENDSEN ? berendsen_factor(sd, k) : 1.0;
        if (lane == 0) s_lambda[r] = f;
    }
}

// Every block of a cluster runs the same sequence of cluster barriers: the
// loop over steps, the rebuild branch (decided from flags that are only
// written before a barrier and cleared after the rebuild's last barrier) and
// the early exit on a list overflow (a per-group flag read after a barrier)
// are the same in every block.
// LJ1: every system has one kind and a Lennard-Jones pair (a force loop with
// the pair type and the one-kind parameters resolved when it is compiled, the
// cutoff a select; staging, if asked for, holds positions only).
template <int TPA, bool LJ1>
__global__ void __launch_bounds__(PK_THREADS, 1) md_persist_kernel(Batch b, PkArgs a) {
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int g = blockIdx.x / C;
    if (g >= a.ngroups) return;  // every block of this cluster

    __shared__ int s_sys[PK_MAXG];
    __shared__ int s_apre[PK_MAXG + 1];
    __shared__ int s_qpre[PK_MAXG + 1];  // force-phase chunk prefix over the group's systems
    __shared__ double s_lambda[PK_MAXG];
    __shared__ int s_rsys[PK_MAXG];      // systems rebuilt at this step
    __shared__ int s_rapre[PK_MAXG + 1];
    __shared__ int s_rcpre[PK_MAXG + 1];
    __shared__ int s_R;
    __shared__ int s_part[PK_THREADS];
    __shared__ int s_lo[PK_WARPS][NL_RUNS], s_pre[PK_WARPS][NL_RUNS + 1];
    __shared__ __align__(16) int s_buf[PK_WARPS][PK_SORT];
    // the force phase's per-warp epilogue buffers reuse the list build's
    // (phases are separated by cluster barriers): 32 FP32 accelerations, their
    // atoms, and the (system slot, chunk) of each buffered chunk
    static_assert(PK_SORT * sizeof(int) >= 32 * sizeof(float4), "epilogue buffer");
    static_assert(NL_RUNS >= 32 && NL_RUNS + 1 >= 2 * 8, "epilogue buffer");
    float4(*s_epa)[32] = reinterpret_cast<float4(*)[32]>(s_buf);
    int(*s_epi)[NL_RUNS] = s_lo;
    int(*s_epq)[NL_RUNS + 1] = s_pre;
    extern __shared__ uint4 s_dyn[];  // staged positions (a.stage atoms), then their kinds (not LJ1)
    uint4* s_pos = s_dyn;
    int* s_kind = reinterpret_cast<int*>(s_dyn + a.stage);

    const int gb = a.group_off[g];
    const int G = a.group_off[g + 1] - gb;
    constexpr int GPW = 32 / TPA;  // atoms of a force-phase chunk (one warp)
    if (threadIdx.x == 0) {
        int acc = 0, chunks = 0;
        for (int r = 0; r < G; r++) {
            int s = a.group_sys[gb + r];
            int n = b.sys[s].end - b.sys[s].begin;
            s_sys[r] = s;
            s_apre[r] = acc;
            s_qpre[r] = chunks;
            acc += n;
            chunks += (n + GPW - 1) / GPW;
        }
        s_apre[G] = acc;
        s_qpre[G] = chunks;
    }
    // the group flag is read only after a cluster barrier: cleared here for this launch
    if (rank == 0 && threadIdx.x == 0) a.group_flag[g] = 0;
    __syncthreads();
    const int A = s_apre[G];
    const int QQ = s_qpre[G];
    const int wib = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int2 ash = pk_share(A, rank, C);  // this block's atoms of the group
    // the force phase hands out chunks from a counter in rank 0's shared
    // memory (one atomic per chunk and warp), so the blocks of the cluster
    // reach its closing barrier together whatever the chunks cost
    __shared__ int s_next;
    int* next_chunk = cluster.map_shared_rank(&s_next, 0);
    bool ran = false;

    for (int step = 0; step < a.nsteps; step++) {
        // ---- 1: [v *= lambda]; v += dt/2 a; x += v dt; fixed-point copy; displacement test
        const bool apply = a.thermo && step > 0;
        // (the previous step's chunks were all taken before its closing barrier)
        if (rank == 0 && threadIdx.x == 0) s_next = 0;
        if (apply) {
            pk_lambdas(b, a, s_sys, G, wib, lane, GPW, s_lambda);
            __syncthreads();
        }
        for (int v = ash.x + threadIdx.x; v < ash.y; v += PK_THREADS) {
            int r = pk_find(s_apre, G, v);
            int s = s_sys[r];
            const SysDev& sd = b.sys[s];
            int i = sd.begin + (v - s_apre[r]);
            double4_32a vel = b.vel[i], acc = b.acc[i], p = b.posq[i];
            if (step == 0 && a.cp_pos) {  // the launch's checkpoint
                a.cp_pos[i] = p;
                a.cp_vel[i] = vel;
                a.cp_acc[i] = acc;
            }
            if (apply) {
                double f = s_lambda[r];
                vel.x *= f;
                vel.y *= f;
                vel.z *= f;
            }
            vel.x = fma(sd.hdt, acc.x, vel.x);
            vel.y = fma(sd.hdt, acc.y, vel.y);
            vel.z = fma(sd.hdt, acc.z, vel.z);
            p.x = fma(vel.x, sd.dt, p.x);
            p.y = fma(vel.y, sd.dt, p.y);
            p.z = fma(vel.z, sd.dt, p.z);
            b.vel[i] = vel;
            b.posq[i] = p;
            flag_nonfinite(p.x, p.y, p.z, s, b.sys_status, b.status);
            uint4 u = fixed_xyz_ortho(sd, p);
            store_fixed_xyz(b.posfx + b.perm[i], u);
            if (fixed_dist2(u, b.pfx_build[i], sd.Lq) > sd.rebuild2_f) b.sys_rebuild[s] = 1u;
        }
        pk_sync(cluster);

        // ---- 2: rebuild the lists of the systems that asked for it
        if (threadIdx.x == 0) {
            int R = 0, ac = 0, cc = 0;
            for (int r = 0; r < G; r++) {
                int s = s_sys[r];
                if (*(volatile const uint32_t*)&b.sys_rebuild[s]) {
                    const SysDev& sd = b.sys[s];
                    s_rsys[R] = s;
                    s_rapre[R] = ac;
                    s_rcpre[R] = cc;
                    ac += sd.end - sd.begin;
                    cc += sd.ncell[0] * sd.ncell[1] * sd.ncell[2];
                    R++;
                }
            }
            s_rapre[R] = ac;
            s_rcpre[R] = cc;
            s_R = R;
        }
        __syncthreads();
        const int R = s_R;
        if (R > 0) {
            const int RA = s_rapre[R], RC = s_rcpre[R];
            const int2 rsh = pk_share(RA, rank, C), csh = pk_share(RC, rank, C);
            // 2a: cell of each atom from its fixed-point copy (written in phase 1:
            // u / 2^32 is the wrapped fraction of the cell, so the cell index is
            // (u * ncell) >> 32, integer arithmetic only), build positions
            for (int v = rsh.x + threadIdx.x; v < rsh.y; v += PK_THREADS) {
                int r = pk_find(s_rapre, R, v);
                const SysDev& sd = b.sys[s_rsys[r]];
                int i = sd.begin + (v - s_rapre[r]);
                int cell = fixed_cell(sd, b.posfx[b.perm[i]]);
                b.atom_cell[i] = cell;
                atomicAdd(&b.cell_count[cell], 1);
                b.pos_build[i] = b.posq[i];
            }
            pk_sync(cluster);
            // 2b: exclusive scan of each system's cell counts (one block per system)
            for (int q = rank; q < R; q += C) {
                int s = s_rsys[q];
                const SysDev& sd = b.sys[s];
                int ncells = sd.ncell[0] * sd.ncell[1] * sd.ncell[2];
                int* count = b.cell_count + sd.cell_begin;
                int* start = b.cell_start + sd.cell_begin + s;
                int t = threadIdx.x;
                int per = (ncells + PK_THREADS - 1) / PK_THREADS;
                int lo = min(t * per, ncells), hi = min(lo + per, ncells);
                int sum = 0;
                for (int c = lo; c < hi; c++) sum += count[c];
                __syncthreads();
                s_part[t] = sum;
                __syncthreads();
                for (int o = 1; o < PK_THREADS; o <<= 1) {
                    int x = t >= o ? s_part[t - o] : 0;
                    __syncthreads();
                    s_part[t] += x;
                    __syncthreads();
                }
                // starts clamped to the system's slice of cell_atoms: stale counts
                // (an interrupted earlier build) keep every later pass in bounds,
                // flag the group, and the host recounts and replays
                int run = sd.begin + s_part[t] - sum;
                for (int c = lo; c < hi; c++) {
                    start[c] = min(run, sd.end);
                    run += count[c];
                    count[c] = 0;
                }
                if (t == PK_THREADS - 1) {
                    start[ncells] = min(sd.begin + s_part[t], sd.end);
                    if (sd.begin + s_part[t] != sd.end) {
                        atomicOr(b.status, ST_CELL_OVF);
                        a.group_flag[g] = 1;
                    }
                }
            }
            pk_sync(cluster);
            // 2c: scatter the atoms into their cells
            for (int v = rsh.x + threadIdx.x; v < rsh.y; v += PK_THREADS) {
                int r = pk_find(s_rapre, R, v);
                int s = s_rsys[r];
                int i = b.sys[s].begin + (v - s_rapre[r]);
                int c = b.atom_cell[i];
                int slot = atomicAdd(&b.cell_count[c], 1);
                int at = b.cell_start[c + s] + slot;
                if (at < b.cell_start[c + s + 1] && at >= b.sys[s].begin && at < b.sys[s].end) {
                    b.cell_atoms[at] = i;
                } else {  // never written out of range: the host recounts and replays
                    atomicOr(b.status, ST_CELL_OVF);
                    a.group_flag[g] = 1;
                }
            }
            pk_sync(cluster);
            // 2d: sort each cell by atom index (warp per cell), leave the counts at zero
            for (int vc = csh.x + wib; vc < csh.y; vc += PK_WARPS) {
                int r = pk_find(s_rcpre, R, vc);
                int s = s_rsys[r];
                int c = b.sys[s].cell_begin + (vc - s_rcpre[r]);
                int lo = b.cell_start[c + s], hi = b.cell_start[c + s + 1];
                int m = hi - lo;
                __syncwarp();
                if (m <= PK_SORT) {
                    for (int x = lane; x < m; x += 32) s_buf[wib][x] = b.cell_atoms[lo + x];
                    __syncwarp();
                    for (int x = lane; x < m; x += 32) {
                        int val = s_buf[wib][x], rk = 0;
                        for (int y = 0; y < m; y++) rk += s_buf[wib][y] < val;
                        b.cell_atoms[lo + rk] = val;
                    }
                } else if (lane == 0) {
                    for (int x = lo + 1; x < hi; x++) {
                        int val = b.cell_atoms[x];
                        int y = x - 1;
                        while (y >= lo && b.cell_atoms[y] > val) {
                            b.cell_atoms[y + 1] = b.cell_atoms[y];
                            y--;
                        }
                        b.cell_atoms[y + 1] = val;
                    }
                }
                if (lane == 0) b.cell_count[c] = 0;
            }
            pk_sync(cluster);
            // 2e: sorted position of each atom, sorted (kind, molecule), fixed-point copies
            for (int v = rsh.x + threadIdx.x; v < rsh.y; v += PK_THREADS) {
                int r = pk_find(s_rapre, R, v);
                const SysDev& sd = b.sys[s_rsys[r]];
                int t = sd.begin + (v - s_rapre[r]);
                int i = b.cell_atoms[t];
                b.perm[i] = t;
                b.km[t] = make_int2(b.kind[i], b.mol[i]);
                uint4 u = fixed_position_ortho(sd, b.posq[i]);
                b.posfx[t] = u;
                b.pfx_build[i] = u;
            }
            pk_sync(cluster);
            // 2f: Verlet list rows, one warp per cell.  The cell's stencil table and
            // each 32-candidate chunk of fixed-point positions are gathered once and
            // tested against every atom of the cell (a cell's atoms share one
            // stencil); each row keeps the candidate order of the per-step list
            // build, so the rows are the same
            for (int vc = csh.x + wib; vc < csh.y; vc += PK_WARPS) {
                int r = pk_find(s_rcpre, R, vc);
                int si = s_rsys[r];
                const SysDev& sd = b.sys[si];
                int local = vc - s_rcpre[r];
                int c = sd.cell_begin + local;
                int lo = b.cell_start[c + si], hi = b.cell_start[c + si + 1];
                if (hi <= lo) continue;  // (the same in every lane)
                __syncwarp();            // the previous cell's readers of s_lo / s_pre are done
                int2 nt = stencil_table(sd, si, local, b.cell_start, lane, s_lo[wib], s_pre[wib]);
                const int nruns = nt.x, total = nt.y;
                __syncwarp();
                // (in registers: the row stores below could alias the system record)
                const float rl2 = sd.rlist2_f;
                const float Lq[3] = {sd.Lq[0], sd.Lq[1], sd.Lq[2]};
                const int maxnb = b.maxnb;
                int* const nbr = b.nbr;
                const unsigned below = (1u << lane) - 1u;
                for (int a0 = lo; a0 < hi; a0 += 32) {  // the cell's atoms, 32 at a time
                    const int na = min(32, hi - a0);
                    const uint4 ua = lane < na ? b.posfx[a0 + lane] : make_uint4(0u, 0u, 0u, 0u);
                    int count = 0;  // row length of atom a0 + lane
                    // four 32-candidate chunks per pass, their gathers in flight together
                    for (int base = 0; base < total; base += 128) {
                        int slot[4];
                        uint4 uj[4];
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            int q = base + 32 * h + lane;
                            slot[h] = q < total ? stencil_slot(s_lo[wib], s_pre[wib], nruns, q) : -1;
                        }
#pragma unroll
                        for (int h = 0; h < 4; h++) uj[h] = slot[h] >= 0 ? b.posfx[slot[h]] : ua;
                        for (int k = 0; k < na; k++) {
                            uint4 ui;
                            ui.x = __shfl_sync(0xffffffffu, ua.x, k);
                            ui.y = __shfl_sync(0xffffffffu, ua.y, k);
                            ui.z = __shfl_sync(0xffffffffu, ua.z, k);
                            const int t = a0 + k;
                            int at = __shfl_sync(0xffffffffu, count, k);
#pragma unroll
                            for (int h = 0; h < 4; h++) {  // candidate order: chunk by chunk
                                if (base + 32 * h >= total) break;  // (the same in every lane)
                                bool keep = slot[h] >= 0 && slot[h] != t && fixed_dist2(ui, uj[h], Lq) < rl2;
                                unsigned mask = __ballot_sync(0xffffffffu, keep);
                                if (keep) {
                                    int pos = at + __popc(mask & below);
                                    if (pos < maxnb) nbr[(size_t)t * maxnb + pos] = slot[h];
                                }
                                at += __popc(mask);
                            }
                            if (lane == k) count = at;
                        }
                    }
                    if (lane < na) {
                        b.nnb[a0 + lane] = min(count, maxnb);
                        if (count > maxnb) {
                            atomicOr(b.status, ST_OVERFLOW);
                            a.group_flag[g] = 1;
                        }
                    }
                }
            }
            pk_sync(cluster);
            if (rank == 0 && threadIdx.x == 0)
                for (int q = 0; q < R; q++) b.sys_rebuild[s_rsys[q]] = 0u;
            // the same value in every block: the caller regrows and replays
            if (*(volatile const int*)&a.group_flag[g]) break;
        }

        // ---- 3: forces (compensated FP32 sums) fused with v += dt/2 a, a = F / m, kinetic energy
        {
            // every block stages the group's fixed-point positions (and kinds) in
            // shared memory (group order: the systems' sorted ranges one after
            // the other), so the neighbour gathers are shared-memory loads
            if (a.stage) {
                for (int v = threadIdx.x; v < A; v += PK_THREADS) {
                    int r = pk_find(s_apre, G, v);
                    int t = b.sys[s_sys[r]].begin + (v - s_apre[r]);
                    s_pos[v] = b.posfx[t];
                    if (!LJ1) s_kind[v] = b.km[t].x;
                }
                __syncthreads();
            }
            // warp chunks of GPW atoms of one system (chunk q of system r covers its
            // atoms q * GPW ...), so a chunk's kinetic energy belongs to one system.
            // The FP64 epilogue (a = F / m widened, v += dt/2 a, kinetic energy)
            // runs once every TPA chunks over the 32 buffered atoms, one atom a
            // lane: GB300 issues one FP64 warp instruction per about 19 cycles and
            // SM, so an epilogue with one atom per TPA lanes would pay TPA times
            // over.  The chunk sums of the kinetic energy take the same tree as a
            // whole-warp butterfly over one atom every TPA lanes (chunk_sum).
            const int sub = lane % TPA;
            int nbuf = 0;  // chunks buffered by this warp (warp-uniform)
            auto flush = [&]() {
                __syncwarp();
                const int c = lane / GPW;  // buffered chunk of this lane
                double ke = 0.0;
                int s = -1, qq = 0;
                if (c < nbuf) {
                    s = s_sys[s_epq[wib][2 * c]];
                    qq = s_epq[wib][2 * c + 1];
                    const int i = s_epi[wib][lane];
                    if (i >= 0) {
                        const SysDev& sd = b.sys[s];
                        const float4 a4 = s_epa[wib][lane];
                        double4_32a vel = b.vel[i];
                        double4_32a ai = make_double4_32a((double)a4.x, (double)a4.y, (double)a4.z, 0.0);
                        vel.x = fma(sd.hdt, ai.x, vel.x);
                        vel.y = fma(sd.hdt, ai.y, vel.y);
                        vel.z = fma(sd.hdt, ai.z, vel.z);
                        b.acc[i] = ai;
                        b.vel[i] = vel;
                        flag_nonfinite(vel.x, vel.y, vel.z, s, b.sys_status, b.status);
                        if (a.thermo) ke = 0.5 * vel.w * fma(vel.x, vel.x, fma(vel.y, vel.y, vel.z * vel.z));
                    }
                }
                if (a.thermo) {  // per chunk, lanes in a fixed order
#pragma unroll
                    for (int o = GPW / 2; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
                    if (c < nbuf && lane % GPW == 0) a.ke[b.sys[s].begin + qq] = ke;
                }
                nbuf = 0;
                __syncwarp();
            };
            int q = 0;
            if (lane == 0) q = atomicAdd(next_chunk, 1);
            q = __shfl_sync(0xffffffffu, q, 0);
            for (; q < QQ;) {
                int r = pk_find(s_qpre, G, q);
                const SysDev& sd = b.sys[s_sys[r]];
                int qq = q - s_qpre[r];
                int local = qq * GPW + lane / TPA;
                bool active = local < sd.end - sd.begin;
                int vv = s_apre[r] + (active ? local : 0);
                int tt = sd.begin + (vv - s_apre[r]);  // sorted position
                int i = b.cell_atoms[tt];
                uint4 pi = b.posfx[tt];
                int2 kmi = b.km[tt];
                const PairDevF* prow = b.ptabf + sd.ptab + kmi.x * sd.nk;
                MixedAcc acc;
                const bool single = sd.nk == 1;
                const int4 ph1 = __ldg(reinterpret_cast<const int4*>(prow));
                const float4 pq1 = __ldg(reinterpret_cast<const float4*>(prow) + 1);
                int cnt = active ? b.nnb[tt] : 0;
                const int* list = b.nbr + (size_t)tt * b.maxnb;
                const int off = sd.begin - s_apre[r];  // sorted position - group slot
                // rows walked as the per-step pair kernel walks them
                walk_row<TPA>(
                    list, cnt, sub,
                    [&](int js, uint4& pj, int2& kmj) {
                        if (a.stage) {
                            pj = s_pos[js - off];
                            kmj = make_int2(LJ1 ? 0 : s_kind[js - off], 0);
                        } else {  // (the neighbour's kind is not needed for one kind)
                            pj = b.posfx[js];
                            kmj = (LJ1 || single) ? make_int2(0, 0) : b.km[js];
                        }
                    },
                    [&](int js, const uint4& pj, const int2& kmj) {
                        mixed_entry<false, false, LJ1>(acc, sd, prow, pi, 0.0f, kmi.y, i, tt, js, pj, kmj, b.cell_atoms,
                                                  nullptr, nullptr, nullptr, true, false, 0.0f, 0.0f, 0.0f, single,
                                                  ph1, pq1, nullptr);
                    });
                group_combine<TPA>(acc);
                if (sub == 0) {
                    // as the per-step path: the compensated sum rounded once to FP32, a = F / m in FP32
                    const int slot = nbuf * GPW + lane / TPA;
                    if (active) {
                        float im = b.inv_mass[i];
                        s_epa[wib][slot] = make_float4(rmul(radd(acc.fxs, acc.fxc), im),
                                                       rmul(radd(acc.fys, acc.fyc), im),
                                                       rmul(radd(acc.fzs, acc.fzc), im), 0.0f);
                    }
                    s_epi[wib][slot] = active ? i : -1;
                }
                if (lane == 0) {
                    s_epq[wib][2 * nbuf] = r;
                    s_epq[wib][2 * nbuf + 1] = qq;
                }
                if (++nbuf == TPA) flush();
                int qn = 0;
                if (lane == 0) qn = atomicAdd(next_chunk, 1);
                q = __shfl_sync(0xffffffffu, qn, 0);
            }
            if (nbuf > 0) flush();
        }
        pk_sync(cluster);

        ran = true;
    }

    // the last step's Berendsen scaling
    if (a.thermo && ran && !*(volatile const int*)&a.group_flag[g]) {
        pk_lambdas(b, a, s_sys, G, wib, lane, GPW, s_lambda);
        __syncthreads();
        for (int v = ash.x + threadIdx.x; v < ash.y; v += PK_THREADS) {
            int r = pk_find(s_apre, G, v);
            int s = s_sys[r];
            int i = b.sys[s].begin + (v - s_apre[r]);
            double f = s_lambda[r];
            double4_32a vel = b.vel[i];
            vel.x *= f;
            vel.y *= f;
            vel.z *= f;
            b.vel[i] = vel;
        }
    }
}

size_t persist_smem_bytes(int stage_atoms) { return (size_t)stage_atoms * (sizeof(uint4) + sizeof(int)); }

template <int TPA, bool LJ1>
cudaError_t launch_persist_tpa(const Batch& b, const PkArgs& a, int cluster, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(a.ngroups * cluster), 1, 1);
    cfg.blockDim = dim3(PK_THREADS, 1, 1);
    // (the shared-memory limit of the kernel was raised to PK_STAGE_MAX atoms when
    // the plan queried its occupancy, so a launch needs no attribute call)
    cfg.dynamicSmemBytes = LJ1 ? (size_t)a.stage * sizeof(uint4) : persist_smem_bytes(a.stage);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, md_persist_kernel<TPA, LJ1>, b, a);
}
template <int TPA>
cudaError_t launch_persist_tpa(const Batch& b, const PkArgs& a, int cluster, cudaStream_t st) {
    return b.lj1 ? launch_persist_tpa<TPA, true>(b, a, cluster, st) : launch_persist_tpa<TPA, false>(b, a, cluster, st);
}

cudaError_t launch_md_persist(const Batch& b, const PkArgs& a, int cluster, cudaStream_t st) {
    if (a.ngroups == 0 || a.nsteps == 0) return cudaSuccess;
    switch (b.tpa) {  // (persistent runs need the per-step kernel's group size: 1, 2, 4 or 8)
        case 1: return launch_persist_tpa<1>(b, a, cluster, st);
        case 2: return launch_persist_tpa<2>(b, a, cluster, st);
        case 4: return launch_persist_tpa<4>(b, a, cluster, st);
        case 8: return launch_persist_tpa<8>(b, a, cluster, st);
        default: return cudaErrorInvalidValue;
    }
}

template <int TPA>
int max_clusters_tpa(int cluster, int stage_atoms) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cluster, 1, 1);
    cfg.blockDim = dim3(PK_THREADS, 1, 1);
    cfg.dynamicSmemBytes = persist_smem_bytes(stage_atoms);
    if (cfg.dynamicSmemBytes > 0 &&
        (cudaFuncSetAttribute(md_persist_kernel<TPA, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)cfg.dynamicSmemBytes) != cudaSuccess ||
         cudaFuncSetAttribute(md_persist_kernel<TPA, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)cfg.dynamicSmemBytes) != cudaSuccess)) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int count = 0;
    // (the one-kind LJ variant has the same registers and static shared memory)
    if (cudaOccupancyMaxActiveClusters(&count, md_persist_kernel<TPA, false>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return count;
}

int persist_max_clusters(int tpa, int cluster, int stage_atoms) {
    switch (tpa) {
        case 1: return max_clusters_tpa<1>(cluster, stage_atoms);
        case 2: return max_clusters_tpa<2>(cluster, stage_atoms);
        case 4: return max_clusters_tpa<4>(cluster, stage_atoms);
        default: return max_clusters_tpa<8>(cluster, stage_atoms);
    }
}

}  // namespace lg
