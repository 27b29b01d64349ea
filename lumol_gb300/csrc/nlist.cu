// nlist.cu -- device cell list and Verlet list.
//
// The reference has no neighbour list: every loop is O(N^2) over i < j
// (lumol-core/src/sys/compute.rs:37-55) with the cutoff test inside the pair
// functions (energy/pairs.rs:185-243, ewald.rs:387-428, wolf.rs:90-117).  The
// list built here is a SUPERSET of those pairs: it holds every j whose minimum
// image lies within rlist = max cutoff + skin (tested in FP32 on wrapped
// copies, with a margin larger than the FP32 error), and the force kernels then
// apply the reference's exact FP64 cutoff test on the unwrapped positions.  The
// list stays valid while no atom moved more than skin / 2 since the build.
//
// All kernels are launched every step (so one step can be captured in a CUDA
// graph) and return at once unless the status word asks for a rebuild.  The
// decision is per system: only the systems with an atom that moved more than
// skin / 2 rebuild, so a system's list (and the order of its force sums) never
// depends on the other systems of the batch.
#include "kernels.h"

namespace lg {

// Rebuild plan: the systems whose list is rebuilt at this build, with prefix
// sums of their atom and cell counts, so that every later kernel walks only
// their atoms and cells (a step in which one system of a large batch rebuilds
// costs that system's work, not the batch's).  Layout of `plan`: R, then the R
// system indices (room for nsys), then R + 1 atom prefix sums, then R + 1 cell
// prefix sums (each with room for nsys + 1).
struct PlanView {
    int R;
    const int* sys;
    const int* apre;
    const int* cpre;
};

__device__ __forceinline__ PlanView plan_view(const int* plan, int nsys) {
    return PlanView{plan[0], plan + 1, plan + 1 + nsys, plan + 2 + 2 * nsys};
}

// index r of the planned system holding virtual index v: the last r with pre[r] <= v
__device__ __forceinline__ int plan_find(const int* pre, int R, int v) {
    int a = 0, b = R - 1;
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (pre[mid] <= v) a = mid;
        else b = mid - 1;
    }
    return a;
}

__global__ void __launch_bounds__(1024) nl_plan_kernel(int nsys, const uint32_t* __restrict__ status,
                                                       const uint32_t* __restrict__ sys_rebuild,
                                                       const SysDev* __restrict__ sys, int* __restrict__ plan) {
    if (!(*status & ST_REBUILD)) return;
    __shared__ int s_r[1024], s_a[1024], s_c[1024];
    int t = threadIdx.x;
    int per = (nsys + blockDim.x - 1) / blockDim.x;
    int lo = min(t * per, nsys), hi = min(lo + per, nsys);
    int r = 0, a = 0, c = 0;
    for (int s = lo; s < hi; s++)
        if (sys_rebuild[s]) {
            const SysDev& d = sys[s];
            r += 1;
            a += d.end - d.begin;
            c += d.ncell[0] * d.ncell[1] * d.ncell[2];
        }
    s_r[t] = r;
    s_a[t] = a;
    s_c[t] = c;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        int vr = t >= o ? s_r[t - o] : 0;
        int va = t >= o ? s_a[t - o] : 0;
        int vc = t >= o ? s_c[t - o] : 0;
        __syncthreads();
        s_r[t] += vr;
        s_a[t] += va;
        s_c[t] += vc;
        __syncthreads();
    }
    int* sl = plan + 1;
    int* apre = plan + 1 + nsys;
    int* cpre = plan + 2 + 2 * nsys;
    int rr = s_r[t] - r, aa = s_a[t] - a, cc = s_c[t] - c;
    for (int s = lo; s < hi; s++)
        if (sys_rebuild[s]) {
            const SysDev& d = sys[s];
            sl[rr] = s;
            apre[rr] = aa;
            cpre[rr] = cc;
            rr += 1;
            aa += d.end - d.begin;
            cc += d.ncell[0] * d.ncell[1] * d.ncell[2];
        }
    if (t == (int)blockDim.x - 1) {
        plan[0] = s_r[t];
        apre[s_r[t]] = s_a[t];
        cpre[s_r[t]] = s_c[t];
    }
}

// Atom pass: cell index of each atom from its wrapped position
// (UnitCell::wrap_vector, cells.rs:263-282), FP32 wrapped copy, reference
// position for the displacement test.
__global__ void nl_bin_kernel(int nsys, const int* __restrict__ plan, const double4_32a* __restrict__ posq,
                              const SysDev* __restrict__ sys, const uint32_t* __restrict__ status,
                              int* __restrict__ atom_cell, int* __restrict__ cell_count, float4* __restrict__ wpos,
                              double4_32a* __restrict__ pos_build) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A; v += gridDim.x * blockDim.x) {
        int r = plan_find(pv.apre, pv.R, v);
        const SysDev& s = sys[pv.sys[r]];
        int i = s.begin + (v - pv.apre[r]);
        double4_32a p = posq[i];
        pos_build[i] = p;
        double w[3] = {p.x, p.y, p.z};
        int c[3];
        if (s.tric) {  // the wrapped fractional coordinates: cells of the fractional grid
            tric_fractional(s, p.x, p.y, p.z, w);
            for (int d = 0; d < 3; d++) {
                w[d] -= floor(w[d]);
                int cd = (int)(w[d] * (double)s.ncell[d]);
                c[d] = min(max(cd, 0), s.ncell[d] - 1);
            }
        } else {
            for (int d = 0; d < 3; d++) {
                w[d] -= floor(w[d] / s.L[d]) * s.L[d];
                int cd = (int)(w[d] * s.invL[d] * (double)s.ncell[d]);
                c[d] = min(max(cd, 0), s.ncell[d] - 1);
            }
        }
        int cell = s.cell_begin + (c[2] * s.ncell[1] + c[1]) * s.ncell[0] + c[0];
        atom_cell[i] = cell;
        atomicAdd(&cell_count[cell], 1);
        wpos[i] = make_float4((float)w[0], (float)w[1], (float)w[2], (float)p.w);
    }
}

// Atom pass of the mixed path: the cell of each atom from its fixed-point
// position (integer arithmetic, as the persistent kernel's list build), and
// the reference position for the displacement test.  (A kernel of its own:
// with the plain path's pass in the same loop body, the z cell index of this
// pass came out as 0 on GB300, for every atom.)
__global__ void nl_bin_fixed_kernel(int nsys, const int* __restrict__ plan, const double4_32a* __restrict__ posq,
                                    const SysDev* __restrict__ sys, const uint32_t* __restrict__ status,
                                    int* __restrict__ atom_cell, int* __restrict__ cell_count,
                                    double4_32a* __restrict__ pos_build) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A; v += gridDim.x * blockDim.x) {
        int r = plan_find(pv.apre, pv.R, v);
        const SysDev& s = sys[pv.sys[r]];
        int i = s.begin + (v - pv.apre[r]);
        double4_32a p = posq[i];
        pos_build[i] = p;
        int cell = fixed_cell(s, fixed_position(s, p));
        atom_cell[i] = cell;
        atomicAdd(&cell_count[cell], 1);
    }
}

// Exclusive scan of the cell counts of one system (one block per rebuilding
// system).  A system's cells hold its atoms at [begin, end) of cell_atoms, and
// its start array has one slot per cell plus an end sentinel, at
// cell_start[cell + system index].  Also zeroes the counts for the scatter.
__global__ void __launch_bounds__(1024) nl_scan_kernel(int nsys, uint32_t* __restrict__ status,
                                                       const int* __restrict__ plan,
                                                       const SysDev* __restrict__ sys, int* __restrict__ cell_count,
                                                       int* __restrict__ cell_start) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    __shared__ int partial[1024];
    for (int r = blockIdx.x; r < pv.R; r += gridDim.x) {
        int s = pv.sys[r];
        const SysDev& d = sys[s];
        int ncells = d.ncell[0] * d.ncell[1] * d.ncell[2];
        int* count = cell_count + d.cell_begin;
        int* start = cell_start + d.cell_begin + s;
        int t = threadIdx.x;
        int per = (ncells + blockDim.x - 1) / blockDim.x;
        int lo = min(t * per, ncells), hi = min(lo + per, ncells);
        int sum = 0;
        for (int c = lo; c < hi; c++) sum += count[c];
        __syncthreads();  // the previous system's readers of partial are done
        partial[t] = sum;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            int v = t >= o ? partial[t - o] : 0;
            __syncthreads();
            partial[t] += v;
            __syncthreads();
        }
        // Every start is clamped to the system's slice [begin, end] of cell_atoms.
        // The counts add up to the system's atoms unless a build was interrupted
        // between binning and sorting (stale counts, only ever too large): then
        // the status word gets ST_CELL_OVF and the clamped ranges keep every later
        // kernel of this build (scatter, sort, sorted order, rows) inside the
        // slice; the host recounts and rebuilds before the list is used.
        int run = d.begin + partial[t] - sum;
        for (int c = lo; c < hi; c++) {
            start[c] = min(run, d.end);
            run += count[c];
            count[c] = 0;
        }
        if (t == (int)blockDim.x - 1) {
            start[ncells] = min(d.begin + partial[t], d.end);
            if (d.begin + partial[t] != d.end) atomicOr(status, ST_CELL_OVF);
        }
    }
}

// Scatter of the atoms into their cells.  A slot beyond the cell's range (or
// the system's slice) is never written: the status word gets ST_CELL_OVF and
// the host recounts and rebuilds.
__global__ void nl_scatter_kernel(int nsys, const int* __restrict__ plan, uint32_t* __restrict__ status,
                                  const SysDev* __restrict__ sys, const int* __restrict__ atom_cell,
                                  int* __restrict__ cell_count, const int* __restrict__ cell_start,
                                  int* __restrict__ cell_atoms) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A; v += gridDim.x * blockDim.x) {
        int r = plan_find(pv.apre, pv.R, v);
        int s = pv.sys[r];
        const SysDev& d = sys[s];
        int i = d.begin + (v - pv.apre[r]);
        int c = atom_cell[i];
        int slot = atomicAdd(&cell_count[c], 1);
        int at = cell_start[c + s] + slot;
        if (at < cell_start[c + s + 1] && at >= d.begin && at < d.end)
            cell_atoms[at] = i;
        else
            atomicOr(status, ST_CELL_OVF);
    }
}

// Sort each cell's atoms by index so that the list order (and so the order of
// the force sums) does not depend on the atomics above: blocks walk the planned
// cells, each atom's slot is its rank among the cell's atoms (indices are
// distinct).  Leaves the counts at zero for the next build.
constexpr int SORT_SMEM = 2048;

__global__ void __launch_bounds__(128) nl_sort_kernel(int nsys, const int* __restrict__ plan,
                                                      const uint32_t* __restrict__ status,
                                                      const SysDev* __restrict__ sys,
                                                      const int* __restrict__ cell_start,
                                                      int* __restrict__ cell_atoms, int* __restrict__ cell_count) {
    if (!(*status & ST_REBUILD)) return;
    __shared__ int buf[SORT_SMEM];
    PlanView pv = plan_view(plan, nsys);
    int C = pv.cpre[pv.R];
    for (int vc = blockIdx.x; vc < C; vc += gridDim.x) {
        int r = plan_find(pv.cpre, pv.R, vc);
        int s = pv.sys[r];
        int c = sys[s].cell_begin + (vc - pv.cpre[r]);
        if (threadIdx.x == 0) cell_count[c] = 0;
        int lo = cell_start[c + s], hi = cell_start[c + s + 1];
        int m = hi - lo;
        if (m <= 1) continue;
        if (m <= SORT_SMEM) {
            __syncthreads();  // the previous cell's readers of buf are done
            for (int a = threadIdx.x; a < m; a += blockDim.x) buf[a] = cell_atoms[lo + a];
            __syncthreads();
            for (int a = threadIdx.x; a < m; a += blockDim.x) {
                int v = buf[a], rank = 0;
                for (int b = 0; b < m; b++) rank += buf[b] < v;
                cell_atoms[lo + rank] = v;
            }
        } else if (threadIdx.x == 0) {
            // very crowded cell: serial insertion sort in place
            for (int a = lo + 1; a < hi; a++) {
                int v = cell_atoms[a];
                int b = a - 1;
                while (b >= lo && cell_atoms[b] > v) {
                    cell_atoms[b + 1] = cell_atoms[b];
                    b--;
                }
                cell_atoms[b + 1] = v;
            }
        }
    }
}

// Position of every atom in the cell-sorted order (perm) and the sorted copies
// of kind, molecule and fixed-point position the mixed kernels read, for the
// planned systems.
__global__ void nl_perm_kernel(int nsys, const int* __restrict__ plan, const uint32_t* __restrict__ status,
                               const SysDev* __restrict__ sys, const int* __restrict__ cell_atoms,
                               const int* __restrict__ kind, const int* __restrict__ mol,
                               const double4_32a* __restrict__ posq, int* __restrict__ perm, int2* __restrict__ km,
                               uint4* __restrict__ posfx, uint4* __restrict__ pfx_build) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A; v += gridDim.x * blockDim.x) {
        int r = plan_find(pv.apre, pv.R, v);
        const SysDev& s = sys[pv.sys[r]];
        int t = s.begin + (v - pv.apre[r]);
        int i = cell_atoms[t];
        perm[i] = t;
        km[t] = make_int2(kind[i], mol[i]);
        uint4 u = fixed_position(s, posq[i]);
        posfx[t] = u;
        pfx_build[i] = u;  // reference point of the displacement test
    }
}

// Warp per atom: keep j != i whose FP32 minimum-image distance is below
// rlist (plus margin).  Warps walk the planned systems' atoms in cell order
// (neighbouring warps share a stencil).  The candidate cells (two cells around
// the atom's per dimension, cells being at least half the list radius wide)
// come as runs of cells contiguous in memory, flattened into one range of
// candidates (per-warp prefix sums in shared memory), so all 32 lanes test
// candidates; candidates keep the run-then-cell-then-index order.  Full list:
// each pair appears in the lists of both atoms.
constexpr int NL_WARPS = 8;

__global__ void __launch_bounds__(32 * NL_WARPS) nl_build_kernel(
    int nsys, const int* __restrict__ plan, const uint32_t* status, const SysDev* __restrict__ sys,
    const float4* __restrict__ wpos, const int* __restrict__ atom_cell, const int* __restrict__ cell_start,
    const int* __restrict__ cell_atoms, const int* __restrict__ perm, const uint4* __restrict__ posfx, int maxnb,
    int* __restrict__ nbr, int* __restrict__ nnb, uint32_t* status_out) {
    __shared__ int s_lo[NL_WARPS][NL_RUNS];
    __shared__ int s_pre[NL_WARPS][NL_RUNS + 1];
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    int wib = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * NL_WARPS + wib; w < A; w += gridDim.x * NL_WARPS) {
        int r = plan_find(pv.apre, pv.R, w);
        int si = pv.sys[r];
        const SysDev& s = sys[si];
        int i = cell_atoms[s.begin + (w - pv.apre[r])];
        // mixed path (perm): the fixed-point copies in the new cell order (written by nl_perm)
        float4 pi = perm ? make_float4(0.f, 0.f, 0.f, 0.f) : wpos[i];
        uint4 ui = perm ? posfx[perm[i]] : make_uint4(0u, 0u, 0u, 0u);
        __syncwarp();  // the previous atom's readers of s_lo / s_pre are done
        int2 nt = stencil_table(s, si, atom_cell[i] - s.cell_begin, cell_start, lane, s_lo[wib], s_pre[wib]);
        int nruns = nt.x, total = nt.y;
        __syncwarp();
        float Lx = s.Lf[0], Ly = s.Lf[1], Lz = s.Lf[2];
        float ix = s.invLf[0], iy = s.invLf[1], iz = s.invLf[2];
        float rl2 = s.rlist2_f;
        int count = 0;
        // with a cell-sorted order (mixed path) the row and its entries are sorted positions
        int row = perm ? perm[i] : i;
        int* out = nbr + (size_t)row * maxnb;
        for (int base = 0; base < total; base += 32) {
            int t = base + lane;
            bool keep = false;
            int j = -1, jout = -1;
            if (t < total) {
                int slot = stencil_slot(s_lo[wib], s_pre[wib], nruns, t);
                if (perm) {  // the same test as the persistent kernel's list build
                    jout = slot;
                    keep = slot != row && fixed_dist2_s(s, ui, posfx[slot]) < rl2;
                } else {
                    j = cell_atoms[slot];
                    jout = j;
                    float4 pj = wpos[j];
                    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                    if (s.tric) {  // wpos holds wrapped fractional coordinates
                        tric_cartesian_f(s, dx - rintf(dx), dy - rintf(dy), dz - rintf(dz), dx, dy, dz);
                    } else {
                        dx -= rintf(dx * ix) * Lx;
                        dy -= rintf(dy * iy) * Ly;
                        dz -= rintf(dz * iz) * Lz;
                    }
                    float r2 = dx * dx + dy * dy + dz * dz;
                    keep = (j != i) && (r2 < rl2);
                }
            }
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                int pos = count + __popc(mask & ((1u << lane) - 1u));
                if (pos < maxnb) out[pos] = jout;
            }
            count += __popc(mask);
        }
        if (lane == 0) {
            nnb[row] = min(count, maxnb);
            if (count > maxnb) atomicOr(status_out, ST_OVERFLOW);
        }
    }
}

// Plain path, after the build: sort each rebuilt row by neighbour index (warp
// per row, rank sort in shared memory) and count its j < i head (nlo).  The
// order of a row's entries only changes the order of the force sums.
constexpr int ROW_SMEM = 512;

__global__ void __launch_bounds__(32 * NL_WARPS) nl_rowsort_kernel(int nsys, const int* __restrict__ plan,
                                                                   const uint32_t* __restrict__ status,
                                                                   const SysDev* __restrict__ sys, int maxnb,
                                                                   int* __restrict__ nbr,
                                                                   const int* __restrict__ nnb,
                                                                   int* __restrict__ nlo) {
    __shared__ int buf[NL_WARPS][ROW_SMEM];
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    int wib = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * NL_WARPS + wib; w < A; w += gridDim.x * NL_WARPS) {
        int r = plan_find(pv.apre, pv.R, w);
        int i = sys[pv.sys[r]].begin + (w - pv.apre[r]);
        int* row = nbr + (size_t)i * maxnb;
        int cnt = nnb[i];
        int below = 0;
        __syncwarp();
        if (cnt <= ROW_SMEM) {
            for (int a = lane; a < cnt; a += 32) buf[wib][a] = row[a];
            __syncwarp();
            for (int a = lane; a < cnt; a += 32) {
                int v = buf[wib][a], rank = 0;
                for (int b = 0; b < cnt; b++) rank += buf[wib][b] < v;
                row[rank] = v;
                below += v < i;
            }
        } else if (lane == 0) {
            // very long row: serial insertion sort in place
            for (int a = 1; a < cnt; a++) {
                int v = row[a];
                int b = a - 1;
                while (b >= 0 && row[b] > v) {
                    row[b + 1] = row[b];
                    b--;
                }
                row[b + 1] = v;
            }
            for (int a = 0; a < cnt; a++) below += row[a] < i;
        }
        for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
        if (lane == 0) nlo[i] = below;
    }
}

// Reverse index of every j < i entry: the slot of i in row j (binary search
// in j's sorted j' > j tail; the list is symmetric).  A row cut short by an
// overflow has no slot for some partners: those get an in-range slot and the
// overflow status makes the caller rebuild and recompute.
__global__ void nl_rev_kernel(int nsys, const int* __restrict__ plan, const uint32_t* __restrict__ status,
                              const SysDev* __restrict__ sys, int maxnb, const int* __restrict__ nbr,
                              const int* __restrict__ nnb, const int* __restrict__ nlo, int* __restrict__ rev) {
    if (!(*status & ST_REBUILD)) return;
    PlanView pv = plan_view(plan, nsys);
    int A = pv.apre[pv.R];
    int wib = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * NL_WARPS + wib; w < A; w += gridDim.x * NL_WARPS) {
        int r = plan_find(pv.apre, pv.R, w);
        int i = sys[pv.sys[r]].begin + (w - pv.apre[r]);
        const int* row = nbr + (size_t)i * maxnb;
        int head = nlo[i];
        for (int k = lane; k < head; k += 32) {
            int j = row[k];
            const int* rj = nbr + (size_t)j * maxnb;
            int a = nlo[j], b = nnb[j];  // first slot with rj[slot] >= i
            while (a < b) {
                int mid = (a + b) >> 1;
                if (rj[mid] < i) a = mid + 1;
                else b = mid;
            }
            rev[(size_t)i * maxnb + k] = min(a, maxnb - 1);
        }
    }
}

// Clears the rebuild requests once the lists are in place.
__global__ void nl_done_kernel(int nsys, uint32_t* status, uint32_t* sys_rebuild) {
    if (!(*status & ST_REBUILD)) return;
    for (int s = threadIdx.x; s < nsys; s += blockDim.x) sys_rebuild[s] = 0;
    __syncthreads();
    if (threadIdx.x == 0) *status &= ~ST_REBUILD;
}

void launch_nlist_build(const Batch& b, cudaStream_t st) {
    int n = b.n;
    if (n == 0) return;
    int tb = 256;
    // grid-stride kernels: enough blocks to fill the device at a full rebuild,
    // few enough that a step with a small (or no) rebuild costs little
    unsigned atoms_grid = (unsigned)std::min((n + tb - 1) / tb, 4 * b.sms);
    unsigned cells_grid = (unsigned)std::min(b.ncells, 16 * b.sms);
    unsigned build_grid = (unsigned)std::min((n + NL_WARPS - 1) / NL_WARPS, 8 * b.sms);
    unsigned scan_grid = (unsigned)std::min(b.nsys, 2 * b.sms);
    nl_plan_kernel<<<1, 1024, 0, st>>>(b.nsys, b.status, b.sys_rebuild, b.sys, b.plan);
    if (b.perm)
        nl_bin_fixed_kernel<<<atoms_grid, tb, 0, st>>>(b.nsys, b.plan, b.posq, b.sys, b.status, b.atom_cell,
                                                       b.cell_count, b.pos_build);
    else
        nl_bin_kernel<<<atoms_grid, tb, 0, st>>>(b.nsys, b.plan, b.posq, b.sys, b.status, b.atom_cell, b.cell_count,
                                                 b.wpos, b.pos_build);
    nl_scan_kernel<<<scan_grid, 1024, 0, st>>>(b.nsys, b.status, b.plan, b.sys, b.cell_count, b.cell_start);
    nl_scatter_kernel<<<atoms_grid, tb, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.atom_cell, b.cell_count,
                                                 b.cell_start, b.cell_atoms);
    nl_sort_kernel<<<cells_grid, 128, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.cell_start, b.cell_atoms,
                                               b.cell_count);
    if (b.perm)
        nl_perm_kernel<<<atoms_grid, tb, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.cell_atoms, b.kind, b.mol,
                                                  b.posq, b.perm, b.km, b.posfx, b.pfx_build);
    nl_build_kernel<<<build_grid, 32 * NL_WARPS, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.wpos, b.atom_cell,
                                                          b.cell_start, b.cell_atoms, b.perm, b.posfx, b.maxnb,
                                                          b.nbr, b.nnb, b.status);
    if (b.pf) {
        nl_rowsort_kernel<<<build_grid, 32 * NL_WARPS, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.maxnb, b.nbr,
                                                                b.nnb, b.nlo);
        nl_rev_kernel<<<build_grid, 32 * NL_WARPS, 0, st>>>(b.nsys, b.plan, b.status, b.sys, b.maxnb, b.nbr, b.nnb,
                                                            b.nlo, b.rev);
    }
    nl_done_kernel<<<1, 256, 0, st>>>(b.nsys, b.status, b.sys_rebuild);
}

}  // namespace lg
