// lower.cu -- the description of every system (particles, topology, pair
// table, Coulomb potential, cell), as Lumol's System holds it, lowered into
// the flat device layout of kernels.h on first use after a change, with the
// host restatements of the reference's scalar arithmetic that feed it
// (potential shifts, TableComputation tables, tail corrections, Ewald
// k-vector factors and self energy).  Compiled with -ffp-contract=off.
#include "engine.h"

namespace lg {
namespace {

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

// UnitCell::k_vector (cells.rs:224-226): (2 PI * inv) * index, the scaled
// matrix times the vector row by row (matrix.rs:389-398).
void k_vector(const HostCell& c, double i0, double i1, double i2, double k[3]) {
    for (int a = 0; a < 3; a++) {
        const double* r = c.inv + 3 * a;
        k[a] = (2.0 * PI) * r[0] * i0 + (2.0 * PI) * r[1] * i1 + (2.0 * PI) * r[2] * i2;
    }
}

// Ewald::prepare + compute_ewald_factors_triclinic (ewald.rs:130-183, 353-379)
void ewald_factors(const HostCell& cell, double alpha, int kmax, int sys, std::vector<KVecDev>& out) {
    // k_vector([1, 1, 1]).max() * kmax (Vector3D::max: the largest component)
    double k111[3];
    k_vector(cell, 1.0, 1.0, 1.0, k111);
    double mx = std::max(std::max(k111[0], k111[1]), k111[2]) * (double)kmax;
    double kmax2 = 1.0001 * mx * mx;
    double alpha_sq_inv_fourth = 0.25 / (alpha * alpha);
    double four_pi_v = 4.0 * PI / cell.volume;
    auto push = [&](int ikx, int iky, int ikz) {
        double k[3];
        k_vector(cell, (double)ikx, (double)iky, (double)ikz, k);
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

}  // namespace

// UnitCell's derived values (cells.rs:108-200) with the reference's
// operations: Matrix3::inverse (matrix.rs:212-249), lengths() from the face
// normals (b ^ c).normalized() (vectors.rs:102-130, 219-228), volume() as
// a * b * c (orthorhombic) or the mixed product a * (b ^ c) (triclinic).
bool cell_init(HostCell& c, const double m[9], int shape) {
    c.shape = shape;
    for (int k = 0; k < 9; k++) c.m[k] = m[k];
    auto M = [&](int i, int j) { return m[3 * i + j]; };
    double det = M(0, 0) * (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2)) - M(0, 1) * (M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0)) +
                 M(0, 2) * (M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0));
    if (!(std::fabs(det) > 1e-30)) return false;
    double id = 1.0 / det;
    double* r = c.inv;
    r[0] = (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2)) * id;
    r[1] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * id;
    r[2] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * id;
    r[3] = (M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2)) * id;
    r[4] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * id;
    r[5] = (M(1, 0) * M(0, 2) - M(0, 0) * M(1, 2)) * id;
    r[6] = (M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1)) * id;
    r[7] = (M(2, 0) * M(0, 1) - M(0, 0) * M(2, 1)) * id;
    r[8] = (M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1)) * id;
    double va[3] = {M(0, 0), M(1, 0), M(2, 0)}, vb[3] = {M(0, 1), M(1, 1), M(2, 1)}, vc[3] = {M(0, 2), M(1, 2), M(2, 2)};
    auto cross = [](const double* x, const double* y, double* z) {
        z[0] = x[1] * y[2] - x[2] * y[1];
        z[1] = x[2] * y[0] - x[0] * y[2];
        z[2] = x[0] * y[1] - x[1] * y[0];
    };
    auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    auto face = [&](const double* x, const double* y, const double* v) {
        double n[3];
        cross(x, y, n);
        double norm = std::sqrt(dot(n, n));
        for (int k = 0; k < 3; k++) n[k] = n[k] / norm;
        return std::fabs(dot(n, v));
    };
    c.len[0] = face(vb, vc, va);
    c.len[1] = face(vc, va, vb);
    c.len[2] = face(va, vb, vc);
    if (shape == LG_CELL_ORTHORHOMBIC) {
        c.volume = M(0, 0) * M(1, 1) * M(2, 2);
    } else {
        double bc[3];
        cross(vb, vc, bc);
        c.volume = dot(va, bc);
    }
    return c.volume > 0.0;
}

void set_host_cell(HostSystem& h, const HostCell& cell) {
    h.cell = cell;
    for (int k = 0; k < 3; k++) h.L[k] = cell.len[k];
    h.has_cell = true;
}

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
    d.barostat = h.barostat;
    d.baro_eta = h.baro_eta;
    for (int k = 0; k < 9; k++) d.baro_m[k] = h.baro_m[k];
}

double max_cutoff(const HostSystem& h) {
    double rc = 0.0;
    for (const lg_pair& p : h.pairs)
        if (p.type != LG_PAIR_ABSENT) rc = std::max(rc, p.cutoff);
    if (h.coul.kind != LG_COULOMB_NONE) rc = std::max(rc, h.coul.cutoff);
    return rc;
}

int check_pair_cutoffs(lg_engine* e, const HostSystem& h) {
    if (!h.has_cell) return LG_OK;
    return check_cell_cutoffs(e, h, h.L);
}

int check_cell_cutoffs(lg_engine* e, const HostSystem& h, const double len[3]) {
    double half = 0.5 * std::min(std::min(len[0], len[1]), len[2]);
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

// The fields of a system's device record that follow from its cell: lengths
// and their inverses in FP64 / FP32, the fixed-point scale, the list radius
// and rebuild threshold, and the cell grid (cells at least half the list
// radius wide: the list builds look two cells around).  A triclinic cell's
// grid divides the fractional coordinates: its cells are at least half the
// list radius apart across every pair of faces.
void cell_geometry(SysDev& d, const HostSystem& h, const HostCell& cell, double skin) {
    // the orthorhombic branches read the diagonal (cells.rs:108-132), even of a
    // matrix that UnitCell::scale_mut gave off-diagonal terms; a triclinic
    // cell's grid spans its face distances
    const bool ortho = cell.shape == LG_CELL_ORTHORHOMBIC;
    const double diag[3] = {cell.m[0], cell.m[4], cell.m[8]};
    const double* L = ortho ? diag : cell.len;
    d.tric = !ortho;
    d.kgen = 0;
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
            if (a != c && cell.inv[3 * a + c] != 0.0) d.kgen = 1;
    for (int k = 0; k < 9; k++) {
        d.H[k] = cell.m[k];
        d.Hi[k] = cell.inv[k];
        d.Hf[k] = (float)cell.m[k];
    }
    for (int k = 0; k < 3; k++) {
        d.L[k] = L[k];
        d.invL[k] = 1.0 / L[k];
        d.Lf[k] = (float)L[k];
        d.invLf[k] = (float)(1.0 / L[k]);
        d.Lq[k] = (float)(L[k] / 4294967296.0);
        d.fxscale[k] = d.invL[k] * 4294967296.0;
    }
    double rc = max_cutoff(h);
    d.rlist = rc + skin;
    d.half_skin2 = 0.25 * skin * skin;
    d.rebuild2_f = 0.99f * (float)d.half_skin2;
    double margin = 1e-5 * std::max(std::max(L[0], L[1]), L[2]) + 1e-4;
    d.rlist2_f = (float)((d.rlist + margin) * (d.rlist + margin));
    for (int k = 0; k < 3; k++) {
        int nc = (int)std::floor(L[k] / (0.5 * (d.rlist + margin)));
        d.ncell[k] = std::max(1, std::min(nc, 128));
    }
}

// k_vector([1, 0, 0]) etc. of the cell (cells.rs:224-226): the columns of
// 2 PI inv; k1 holds their one non-zero component for an orthorhombic cell.
void ewald_k1(SysDev& d, const HostCell& cell) {
    for (int a = 0; a < 3; a++) {
        double e[3] = {0.0, 0.0, 0.0};
        e[a] = 1.0;
        double k[3];
        k_vector(cell, e[0], e[1], e[2], k);
        for (int c = 0; c < 3; c++) d.kax[3 * a + c] = k[c];
        d.k1[a] = k[a];
    }
}

// Tail corrections (sys/energy.rs:63-79, compute.rs:219-229), kinds in index
// order, at the current volume.
void tail_corrections(HostSystem& h) {
    double volume = h.cell.volume;
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
}

int set_cell_fast(lg_engine* e, int s, const HostCell& cell) {
    HostSystem& h = e->sys[s];
    SysDev d = e->h_sysdev[s];
    cell_geometry(d, h, cell, e->skin);
    const SysDev& old = e->h_sysdev[s];
    if (d.ncell[0] != old.ncell[0] || d.ncell[1] != old.ncell[1] || d.ncell[2] != old.ncell[2]) return -1;
    std::vector<KVecDev> kv;
    if (h.coul.kind == LG_COULOMB_EWALD) {
        ewald_k1(d, cell);
        ewald_factors(cell, h.alpha, h.coul.kmax, s, kv);
        if ((int)kv.size() != old.kend - old.kbegin) return -1;  // another k-vector set: lower again
    }
    set_host_cell(h, cell);
    tail_corrections(h);
    e->h_sysdev[s] = d;
    cudaStream_t st = e->stream;
    double hc[3] = {h.tail_energy, h.tail_virial, h.ewald_self};
    CUDA_TRY(e, cudaMemcpyAsync(e->sysdev.p + s, &e->h_sysdev[s], sizeof(SysDev), cudaMemcpyHostToDevice, st));
    CUDA_TRY(e, cudaMemcpyAsync(e->host_const.p + (size_t)s * RED_STRIDE, hc, 3 * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    if (!kv.empty()) {
        std::vector<KVecF> kf(kv.size());
        for (size_t k = 0; k < kv.size(); k++)
            kf[k] = KVecF{kv[k].ikx, kv[k].iky, kv[k].ikz, kv[k].sys, (float)kv[k].field[0], (float)kv[k].field[1],
                          (float)kv[k].field[2], (float)kv[k].energy};
        CUDA_TRY(e, cudaMemcpyAsync(e->kvec.p + d.kbegin, kv.data(), kv.size() * sizeof(KVecDev),
                                    cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->kvecf.p + d.kbegin, kf.data(), kf.size() * sizeof(KVecF),
                                    cudaMemcpyHostToDevice, st));
    }
    // positions keep their values in Angstrom: every list of the system is rebuilt
    uint32_t one = 1u;
    CUDA_TRY(e, cudaMemcpyAsync(e->sys_rebuild.p + s, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    launch_request_rebuild_flag(e->b, st);
    CUDA_TRY(e, cudaStreamSynchronize(st));  // the host copies above live on this stack
    e->shadow_valid = false;
    e->pk_cluster = 0;  // the persistent plan weighs systems by their density
    return LG_OK;
}

int commit(lg_engine* e) {
    if (!e->dirty) return LG_OK;
    e->shadow_valid = false;
    int nsys = e->nsys;
    const std::vector<int64_t> old_begin = e->begin;
    const int old_n = e->b.n, old_nsys = e->b.nsys;
    std::vector<int64_t> new_begin(nsys + 1, 0);
    for (int s = 0; s < nsys; s++) {
        const HostSystem& h = e->sys[s];
        if (!h.has_cell) return fail(e, LG_ERR_STATE, "system " + std::to_string(s) + " has no cell");
        if (h.nk == 0 && h.n > 0)
            return fail(e, LG_ERR_STATE, "system " + std::to_string(s) + " has no pair table");
        new_begin[s + 1] = new_begin[s] + h.n;
    }
    int64_t n = new_begin[nsys];
    if (n > (int64_t)0x7fffffff / 64) return fail(e, LG_ERR_ARGUMENT, "too many atoms");
    cudaStream_t st = e->stream;

    // Systems that stay (carry_from) keep their positions, velocities,
    // accelerations, thermostat counters, status flags and Monte Carlo chains
    // through the re-lowering: staged here, put back at their new offsets at
    // the end.  The staging reuses the checkpoint buffers when the batch does
    // not grow, so a system leaving allocates nothing.
    std::vector<int> carry(nsys, -1);
    bool any_carry = false;
    if (old_n > 0 && (int)old_begin.size() == old_nsys + 1) {
        for (int s = 0; s < nsys && s < (int)e->carry_from.size(); s++) {
            int o = e->carry_from[s];
            if (o >= 0 && o < old_nsys && old_begin[o + 1] - old_begin[o] == e->sys[s].n) {
                carry[s] = o;
                any_carry = true;
            }
        }
    }
    DBuf<double4_32a> tpos, tvel, tacc;
    double4_32a *sp = nullptr, *sv = nullptr, *sa = nullptr;
    std::vector<unsigned long long> old_count;
    std::vector<uint32_t> old_status;
    std::vector<McState> old_mc;
    if (any_carry) {
        if ((size_t)n <= e->cp_pos.cap && (size_t)n <= e->cp_vel.cap && (size_t)n <= e->cp_acc.cap) {
            sp = e->cp_pos.p;
            sv = e->cp_vel.p;
            sa = e->cp_acc.p;
        } else {
            CUDA_TRY(e, tpos.alloc(old_n));
            CUDA_TRY(e, tvel.alloc(old_n));
            CUDA_TRY(e, tacc.alloc(old_n));
            sp = tpos.p;
            sv = tvel.p;
            sa = tacc.p;
        }
        size_t bytes = (size_t)old_n * sizeof(double4_32a);
        CUDA_TRY(e, cudaMemcpyAsync(sp, e->posq.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(sv, e->vel.p, bytes, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(sa, e->acc.p, bytes, cudaMemcpyDeviceToDevice, st));
        old_count.resize(old_nsys);
        old_status.resize(old_nsys);
        old_mc.resize(old_nsys);
        CUDA_TRY(e, cudaMemcpyAsync(old_count.data(), e->md_count.p, old_nsys * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, st));
        CUDA_TRY(e, cudaMemcpyAsync(old_status.data(), e->sys_status.p, old_nsys * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, st));
        CUDA_TRY(e, cudaMemcpyAsync(old_mc.data(), e->mc_chains.p, old_nsys * sizeof(McState),
                                    cudaMemcpyDeviceToHost, st));
        CUDA_TRY(e, cudaStreamSynchronize(st));
    }
    e->begin = new_begin;

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
        cell_geometry(d, h, h.cell, e->skin);
        const int cells = d.ncell[0] * d.ncell[1] * d.ncell[2];
        d.cell_begin = cell_total;
        cell_total += cells;
        d.tile_begin = (int)h_tiles.size();
        for (int64_t a = 0; a < h.n; a += VV_TILE) h_tiles.push_back(make_int2(s, (int)(base + a)));
        d.tile_end = (int)h_tiles.size();
        double volume = h.cell.volume;
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
            ewald_k1(d, h.cell);
            d.kbegin = (int)h_kvec.size();
            ewald_factors(h.cell, h.alpha, h.coul.kmax, s, h_kvec);
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

        tail_corrections(h);
        double* hc = &h_const[(size_t)s * RED_STRIDE];
        hc[0] = h.tail_energy;
        hc[1] = h.tail_virial;
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
    CUDA_TRY(e, e->sys_status.alloc(nsys));
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
    CUDA_TRY(e, e->qf.alloc(mixed && nkv ? n : 1));
    CUDA_TRY(e, e->kvec.alloc(nkv));
    CUDA_TRY(e, e->eikr.alloc(nkv ? (size_t)kdim * 3 * n : 1));
    CUDA_TRY(e, e->rho.alloc(nkv));
    CUDA_TRY(e, e->kred.alloc((size_t)nkv * 7));
    CUDA_TRY(e, e->fpart.alloc(nkv ? (size_t)max_chunks * 3 * n : 1));

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
    CUDA_TRY(e, cudaMemsetAsync(e->sys_status.p, 0, nsys * sizeof(uint32_t), st));
    std::vector<uint32_t> all_rebuild(nsys, 1u);
    CUDA_TRY(e, cudaMemcpyAsync(e->sys_rebuild.p, all_rebuild.data(), nsys * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                st));
    CUDA_TRY(e, cudaStreamSynchronize(st));

    if (e->h_out_cap < (size_t)nsys) {  // page-locked: reallocated only when the batch grows
        if (e->h_out) cudaFreeHost(e->h_out);
        e->h_out = nullptr;
        e->h_out_cap = 0;
        CUDA_TRY(e, cudaMallocHost((void**)&e->h_out, (size_t)nsys * RED_STRIDE * sizeof(double)));
        e->h_out_cap = (size_t)nsys;
    }

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
    b.sys_status = e->sys_status.p;
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
    if (any_carry) {  // the chains of the systems that stay; the others' as lg_mc_setup left them
        e->h_mc.resize(nsys, McState{});
        for (int s = 0; s < nsys; s++)
            if (carry[s] >= 0) e->h_mc[s] = old_mc[carry[s]];
    }
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
    // a triclinic cell's minimum image is in the general kernels only (and
    // keeps its batch off the persistent kernel)
    for (int s = 0; s < nsys; s++) b.pair_general |= e->h_sysdev[s].tric ? 1 : 0;
    b.norestr = 1;
    for (const PairDevF& q : h_ptabf) b.norestr &= (q.type == 0 || q.restriction == 0) ? 1 : 0;
    for (int s = 0; s < nsys; s++) b.norestr &= (e->h_sysdev[s].coul_restr == 0 && !e->h_sysdev[s].tric) ? 1 : 0;
    b.lj1 = nsys > 0 ? 1 : 0;
    for (int s = 0; s < nsys; s++) {
        const SysDev& d = e->h_sysdev[s];
        if (d.nk != 1 || d.ptab < 0 || (size_t)d.ptab >= h_ptabf.size() || h_ptabf[d.ptab].type != 2) b.lj1 = 0;
    }
    b.kvecf = e->kvecf.p;
    b.eikrf = e->eikrf.p;
    b.rhof = e->rhof.p;
    b.qf = e->qf.p;
    if (any_carry) {
        std::vector<unsigned long long> count(nsys, 0ull);
        std::vector<uint32_t> status(nsys, 0u);
        for (int s = 0; s < nsys; s++) {
            int o = carry[s];
            if (o < 0) continue;
            int m = (int)e->sys[s].n;
            // x, v and a at the new offsets (charges and masses from the new description)
            launch_carry_vectors(sp + old_begin[o], e->posq.p + new_begin[s], m, true, st);
            launch_carry_vectors(sv + old_begin[o], e->vel.p + new_begin[s], m, true, st);
            launch_carry_vectors(sa + old_begin[o], e->acc.p + new_begin[s], m, false, st);
            count[s] = old_count[o];
            status[s] = old_status[o];
        }
        CUDA_TRY(e, cudaMemcpyAsync(e->md_count.p, count.data(), nsys * sizeof(unsigned long long),
                                    cudaMemcpyHostToDevice, st));
        CUDA_TRY(e, cudaMemcpyAsync(e->sys_status.p, status.data(), nsys * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                    st));
    }
    for (int s = 0; s < nsys; s++) {  // VelocityVerlet / LeapFrog::setup of a carried system
        HostSystem& h = e->sys[s];
        if (h.reset_acc && carry[s] >= 0 && h.n)
            CUDA_TRY(e, cudaMemsetAsync(e->acc.p + new_begin[s], 0, h.n * sizeof(double4_32a), st));
        h.reset_acc = false;
    }
    CUDA_TRY(e, cudaGetLastError());
    CUDA_TRY(e, cudaStreamSynchronize(st));  // the staging buffers are released on return
    e->carry_from.resize(nsys);
    for (int s = 0; s < nsys; s++) e->carry_from[s] = s;
    e->dirty = false;
    e->tuned = false;
    e->pk_cluster = 0;
    return LG_OK;
}

int commit_carried(lg_engine* e) {
    if (!e->dirty) return LG_OK;
    bool carried = e->carry_from.size() == (size_t)e->nsys;
    for (int s = 0; carried && s < e->nsys; s++) carried = e->carry_from[s] >= 0;
    if (!carried) return fail(e, LG_ERR_STATE, "no device state: call lg_md_set_state first");
    return commit(e);
}

}  // namespace lg
