// lumol_oracle.cpp -- CPU oracle for the lumol-gb300 parity tests.
//
// TEST INFRASTRUCTURE ONLY: a C++17 restatement of lumol-core's CPU arithmetic,
// used as the checker for the GPU engine.  It is never linked into, loaded by or
// called from the product.
//
// Every function keeps the reference's operation order, and the file is built
// with -ffp-contract=off because Rust never contracts a*b+c into an FMA.  The
// O(N^2) loops are parallelised over i with OpenMP and per-thread force buffers,
// the same structure as rayon + ThreadLocalVec (lumol-core/src/utils/thread_vec.rs).
// Summation order across threads is therefore not fixed, exactly as in the
// reference (rayon's sum is not ordered either).

#include "lumol_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <tuple>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double FRAC_2_SQRT_PI = 1.12837916709551257390;
// lumol-core/src/consts.rs:9,15
constexpr double K_BOLTZMANN = 8.31446284161522e-7;
constexpr double FOUR_PI_EPSILON_0 = 7.197589831304046;

struct V3 {
    double v[3];
    double& operator[](int k) { return v[k]; }
    double operator[](int k) const { return v[k]; }
};
struct M3 {
    double m[3][3];
};

inline V3 vzero() { return V3{{0.0, 0.0, 0.0}}; }
inline V3 vsub(const V3& a, const V3& b) { return V3{{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
inline V3 vadd(const V3& a, const V3& b) { return V3{{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
inline V3 vscale(double s, const V3& a) { return V3{{s * a[0], s * a[1], s * a[2]}}; }
inline V3 vdiv(const V3& a, double s) { return V3{{a[0] / s, a[1] / s, a[2] / s}}; }
// types/vectors.rs: dot = x*x' + y*y' + z*z' evaluated left to right
inline double vdot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
// cross product, Vector3D ^ Vector3D (types/vectors.rs:221-228)
inline V3 vcross(const V3& a, const V3& b) {
    return V3{{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}
inline double vnorm2(const V3& a) { return vdot(a, a); }
inline double vnorm(const V3& a) { return std::sqrt(vnorm2(a)); }
inline V3 vnormalized(const V3& a) { return vdiv(a, vnorm(a)); }
inline M3 mzero() {
    M3 r;
    std::memset(&r, 0, sizeof(r));
    return r;
}
// types/vectors.rs:150-156
inline M3 tensorial(const V3& a, const V3& b) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = a[i] * b[j];
    return r;
}
inline void madd(M3& a, const M3& b) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a.m[i][j] += b.m[i][j];
}
inline M3 mscale(double s, const M3& a) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = s * a.m[i][j];
    return r;
}

struct Complex {
    double re, im;
};
// types/complex.rs:40-63, 152-154
inline Complex cmul(const Complex& a, const Complex& b) {
    return Complex{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
inline Complex cconj(const Complex& a) { return Complex{a.re, -a.im}; }
inline double cnorm2(const Complex& a) { return a.re * a.re + a.im * a.im; }

// ---------------------------------------------------------------------------
// UnitCell (lumol-core/src/sys/config/cells.rs), orthorhombic or triclinic
// ---------------------------------------------------------------------------
// Matrix3 * Vector3D (types/matrix.rs:389-398)
inline V3 mat_vec(const M3& m, const V3& v) {
    return V3{{m.m[0][0] * v[0] + m.m[0][1] * v[1] + m.m[0][2] * v[2],
               m.m[1][0] * v[0] + m.m[1][1] * v[1] + m.m[1][2] * v[2],
               m.m[2][0] * v[0] + m.m[2][1] * v[1] + m.m[2][2] * v[2]}};
}

struct Cell {
    int shape = ORC_CELL_ORTHORHOMBIC;
    double a, b, c;  // the orthorhombic branches' lengths: the diagonal (cells.rs:108-132)
    M3 cell;         // UnitCell::matrix
    M3 inv;          // Matrix3::inverse, types/matrix.rs:212-227

    void init(double la, double lb, double lc) {
        double m[9] = {la, 0.0, 0.0, 0.0, lb, 0.0, 0.0, 0.0, lc};
        init_matrix(m, ORC_CELL_ORTHORHOMBIC);
    }
    void init_matrix(const double* mm, int sh) {
        shape = sh;
        double m[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m[i][j] = cell.m[i][j] = mm[3 * i + j];
        a = m[0][0];
        b = m[1][1];
        c = m[2][2];
        double det = m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) -
                     m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                     m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        double id = 1.0 / det;
        inv.m[0][0] = (m[1][1] * m[2][2] - m[2][1] * m[1][2]) * id;
        inv.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
        inv.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
        inv.m[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
        inv.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
        inv.m[1][2] = (m[1][0] * m[0][2] - m[0][0] * m[1][2]) * id;
        inv.m[2][0] = (m[1][0] * m[2][1] - m[2][0] * m[1][1]) * id;
        inv.m[2][1] = (m[2][0] * m[0][1] - m[0][0] * m[2][1]) * id;
        inv.m[2][2] = (m[0][0] * m[1][1] - m[1][0] * m[0][1]) * id;
    }
    V3 vect(int k) const { return V3{{cell.m[0][k], cell.m[1][k], cell.m[2][k]}}; }
    // cells.rs:185-200
    double volume() const {
        if (shape == ORC_CELL_ORTHORHOMBIC) return a * b * c;
        return vdot(vect(0), vcross(vect(1), vect(2)));
    }
    // cells.rs:134-146: distances between opposite faces
    V3 lengths() const {
        V3 va = vect(0), vb = vect(1), vc = vect(2);
        auto face = [](const V3& x, const V3& y, const V3& v) {
            V3 n = vcross(x, y);
            double norm = std::sqrt(vdot(n, n));
            n = V3{{n[0] / norm, n[1] / norm, n[2] / norm}};
            return std::fabs(vdot(n, v));
        };
        return V3{{face(vb, vc, va), face(vc, va, vb), face(va, vb, vc)}};
    }
    // cells.rs:284-301
    void vector_image(V3& v) const {
        if (shape == ORC_CELL_TRICLINIC) {
            V3 f = mat_vec(inv, v);
            for (int k = 0; k < 3; k++) f[k] -= std::round(f[k]);
            v = mat_vec(cell, f);
            return;
        }
        v[0] -= std::round(v[0] / a) * a;
        v[1] -= std::round(v[1] / b) * b;
        v[2] -= std::round(v[2] / c) * c;
    }
    // cells.rs:263-282
    void wrap_vector(V3& v) const {
        if (shape == ORC_CELL_TRICLINIC) {
            V3 f = mat_vec(inv, v);
            for (int k = 0; k < 3; k++) f[k] -= std::floor(f[k]);
            v = mat_vec(cell, f);
            return;
        }
        v[0] -= std::floor(v[0] / a) * a;
        v[1] -= std::floor(v[1] / b) * b;
        v[2] -= std::floor(v[2] / c) * c;
    }
    // cells.rs:224-226: 2 PI * inv * index
    V3 k_vector(double i0, double i1, double i2) const {
        M3 s = mscale(2.0 * PI, inv);
        return V3{{s.m[0][0] * i0 + s.m[0][1] * i1 + s.m[0][2] * i2,
                   s.m[1][0] * i0 + s.m[1][1] * i1 + s.m[1][2] * i2,
                   s.m[2][0] * i0 + s.m[2][1] * i1 + s.m[2][2] * i2}};
    }
    // cells.rs:316-320
    double distance(const V3& u, const V3& v) const {
        V3 d = vsub(v, u);
        vector_image(d);
        return vnorm(d);
    }
};

// ---------------------------------------------------------------------------
// Potentials (lumol-core/src/energy/functions.rs)
// ---------------------------------------------------------------------------

// f64::powi(x, 6) as lowered by LLVM (repeated squaring): x^2 * (x^2)^2
inline double powi6(double x) {
    double x2 = x * x;
    double x4 = x2 * x2;
    return x2 * x4;
}

struct PairPot {
    orc_pair d;
    double shift = 0.0;
    // TableComputation (energy/computations.rs:63-144): tabulated at r = i delta
    std::vector<double> te, tf;
    double tdelta = 0.0;

    // TableComputation::new (computations.rs:101-121); call after d is set
    void build_table() {
        te.clear();
        tf.clear();
        if (d.table_size <= 0) return;
        tdelta = d.table_max / (double)d.table_size;
        for (int32_t i = 0; i < d.table_size; i++) {
            double r = (double)i * tdelta;
            te.push_back(pot_energy(r));
            tf.push_back(pot_force(r));
        }
    }
    // Computation::compute_energy / compute_force (computations.rs:123-144)
    static double interpolate(const std::vector<double>& t, double delta, double r) {
        double binf = std::floor(r / delta);
        if (binf < 0.0 || binf >= (double)t.size()) return 0.0;
        size_t bin = (size_t)binf;
        if (bin < t.size() - 1) {
            double dx = r - (double)bin * delta;
            double slope = (t[bin + 1] - t[bin]) / delta;
            return t[bin] + dx * slope;
        }
        return 0.0;
    }
    // the PairPotential's energy / force: the table when there is one
    double comp_energy(double r) const { return d.table_size > 0 ? interpolate(te, tdelta, r) : pot_energy(r); }
    double comp_force(double r) const { return d.table_size > 0 ? interpolate(tf, tdelta, r) : pot_force(r); }

    // Potential::energy
    double pot_energy(double r) const {
        switch (d.type) {
            case ORC_PAIR_LJ: {  // functions.rs:85-88
                double s6 = powi6(d.p0 / r);
                return 4.0 * d.p1 * (s6 * s6 - s6);
            }
            case ORC_PAIR_BUCKINGHAM: {  // functions.rs:287-292
                double r3 = r * r * r;
                double r6 = r3 * r3;
                double e = std::exp(-r / d.p2);
                return d.p0 * e - d.p1 / r6;
            }
            case ORC_PAIR_HARMONIC: {  // functions.rs:135-139
                double dx = r - d.p1;
                return 0.5 * d.p0 * dx * dx;
            }
            case ORC_PAIR_BMH: {  // functions.rs:354-359
                double r2 = r * r;
                double r6 = r2 * r2 * r2;
                double e = std::exp((d.p3 - r) / d.p4);
                return d.p0 * e - d.p1 / r6 + d.p2 / (r6 * r2);
            }
            case ORC_PAIR_MORSE: {  // functions.rs:415-418
                double rc = 1.0 - std::exp((d.p1 - r) * d.p0);
                return d.p2 * rc * rc;
            }
            case ORC_PAIR_GAUSSIAN:  // functions.rs:475-477
                return -d.p0 * std::exp(-d.p1 * r * r);
            case ORC_PAIR_MIE: {  // functions.rs:553-558
                double sr = d.p0 / r;
                return mie_prefac() * (std::pow(sr, d.p2) - std::pow(sr, d.p3));
            }
            default:
                return 0.0;
        }
    }
    // Mie::new prefactor (functions.rs:540-549)
    double mie_prefac() const {
        double n = d.p2, mm = d.p3;
        return n / (n - mm) * std::pow(n / mm, mm / (n - mm)) * d.p1;
    }
    // Potential::force
    double pot_force(double r) const {
        switch (d.type) {
            case ORC_PAIR_LJ: {  // functions.rs:90-93
                double s6 = powi6(d.p0 / r);
                return -24.0 * d.p1 * (s6 - 2.0 * (s6 * s6)) / r;
            }
            case ORC_PAIR_BUCKINGHAM: {  // functions.rs:294-299
                double r3 = r * r * r;
                double r7 = r3 * r3 * r;
                double e = std::exp(-r / d.p2);
                return d.p0 / d.p2 * e - 6.0 * d.p1 / r7;
            }
            case ORC_PAIR_HARMONIC:  // functions.rs:141-143
                return d.p0 * (d.p1 - r);
            case ORC_PAIR_BMH: {  // functions.rs:361-366
                double r2 = r * r;
                double r7 = r2 * r2 * r2 * r;
                double e = std::exp((d.p3 - r) / d.p4);
                return d.p0 / d.p4 * e - 6.0 * d.p1 / r7 + 8.0 * d.p2 / (r7 * r2);
            }
            case ORC_PAIR_MORSE: {  // functions.rs:420-423, as written there
                double e = std::exp((d.p1 - r) * d.p0);
                return 2.0 * d.p2 * (1.0 - e * e) * d.p0;
            }
            case ORC_PAIR_GAUSSIAN:  // functions.rs:479-481
                return 2.0 * d.p1 * r * pot_energy(r);
            case ORC_PAIR_MIE: {  // functions.rs:560-565
                double sr = d.p0 / r;
                double rep = std::pow(sr, d.p2), att = std::pow(sr, d.p3);
                return mie_prefac() * (d.p2 * rep - d.p3 * att) / r;
            }
            default:
                return 0.0;
        }
    }
    double pot_tail_energy(double rc) const {
        switch (d.type) {
            case ORC_PAIR_LJ: {  // functions.rs:97-103
                double s3 = d.p0 * d.p0 * d.p0;
                double rc3 = rc * rc * rc;
                double s9 = s3 * s3 * s3;
                double rc9 = rc3 * rc3 * rc3;
                return 4.0 / 3.0 * d.p1 * s3 * (1.0 / 3.0 * s9 / rc9 - s3 / rc3);
            }
            case ORC_PAIR_BUCKINGHAM: {  // functions.rs:303-309
                double rc2 = rc * rc;
                double rc3 = rc2 * rc;
                double e = std::exp(-rc / d.p2);
                double factor = rc2 - 2.0 * rc * d.p2 + 2.0 * d.p2 * d.p2;
                return d.p0 * d.p2 * e * factor - d.p1 / (3.0 * rc3);
            }
            case ORC_PAIR_BMH: {  // functions.rs:370-376
                double rc2 = rc * rc;
                double rc3 = rc2 * rc;
                double e = std::exp((d.p3 - rc) / d.p4);
                double factor = rc2 - 2.0 * rc * d.p4 + 2.0 * d.p4 * d.p4;
                return d.p0 * d.p4 * e * factor - d.p1 / (3.0 * rc3) + d.p2 / (5.0 * rc2 * rc3);
            }
            case ORC_PAIR_GAUSSIAN: {  // functions.rs:485-488
                double b = d.p1;
                return pot_energy(rc) * rc / (2.0 * b) -
                       d.p0 * std::sqrt(PI) * std::erfc(std::sqrt(b) * rc) / (4.0 * std::pow(b, 3.0 / 2.0));
            }
            case ORC_PAIR_MIE: {  // functions.rs:569-579
                if (d.p3 <= 3.0) return 0.0;
                double src = d.p0 / rc;
                double n3 = d.p2 - 3.0, m3 = d.p3 - 3.0;
                double s3 = d.p0 * d.p0 * d.p0;  // f64::powi(sigma, 3)
                return mie_prefac() * s3 * (std::pow(src, n3) / n3 - std::pow(src, m3) / m3);
            }
            default:
                return 0.0;
        }
    }
    double pot_tail_virial(double rc) const {
        switch (d.type) {
            case ORC_PAIR_LJ: {  // functions.rs:105-111
                double s3 = d.p0 * d.p0 * d.p0;
                double rc3 = rc * rc * rc;
                double s9 = s3 * s3 * s3;
                double rc9 = rc3 * rc3 * rc3;
                return 8.0 * d.p1 * s3 * (2.0 / 3.0 * s9 / rc9 - s3 / rc3);
            }
            case ORC_PAIR_BUCKINGHAM: {  // functions.rs:311-318, including the "+ 8.0"
                double rc2 = rc * rc;
                double rc3 = rc2 * rc;
                double e = std::exp(-rc / d.p2);
                double factor = rc3 + 3.0 * rc2 * d.p2 + 6.0 * rc * d.p2 * d.p2 +
                                6.0 * d.p2 * d.p2 * d.p2;
                return d.p0 * e * factor - 20.0 * d.p1 / rc3 + 8.0;
            }
            case ORC_PAIR_BMH: {  // functions.rs:378-385
                double rc2 = rc * rc;
                double rc3 = rc2 * rc;
                double e = std::exp((d.p3 - rc) / d.p4);
                double factor = rc3 + 3.0 * rc2 * d.p4 + 6.0 * rc * d.p4 * d.p4 + 6.0 * d.p4 * d.p4 * d.p4;
                return d.p0 * e * factor - 20.0 * d.p1 / rc3 + 8.0 * d.p2 / (5.0 * rc2 * rc3);
            }
            case ORC_PAIR_GAUSSIAN: {  // functions.rs:490-493
                double b = d.p1;
                return 3.0 * std::sqrt(PI) * d.p0 * std::erfc(std::sqrt(b) * rc) / (4.0 * std::pow(b, 3.0 / 2.0)) -
                       pot_energy(rc) * rc * (2.0 * b * rc * rc + 3.0) / (2.0 * b);
            }
            case ORC_PAIR_MIE: {  // functions.rs:581-591
                if (d.p3 <= 3.0) return 0.0;
                double src = d.p0 / rc;
                double n3 = d.p2 - 3.0, m3 = d.p3 - 3.0;
                double s3 = d.p0 * d.p0 * d.p0;
                return mie_prefac() * s3 * (std::pow(src, n3) * d.p2 / n3 - std::pow(src, m3) * d.p3 / m3);
            }
            default:
                return 0.0;
        }
    }

    // PairInteraction (energy/pairs.rs:185-296)
    double energy(double r) const {
        if (r >= d.cutoff) return 0.0;
        double e = comp_energy(r);
        return d.shifted ? e - shift : e;
    }
    double force(double r) const {
        if (r >= d.cutoff) return 0.0;
        return comp_force(r);
    }
    // PairPotential::virial default (energy/mod.rs:137-142) behind the cutoff test
    M3 virial(const V3& r) const {
        if (vnorm(r) >= d.cutoff) return mzero();
        double fact = comp_force(vnorm(r));
        V3 rn = vnormalized(r);
        V3 f = vscale(fact, rn);
        return tensorial(f, r);
    }
    double tail_energy() const { return d.tail ? pot_tail_energy(d.cutoff) : 0.0; }
    double tail_virial_scalar() const { return d.tail ? pot_tail_virial(d.cutoff) : 0.0; }
};

struct Bonded {
    orc_bonded d;
    bool present() const { return d.type != 0; }
    // Potential::energy / force of Harmonic (functions.rs:135-143), CosineHarmonic
    // (functions.rs:190-207, cos x0 taken at construction), Torsion (functions.rs:244-256)
    // and Morse (functions.rs:414-424, the force as written there)
    double energy(double x) const {
        if (d.type == ORC_PAIR_MORSE) {
            double rc = 1.0 - std::exp((d.x0 - x) * d.a);
            return d.k * rc * rc;
        }
        if (d.type == ORC_BONDED_COSINE_HARMONIC) {
            double dr = std::cos(x) - std::cos(d.x0);
            return 0.5 * d.k * dr * dr;
        }
        if (d.type == ORC_BONDED_TORSION) {
            double n = (double)d.n;
            double cs = std::cos(n * x - d.x0);
            return d.k * (1.0 + cs);
        }
        if (d.type != ORC_PAIR_HARMONIC) return 0.0;
        double dx = x - d.x0;
        return 0.5 * d.k * dx * dx;
    }
    double force(double x) const {
        if (d.type == ORC_PAIR_MORSE) {
            double ex = std::exp((d.x0 - x) * d.a);
            return 2.0 * d.k * (1.0 - ex * ex) * d.a;
        }
        if (d.type == ORC_BONDED_COSINE_HARMONIC) return d.k * (std::cos(x) - std::cos(d.x0)) * std::sin(x);
        if (d.type == ORC_BONDED_TORSION) {
            double n = (double)d.n;
            double sn = std::sin(n * x - d.x0);
            return d.k * n * sn;
        }
        if (d.type != ORC_PAIR_HARMONIC) return 0.0;
        return d.k * (d.x0 - x);
    }
};

// UnitCell::dihedral_and_derivatives (cells.rs:379-411); image(v) applies the
// cell's vector_image
template <typename Image>
double dihedral_and_derivatives(const V3& r1, const V3& r2, const V3& r3, const V3& r4, Image image, V3& d1,
                                V3& d2, V3& d3, V3& d4) {
    V3 r12 = vsub(r2, r1);
    image(r12);
    V3 r23 = vsub(r3, r2);
    image(r23);
    V3 r34 = vsub(r4, r3);
    image(r34);
    V3 u = vcross(r12, r23);
    V3 v = vcross(r23, r34);
    double u_norm2 = vnorm2(u);
    double v_norm2 = vnorm2(v);
    double r23_norm2 = vnorm2(r23);
    double r23_norm = std::sqrt(r23_norm2);
    d1 = vscale(-r23_norm / u_norm2, u);
    d4 = vscale(r23_norm / v_norm2, v);
    double r23_r34 = vdot(r23, r34);
    double r12_r23 = vdot(r12, r23);
    d2 = vadd(vscale(-r12_r23 / r23_norm2 - 1.0, d1), vscale(r23_r34 / r23_norm2, d4));
    d3 = vadd(vscale(-r23_r34 / r23_norm2 - 1.0, d4), vscale(r12_r23 / r23_norm2, d1));
    return std::atan2(vdot(vscale(r23_norm, v), r12), vdot(u, v));
}

// BondPath (energy/restrictions.rs:37-50)
enum BondPath { PATH_NONE, PATH_SAME, PATH_ONE, PATH_TWO, PATH_THREE, PATH_FAR };

struct RestrictionInfo {
    bool excluded;
    double scaling;
};

// PairRestriction::information (energy/restrictions.rs:85-115)
RestrictionInfo information(int restriction, double scale14, BondPath path) {
    bool same = path != PATH_NONE;
    bool excluded = false;
    switch (restriction) {
        case ORC_RESTRICT_NONE: excluded = false; break;
        case ORC_RESTRICT_INTER: excluded = same; break;
        case ORC_RESTRICT_INTRA: excluded = !same; break;
        case ORC_RESTRICT_EXCLUDE12: excluded = path == PATH_ONE; break;
        case ORC_RESTRICT_EXCLUDE13:
        case ORC_RESTRICT_SCALE14: excluded = path == PATH_ONE || path == PATH_TWO; break;
        case ORC_RESTRICT_EXCLUDE14:
            excluded = path == PATH_ONE || path == PATH_TWO || path == PATH_THREE;
            break;
    }
    double scaling = 1.0;
    if (restriction == ORC_RESTRICT_SCALE14 && path == PATH_THREE) scaling = scale14;
    return RestrictionInfo{excluded, scaling};
}

}  // namespace

// ---------------------------------------------------------------------------
// The system
// ---------------------------------------------------------------------------
struct orc_system {
    int64_t n = 0;
    std::vector<V3> pos;
    std::vector<int32_t> kind;
    std::vector<double> charge, mass;
    std::vector<int32_t> mol;
    std::vector<std::pair<int64_t, int64_t>> mol_range;  // [start, end) per molecule
    int32_t nk = 0;
    std::vector<PairPot> pairs;
    std::vector<Bonded> bond_pots, angle_pots, dihedral_pots;
    std::vector<std::pair<int32_t, int32_t>> bonds;          // i < j
    std::vector<std::tuple<int32_t, int32_t, int32_t>> angles;  // i < k
    std::vector<std::tuple<int32_t, int32_t, int32_t, int32_t>> dihedrals;
    // bond distances flags per molecule, indexed by (i - start, j - start)
    std::vector<std::vector<uint8_t>> distances;
    Cell cell;
    orc_coulomb coul;
    double ewald_alpha = 0.0;

    // Ewald state (energy/global/ewald.rs:187-196)
    struct KFactor {
        int ikx, iky, ikz;
        double energy;
        V3 field;
        M3 virial;
    };
    std::vector<KFactor> factors;
    double kmax2 = 0.0;
    int kmax = 0;
    std::vector<Complex> eikr;  // [(k + kmax)][axis][atom]
    std::vector<Complex> rho;
    bool factors_ready = false;

    // Wolf constants (wolf.rs:68-84)
    double wolf_alpha = 0.0, wolf_ec = 0.0, wolf_fc = 0.0;

    // EnergyCache (sys/cache.rs:22-42)
    std::vector<double> pairs_cache;
    double c_pairs = 0, c_tail = 0, c_bonds = 0, c_angles = 0, c_coulomb = 0;
    bool has_pending = false;
    int64_t pending_mol = -1;
    std::vector<double> pending_new_pairs;  // rows of the moved molecule: [local i][j]
    double pending_pairs_delta = 0, pending_coulomb_delta = 0;
    std::vector<Complex> pending_delta_rho;
    // move_all_molecules_cost (cache.rs:238-292): the pending update, and the
    // configuration before the move (the Resize move's `previous`)
    bool pending_all = false;
    std::vector<double> pending_all_pairs;  // [i * n + j], between molecules
    double pending_all_tail = 0, pending_all_coulomb = 0;
    Cell saved_cell;
    std::vector<V3> saved_pos;

    const PairPot* pair(int64_t i, int64_t j) const {
        const PairPot& p = pairs[(size_t)kind[i] * nk + kind[j]];
        return p.d.type == ORC_PAIR_ABSENT ? nullptr : &p;
    }

    // Configuration::nearest_image (configuration.rs:399-403)
    V3 nearest_image(int64_t i, int64_t j) const {
        V3 d = vsub(pos[i], pos[j]);
        cell.vector_image(d);
        return d;
    }
    double distance(int64_t i, int64_t j) const { return cell.distance(pos[i], pos[j]); }

    // Configuration::bond_path (configuration.rs:124-145)
    BondPath bond_path(int64_t i, int64_t j) const {
        if (mol[i] != mol[j]) return PATH_NONE;
        if (i == j) return PATH_SAME;
        int64_t m = mol[i];
        int64_t start = mol_range[m].first, size = mol_range[m].second - start;
        uint8_t flags = distances[m][(size_t)(i - start) * size + (j - start)];
        if (flags & 1) return PATH_ONE;
        if (flags & 2) return PATH_TWO;
        if (flags & 4) return PATH_THREE;
        return PATH_FAR;
    }

    ~orc_system() = default;
};

namespace {

// Bonding::rebuild (sys/config/bonding.rs:78-157) restated per molecule
void rebuild_bonding(orc_system* s) {
    std::set<std::pair<int32_t, int32_t>> bonds(s->bonds.begin(), s->bonds.end());
    std::set<std::tuple<int32_t, int32_t, int32_t>> angles;
    std::set<std::tuple<int32_t, int32_t, int32_t, int32_t>> dihedrals;
    auto make_angle = [](int32_t a, int32_t b, int32_t c) {
        return std::make_tuple(std::min(a, c), b, std::max(a, c));
    };
    auto make_dihedral = [](int32_t a, int32_t b, int32_t c, int32_t d) {
        if (std::max(a, b) < std::max(c, d)) return std::make_tuple(a, b, c, d);
        return std::make_tuple(d, c, b, a);
    };
    for (auto& b1 : bonds) {
        for (auto& b2 : bonds) {
            if (b1 == b2) continue;
            std::tuple<int32_t, int32_t, int32_t> angle;
            if (b1.first == b2.second) angle = make_angle(b2.first, b2.second, b1.second);
            else if (b1.second == b2.first) angle = make_angle(b1.first, b1.second, b2.second);
            else if (b1.second == b2.second) angle = make_angle(b1.first, b1.second, b2.first);
            else if (b1.first == b2.first) angle = make_angle(b1.second, b1.first, b2.second);
            else continue;
            angles.insert(angle);
            int32_t ai = std::get<0>(angle), aj = std::get<1>(angle), ak = std::get<2>(angle);
            for (auto& b3 : bonds) {
                if (b2 == b3) continue;
                if (ak == b3.first && aj != b3.second)
                    dihedrals.insert(make_dihedral(ai, aj, ak, b3.second));
                else if (ak == b3.second && aj != b3.first)
                    dihedrals.insert(make_dihedral(ai, aj, ak, b3.first));
                else if (ai == b3.second && aj != b3.first)
                    dihedrals.insert(make_dihedral(b3.first, ai, aj, ak));
                else if (ai == b3.first && aj != b3.second)
                    dihedrals.insert(make_dihedral(b3.second, ai, aj, ak));
            }
        }
    }
    s->angles.assign(angles.begin(), angles.end());
    s->dihedrals.assign(dihedrals.begin(), dihedrals.end());

    // rebuild_connections (bonding.rs:159-186)
    s->distances.assign(s->mol_range.size(), {});
    for (size_t m = 0; m < s->mol_range.size(); m++) {
        int64_t size = s->mol_range[m].second - s->mol_range[m].first;
        s->distances[m].assign((size_t)(size * size), 0);
    }
    auto add = [&](int32_t i, int32_t j, uint8_t term) {
        int64_t m = s->mol[i];
        int64_t start = s->mol_range[m].first, size = s->mol_range[m].second - start;
        s->distances[m][(size_t)(i - start) * size + (j - start)] |= term;
    };
    for (auto& b : s->bonds) {
        add(b.first, b.second, 1);
        add(b.second, b.first, 1);
    }
    for (auto& a : s->angles) {
        add(std::get<0>(a), std::get<2>(a), 2);
        add(std::get<2>(a), std::get<0>(a), 2);
    }
    for (auto& d : s->dihedrals) {
        add(std::get<0>(d), std::get<3>(d), 4);
        add(std::get<3>(d), std::get<0>(d), 4);
    }
}

int nthreads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
int thread_id() {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

// ---------------------------------------------------------------------------
// Pair potentials: sys/compute.rs:30-59, sys/energy.rs:32-79, compute.rs:198-231
// ---------------------------------------------------------------------------
double pair_energy_ij(const orc_system* s, BondPath path, double r, int64_t i, int64_t j) {
    const PairPot* p = s->pair(i, j);
    if (!p) return 0.0;
    RestrictionInfo info = information(p->d.restriction, p->d.scale14, path);
    if (info.excluded) return 0.0;
    return info.scaling * p->energy(r);
}

double pairs_energy(const orc_system* s) {
    double total = 0.0;
    int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
    for (int64_t i = 0; i < n; i++) {
        double local = 0.0;
        for (int64_t j = i + 1; j < n; j++) {
            double r = vnorm(s->nearest_image(i, j));
            BondPath path = s->bond_path(i, j);
            local += pair_energy_ij(s, path, r, i, j);
        }
        total += local;
    }
    return total;
}

double pairs_tail(const orc_system* s) {
    double energy = 0.0;
    double volume = s->cell.volume();
    std::vector<int64_t> counts(s->nk, 0);
    for (int64_t i = 0; i < s->n; i++) counts[s->kind[i]]++;
    for (int a = 0; a < s->nk; a++) {
        if (!counts[a]) continue;
        for (int b = 0; b < s->nk; b++) {
            if (!counts[b]) continue;
            double two_pi_density = 2.0 * PI * (double)counts[a] * (double)counts[b] / volume;
            const PairPot& p = s->pairs[(size_t)a * s->nk + b];
            if (p.d.type != ORC_PAIR_ABSENT) energy += two_pi_density * p.tail_energy();
        }
    }
    return energy;
}

M3 pairs_tail_virial(const orc_system* s) {
    M3 virial = mzero();
    double volume = s->cell.volume();
    std::vector<int64_t> counts(s->nk, 0);
    for (int64_t i = 0; i < s->n; i++) counts[s->kind[i]]++;
    for (int a = 0; a < s->nk; a++) {
        if (!counts[a]) continue;
        for (int b = 0; b < s->nk; b++) {
            if (!counts[b]) continue;
            double two_pi_density = 2.0 * PI * (double)counts[a] * (double)counts[b] / volume;
            const PairPot& p = s->pairs[(size_t)a * s->nk + b];
            if (p.d.type == ORC_PAIR_ABSENT) continue;
            // PairInteraction::tail_virial: tail_virial(rc) * (Matrix3::one() / 3.0)
            M3 t = mzero();
            if (p.d.tail) {
                double w = p.tail_virial_scalar();
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) t.m[k][l] = w * ((k == l ? 1.0 : 0.0) / 3.0);
            }
            madd(virial, mscale(two_pi_density, t));
        }
    }
    return virial;
}

void reduce_thread_forces(const std::vector<std::vector<V3>>& tl, int64_t n, double* out) {
    for (auto& buf : tl)
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) out[3 * i + k] += buf[i][k];
}

void pairs_forces(const orc_system* s, double* out) {
    int64_t n = s->n;
    std::vector<std::vector<V3>> tl(nthreads(), std::vector<V3>(n, vzero()));
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        auto& forces = tl[thread_id()];
        V3 force_i = vzero();
        for (int64_t j = i + 1; j < n; j++) {
            BondPath path = s->bond_path(i, j);
            V3 d = s->nearest_image(i, j);
            V3 dn = vnormalized(d);
            double r = vnorm(d);
            const PairPot* p = s->pair(i, j);
            if (p) {
                RestrictionInfo info = information(p->d.restriction, p->d.scale14, path);
                if (!info.excluded) {
                    V3 f = vscale(info.scaling * p->force(r), dn);
                    force_i = vadd(force_i, f);
                    forces[j] = vsub(forces[j], f);
                }
            }
        }
        forces[i] = vadd(forces[i], force_i);
    }
    reduce_thread_forces(tl, n, out);
}

M3 pairs_virial(const orc_system* s) {
    int64_t n = s->n;
    std::vector<M3> partial(nthreads(), mzero());
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        M3 local = mzero();
        for (int64_t j = i + 1; j < n; j++) {
            BondPath path = s->bond_path(i, j);
            const PairPot* p = s->pair(i, j);
            if (p) {
                RestrictionInfo info = information(p->d.restriction, p->d.scale14, path);
                if (!info.excluded) {
                    V3 d = s->nearest_image(i, j);
                    madd(local, mscale(info.scaling, p->virial(d)));
                }
            }
        }
        madd(partial[thread_id()], local);
    }
    M3 total = mzero();
    for (auto& m : partial) madd(total, m);
    return total;
}

// ---------------------------------------------------------------------------
// Bonds and angles: compute.rs:62-84, 233-241; energy.rs:90-120; cells.rs:322-362
// ---------------------------------------------------------------------------
const Bonded* bond_pot(const orc_system* s, int32_t i, int32_t j) {
    const Bonded& b = s->bond_pots[(size_t)s->kind[i] * s->nk + s->kind[j]];
    return b.present() ? &b : nullptr;
}
const Bonded* angle_pot(const orc_system* s, int32_t i, int32_t j, int32_t k) {
    size_t nk = s->nk;
    const Bonded& b = s->angle_pots[((size_t)s->kind[i] * nk + s->kind[j]) * nk + s->kind[k]];
    return b.present() ? &b : nullptr;
}

const Bonded* dihedral_pot(const orc_system* s, int32_t i, int32_t j, int32_t k, int32_t l) {
    size_t nk = s->nk;
    if (s->dihedral_pots.empty()) return nullptr;
    const Bonded& b =
        s->dihedral_pots[(((size_t)s->kind[i] * nk + s->kind[j]) * nk + s->kind[k]) * nk + s->kind[l]];
    return b.present() ? &b : nullptr;
}
double cell_dihedral(const orc_system* s, int32_t i, int32_t j, int32_t k, int32_t l, V3& d1, V3& d2, V3& d3,
                     V3& d4) {
    return dihedral_and_derivatives(s->pos[i], s->pos[j], s->pos[k], s->pos[l],
                                    [&](V3& v) { s->cell.vector_image(v); }, d1, d2, d3, d4);
}
// EnergyEvaluator::dihedrals (sys/energy.rs:130-141); UnitCell::dihedral (cells.rs:364-375)
// is the angle of dihedral_and_derivatives
double dihedrals_energy(const orc_system* s) {
    double e = 0.0;
    for (auto& d : s->dihedrals) {
        int32_t i = std::get<0>(d), j = std::get<1>(d), k = std::get<2>(d), l = std::get<3>(d);
        const Bonded* p = dihedral_pot(s, i, j, k, l);
        if (!p) continue;
        V3 d1, d2, d3, d4;
        e += p->energy(cell_dihedral(s, i, j, k, l, d1, d2, d3, d4));
    }
    return e;
}

double bonds_energy(const orc_system* s) {
    double e = 0.0;
    for (auto& b : s->bonds) {
        double r = vnorm(s->nearest_image(b.first, b.second));
        const Bonded* p = bond_pot(s, b.first, b.second);
        if (p) e += p->energy(r);
    }
    return e;
}

// UnitCell::angle (cells.rs:322-330)
double cell_angle(const orc_system* s, int32_t i, int32_t j, int32_t k) {
    V3 r12 = vsub(s->pos[i], s->pos[j]);
    s->cell.vector_image(r12);
    V3 r23 = vsub(s->pos[k], s->pos[j]);
    s->cell.vector_image(r23);
    return std::acos(vdot(r12, r23) / (vnorm(r12) * vnorm(r23)));
}

double angles_energy(const orc_system* s) {
    double e = 0.0;
    for (auto& a : s->angles) {
        int32_t i = std::get<0>(a), j = std::get<1>(a), k = std::get<2>(a);
        double theta = cell_angle(s, i, j, k);
        const Bonded* p = angle_pot(s, i, j, k);
        if (p) e += p->energy(theta);
    }
    return e;
}

void bonded_forces(const orc_system* s, int terms, double* out) {
    if (terms & ORC_TERM_BONDS) {
        for (auto& b : s->bonds) {
            V3 d = s->nearest_image(b.first, b.second);
            V3 dn = vnormalized(d);
            double r = vnorm(d);
            const Bonded* p = bond_pot(s, b.first, b.second);
            if (p) {
                V3 f = vscale(p->force(r), dn);
                for (int k = 0; k < 3; k++) {
                    out[3 * b.first + k] += f[k];
                    out[3 * b.second + k] -= f[k];
                }
            }
        }
    }
    if (terms & ORC_TERM_ANGLES) {
        for (auto& a : s->angles) {
            int32_t i = std::get<0>(a), j = std::get<1>(a), k = std::get<2>(a);
            // UnitCell::angle_and_derivatives (cells.rs:335-362)
            V3 r12 = vsub(s->pos[i], s->pos[j]);
            s->cell.vector_image(r12);
            V3 r23 = vsub(s->pos[k], s->pos[j]);
            s->cell.vector_image(r23);
            double r12_norm = vnorm(r12), r23_norm = vnorm(r23);
            V3 r12n = vdiv(r12, r12_norm), r23n = vdiv(r23, r23_norm);
            double cos = vdot(r12n, r23n);
            double sin_inv = 1.0 / std::sqrt(1.0 - cos * cos);
            V3 d1 = vdiv(vscale(sin_inv, vsub(vscale(cos, r12n), r23n)), r12_norm);
            V3 d3 = vdiv(vscale(sin_inv, vsub(vscale(cos, r23n), r12n)), r23_norm);
            V3 sum = vadd(d1, d3);
            V3 d2 = V3{{-sum[0], -sum[1], -sum[2]}};
            double theta = std::acos(cos);
            const Bonded* p = angle_pot(s, i, j, k);
            if (p) {
                double f = p->force(theta);
                for (int c = 0; c < 3; c++) {
                    out[3 * i + c] += f * d1[c];
                    out[3 * j + c] += f * d2[c];
                    out[3 * k + c] += f * d3[c];
                }
            }
        }
    }
}

// dihedral forces (compute.rs:86-96)
void dihedral_forces(const orc_system* s, double* out) {
    for (auto& d : s->dihedrals) {
        int32_t q[4] = {std::get<0>(d), std::get<1>(d), std::get<2>(d), std::get<3>(d)};
        const Bonded* p = dihedral_pot(s, q[0], q[1], q[2], q[3]);
        if (!p) continue;
        V3 dv[4];
        double phi = cell_dihedral(s, q[0], q[1], q[2], q[3], dv[0], dv[1], dv[2], dv[3]);
        double f = p->force(phi);
        for (int a = 0; a < 4; a++)
            for (int c = 0; c < 3; c++) out[3 * q[a] + c] += f * dv[a][c];
    }
}

M3 bonds_virial(const orc_system* s) {
    M3 virial = mzero();
    for (auto& b : s->bonds) {
        V3 r = s->nearest_image(b.first, b.second);
        const Bonded* p = bond_pot(s, b.first, b.second);
        if (p) {
            // BondPotential::virial (energy/mod.rs:188-193)
            double fact = p->force(vnorm(r));
            V3 f = vscale(fact, vnormalized(r));
            madd(virial, tensorial(f, r));
        }
    }
    return virial;
}

// ---------------------------------------------------------------------------
// Ewald (energy/global/ewald.rs)
// ---------------------------------------------------------------------------
RestrictionInfo coul_info(const orc_system* s, int64_t i, int64_t j) {
    return information(s->coul.restriction, s->coul.scale14, s->bond_path(i, j));
}

// Ewald::prepare + compute_ewald_factors_triclinic (ewald.rs:130-183, 353-379)
void ewald_prepare(orc_system* s) {
    if (s->factors_ready) return;
    s->factors_ready = true;
    V3 k111 = s->cell.k_vector(1.0, 1.0, 1.0);
    double max = std::max(std::max(k111[0], k111[1]), k111[2]) * (double)s->kmax;
    s->kmax2 = 1.0001 * max * max;

    double alpha = s->ewald_alpha;
    double alpha_sq_inv_fourth = 0.25 / (alpha * alpha);
    double four_pi_v = 4.0 * PI / s->cell.volume();
    s->factors.clear();
    auto push = [&](V3 k, double k2, int ikx, int iky, int ikz) {
        orc_system::KFactor f;
        f.ikx = ikx;
        f.iky = iky;
        f.ikz = ikz;
        f.energy = four_pi_v * std::exp(-k2 * alpha_sq_inv_fourth) / k2;
        f.field = vscale(2.0 * f.energy, k);
        double virial_factor = -2.0 * (1.0 / k2 + alpha_sq_inv_fourth);
        M3 kk = tensorial(k, k);
        M3 v;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                v.m[a][b] = (a == b ? 1.0 : 0.0) + virial_factor * kk.m[a][b];
        f.virial = mscale(f.energy, v);
        s->factors.push_back(f);
    };
    int kmax = s->kmax;
    for (int ikx = 1; ikx < kmax; ikx++)
        for (int iky = -kmax; iky < kmax; iky++)
            for (int ikz = -kmax; ikz < kmax; ikz++) {
                V3 k = s->cell.k_vector(ikx, iky, ikz);
                double k2 = vnorm2(k);
                if (k2 > s->kmax2) continue;
                push(k, k2, ikx, iky, ikz);
            }
    for (int iky = 1; iky < kmax; iky++)
        for (int ikz = -kmax; ikz < kmax; ikz++) {
            V3 k = s->cell.k_vector(0.0, iky, ikz);
            double k2 = vnorm2(k);
            if (k2 > s->kmax2) continue;
            push(k, k2, 0, iky, ikz);
        }
    for (int ikz = 1; ikz < kmax; ikz++) {
        V3 k = s->cell.k_vector(0.0, 0.0, ikz);
        double k2 = vnorm2(k);
        if (k2 > s->kmax2) continue;
        push(k, k2, 0, 0, ikz);
    }
}

inline Complex& eikr_at(orc_system* s, int k, int axis, int64_t i) {
    return s->eikr[((size_t)(k + s->kmax) * 3 + axis) * s->n + i];
}

// Ewald::eik_dot_r (ewald.rs:633-674)
void eik_dot_r(orc_system* s) {
    int64_t n = s->n;
    int kmax = s->kmax;
    s->eikr.assign((size_t)(2 * kmax + 1) * 3 * n, Complex{0.0, 0.0});
    for (int spatial = 0; spatial < 3; spatial++) {
        double idx[3] = {0.0, 0.0, 0.0};
        idx[spatial] = 1.0;
        V3 k = s->cell.k_vector(idx[0], idx[1], idx[2]);
        for (int64_t i = 0; i < n; i++) {
            double phi = vdot(k, s->pos[i]);
            eikr_at(s, 0, spatial, i) = Complex{1.0, 0.0};
            eikr_at(s, 1, spatial, i) = Complex{1.0 * std::cos(phi), 1.0 * std::sin(phi)};
            eikr_at(s, -1, spatial, i) = cconj(eikr_at(s, 1, spatial, i));
        }
    }
    for (int spatial = 0; spatial < 3; spatial++)
        for (int k = 2; k <= kmax; k++)
            for (int64_t i = 0; i < n; i++) {
                eikr_at(s, k, spatial, i) = cmul(eikr_at(s, k - 1, spatial, i), eikr_at(s, 1, spatial, i));
                eikr_at(s, -k, spatial, i) = cconj(eikr_at(s, k, spatial, i));
            }
    s->rho.assign(s->factors.size(), Complex{0.0, 0.0});
    size_t nk = s->factors.size();
#pragma omp parallel for schedule(dynamic, 8)
    for (size_t f = 0; f < nk; f++) {
        const auto& kf = s->factors[f];
        Complex partial{0.0, 0.0};
        for (int64_t i = 0; i < n; i++) {
            Complex phi = cmul(cmul(eikr_at(s, kf.ikx, 0, i), eikr_at(s, kf.iky, 1, i)),
                               eikr_at(s, kf.ikz, 2, i));
            partial.re += s->charge[i] * phi.re;
            partial.im += s->charge[i] * phi.im;
        }
        s->rho[f] = partial;
    }
}

// ewald.rs:383-398
double ewald_real_energy_pair(const orc_system* s, RestrictionInfo info, double qiqj, double r) {
    if (r > s->coul.cutoff) return 0.0;
    double alpha = s->ewald_alpha;
    if (info.excluded) return -qiqj / FOUR_PI_EPSILON_0 * std::erf(alpha * r) / r;
    return qiqj / FOUR_PI_EPSILON_0 * std::erfc(alpha * r) / r;
}

// ewald.rs:402-428
double ewald_real_force_pair(const orc_system* s, RestrictionInfo info, double qiqj, double r) {
    if (r > s->coul.cutoff) return 0.0;
    double alpha = s->ewald_alpha;
    if (info.excluded)
        return qiqj / (FOUR_PI_EPSILON_0 * r * r) *
               (alpha * FRAC_2_SQRT_PI * std::exp(-alpha * alpha * r * r) - std::erf(alpha * r) / r);
    return qiqj / (FOUR_PI_EPSILON_0 * r * r) *
           (alpha * FRAC_2_SQRT_PI * std::exp(-alpha * alpha * r * r) + std::erfc(alpha * r) / r);
}

// Wolf (wolf.rs:90-117)
double wolf_energy_pair(const orc_system* s, double qiqj, double r) {
    if (r > s->coul.cutoff) return 0.0;
    return qiqj * (std::erfc(s->wolf_alpha * r) / r - s->wolf_ec) / FOUR_PI_EPSILON_0;
}
double wolf_energy_self(const orc_system* s, double qi) {
    return qi * qi * 0.5 * (s->wolf_ec + s->wolf_alpha * FRAC_2_SQRT_PI) / FOUR_PI_EPSILON_0;
}
double wolf_force_pair(const orc_system* s, double qiqj, double r) {
    if (r > s->coul.cutoff) return 0.0;
    double rij2 = r * r;
    double alpha_rij = s->wolf_alpha * r;
    double exp_alpha_rij = std::exp(-alpha_rij * alpha_rij);
    double factor = std::erfc(alpha_rij) / rij2 + s->wolf_alpha * FRAC_2_SQRT_PI * exp_alpha_rij / r;
    return qiqj * (factor - s->wolf_fc) / (r * FOUR_PI_EPSILON_0);
}

// Ewald real_space_energy (ewald.rs:431-457), Wolf energy (wolf.rs:177-207)
double coulomb_real_energy(const orc_system* s) {
    int64_t n = s->n;
    double total = 0.0;
    bool ewald = s->coul.kind == ORC_COULOMB_EWALD;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
    for (int64_t i = 0; i < n; i++) {
        double qi = s->charge[i];
        if (qi == 0.0) continue;
        double local = 0.0;
        for (int64_t j = i + 1; j < n; j++) {
            double qj = s->charge[j];
            if (qj == 0.0) continue;
            RestrictionInfo info = coul_info(s, i, j);
            if (ewald) {
                double r = s->distance(i, j);
                local += ewald_real_energy_pair(s, info, qi * qj, r);
            } else {
                if (info.excluded) continue;
                double r = s->distance(i, j);
                local += info.scaling * wolf_energy_pair(s, qi * qj, r);
            }
        }
        if (!ewald) local = local - wolf_energy_self(s, qi);
        total += local;
    }
    return total;
}

// ewald.rs:461-500, wolf.rs:209-249
void coulomb_real_forces(const orc_system* s, double* out) {
    int64_t n = s->n;
    bool ewald = s->coul.kind == ORC_COULOMB_EWALD;
    std::vector<std::vector<V3>> tl(nthreads(), std::vector<V3>(n, vzero()));
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        auto& forces = tl[thread_id()];
        double qi = s->charge[i];
        if (qi == 0.0) continue;
        V3 force_i = vzero();
        for (int64_t j = i + 1; j < n; j++) {
            double qj = s->charge[j];
            if (qj == 0.0) continue;
            RestrictionInfo info = coul_info(s, i, j);
            V3 rij = s->nearest_image(i, j);
            V3 f;
            if (ewald) {
                f = vscale(ewald_real_force_pair(s, info, qi * qj, vnorm(rij)), rij);
            } else {
                if (info.excluded) continue;
                f = vscale(info.scaling * wolf_force_pair(s, qi * qj, vnorm(rij)), rij);
            }
            force_i = vadd(force_i, f);
            forces[j] = vsub(forces[j], f);
        }
        forces[i] = vadd(forces[i], force_i);
    }
    reduce_thread_forces(tl, n, out);
}

// ewald.rs:502-530, wolf.rs:251-282
M3 coulomb_real_virial(const orc_system* s) {
    int64_t n = s->n;
    bool ewald = s->coul.kind == ORC_COULOMB_EWALD;
    std::vector<M3> partial(nthreads(), mzero());
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        double qi = s->charge[i];
        if (qi == 0.0) continue;
        M3 local = mzero();
        for (int64_t j = i + 1; j < n; j++) {
            double qj = s->charge[j];
            if (qj == 0.0) continue;
            RestrictionInfo info = coul_info(s, i, j);
            V3 rij = s->nearest_image(i, j);
            V3 f;
            if (ewald) {
                f = vscale(ewald_real_force_pair(s, info, qi * qj, vnorm(rij)), rij);
            } else {
                if (info.excluded) continue;
                f = vscale(info.scaling * wolf_force_pair(s, qi * qj, vnorm(rij)), rij);
            }
            madd(local, tensorial(f, rij));
        }
        madd(partial[thread_id()], local);
    }
    M3 total = mzero();
    for (auto& m : partial) madd(total, m);
    return total;
}

// ewald.rs:619-626
double ewald_self_energy(const orc_system* s) {
    double q2 = 0.0;
    for (int64_t i = 0; i < s->n; i++) q2 += s->charge[i] * s->charge[i];
    return -s->ewald_alpha / std::sqrt(PI) * q2 / FOUR_PI_EPSILON_0;
}

// ewald.rs:677-688
double ewald_kspace_energy(orc_system* s) {
    eik_dot_r(s);
    double e = 0.0;
    for (size_t f = 0; f < s->factors.size(); f++) e += s->factors[f].energy * cnorm2(s->rho[f]);
    return e / FOUR_PI_EPSILON_0;
}

// ewald.rs:690-720
void ewald_kspace_forces(orc_system* s, double* out) {
    eik_dot_r(s);
    int64_t n = s->n;
    size_t nk = s->factors.size();
    std::vector<std::vector<V3>> tl(nthreads(), std::vector<V3>(n, vzero()));
#pragma omp parallel for schedule(dynamic, 4)
    for (size_t f = 0; f < nk; f++) {
        auto& field = tl[thread_id()];
        const auto& kf = s->factors[f];
        Complex rc = cconj(s->rho[f]);
        for (int64_t i = 0; i < n; i++) {
            Complex e = cmul(cmul(eikr_at(s, kf.ikx, 0, i), eikr_at(s, kf.iky, 1, i)),
                             eikr_at(s, kf.ikz, 2, i));
            Complex partial = cmul(e, rc);
            field[i] = vadd(field[i], vscale(partial.im, kf.field));
        }
    }
    std::vector<double> fieldsum(3 * n, 0.0);
    reduce_thread_forces(tl, n, fieldsum.data());
    for (int64_t i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) out[3 * i + k] += s->charge[i] * fieldsum[3 * i + k] / FOUR_PI_EPSILON_0;
    }
}

// ewald.rs:723-733
M3 ewald_kspace_virial(orc_system* s) {
    eik_dot_r(s);
    M3 v = mzero();
    for (size_t f = 0; f < s->factors.size(); f++) madd(v, mscale(cnorm2(s->rho[f]), s->factors[f].virial));
    M3 r;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) r.m[a][b] = v.m[a][b] / FOUR_PI_EPSILON_0;
    return r;
}

double coulomb_energy_terms(orc_system* s, int terms) {
    double e = 0.0;
    if (s->coul.kind == ORC_COULOMB_NONE) return 0.0;
    if (s->coul.kind == ORC_COULOMB_EWALD) ewald_prepare(s);
    if (terms & ORC_TERM_COUL_REAL) e += coulomb_real_energy(s);
    if (s->coul.kind == ORC_COULOMB_EWALD) {
        if (terms & ORC_TERM_COUL_SELF) e += ewald_self_energy(s);
        if (terms & ORC_TERM_COUL_KSPACE) e += ewald_kspace_energy(s);
    }
    return e;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

orc_system* orc_create(const orc_desc* d) {
    orc_system* s = new orc_system();
    s->n = d->n;
    s->pos.resize(d->n);
    for (int64_t i = 0; i < d->n; i++)
        for (int k = 0; k < 3; k++) s->pos[i][k] = d->positions[3 * i + k];
    s->kind.assign(d->kinds, d->kinds + d->n);
    s->charge.assign(d->charges, d->charges + d->n);
    s->mass.assign(d->masses, d->masses + d->n);
    s->mol.assign(d->molecules, d->molecules + d->n);
    int32_t nmol = 0;
    for (int64_t i = 0; i < d->n; i++) nmol = std::max(nmol, s->mol[i] + 1);
    s->mol_range.assign(nmol, {INT64_MAX, 0});
    for (int64_t i = 0; i < d->n; i++) {
        auto& r = s->mol_range[s->mol[i]];
        r.first = std::min(r.first, i);
        r.second = std::max(r.second, i + 1);
    }
    s->nk = d->n_kinds;
    s->pairs.resize((size_t)s->nk * s->nk);
    for (size_t p = 0; p < s->pairs.size(); p++) {
        s->pairs[p].d = d->pairs[p];
        // PairInteraction::shifted: shift = potential.energy(cutoff) (pairs.rs:86-95)
        s->pairs[p].build_table();
        if (d->pairs[p].shifted) s->pairs[p].shift = s->pairs[p].comp_energy(d->pairs[p].cutoff);
    }
    s->bond_pots.resize((size_t)s->nk * s->nk);
    for (size_t p = 0; p < s->bond_pots.size(); p++) s->bond_pots[p].d = d->bond_pots ? d->bond_pots[p] : orc_bonded{0, 0, 0, 0, 0};
    s->angle_pots.resize((size_t)s->nk * s->nk * s->nk);
    for (size_t p = 0; p < s->angle_pots.size(); p++) s->angle_pots[p].d = d->angle_pots ? d->angle_pots[p] : orc_bonded{0, 0, 0, 0, 0};
    if (d->dihedral_pots) {
        s->dihedral_pots.resize((size_t)s->nk * s->nk * s->nk * s->nk);
        for (size_t p = 0; p < s->dihedral_pots.size(); p++) s->dihedral_pots[p].d = d->dihedral_pots[p];
    }
    for (int64_t b = 0; b < d->n_bonds; b++) {
        int32_t i = d->bonds[2 * b], j = d->bonds[2 * b + 1];
        s->bonds.push_back({std::min(i, j), std::max(i, j)});
    }
    std::sort(s->bonds.begin(), s->bonds.end());
    s->bonds.erase(std::unique(s->bonds.begin(), s->bonds.end()), s->bonds.end());
    rebuild_bonding(s);
    if (d->cell_shape == ORC_CELL_TRICLINIC) s->cell.init_matrix(d->cell_matrix, ORC_CELL_TRICLINIC);
    else s->cell.init(d->cell[0], d->cell[1], d->cell[2]);
    s->coul = d->coulomb;
    s->kmax = d->coulomb.kmax;
    if (s->coul.kind == ORC_COULOMB_EWALD) {
        // Ewald::new: alpha defaults to PI / cutoff (ewald.rs:278-279)
        s->ewald_alpha = d->coulomb.alpha > 0.0 ? d->coulomb.alpha : PI / d->coulomb.cutoff;
    } else if (s->coul.kind == ORC_COULOMB_WOLF) {
        double cutoff = d->coulomb.cutoff;
        double alpha = PI / cutoff;
        double ac = alpha * cutoff;
        double ac2 = ac * ac;
        s->wolf_alpha = alpha;
        s->wolf_ec = std::erfc(ac) / cutoff;
        s->wolf_fc = std::erfc(ac) / (cutoff * cutoff) + FRAC_2_SQRT_PI * alpha * std::exp(-ac2) / cutoff;
    }
    return s;
}

void orc_destroy(orc_system* s) { delete s; }

int orc_num_threads(void) { return nthreads(); }
void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_set_positions(orc_system* s, const double* p) {
    for (int64_t i = 0; i < s->n; i++)
        for (int k = 0; k < 3; k++) s->pos[i][k] = p[3 * i + k];
}
void orc_get_positions(const orc_system* s, double* p) {
    for (int64_t i = 0; i < s->n; i++)
        for (int k = 0; k < 3; k++) p[3 * i + k] = s->pos[i][k];
}

int64_t orc_n_angles(const orc_system* s) { return (int64_t)s->angles.size(); }
void orc_angles(const orc_system* s, int32_t* out) {
    for (size_t a = 0; a < s->angles.size(); a++) {
        out[3 * a] = std::get<0>(s->angles[a]);
        out[3 * a + 1] = std::get<1>(s->angles[a]);
        out[3 * a + 2] = std::get<2>(s->angles[a]);
    }
}

// PotentialEnergy::compute (compute.rs:111-128), per term
double orc_energy(orc_system* s, int terms) {
    double e = 0.0;
    if (terms & ORC_TERM_PAIRS) e += pairs_energy(s);
    if (terms & ORC_TERM_TAIL) e += pairs_tail(s);
    if (terms & ORC_TERM_BONDS) e += bonds_energy(s);
    if (terms & ORC_TERM_ANGLES) e += angles_energy(s);
    if (terms & ORC_TERM_DIHEDRALS) e += dihedrals_energy(s);
    e += coulomb_energy_terms(s, terms);
    return e;
}

// Forces::compute (compute.rs:30-108), per term
void orc_forces(orc_system* s, int terms, double* out) {
    if (terms & ORC_TERM_PAIRS) pairs_forces(s, out);
    bonded_forces(s, terms, out);
    if (terms & ORC_TERM_DIHEDRALS) dihedral_forces(s, out);
    if (s->coul.kind != ORC_COULOMB_NONE) {
        if (s->coul.kind == ORC_COULOMB_EWALD) ewald_prepare(s);
        if (terms & ORC_TERM_COUL_REAL) coulomb_real_forces(s, out);
        if (s->coul.kind == ORC_COULOMB_EWALD && (terms & ORC_TERM_COUL_KSPACE)) ewald_kspace_forces(s, out);
    }
}

// AtomicVirial::compute (compute.rs:198-254), per term
void orc_virial(orc_system* s, int terms, double* out) {
    M3 v = mzero();
    if (terms & ORC_TERM_PAIRS) madd(v, pairs_virial(s));
    if (terms & ORC_TERM_TAIL) madd(v, pairs_tail_virial(s));
    if (terms & ORC_TERM_BONDS) madd(v, bonds_virial(s));
    if (s->coul.kind != ORC_COULOMB_NONE) {
        if (s->coul.kind == ORC_COULOMB_EWALD) ewald_prepare(s);
        if (terms & ORC_TERM_COUL_REAL) madd(v, coulomb_real_virial(s));
        if (s->coul.kind == ORC_COULOMB_EWALD && (terms & ORC_TERM_COUL_KSPACE)) madd(v, ewald_kspace_virial(s));
    }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) out[3 * a + b] = v.m[a][b];
}

// Molecule::center_of_mass (sys/config/molecules.rs:256-264)
V3 center_of_mass(const orc_system* s, size_t m) {
    double total = 0.0;
    V3 com{{0.0, 0.0, 0.0}};
    for (int64_t i = s->mol_range[m].first; i < s->mol_range[m].second; i++) {
        total += s->mass[i];
        com = vadd(com, vscale(s->mass[i], s->pos[i]));
    }
    return V3{{com[0] / total, com[1] / total, com[2] / total}};
}

// MolecularVirial::compute (compute.rs:278-362), per term: the pair potentials
// between molecules with the molecular definition (Allen & Tildesley 2.54,
// 2.61, 2.63), the tail correction, bonds ignored; real-space Coulomb with
// the same definition (Ewald ewald.rs:533-571, Wolf wolf.rs:285-320) and the
// Ewald k-space atomic virial minus sum_i F_k,i (x) (x_i - com) (ewald.rs:736-752).
void orc_molecular_virial(orc_system* s, int terms, double* out) {
    size_t nm = s->mol_range.size();
    std::vector<V3> com(nm);
    for (size_t m = 0; m < nm; m++) com[m] = center_of_mass(s, m);
    bool ewald = s->coul.kind == ORC_COULOMB_EWALD;
    bool coul = s->coul.kind != ORC_COULOMB_NONE && (terms & ORC_TERM_COUL_REAL);
    if (ewald) ewald_prepare(s);
    std::vector<M3> partial(nthreads(), mzero());
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t mi = 0; mi < (int64_t)nm; mi++) {
        M3 local = mzero();
        for (size_t mj = (size_t)mi + 1; mj < nm; mj++) {
            V3 rij = vsub(com[mi], com[mj]);
            s->cell.vector_image(rij);
            for (int64_t a = s->mol_range[mi].first; a < s->mol_range[mi].second; a++) {
                for (int64_t b = s->mol_range[mj].first; b < s->mol_range[mj].second; b++) {
                    V3 rab = s->nearest_image(a, b);
                    double dot = vdot(rab, rij), n2 = vdot(rab, rab);
                    if (terms & ORC_TERM_PAIRS) {
                        const PairPot* p = s->pair(a, b);
                        if (p) {
                            RestrictionInfo info = information(p->d.restriction, p->d.scale14, s->bond_path(a, b));
                            if (!info.excluded) madd(local, mscale(dot / n2, mscale(info.scaling, p->virial(rab))));
                        }
                    }
                    double qa = s->charge[a], qb = s->charge[b];
                    if (coul && qa != 0.0 && qb != 0.0) {
                        RestrictionInfo info = coul_info(s, a, b);
                        V3 f;
                        if (ewald) {
                            f = vscale(ewald_real_force_pair(s, info, qa * qb, vnorm(rab)), rab);
                        } else {
                            if (info.excluded) continue;
                            f = vscale(info.scaling * wolf_force_pair(s, qa * qb, vnorm(rab)), rab);
                        }
                        madd(local, mscale(dot / n2, tensorial(f, rab)));
                    }
                }
            }
        }
        madd(partial[thread_id()], local);
    }
    M3 v = mzero();
    for (auto& m : partial) madd(v, m);
    if (terms & ORC_TERM_TAIL) madd(v, pairs_tail_virial(s));
    if (ewald && (terms & ORC_TERM_COUL_KSPACE)) {
        madd(v, ewald_kspace_virial(s));
        std::vector<double> fk(3 * (size_t)s->n, 0.0);
        ewald_kspace_forces(s, fk.data());
        M3 correction = mzero();
        for (size_t m = 0; m < nm; m++)
            for (int64_t i = s->mol_range[m].first; i < s->mol_range[m].second; i++) {
                V3 fi{{fk[3 * i], fk[3 * i + 1], fk[3 * i + 2]}};
                madd(correction, tensorial(fi, vsub(s->pos[i], com[m])));
            }
        madd(v, mscale(-1.0, correction));
    }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) out[3 * a + b] = v.m[a][b];
}

int64_t orc_pairset(orc_system* s, int family, int32_t* out, int64_t cap) {
    int64_t count = 0;
    for (int64_t i = 0; i < s->n; i++) {
        for (int64_t j = i + 1; j < s->n; j++) {
            bool in = false;
            if (family == 0) {
                // the pair contributes iff the potential exists, is not excluded and r < cutoff
                const PairPot* p = s->pair(i, j);
                if (!p) continue;
                RestrictionInfo info = information(p->d.restriction, p->d.scale14, s->bond_path(i, j));
                if (info.excluded) continue;
                double r = vnorm(s->nearest_image(i, j));
                in = !(r >= p->d.cutoff);
            } else {
                if (s->coul.kind == ORC_COULOMB_NONE) continue;
                if (s->charge[i] == 0.0 || s->charge[j] == 0.0) continue;
                RestrictionInfo info = coul_info(s, i, j);
                if (s->coul.kind == ORC_COULOMB_WOLF && info.excluded) continue;
                double r = vnorm(s->nearest_image(i, j));
                in = !(r > s->coul.cutoff);
            }
            if (in) {
                if (count < cap) {
                    out[2 * count] = (int32_t)i;
                    out[2 * count + 1] = (int32_t)j;
                }
                count++;
            }
        }
    }
    return count;
}

// KineticEnergy (compute.rs:133-144)
double orc_kinetic_energy(const orc_system* s, const double* v) {
    double e = 0.0;
    for (int64_t i = 0; i < s->n; i++) {
        V3 vi{{v[3 * i], v[3 * i + 1], v[3 * i + 2]}};
        e += 0.5 * s->mass[i] * vnorm2(vi);
    }
    return e;
}

// Temperature (compute.rs:164-172) with DegreesOfFreedom::Particles (system.rs:249-255)
double orc_temperature(const orc_system* s, const double* v) {
    double k = orc_kinetic_energy(s, v);
    double dof = (double)(3 * s->n);
    return 2.0 * k / (dof * K_BOLTZMANN);
}

void orc_velocity_verlet(orc_system* s, double* x, double* v, double* a, double dt, int64_t nsteps,
                         double T0, double tau) {
    int64_t n = s->n;
    std::vector<double> f(3 * n);
    for (int64_t step = 0; step < nsteps; step++) {
        // integrators.rs:48-53
        for (int64_t i = 0; i < 3 * n; i++) {
            v[i] += 0.5 * dt * a[i];
            x[i] += v[i] * dt;
        }
        orc_set_positions(s, x);
        std::fill(f.begin(), f.end(), 0.0);
        orc_forces(s, ORC_TERM_ALL, f.data());
        // integrators.rs:55-68
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) a[3 * i + k] = f[3 * i + k] / s->mass[i];
        for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * dt * a[i];
        // BerendsenThermostat::apply (thermostats.rs:112-121)
        if (tau > 0.0) {
            double T = orc_temperature(s, v);
            double factor = std::sqrt(1.0 + (T0 / T - 1.0) / tau);
            for (int64_t i = 0; i < 3 * n; i++) v[i] *= factor;
        }
    }
}

// ---- integrators, thermostats and controls ------------------------------------

// The CSVR noise stream of one thermostat application: SplitMix64 from
// (seed, count), uniforms from the top 53 bits, Box-Muller normals (cosine
// branch), Gamma(a >= 1) by Marsaglia and Tsang (ACM TOMS 26 (2000) 363-372).
// The engine draws the same numbers; the reference draws from rand_xorshift /
// rand_distr (third-party, not restated), so only the distribution matches it.
struct Noise {
    uint64_t st;
    Noise(uint64_t seed, uint64_t count) : st(seed ^ (count * 0xD1B54A32D192ED03ull)) {}
    uint64_t next() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((double)(next() >> 11) + 0.5) * 0x1.0p-53; }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * PI * u2);
    }
    double gamma(double a) {
        double d = a - 1.0 / 3.0;
        double c = 1.0 / std::sqrt(9.0 * d);
        for (int it = 0; it < 64; it++) {
            double x = normal();
            double v = 1.0 + c * x;
            if (v <= 0.0) continue;
            v = v * v * v;
            double u = uniform();
            double x2 = x * x;
            if (u < 1.0 - 0.0331 * x2 * x2) return d * v;
            if (std::log(u) < 0.5 * x2 + d * (1.0 - v + std::log(v))) return d * v;
        }
        return d;
    }
};

// Verlet::setup (integrators.rs:92-104): x_prev = x - v dt
void orc_verlet_setup(const orc_system* s, const double* x, const double* v, double dt, double* prev) {
    for (int64_t i = 0; i < 3 * s->n; i++) prev[i] = x[i] - v[i] * dt;
}

// MolecularDynamics::propagate (md/molecular_dynamics.rs:66-76): integrate,
// thermostat, controls, `nsteps` times.
void orc_md_run(orc_system* s, double* x, double* v, double* state, int integrator, double dt, int thermostat,
                double T0, double tau, double tol, uint64_t seed, uint64_t* count, uint32_t controls,
                int64_t nsteps) {
    int64_t n = s->n;
    std::vector<double> f(3 * n);
    const double dt2 = dt * dt;
    auto forces = [&]() {
        orc_set_positions(s, x);
        std::fill(f.begin(), f.end(), 0.0);
        orc_forces(s, ORC_TERM_ALL, f.data());
    };
    for (int64_t step = 0; step < nsteps; step++) {
        if (integrator == 0) {  // VelocityVerlet::integrate (integrators.rs:44-69)
            double* a = state;
            for (int64_t i = 0; i < 3 * n; i++) {
                v[i] += 0.5 * dt * a[i];
                x[i] += v[i] * dt;
            }
            forces();
            for (int64_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) a[3 * i + k] = f[3 * i + k] / s->mass[i];
            for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * dt * a[i];
        } else if (integrator == 1) {  // Verlet::integrate (integrators.rs:106-122)
            double* prev = state;
            forces();
            for (int64_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) {
                    int64_t c = 3 * i + k;
                    double tmp = x[c];
                    x[c] = 2.0 * x[c] - prev[c] + dt2 / s->mass[i] * f[c];
                    v[c] = (x[c] - prev[c]) / (2.0 * dt);
                    prev[c] = tmp;
                }
        } else {  // LeapFrog::integrate (integrators.rs:151-168)
            double* a = state;
            for (int64_t i = 0; i < 3 * n; i++) x[i] += v[i] * dt + 0.5 * a[i] * dt2;
            forces();
            for (int64_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) {
                    int64_t c = 3 * i + k;
                    double an = f[c] / s->mass[i];
                    v[c] += 0.5 * (a[c] + an) * dt;
                    a[c] = an;
                }
        }
        // Thermostat::apply (thermostats.rs:66-73, 112-121, 195-210)
        if (thermostat == 1) {
            double T = orc_temperature(s, v);
            double factor = std::sqrt(1.0 + (T0 / T - 1.0) / tau);
            for (int64_t i = 0; i < 3 * n; i++) v[i] *= factor;
        } else if (thermostat == 2) {
            double T = orc_temperature(s, v);
            if (std::fabs(T - T0) > tol) {  // velocities::scale (velocities.rs:16-22)
                double factor = std::sqrt(T0 / T);
                for (int64_t i = 0; i < 3 * n; i++) v[i] *= factor;
            }
        } else if (thermostat == 3) {
            *count += 1;
            double kinetic = orc_kinetic_energy(s, v);
            double kinetic_factor = (K_BOLTZMANN * T0 / 2.0) / kinetic;
            double exp_1 = std::exp(-1.0 / tau);
            double exp_2 = (1.0 - exp_1) * kinetic_factor;
            int64_t dn = 3 * n - 1;  // sum_noises(dof - 1) (thermostats.rs:166-192)
            Noise r(seed, *count);
            double gauss = 0.0, wiener = 0.0;
            if (dn == 1) {
                gauss = r.normal();
                wiener = gauss * gauss;
            } else if (dn > 1) {
                gauss = r.normal();
                if (dn % 2 == 0) wiener = 2.0 * r.gamma((double)(dn / 2));
                else wiener = 2.0 * r.gamma((double)((dn - 1) / 2)) + gauss * gauss;
            }
            double scale = exp_1 + exp_2 * (gauss * gauss + wiener) + 2.0 * gauss * std::sqrt(exp_1 * exp_2);
            double alpha = std::sqrt(scale);
            for (int64_t i = 0; i < 3 * n; i++) v[i] *= alpha;
        }
        // Control::control (controls.rs:29-43, 80-89)
        if (controls & 1u) {  // RemoveTranslation
            double total = 0.0;
            for (int64_t i = 0; i < n; i++) total += s->mass[i];
            double com[3] = {0.0, 0.0, 0.0};
            for (int64_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) com[k] += v[3 * i + k] * s->mass[i] / total;
            for (int64_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) v[3 * i + k] -= com[k];
        }
        if (controls & 4u) {  // RemoveRotation (controls.rs:47-71)
            double total = 0.0, com[3] = {0.0, 0.0, 0.0};  // Configuration::center_of_mass (configuration.rs:270-278)
            for (int64_t i = 0; i < n; i++) {
                total += s->mass[i];
                for (int k = 0; k < 3; k++) com[k] += s->mass[i] * x[3 * i + k];
            }
            for (int k = 0; k < 3; k++) com[k] = com[k] / total;
            double L[3] = {0.0, 0.0, 0.0}, I[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int64_t i = 0; i < n; i++) {
                double d[3], vv[3];
                for (int k = 0; k < 3; k++) {
                    d[k] = x[3 * i + k] - com[k];
                    vv[k] = v[3 * i + k];
                }
                double cr[3] = {d[1] * vv[2] - d[2] * vv[1], d[2] * vv[0] - d[0] * vv[2], d[0] * vv[1] - d[1] * vv[0]};
                for (int k = 0; k < 3; k++) L[k] += s->mass[i] * cr[k];
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) I[a][b] += -s->mass[i] * (d[a] * d[b]);
            }
            double tr = I[0][0] + I[1][1] + I[2][2];
            for (int k = 0; k < 3; k++) I[k][k] += tr;
            // Matrix3::inverse (types/matrix.rs:212-249)
            double det = I[0][0] * (I[1][1] * I[2][2] - I[2][1] * I[1][2]) -
                         I[0][1] * (I[1][0] * I[2][2] - I[1][2] * I[2][0]) +
                         I[0][2] * (I[1][0] * I[2][1] - I[1][1] * I[2][0]);
            double id = 1.0 / det;
            double r[3][3];
            r[0][0] = (I[1][1] * I[2][2] - I[2][1] * I[1][2]) * id;
            r[0][1] = (I[0][2] * I[2][1] - I[0][1] * I[2][2]) * id;
            r[0][2] = (I[0][1] * I[1][2] - I[0][2] * I[1][1]) * id;
            r[1][0] = (I[1][2] * I[2][0] - I[1][0] * I[2][2]) * id;
            r[1][1] = (I[0][0] * I[2][2] - I[0][2] * I[2][0]) * id;
            r[1][2] = (I[1][0] * I[0][2] - I[0][0] * I[1][2]) * id;
            r[2][0] = (I[1][0] * I[2][1] - I[2][0] * I[1][1]) * id;
            r[2][1] = (I[2][0] * I[0][1] - I[0][0] * I[2][1]) * id;
            r[2][2] = (I[0][0] * I[1][1] - I[1][0] * I[0][1]) * id;
            double w[3];
            for (int a = 0; a < 3; a++) w[a] = r[a][0] * L[0] + r[a][1] * L[1] + r[a][2] * L[2];
            for (int64_t i = 0; i < n; i++) {
                double d[3];
                for (int k = 0; k < 3; k++) d[k] = x[3 * i + k] - com[k];
                v[3 * i] -= d[1] * w[2] - d[2] * w[1];
                v[3 * i + 1] -= d[2] * w[0] - d[0] * w[2];
                v[3 * i + 2] -= d[0] * w[1] - d[1] * w[0];
            }
        }
        if (controls & 2u) {  // Rewrap: Molecule::wrap (sys/config/molecules.rs:256-296)
            for (auto& mr : s->mol_range) {
                double total = 0.0, com[3] = {0.0, 0.0, 0.0};
                for (int64_t i = mr.first; i < mr.second; i++) {
                    total += s->mass[i];
                    for (int k = 0; k < 3; k++) com[k] += s->mass[i] * x[3 * i + k];
                }
                V3 c{{com[0] / total, com[1] / total, com[2] / total}};
                V3 w = c;
                s->cell.wrap_vector(w);  // UnitCell::wrap_vector (cells.rs:263-282)
                double delta[3];
                for (int k = 0; k < 3; k++) delta[k] = w[k] - c[k];
                for (int64_t i = mr.first; i < mr.second; i++)
                    for (int k = 0; k < 3; k++) x[3 * i + k] += delta[k];
            }
        }
    }
    orc_set_positions(s, x);
}

void orc_bonded_eval(const orc_bonded* p, double x, double* energy, double* force) {
    Bonded b;
    b.d = *p;
    *energy = b.energy(x);
    *force = b.force(x);
}

void orc_dihedral_geometry(const double cell[3], const double* r1, const double* r2, const double* r3,
                           const double* r4, double* phi, double* derivatives) {
    Cell c;
    c.init(cell[0], cell[1], cell[2]);
    auto v = [](const double* r) { return V3{{r[0], r[1], r[2]}}; };
    V3 d[4];
    *phi = dihedral_and_derivatives(v(r1), v(r2), v(r3), v(r4), [&](V3& x) { c.vector_image(x); }, d[0], d[1],
                                    d[2], d[3]);
    for (int a = 0; a < 4; a++)
        for (int k = 0; k < 3; k++) derivatives[3 * a + k] = d[a][k];
}

int64_t orc_n_dihedrals(const orc_system* s) { return (int64_t)s->dihedrals.size(); }

void orc_dihedrals(const orc_system* s, int32_t* out) {
    size_t k = 0;
    for (auto& d : s->dihedrals) {
        out[k++] = std::get<0>(d);
        out[k++] = std::get<1>(d);
        out[k++] = std::get<2>(d);
        out[k++] = std::get<3>(d);
    }
}

void orc_pair_eval(const orc_pair* d, double r, double* energy, double* force, double* tail_energy,
                   double* tail_virial) {
    PairPot p;
    p.d = *d;
    p.build_table();
    if (d->shifted) p.shift = p.comp_energy(d->cutoff);
    *energy = p.energy(r);
    *force = p.force(r);
    *tail_energy = p.tail_energy();
    *tail_virial = p.tail_virial_scalar();
}

// UnitCell::scale_mut of the orthorhombic cell (cells.rs:201-207) to new lengths;
// Ewald::prepare recomputes its k-vectors for the new cell (ewald.rs:353-379).
void orc_set_cell(orc_system* s, double a, double b, double c) {
    s->cell.init(a, b, c);
    s->factors_ready = false;
}
void orc_get_cell(const orc_system* s, double* out) {
    out[0] = s->cell.a;
    out[1] = s->cell.b;
    out[2] = s->cell.c;
}
// Any cell: its matrix (row-major) and shape
void orc_set_cell_matrix(orc_system* s, const double* m, int32_t shape) {
    s->cell.init_matrix(m, shape);
    s->factors_ready = false;
}
void orc_get_cell_matrix(const orc_system* s, double* out) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[3 * i + j] = s->cell.cell.m[i][j];
}
// UnitCell::lengths and volume (cells.rs:134-146, 185-200)
void orc_cell_info(const orc_system* s, double* lengths, double* volume) {
    V3 l = s->cell.lengths();
    for (int k = 0; k < 3; k++) lengths[k] = l[k];
    *volume = s->cell.volume();
}
// UnitCell::vector_image (wrap == 0) or wrap_vector (wrap != 0) of v, and
// the fractional / Cartesian round trip (wrap == 2), in place
void orc_cell_apply(const orc_system* s, double* v, int32_t wrap) {
    V3 x{{v[0], v[1], v[2]}};
    if (wrap == 2) x = mat_vec(s->cell.cell, mat_vec(s->cell.inv, x));
    else if (wrap) s->cell.wrap_vector(x);
    else s->cell.vector_image(x);
    for (int k = 0; k < 3; k++) v[k] = x[k];
}

// UnitCell::scale_mut(f * Matrix3::one()) (cells.rs:201-207): cell * (f 1)
static void scale_cell(orc_system* s, double f) {
    M3 one = mscale(f, M3{{{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}}});
    double m[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            m[3 * i + j] = s->cell.cell.m[i][0] * one.m[0][j] + s->cell.cell.m[i][1] * one.m[1][j] +
                           s->cell.cell.m[i][2] * one.m[2][j];
    orc_set_cell_matrix(s, m, s->cell.shape);
}

// Interactions::maximum_cutoff (interactions.rs:173-190): pair and Coulomb cutoffs
double orc_maximum_cutoff(const orc_system* s) {
    double rc = 0.0;
    for (const PairPot& p : s->pairs)
        if (p.d.type != ORC_PAIR_ABSENT) rc = std::max(rc, p.d.cutoff);
    if (s->coul.kind != ORC_COULOMB_NONE) rc = std::max(rc, s->coul.cutoff);
    return rc;
}

// BerendsenBarostat::integrate (lumol-sim/src/md/integrators.rs:213-250), then
// the Berendsen thermostat when tau_thermostat > 0 (thermostats.rs:112-121), as
// MolecularDynamics::propagate does, `nsteps` times.  `eta` (in / out) is the
// scaling factor the next step applies (1 after setup).  Returns 1 where the
// reference panics (a cell length at or below twice the maximum cutoff), with
// the state of that step's first half.
int orc_berendsen_barostat_run(orc_system* s, double* x, double* v, double* a, double* eta, double dt,
                               double pressure, double tau, double T0, double tau_thermostat, int64_t nsteps) {
    const double WATER_COMPRESSIBILITY = 7372.0;  // integrators.rs:171
    int64_t n = s->n;
    std::vector<double> f(3 * n);
    for (int64_t step = 0; step < nsteps; step++) {
        for (int64_t i = 0; i < 3 * n; i++) {
            v[i] += 0.5 * dt * a[i];
            x[i] *= *eta;
            x[i] += v[i] * dt;
        }
        double e3 = *eta * *eta * *eta;
        scale_cell(s, e3);
        double rc = orc_maximum_cutoff(s);
        V3 len = s->cell.lengths();
        if (0.5 * len[0] <= rc || 0.5 * len[1] <= rc || 0.5 * len[2] <= rc) return 1;
        // System::pressure (Pressure, compute.rs:399-431): (N_f k_B T + Tr W) / (3 V)
        orc_set_positions(s, x);
        double w[9];
        orc_virial(s, ORC_TERM_ALL, w);
        double T = orc_temperature(s, v);
        double dof = (double)(3 * n);
        double P = (dof * K_BOLTZMANN * T + (w[0] + w[4] + w[8])) / (3.0 * s->cell.volume());
        double eta3 = 1.0 - WATER_COMPRESSIBILITY / tau * (pressure - P);
        *eta = std::cbrt(eta3);
        std::fill(f.begin(), f.end(), 0.0);
        orc_forces(s, ORC_TERM_ALL, f.data());
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) a[3 * i + k] = f[3 * i + k] / s->mass[i];
        for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * dt * a[i];
        if (tau_thermostat > 0.0) {
            double Tt = orc_temperature(s, v);
            double factor = std::sqrt(1.0 + (T0 / Tt - 1.0) / tau_thermostat);
            for (int64_t i = 0; i < 3 * n; i++) v[i] *= factor;
        }
    }
    return 0;
}

// AnisoBerendsenBarostat::integrate (lumol-sim/src/md/integrators.rs:296-342)
// `nsteps` times: v += dt/2 a; x = eta x; x += v dt; cell * eta; the panic
// check on the face distances; eta = 1 - dt 7372 / tau (stress0 - Stress)
// made symmetric, with Stress = (sum m v (x) v + W) / V (compute.rs:466-480);
// then the forces.  `eta` (9, in / out) starts at the identity.  Returns 1
// where the reference panics.
int orc_aniso_barostat_run(orc_system* s, double* x, double* v, double* a, double* eta, double dt,
                           const double* stress0, double tau, int64_t nsteps) {
    const double WATER_COMPRESSIBILITY = 7372.0;  // integrators.rs:171
    int64_t n = s->n;
    std::vector<double> f(3 * n);
    for (int64_t step = 0; step < nsteps; step++) {
        for (int64_t i = 0; i < n; i++) {
            for (int k = 0; k < 3; k++) v[3 * i + k] += 0.5 * dt * a[3 * i + k];
            V3 p{{x[3 * i], x[3 * i + 1], x[3 * i + 2]}};
            M3 m;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) m.m[r][c] = eta[3 * r + c];
            p = mat_vec(m, p);
            for (int k = 0; k < 3; k++) x[3 * i + k] = p[k] + v[3 * i + k] * dt;
        }
        // self.cell *= factor (matrix.rs:365-388)
        double cm[9];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                cm[3 * r + c] = s->cell.cell.m[r][0] * eta[c] + s->cell.cell.m[r][1] * eta[3 + c] +
                                s->cell.cell.m[r][2] * eta[6 + c];
        orc_set_cell_matrix(s, cm, s->cell.shape);
        double rc = orc_maximum_cutoff(s);
        V3 len = s->cell.lengths();
        if (0.5 * len[0] <= rc || 0.5 * len[1] <= rc || 0.5 * len[2] <= rc) return 1;
        orc_set_positions(s, x);
        double w[9];
        orc_virial(s, ORC_TERM_ALL, w);
        double kin[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t i = 0; i < n; i++)  // kinetic += mass * velocity.tensorial(velocity)
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) kin[3 * r + c] += s->mass[i] * (v[3 * i + r] * v[3 * i + c]);
        double volume = s->cell.volume();
        double factor = dt * WATER_COMPRESSIBILITY / tau;
        for (int k = 0; k < 9; k++) {
            double stress = (kin[k] + w[k]) / volume;
            eta[k] = (k % 4 == 0 ? 1.0 : 0.0) - factor * (stress0[k] - stress);
        }
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < r; c++) {
                eta[3 * r + c] = 0.5 * (eta[3 * r + c] + eta[3 * c + r]);
                eta[3 * c + r] = eta[3 * r + c];
            }
        std::fill(f.begin(), f.end(), 0.0);
        orc_forces(s, ORC_TERM_ALL, f.data());
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) a[3 * i + k] = f[3 * i + k] / s->mass[i];
        for (int64_t i = 0; i < 3 * n; i++) v[i] += 0.5 * dt * a[i];
    }
    return 0;
}

// EnergyCache::init (cache.rs:75-98)
void orc_cache_init(orc_system* s) {
    int64_t n = s->n;
    s->pairs_cache.assign((size_t)(n * n), 0.0);
    s->c_pairs = 0.0;
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = i + 1; j < n; j++) {
            double r = vnorm(s->nearest_image(i, j));
            double e = pair_energy_ij(s, s->bond_path(i, j), r, i, j);
            s->pairs_cache[(size_t)(i * n + j)] = e;
            s->pairs_cache[(size_t)(j * n + i)] = e;
            s->c_pairs += e;
        }
    s->c_tail = pairs_tail(s);
    s->c_bonds = bonds_energy(s);
    s->c_angles = angles_energy(s) + dihedrals_energy(s);  // intramolecular angular terms
    s->c_coulomb = coulomb_energy_terms(s, ORC_TERM_ALL);
    s->has_pending = false;
}

// EnergyCache::energy (cache.rs:100-114)
double orc_cache_energy(const orc_system* s) {
    double e = 0.0;
    e += s->c_pairs;
    e += s->c_tail;
    e += s->c_bonds;
    e += s->c_angles;
    e += s->c_coulomb;
    return e;
}

// EnergyCache::move_molecule_cost (cache.rs:145-220) with the Coulomb
// GlobalCache costs of Ewald (ewald.rs:572-613, 758-839) and Wolf (wolf.rs:121-165)
double orc_move_molecule_cost(orc_system* s, int64_t molid, const double* newp) {
    int64_t n = s->n;
    int64_t start = s->mol_range[molid].first, end = s->mol_range[molid].second;
    int64_t msize = end - start;
    std::vector<V3> newpos(msize);
    for (int64_t a = 0; a < msize; a++)
        for (int k = 0; k < 3; k++) newpos[a][k] = newp[3 * a + k];

    s->pending_new_pairs.assign((size_t)(msize * n), 0.0);
    double pairs_delta = 0.0;
    for (int64_t a = 0; a < msize; a++) {
        int64_t part_i = start + a;
        for (int64_t part_j = 0; part_j < n; part_j++) {
            if (part_j >= start && part_j < end) continue;
            double r = s->cell.distance(s->pos[part_j], newpos[a]);
            double e = pair_energy_ij(s, s->bond_path(part_i, part_j), r, part_i, part_j);
            pairs_delta += e;
            s->pending_new_pairs[(size_t)(a * n + part_j)] += e;
            pairs_delta -= s->pairs_cache[(size_t)(part_i * n + part_j)];
        }
    }

    double coulomb_delta = 0.0;
    s->pending_delta_rho.clear();
    if (s->coul.kind != ORC_COULOMB_NONE) {
        double old_e = 0.0, new_e = 0.0;
        bool ewald = s->coul.kind == ORC_COULOMB_EWALD;
        for (int64_t a = 0; a < msize; a++) {
            int64_t part_i = start + a;
            double qi = s->charge[part_i];
            if (qi == 0.0) continue;
            for (int64_t part_j = 0; part_j < n; part_j++) {
                if (part_j >= start && part_j < end) continue;
                double qj = s->charge[part_j];
                if (qj == 0.0) continue;
                RestrictionInfo info = coul_info(s, part_i, part_j);
                if (ewald) {
                    double old_r = s->distance(part_i, part_j);
                    double new_r = s->cell.distance(newpos[a], s->pos[part_j]);
                    old_e += ewald_real_energy_pair(s, info, qi * qj, old_r);
                    new_e += ewald_real_energy_pair(s, info, qi * qj, new_r);
                } else {
                    if (info.excluded) continue;
                    double old_r = s->distance(part_i, part_j);
                    double new_r = s->cell.distance(newpos[a], s->pos[part_j]);
                    old_e += info.scaling * wolf_energy_pair(s, qi * qj, old_r);
                    new_e += info.scaling * wolf_energy_pair(s, qi * qj, new_r);
                }
            }
        }
        coulomb_delta = new_e - old_e;
        if (ewald) {
            ewald_prepare(s);
            // k_space_move_molecule_cost: uses the rho / eikr of the last eik_dot_r call
            if (s->rho.size() != s->factors.size()) eik_dot_r(s);
            double old_k = 0.0;
            for (size_t f = 0; f < s->factors.size(); f++) old_k += s->factors[f].energy * cnorm2(s->rho[f]);
            old_k /= FOUR_PI_EPSILON_0;
            // delta_rho_move_rigid_molecules (ewald.rs:758-805)
            int kmax = s->kmax;
            std::vector<Complex> ne((size_t)(2 * kmax + 1) * 3 * msize);
            auto at = [&](int k, int axis, int64_t a) -> Complex& {
                return ne[((size_t)(k + kmax) * 3 + axis) * msize + a];
            };
            for (int spatial = 0; spatial < 3; spatial++) {
                double idx[3] = {0.0, 0.0, 0.0};
                idx[spatial] = 1.0;
                V3 k = s->cell.k_vector(idx[0], idx[1], idx[2]);
                for (int64_t a = 0; a < msize; a++) {
                    double phi = vdot(k, newpos[a]);
                    at(0, spatial, a) = Complex{1.0, 0.0};
                    at(1, spatial, a) = Complex{1.0 * std::cos(phi), 1.0 * std::sin(phi)};
                    at(-1, spatial, a) = cconj(at(1, spatial, a));
                }
            }
            for (int spatial = 0; spatial < 3; spatial++)
                for (int k = 2; k <= kmax; k++)
                    for (int64_t a = 0; a < msize; a++) {
                        at(k, spatial, a) = cmul(at(k - 1, spatial, a), at(1, spatial, a));
                        at(-k, spatial, a) = cconj(at(k, spatial, a));
                    }
            s->pending_delta_rho.assign(s->factors.size(), Complex{0.0, 0.0});
            for (size_t f = 0; f < s->factors.size(); f++) {
                const auto& kf = s->factors[f];
                Complex partial{0.0, 0.0};
                for (int64_t a = 0; a < msize; a++) {
                    int64_t part_i = start + a;
                    Complex old_phi = cmul(cmul(eikr_at(s, kf.ikx, 0, part_i), eikr_at(s, kf.iky, 1, part_i)),
                                           eikr_at(s, kf.ikz, 2, part_i));
                    Complex new_phi = cmul(cmul(at(kf.ikx, 0, a), at(kf.iky, 1, a)), at(kf.ikz, 2, a));
                    double q = s->charge[part_i];
                    partial.re += q * (new_phi.re - old_phi.re);
                    partial.im += q * (new_phi.im - old_phi.im);
                }
                s->pending_delta_rho[f] = partial;
            }
            double new_k = 0.0;
            for (size_t f = 0; f < s->factors.size(); f++) {
                Complex r{s->rho[f].re + s->pending_delta_rho[f].re, s->rho[f].im + s->pending_delta_rho[f].im};
                new_k += s->factors[f].energy * cnorm2(r);
            }
            new_k /= FOUR_PI_EPSILON_0;
            coulomb_delta += new_k - old_k;
        }
    }

    s->pending_mol = molid;
    s->pending_pairs_delta = pairs_delta;
    s->pending_coulomb_delta = coulomb_delta;
    s->has_pending = true;
    return pairs_delta + coulomb_delta;
}

// EnergyCache::move_all_molecules_cost (cache.rs:238-292) for the configuration
// a Resize move prepared (resize.rs:70-107): the new cell and positions are
// installed (the Resize move changed the System before the cost), pairs
// between different molecules are evaluated again against the cache, the
// Coulomb energy and the tail correction in full.  orc_cache_update keeps the
// new configuration, orc_cache_restore puts the previous one back.
double orc_move_all_molecules_cost(orc_system* s, const double* cell, const double* newp) {
    int64_t n = s->n;
    s->saved_cell = s->cell;
    s->saved_pos = s->pos;
    orc_set_cell_matrix(s, cell, s->cell.shape);  // (the shape is kept: cells.rs:201-207)
    orc_set_positions(s, newp);
    s->pending_all_pairs.assign((size_t)(n * n), 0.0);
    double pairs_delta = 0.0;
    for (size_t mi = 0; mi < s->mol_range.size(); mi++)
        for (size_t mj = mi + 1; mj < s->mol_range.size(); mj++)
            for (int64_t i = s->mol_range[mi].first; i < s->mol_range[mi].second; i++)
                for (int64_t j = s->mol_range[mj].first; j < s->mol_range[mj].second; j++) {
                    double r = s->distance(i, j);
                    double e = pair_energy_ij(s, s->bond_path(i, j), r, i, j);
                    pairs_delta += e;
                    s->pending_all_pairs[(size_t)(i * n + j)] += e;
                    s->pending_all_pairs[(size_t)(j * n + i)] += e;
                    pairs_delta -= s->pairs_cache[(size_t)(i * n + j)];
                }
    double new_coulomb = coulomb_energy_terms(s, ORC_TERM_ALL);
    double tail = pairs_tail(s);
    double cost = pairs_delta + (tail - s->c_tail) + (new_coulomb - s->c_coulomb);
    s->pending_pairs_delta = pairs_delta;
    s->pending_all_tail = tail;
    s->pending_all_coulomb = new_coulomb;
    s->pending_all = true;
    s->has_pending = false;
    return cost;
}

// Resize::restore (resize.rs:121-124): the previous configuration back; the
// pending update is dropped.
void orc_cache_restore(orc_system* s) {
    if (s->pending_all) {
        s->cell = s->saved_cell;
        s->factors_ready = false;
        s->pos = s->saved_pos;
    }
    s->pending_all = false;
    s->has_pending = false;
}

// EnergyCache::update (cache.rs:118-127) running the closure of cache.rs:190-218
// (or of cache.rs:274-290 after move_all_molecules_cost)
void orc_cache_update(orc_system* s) {
    if (s->pending_all) {
        int64_t n = s->n;
        s->c_pairs += s->pending_pairs_delta;
        s->c_tail = s->pending_all_tail;
        s->c_coulomb = s->pending_all_coulomb;
        for (size_t mi = 0; mi < s->mol_range.size(); mi++)
            for (size_t mj = mi + 1; mj < s->mol_range.size(); mj++)
                for (int64_t i = s->mol_range[mi].first; i < s->mol_range[mi].second; i++)
                    for (int64_t j = s->mol_range[mj].first; j < s->mol_range[mj].second; j++) {
                        double e = s->pending_all_pairs[(size_t)(i * n + j)];
                        s->pairs_cache[(size_t)(i * n + j)] = e;
                        s->pairs_cache[(size_t)(j * n + i)] = e;
                    }
        s->pending_all = false;
        return;
    }
    if (!s->has_pending) return;
    int64_t n = s->n;
    int64_t start = s->mol_range[s->pending_mol].first, end = s->mol_range[s->pending_mol].second;
    s->c_pairs += s->pending_pairs_delta;
    s->c_coulomb += s->pending_coulomb_delta;
    for (int64_t i = start; i < end; i++)
        for (int64_t j = 0; j < n; j++) {
            if (j >= start && j < end) continue;
            double e = s->pending_new_pairs[(size_t)((i - start) * n + j)];
            s->pairs_cache[(size_t)(i * n + j)] = e;
            s->pairs_cache[(size_t)(j * n + i)] = e;
        }
    // SharedEwald::update: rho += delta (ewald.rs:826-830, 947-955)
    for (size_t f = 0; f < s->pending_delta_rho.size() && f < s->rho.size(); f++) {
        s->rho[f].re += s->pending_delta_rho[f].re;
        s->rho[f].im += s->pending_delta_rho[f].im;
    }
    s->has_pending = false;
}

}  // extern "C"
