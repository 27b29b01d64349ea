// replay.cpp -- the call sequence Lumol's host code makes, replayed through
// the C ABI of include/lumol_gb300.h (no Python, no ctypes): a C++ stand-in
// for the Rust binding, which cannot be compiled in this image.
//
//   Forces::compute           forces zeroed, then GlobalPotential::forces
//   (sys/compute.rs:30-59)     accumulates into them: lg_compute twice
//                              gives twice the forces
//   PotentialEnergy::compute   lg_compute with LG_WANT_ENERGY
//   (compute.rs:111-128)
//   AtomicVirial::compute      lg_compute with LG_WANT_VIRIAL
//   (compute.rs:198-254)
//   VelocityVerlet             setup (accelerations := 0), then one
//   (md/integrators.rs:22-70)  integrate per Simulation::run step: ten
//                              lg_md_integrate(1) calls equal one
//                              lg_md_run(10) bit for bit
//   System::set_pair_potential a cutoff above half the cell fails with the
//   (sys/system.rs:122-131)    reference's panic message
//
// Usage: replay <input file>.  The input holds "n L cutoff alpha kmax", a line
// "sigma0 sigma1 epsilon0 epsilon1" (LJ of the two kinds in internal units,
// Lorentz-Berthelot mixing below), then n lines "kind charge mass x y z".
// Prints one JSON line; exits 0 when every check passed, 1 on a failed check,
// 3 when no device is visible (the engine has no CPU fallback).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lumol_gb300.h"

static int failures = 0;
static void check(bool ok, const char* what) {
    if (!ok) {
        std::fprintf(stderr, "replay: check failed: %s\n", what);
        failures++;
    }
}

struct Input {
    long n = 0;
    double L = 0, cutoff = 0, alpha = 0;
    int kmax = 0;
    double sigma[2] = {0, 0}, eps[2] = {0, 0};
    std::vector<int> kind, mol;
    std::vector<double> q, m, x;
};

static bool read_input(const char* path, Input& in) {
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    if (std::fscanf(f, "%ld %lf %lf %lf %d", &in.n, &in.L, &in.cutoff, &in.alpha, &in.kmax) != 5) return false;
    if (std::fscanf(f, "%lf %lf %lf %lf", &in.sigma[0], &in.sigma[1], &in.eps[0], &in.eps[1]) != 4) return false;
    in.kind.resize(in.n);
    in.mol.resize(in.n);
    in.q.resize(in.n);
    in.m.resize(in.n);
    in.x.resize(3 * in.n);
    for (long i = 0; i < in.n; i++) {
        if (std::fscanf(f, "%d %lf %lf %lf %lf %lf", &in.kind[i], &in.q[i], &in.m[i], &in.x[3 * i], &in.x[3 * i + 1],
                        &in.x[3 * i + 2]) != 6)
            return false;
        in.mol[i] = (int)i;
    }
    std::fclose(f);
    return true;
}

// NaCl-like pair table: LJ with Lorentz-Berthelot parameters between two kinds
static std::vector<lg_pair> pair_table(const Input& in) {
    const double* sigma = in.sigma;
    const double* eps = in.eps;
    std::vector<lg_pair> t(4);
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            lg_pair& p = t[a * 2 + b];
            std::memset(&p, 0, sizeof(p));
            p.type = LG_PAIR_LJ;
            p.p0 = 0.5 * (sigma[a] + sigma[b]);
            p.p1 = std::sqrt(eps[a] * eps[b]);
            p.cutoff = in.cutoff;
            p.scale14 = 1.0;
        }
    return t;
}

static lg_engine* make_engine(const Input& in, int* status) {
    lg_options opt{0, LG_PRECISION_FP64, 1.0, 0, 0};
    lg_engine* e = nullptr;
    *status = lg_create(&opt, 1, &e);
    if (*status != LG_OK) return nullptr;
    double cell[9] = {in.L, 0, 0, 0, in.L, 0, 0, 0, in.L};
    check(lg_set_cell(e, 0, cell) == LG_OK, "lg_set_cell");
    check(lg_set_particles(e, 0, in.n, in.kind.data(), in.q.data(), in.m.data(), in.mol.data()) == LG_OK,
          "lg_set_particles");
    std::vector<lg_pair> table = pair_table(in);
    check(lg_set_pairs(e, 0, 2, table.data()) == LG_OK, "lg_set_pairs");
    lg_coulomb c;
    std::memset(&c, 0, sizeof(c));
    c.kind = LG_COULOMB_EWALD;
    c.kmax = in.kmax;
    c.cutoff = in.cutoff;
    c.alpha = in.alpha;
    c.scale14 = 1.0;
    check(lg_set_coulomb(e, 0, &c) == LG_OK, "lg_set_coulomb");
    return e;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: replay <input>\n");
        return 2;
    }
    Input in;
    if (!read_input(argv[1], in)) {
        std::fprintf(stderr, "replay: cannot read %s\n", argv[1]);
        return 2;
    }
    int status = 0;
    lg_engine* e = make_engine(in, &status);
    if (!e) {
        std::printf("{\"status\": %d, \"error\": \"%s\"}\n", status, lg_last_error(nullptr));
        return status == LG_ERR_NO_DEVICE ? 3 : 1;
    }
    const long n3 = 3 * in.n;

    // Forces::compute: zeroed, then accumulated into (twice: doubled)
    std::vector<double> f1(n3, 0.0), f2(n3, 0.0);
    check(lg_compute(e, 0, in.x.data(), LG_TERM_ALL, LG_WANT_FORCES, f1.data(), nullptr, nullptr) == LG_OK,
          "forces");
    check(lg_compute(e, 0, in.x.data(), LG_TERM_ALL, LG_WANT_FORCES, f2.data(), nullptr, nullptr) == LG_OK,
          "forces again");
    check(lg_compute(e, 0, in.x.data(), LG_TERM_ALL, LG_WANT_FORCES, f2.data(), nullptr, nullptr) == LG_OK,
          "forces accumulated");
    double fmax = 0.0, sum[3] = {0, 0, 0};
    for (long i = 0; i < n3; i++) {
        check(f2[i] == 2.0 * f1[i], "forces accumulate into the caller's array");
        fmax = std::fmax(fmax, std::fabs(f1[i]));
        sum[i % 3] += f1[i];
    }
    // PotentialEnergy and AtomicVirial
    double energy = 0.0, virial[9];
    check(lg_compute(e, 0, in.x.data(), LG_TERM_ALL, LG_WANT_ENERGY, nullptr, &energy, nullptr) == LG_OK, "energy");
    check(lg_compute(e, 0, in.x.data(), LG_TERM_ALL, LG_WANT_VIRIAL, nullptr, nullptr, virial) == LG_OK, "virial");
    check(std::isfinite(energy), "finite energy");

    // VelocityVerlet: setup, then integrate once per step
    std::vector<double> x(in.x), v(n3, 0.0);
    lg_md_params p;
    std::memset(&p, 0, sizeof(p));
    p.integrator = LG_INTEGRATOR_VELOCITY_VERLET;
    p.timestep = 1.0;
    check(lg_md_setup_ex(e, 0, &p) == LG_OK, "md setup");
    for (int step = 0; step < 10; step++)
        check(lg_md_integrate(e, x.data(), v.data(), 1) == LG_OK, "integrate");
    lg_engine* e2 = make_engine(in, &status);
    std::vector<double> x2(in.x), v2(n3, 0.0);
    check(lg_md_setup_ex(e2, 0, &p) == LG_OK, "md setup (run)");
    check(lg_md_set_state(e2, 0, x2.data(), v2.data()) == LG_OK, "set state");
    check(lg_md_run(e2, 10) == LG_OK, "run");
    check(lg_md_get_state(e2, 0, x2.data(), v2.data()) == LG_OK, "get state");
    bool same = true;
    for (long i = 0; i < n3; i++) same = same && x[i] == x2[i] && v[i] == v2[i];
    check(same, "ten integrate calls equal one ten-step run");

    // set_pair_potential's check of the cutoff against half the cell
    Input wide = in;
    wide.cutoff = 0.75 * in.L;
    std::vector<lg_pair> big = pair_table(wide);
    int rc = lg_set_pairs(e2, 0, 2, big.data());
    check(rc == LG_ERR_ARGUMENT, "cutoff above half the cell is refused");
    check(std::strstr(lg_last_error(e2), "cutoff bigger than half of the smallest cell length") != nullptr,
          "the reference's message");

    double xsum = 0.0;
    for (long i = 0; i < n3; i++) xsum += x[i];
    std::printf("{\"status\": 0, \"energy\": %.17g, \"virial\": [%.17g, %.17g, %.17g, %.17g, %.17g, %.17g, "
                "%.17g, %.17g, %.17g], \"force_max\": %.17g, \"force_sum\": [%.17g, %.17g, %.17g], "
                "\"positions_sum_after_10_steps\": %.17g, \"failures\": %d}\n",
                energy, virial[0], virial[1], virial[2], virial[3], virial[4], virial[5], virial[6], virial[7],
                virial[8], fmax, sum[0], sum[1], sum[2], xsum, failures);
    lg_destroy(e);
    lg_destroy(e2);
    return failures ? 1 : 0;
}
