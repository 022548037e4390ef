// adjoint_vjp_selftest.cc -- host check of the general reverse-mode product
// (what lg_adjoint_vjp computes) from a state in mid-run.
//
// A Sedov problem whose every element holds energy runs npre cycles; from
// there, ncycles frozen-step cycles are recorded and differentiated.  The
// objective is J = sum over the eleven carried fields of seed_f . final_f,
// the seeds random normal (one field only if a name is given).  For each
// initial field, the adjoint's directional derivative along a random
// direction is compared with central differences of the oracle replaying the
// recorded run's branch decisions (Richardson over relative steps rel and
// rel/10), and dJ/dhgcoef likewise.
// Usage: adjoint_vjp_selftest nx npre ncycles [seed-field|all]
//        (prints one line per field, then WORST; needs the oracle compiled
//        with -DORC_TAPE)
// Environment: LG_FD_REL  relative step (default 1e-6)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "adjoint_host.h"

using hostadj::fld;
using std::vector;

namespace {

const char *const kFields[11] = {"x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"};

struct Case {
    int nx, nreg, npre, ncyc, E, N;
    double hg;
    vector<double> dts;   // npre + ncyc frozen steps
    vector<double> seed;  // 6N + 5E, in kFields order
    orc_domain *tape;     // the recorded run
};

size_t offset(const Case &c, int f)
{
    return f < 6 ? (size_t)f * c.N : 6 * (size_t)c.N + (size_t)(f - 6) * c.E;
}

// J after ncyc cycles from `state` (6N + 5E) at cycle npre, branches replayed
double objective(const Case &c, const vector<double> &state, double hg)
{
    orc_domain *d = orc_create_ex(c.nx, c.nreg, 1, 1, hg, 1.0);
    orc_dt_freeze(d, c.dts.data(), (int)c.dts.size());
    orc_set_scalar(d, "cycle", c.npre);
    for (int f = 0; f < 11; ++f) {
        size_t n;
        double *dst = orc_field_f64(d, kFields[f], &n);
        memcpy(dst, &state[offset(c, f)], 8 * n);
    }
    if (orc_tape_replay(d, c.tape) != 0 || orc_step(d, c.ncyc) != 0) {
        fprintf(stderr, "replayed forward failed\n");
        exit(2);
    }
    double J = 0.;
    for (int f = 0; f < 11; ++f) {
        const vector<double> v = fld(d, kFields[f]);
        for (size_t k = 0; k < v.size(); ++k) J += c.seed[offset(c, f) + k] * v[k];
    }
    orc_destroy(d);
    return J;
}

}  // namespace

int main(int argc, char **argv)
{
    Case c;
    c.nx = argc > 1 ? atoi(argv[1]) : 6;
    c.npre = argc > 2 ? atoi(argv[2]) : 5;
    c.ncyc = argc > 3 ? atoi(argv[3]) : 8;
    const char *only = argc > 4 ? argv[4] : "all";
    c.nreg = 11;
    c.hg = 3.0;
    c.E = c.nx * c.nx * c.nx;
    c.N = (c.nx + 1) * (c.nx + 1) * (c.nx + 1);
    const double rel = getenv("LG_FD_REL") ? atof(getenv("LG_FD_REL")) : 1e-6;

    // initial energy: the set-up field plus 1e-3..2e-3 of the origin energy
    // on every element; the time steps of its free run
    vector<double> e0;
    {
        orc_domain *d = orc_create_ex(c.nx, c.nreg, 1, 1, c.hg, 1.0);
        e0 = fld(d, "e");
        std::mt19937_64 g(11);
        std::uniform_real_distribution<double> u(0.0, 1.0);
        const double eo = e0[0];
        for (double &v : e0) v += 1e-3 * eo * (1.0 + u(g));
        size_t n;
        double *e = orc_field_f64(d, "e", &n);
        memcpy(e, e0.data(), 8 * n);
        orc_dt_record(d, c.npre + c.ncyc);
        if (orc_step(d, c.npre + c.ncyc) != 0) return 2;
        c.dts.assign(orc_dt_recorded(d), orc_dt_recorded(d) + c.npre + c.ncyc);
        orc_destroy(d);
    }
    orc_domain *d = orc_create_ex(c.nx, c.nreg, 1, 1, c.hg, 1.0);
    {
        size_t n;
        double *e = orc_field_f64(d, "e", &n);
        memcpy(e, e0.data(), 8 * n);
    }
    orc_dt_freeze(d, c.dts.data(), (int)c.dts.size());
    if (orc_step(d, c.npre) != 0) return 2;
    if (orc_tape_record(d, c.ncyc) != 0) {
        fprintf(stderr, "no decision tape (oracle built without -DORC_TAPE)\n");
        return 2;
    }
    c.tape = d;
    hostadj::Tape tape(d, c.ncyc);
    const vector<double> base(tape.snaps.begin(), tape.snaps.begin() + tape.snapD);

    c.seed.assign(tape.snapD, 0.);
    {
        std::mt19937_64 g(3);
        std::normal_distribution<double> nd(0.0, 1.0);
        for (int f = 0; f < 11; ++f) {
            const size_t cnt = f < 6 ? c.N : c.E;
            for (size_t k = 0; k < cnt; ++k) {
                const double v = nd(g);
                if (!strcmp(only, "all") || !strcmp(only, kFields[f])) c.seed[offset(c, f) + k] = v;
            }
        }
    }
    hostadj::Adjoint adj(d, c.hg);
    memcpy(adj.nbar.data(), c.seed.data(), 8 * 6 * (size_t)c.N);
    memcpy(adj.ebar.data(), c.seed.data() + 6 * (size_t)c.N, 8 * 5 * (size_t)c.E);
    const double hgb = adj.backward(tape, c.dts.data() + c.npre);

    double worst = 0.;
    std::mt19937_64 g(5);
    std::normal_distribution<double> nd(0.0, 1.0);
    auto richardson = [&](auto J_of) {
        double fd[2];
        for (int t = 0; t < 2; ++t) {
            const double h = t ? rel / 10 : rel;
            fd[t] = (J_of(h) - J_of(-h)) / (2 * h);
        }
        return fd[1] + (fd[1] - fd[0]) / 99;
    };
    for (int f = 0; f < 11; ++f) {
        const size_t off = offset(c, f), cnt = f < 6 ? c.N : c.E;
        double scale = 1e-3;  // the direction's size: the field's own
        for (size_t k = 0; k < cnt; ++k) scale = std::max(scale, std::fabs(base[off + k]));
        const double *grad = f < 6 ? &adj.nbar[(size_t)f * c.N] : &adj.ebar[(size_t)(f - 6) * c.E];
        vector<double> dir(cnt);
        double ad = 0.;
        for (size_t k = 0; k < cnt; ++k) {
            dir[k] = nd(g) * scale;
            ad += grad[k] * dir[k];
        }
        const double fd = richardson([&](double h) {
            vector<double> s = base;
            for (size_t k = 0; k < cnt; ++k) s[off + k] += h * dir[k];
            return objective(c, s, c.hg);
        });
        const double err = std::fabs(ad - fd) / std::max(std::fabs(fd), 1e-300);
        printf("%-3s adjoint % .10e fd % .10e rel %.2e\n", kFields[f], ad, fd, err);
        worst = std::max(worst, err);
    }
    {
        const double fd = richardson([&](double h) { return objective(c, base, c.hg * (1 + h)); }) / c.hg;
        const double err = std::fabs(hgb - fd) / std::max(std::fabs(fd), 1e-300);
        printf("hg  adjoint % .10e fd % .10e rel %.2e\n", hgb, fd, err);
        worst = std::max(worst, err);
    }
    printf("WORST %.3e\n", worst);
    orc_destroy(d);
    return 0;
}
