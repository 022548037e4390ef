// adjoint_cycle_selftest.cc -- host check of the whole-cycle adjoint.
//
// The oracle (oracle/lulesh_oracle.c) runs the forward cycles with frozen
// time steps; the adjoint item functions of lulesh_gb300/csrc/lg_adjoint_cycle.h
// -- the same code the GPU adjoint kernels run -- are looped over elements
// and nodes on the host, cycle by cycle in reverse.  The gradient of
// J = sum(e * volo over a mask) with respect to the initial energy field and
// hgcoef is compared with central finite differences of the oracle.
// Usage: adjoint_cycle_selftest nx ncycles [nnoise [dump.bin]]
//        (prints per-check errors, then WORST; dump.bin receives nx, ncycles,
//        the initial energy field, the frozen steps, the mask and the
//        gradients, for comparing another implementation on the same inputs)
// Environment: LG_FD_REL  relative step (default 1e-6)
//              LG_FD_BRANCH=1  differences replay the forward run's branch
//                 decisions (orc_tape_replay; needs the oracle compiled with
//                 -DORC_TAPE) instead of re-deciding them
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "adjoint_host.h"

using hostadj::fld;
using hostadj::ifld;
using std::vector;

struct Run {
    int nx, nreg, ncyc;
    double hg;
    vector<double> e0, dts;
    vector<unsigned char> mask;
};

static orc_domain *fresh(const Run &r, const vector<double> &e0, double hg)
{
    orc_domain *d = orc_create_ex(r.nx, r.nreg, 1, 1, hg, 1.0);
    size_t n;
    double *e = orc_field_f64(d, "e", &n);
    memcpy(e, e0.data(), sizeof(double) * n);
    if (!r.dts.empty()) orc_dt_freeze(d, r.dts.data(), (int)r.dts.size());
    return d;
}

static orc_domain *g_tape = nullptr;  // recorded run the differences replay

static double objective(const Run &r, const vector<double> &e0, double hg)
{
    orc_domain *d = fresh(r, e0, hg);
    if (g_tape && orc_tape_replay(d, g_tape) != 0) {
        fprintf(stderr, "no decision tape (oracle built without -DORC_TAPE)\n");
        exit(2);
    }
    if (orc_step(d, r.ncyc) != 0) {
        fprintf(stderr, "forward failed\n");
        exit(2);
    }
    const vector<double> e = fld(d, "e"), volo = fld(d, "volo");
    double J = 0;
    for (size_t i = 0; i < e.size(); ++i)
        if (r.mask[i]) J += e[i] * volo[i];
    orc_destroy(d);
    return J;
}

int main(int argc, char **argv)
{
    Run r;
    r.nx = argc > 1 ? atoi(argv[1]) : 5;
    r.ncyc = argc > 2 ? atoi(argv[2]) : 3;
    const int nnoise = argc > 3 ? atoi(argv[3]) : 40;
    r.nreg = 3;
    r.hg = 3.0;
    // noisy initial energy: the set-up field plus noise near the origin
    {
        orc_domain *d = orc_create_ex(r.nx, r.nreg, 1, 1, r.hg, 1.0);
        r.e0 = fld(d, "e");
        std::mt19937_64 g(11);
        std::normal_distribution<double> nd(0.0, 1e-3 * r.e0[0]);
        const int E = (int)r.e0.size();
        for (int i = 0; i < std::min(E, nnoise); ++i) r.e0[i] += nd(g);
        orc_destroy(d);
    }
    // time steps from the forward run of e0, and the mask (centroid r < 0.5
    // of the domain size 1.125 scaled to this mesh: r < 0.45)
    {
        orc_domain *d = fresh(r, r.e0, r.hg);
        orc_dt_record(d, r.ncyc);
        orc_step(d, r.ncyc);
        r.dts.assign(orc_dt_recorded(d), orc_dt_recorded(d) + r.ncyc);
        const vector<int> nl = ifld(d, "nodelist");
        const vector<double> x = fld(d, "x"), y = fld(d, "y"), z = fld(d, "z");
        const int E = r.nx * r.nx * r.nx;
        r.mask.assign(E, 0);
        for (int k = 0; k < E; ++k) {
            double cx = 0, cy = 0, cz = 0;
            for (int j = 0; j < 8; ++j) {
                cx += x[nl[8 * k + j]] / 8;
                cy += y[nl[8 * k + j]] / 8;
                cz += z[nl[8 * k + j]] / 8;
            }
            r.mask[k] = std::sqrt(cx * cx + cy * cy + cz * cz) < 0.45;
        }
        orc_destroy(d);
    }

    // forward with stored states and temporaries, then the reverse sweep
    orc_domain *d = fresh(r, r.e0, r.hg);
    const int E = r.nx * r.nx * r.nx;
    const bool branch = getenv("LG_FD_BRANCH") && atoi(getenv("LG_FD_BRANCH"));
    if (branch) {
        if (orc_tape_record(d, r.ncyc) != 0) {
            fprintf(stderr, "no decision tape (oracle built without -DORC_TAPE)\n");
            return 2;
        }
        g_tape = d;
    }
    hostadj::Tape tape(d, r.ncyc);
    hostadj::Adjoint adj(d, r.hg);
    for (int i = 0; i < E; ++i)
        if (r.mask[i]) adj.ebar[i] = adj.volo[i];
    const double hgb = adj.backward(tape, r.dts.data());
    const vector<double> &ebar = adj.ebar;

    // finite differences
    double worst = 0.;
    std::mt19937_64 g(5);
    std::uniform_real_distribution<double> u(-1, 1);
    const double rel = getenv("LG_FD_REL") ? atof(getenv("LG_FD_REL")) : 1e-6;
    const double scale = rel * r.e0[0];
    for (int trial = 0; trial < 6; ++trial) {
        vector<double> dir(E, 0.);
        double ad = 0.;
        // trial 0..2: single elements; 3..5: random directions near the origin
        if (trial < 3) {
            const int k = trial == 0 ? 0 : trial == 1 ? 1 : r.nx + 1;
            dir[k] = scale;
        } else {
            // relative step of a vector: |dir| = rel * |e0| over the perturbed entries
            const int m = std::min(E, std::max(nnoise, 1));
            double dn = 0., en = 0.;
            for (int k = 0; k < m; ++k) {
                dir[k] = u(g);
                dn += dir[k] * dir[k];
                en += r.e0[k] * r.e0[k];
            }
            for (int k = 0; k < m; ++k) dir[k] *= rel * std::sqrt(en / dn);
        }
        for (int k = 0; k < E; ++k) ad += ebar[k] * dir[k];
        vector<double> ep = r.e0, em = r.e0;
        for (int k = 0; k < E; ++k) {
            ep[k] += dir[k];
            em[k] -= dir[k];
        }
        const double fd = (objective(r, ep, r.hg) - objective(r, em, r.hg)) / 2;
        const double err = std::fabs(ad - fd) / std::max(std::fabs(fd), 1e-300);
        printf("e0 dir %d: adjoint % .10e fd % .10e rel %.2e\n", trial, ad, fd, err);
        worst = std::max(worst, err);
    }
    {
        const double h = rel * r.hg;
        const double fd = (objective(r, r.e0, r.hg + h) - objective(r, r.e0, r.hg - h)) / (2 * h);
        const double err = std::fabs(hgb - fd) / std::max(std::fabs(fd), 1e-300);
        printf("hgcoef: adjoint % .10e fd % .10e rel %.2e\n", hgb, fd, err);
        worst = std::max(worst, err);
    }
    printf("WORST %.3e\n", worst);
    if (argc > 4) {
        FILE *f = fopen(argv[4], "wb");
        const int hdr[2] = {r.nx, r.ncyc};
        fwrite(hdr, sizeof(int), 2, f);
        fwrite(r.e0.data(), sizeof(double), E, f);
        fwrite(r.dts.data(), sizeof(double), r.ncyc, f);
        fwrite(r.mask.data(), 1, E, f);
        fwrite(ebar.data(), sizeof(double), E, f);
        fwrite(&hgb, sizeof(double), 1, f);
        fclose(f);
    }
    orc_destroy(d);
    return 0;
}
