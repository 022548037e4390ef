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

#include "lg_adjoint_cycle.h"
#include "lulesh_oracle.h"

using namespace lg;
using std::vector;

static vector<double> fld(orc_domain *d, const char *n)
{
    size_t c;
    double *p = orc_field_f64(d, n, &c);
    return vector<double>(p, p + c);
}
static vector<int> ifld(orc_domain *d, const char *n)
{
    size_t c;
    int *p = orc_field_i32(d, n, &c);
    return vector<int>(p, p + c);
}

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

    // forward with stored states and temporaries
    orc_domain *d = fresh(r, r.e0, r.hg);
    const int E = r.nx * r.nx * r.nx, N = (r.nx + 1) * (r.nx + 1) * (r.nx + 1);
    const char *nodeF[6] = {"x", "y", "z", "xd", "yd", "zd"};
    const char *elemF[5] = {"e", "p", "q", "v", "ss"};
    const char *tempF[8] = {"vnew", "vdov", "delx_xi", "delx_eta", "delx_zeta",
                            "delv_xi", "delv_eta", "delv_zeta"};
    const size_t snapD = 6 * (size_t)N + 5 * (size_t)E;
    vector<double> snaps((r.ncyc + 1) * snapD), temps(r.ncyc * 8 * (size_t)E);
    const bool branch = getenv("LG_FD_BRANCH") && atoi(getenv("LG_FD_BRANCH"));
    if (branch) {
        if (orc_tape_record(d, r.ncyc) != 0) {
            fprintf(stderr, "no decision tape (oracle built without -DORC_TAPE)\n");
            return 2;
        }
        g_tape = d;
    }
    auto save = [&](int c) {
        double *b = &snaps[c * snapD];
        for (int i = 0; i < 6; ++i) {
            const vector<double> f = fld(d, nodeF[i]);
            memcpy(b + (size_t)i * N, f.data(), 8 * (size_t)N);
        }
        for (int i = 0; i < 5; ++i) {
            const vector<double> f = fld(d, elemF[i]);
            memcpy(b + 6 * (size_t)N + (size_t)i * E, f.data(), 8 * (size_t)E);
        }
    };
    for (int c = 0; c < r.ncyc; ++c) {
        save(c);
        orc_step(d, 1);
        for (int t = 0; t < 8; ++t) {
            const vector<double> f = fld(d, tempF[t]);
            memcpy(&temps[(c * 8 + t) * (size_t)E], f.data(), 8 * (size_t)E);
        }
    }
    save(r.ncyc);

    // host DevState for the item functions
    DevState s{};
    s.E = E;
    s.N = N;
    vector<double> volo = fld(d, "volo"), mass = fld(d, "elemMass"), nmass = fld(d, "nodalMass");
    vector<int> nl = ifld(d, "nodelist"), nlT(8 * (size_t)E);
    for (int k = 0; k < E; ++k)
        for (int j = 0; j < 8; ++j) nlT[(size_t)j * E + k] = nl[8 * k + j];
    vector<int> nes = ifld(d, "nodeElemStart"), ncl = ifld(d, "nodeElemCornerList");
    vector<int> lxim = ifld(d, "lxim"), lxip = ifld(d, "lxip"), letam = ifld(d, "letam"),
                letap = ifld(d, "letap"), lzetam = ifld(d, "lzetam"), lzetap = ifld(d, "lzetap"),
                bc = ifld(d, "elemBC");
    vector<uint8_t> symm(N, 0);
    for (int v : ifld(d, "symmX")) symm[v] |= 1;
    for (int v : ifld(d, "symmY")) symm[v] |= 2;
    for (int v : ifld(d, "symmZ")) symm[v] |= 4;
    s.volo = volo.data();
    s.elemMass = mass.data();
    s.nodalMass = nmass.data();
    s.nodelistT = nlT.data();
    s.nodeElemStart = nes.data();
    s.nodeElemCornerList = ncl.data();
    s.lxim = lxim.data(); s.lxip = lxip.data(); s.letam = letam.data(); s.letap = letap.data();
    s.lzetam = lzetam.data(); s.lzetap = lzetap.data(); s.elemBC = bc.data();
    s.symm = symm.data();
    s.prm = {1e-7, 1e-7, 1e-7, 1e-10, 1e-7, r.hg, 4.0 / 3.0, 1e12, 1.0, 2.0, 0.5, 2.0 / 3.0, 2.0,
             1e9, 1e-9, 0.0, -1e15, 0.1, 1.0};

    // reverse neighbour map (as lg_adjoint.cu builds it)
    vector<int> revStart(E + 1, 0), revEntry;
    {
        vector<vector<int>> lists(E);
        const vector<int> *nb[6] = {&lxim, &lxip, &letam, &letap, &lzetam, &lzetap};
        const int mm[3] = {XI_M, ETA_M, ZETA_M}, ms[3] = {XI_M_SYMM, ETA_M_SYMM, ZETA_M_SYMM},
                  mf[3] = {XI_M_FREE, ETA_M_FREE, ZETA_M_FREE};
        const int pm[3] = {XI_P, ETA_P, ZETA_P}, ps[3] = {XI_P_SYMM, ETA_P_SYMM, ZETA_P_SYMM},
                  pf[3] = {XI_P_FREE, ETA_P_FREE, ZETA_P_FREE};
        auto uses = [](int bits, int mask, int sym, int fr) {
            const int b = bits & mask;
            return b == 0 || (b != sym && b != fr && b == (mask & ~(sym | fr)));
        };
        for (int j = 0; j < E; ++j)
            for (int dd = 0; dd < 3; ++dd) {
                if (uses(bc[j], mm[dd], ms[dd], mf[dd])) lists[(*nb[2 * dd])[j]].push_back(j * 6 + 2 * dd);
                if (uses(bc[j], pm[dd], ps[dd], pf[dd])) lists[(*nb[2 * dd + 1])[j]].push_back(j * 6 + 2 * dd + 1);
            }
        for (int k = 0; k < E; ++k) {
            revStart[k + 1] = revStart[k] + (int)lists[k].size();
            revEntry.insert(revEntry.end(), lists[k].begin(), lists[k].end());
        }
    }

    // adjoint arrays
    vector<double> nbar(6 * (size_t)N, 0.), ebar(5 * (size_t)E, 0.), vnewb(E), dxb(3 * (size_t)E),
        dvb(3 * (size_t)E), slot(6 * (size_t)E), corner(48 * (size_t)E), fb(3 * (size_t)N), hgpart(1);
    for (int i = 0; i < E; ++i)
        if (r.mask[i]) ebar[i] = volo[i];
    adj::AdjArgs A;
    for (int i = 0; i < 6; ++i) A.nb[i] = &nbar[(size_t)i * N];
    A.eb = &ebar[0]; A.pb = &ebar[E]; A.qb = &ebar[2 * (size_t)E]; A.vb = &ebar[3 * (size_t)E];
    A.ssb = &ebar[4 * (size_t)E];
    A.vnewb = vnewb.data();
    for (int i = 0; i < 3; ++i) {
        A.delxb[i] = &dxb[(size_t)i * E];
        A.delvb[i] = &dvb[(size_t)i * E];
    }
    A.slot = slot.data(); A.corner = corner.data(); A.fb = fb.data(); A.hgPart = hgpart.data();
    A.revStart = revStart.data(); A.revEntry = revEntry.data(); A.hg = r.hg;
    auto snap_at = [&](int c) {
        adj::Snap sn;
        double *b = &snaps[c * snapD];
        for (int i = 0; i < 6; ++i) sn.n[i] = b + (size_t)i * N;
        for (int i = 0; i < 5; ++i) sn.el[i] = b + 6 * (size_t)N + (size_t)i * E;
        return sn;
    };
    double hgb = 0.;
    for (int c = r.ncyc - 1; c >= 0; --c) {
        A.s0 = snap_at(c);
        A.s1 = snap_at(c + 1);
        for (int t = 0; t < 8; ++t) A.tc.t[t] = &temps[(c * 8 + t) * (size_t)E];
        A.dt = r.dts[c];
        for (int k = 0; k < E; ++k) adj::adj_material(s, A, k);
        for (int k = 0; k < E; ++k) adj::adj_qslots(s, A, k);
        for (int k = 0; k < E; ++k) adj::adj_kinematics(s, A, k);
        for (int n = 0; n < N; ++n) adj::adj_nodes(s, A, n);
        for (int k = 0; k < E; ++k) hgb += adj::adj_forces(s, A, k);
        for (int n = 0; n < N; ++n) adj::adj_gather(s, A, n);
    }

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
