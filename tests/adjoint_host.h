// adjoint_host.h -- the GPU adjoint's item functions (lg_adjoint_cycle.h)
// looped on the host over states the oracle stored, for the host checks
// adjoint_cycle_selftest.cc and adjoint_vjp_selftest.cc.
#pragma once
#include <cstring>
#include <vector>

#include "lg_adjoint_cycle.h"
#include "lulesh_oracle.h"

namespace hostadj {

using std::vector;

inline vector<double> fld(orc_domain *d, const char *n)
{
    size_t c;
    double *p = orc_field_f64(d, n, &c);
    return vector<double>(p, p + c);
}
inline vector<int> ifld(orc_domain *d, const char *n)
{
    size_t c;
    int *p = orc_field_i32(d, n, &c);
    return vector<int>(p, p + c);
}

inline const char *const kNodeF[6] = {"x", "y", "z", "xd", "yd", "zd"};
inline const char *const kElemF[5] = {"e", "p", "q", "v", "ss"};
inline const char *const kTempF[8] = {"vnew", "vdov", "delx_xi", "delx_eta", "delx_zeta",
                                      "delv_xi", "delv_eta", "delv_zeta"};

// Forward cycles of d with the carried state stored before each cycle and
// after the last, and each cycle's kinematic temporaries.
struct Tape {
    int E, N, ncyc;
    size_t snapD;
    vector<double> snaps, temps;
    Tape(orc_domain *d, int ncycles)
    {
        E = (int)orc_get_scalar(d, "numElem");
        N = (int)orc_get_scalar(d, "numNode");
        ncyc = ncycles;
        snapD = 6 * (size_t)N + 5 * (size_t)E;
        snaps.resize((ncyc + 1) * snapD);
        temps.resize(ncyc * 8 * (size_t)E);
        for (int c = 0; c < ncyc; ++c) {
            save(d, c);
            orc_step(d, 1);
            for (int t = 0; t < 8; ++t) {
                const vector<double> f = fld(d, kTempF[t]);
                memcpy(&temps[(c * 8 + t) * (size_t)E], f.data(), 8 * (size_t)E);
            }
        }
        save(d, ncyc);
    }
    void save(orc_domain *d, int c)
    {
        double *b = &snaps[c * snapD];
        for (int i = 0; i < 6; ++i) {
            const vector<double> f = fld(d, kNodeF[i]);
            memcpy(b + (size_t)i * N, f.data(), 8 * (size_t)N);
        }
        for (int i = 0; i < 5; ++i) {
            const vector<double> f = fld(d, kElemF[i]);
            memcpy(b + 6 * (size_t)N + (size_t)i * E, f.data(), 8 * (size_t)E);
        }
    }
    lg::adj::Snap snap(int c)
    {
        lg::adj::Snap sn;
        double *b = &snaps[c * snapD];
        for (int i = 0; i < 6; ++i) sn.n[i] = b + (size_t)i * N;
        for (int i = 0; i < 5; ++i) sn.el[i] = b + 6 * (size_t)N + (size_t)i * E;
        return sn;
    }
};

// The topology, masses and adjoint arrays; backward() runs the reverse
// sweep over a Tape.  nbar (6 x N: x y z xd yd zd) and ebar (5 x E: e p q v
// ss) hold the adjoint of the state: the caller seeds them with dJ/d(final
// state) and reads dJ/d(initial state) back.
struct Adjoint {
    int E, N;
    lg::DevState s{};
    vector<double> volo, mass, nmass;
    vector<int> nlT, nes, ncl, lxim, lxip, letam, letap, lzetam, lzetap, bc;
    vector<uint8_t> symm;
    vector<int> revStart, revEntry;
    vector<double> nbar, ebar, vnewb, dxb, dvb, slot, corner, fb, hgpart;
    lg::adj::AdjArgs A;

    Adjoint(orc_domain *d, double hg)
    {
        E = (int)orc_get_scalar(d, "numElem");
        N = (int)orc_get_scalar(d, "numNode");
        s.E = E;
        s.N = N;
        volo = fld(d, "volo");
        mass = fld(d, "elemMass");
        nmass = fld(d, "nodalMass");
        const vector<int> nl = ifld(d, "nodelist");
        nlT.resize(8 * (size_t)E);
        for (int k = 0; k < E; ++k)
            for (int j = 0; j < 8; ++j) nlT[(size_t)j * E + k] = nl[8 * k + j];
        nes = ifld(d, "nodeElemStart");
        ncl = ifld(d, "nodeElemCornerList");
        lxim = ifld(d, "lxim"); lxip = ifld(d, "lxip"); letam = ifld(d, "letam");
        letap = ifld(d, "letap"); lzetam = ifld(d, "lzetam"); lzetap = ifld(d, "lzetap");
        bc = ifld(d, "elemBC");
        symm.assign(N, 0);
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
        s.prm = {1e-7, 1e-7, 1e-7, 1e-10, 1e-7, hg, 4.0 / 3.0, 1e12, 1.0, 2.0, 0.5, 2.0 / 3.0, 2.0,
                 1e9, 1e-9, 0.0, -1e15, 0.1, 1.0};
        reverse_neighbours();
        nbar.assign(6 * (size_t)N, 0.);
        ebar.assign(5 * (size_t)E, 0.);
        vnewb.resize(E);
        dxb.resize(3 * (size_t)E);
        dvb.resize(3 * (size_t)E);
        slot.resize(6 * (size_t)E);
        corner.resize(48 * (size_t)E);
        fb.resize(3 * (size_t)N);
        hgpart.resize(1);
        for (int i = 0; i < 6; ++i) A.nb[i] = &nbar[(size_t)i * N];
        A.eb = &ebar[0]; A.pb = &ebar[E]; A.qb = &ebar[2 * (size_t)E]; A.vb = &ebar[3 * (size_t)E];
        A.ssb = &ebar[4 * (size_t)E];
        A.vnewb = vnewb.data();
        for (int i = 0; i < 3; ++i) {
            A.delxb[i] = &dxb[(size_t)i * E];
            A.delvb[i] = &dvb[(size_t)i * E];
        }
        A.slot = slot.data(); A.corner = corner.data(); A.fb = fb.data(); A.hgPart = hgpart.data();
        A.revStart = revStart.data(); A.revEntry = revEntry.data(); A.hg = hg;
    }

    // for each element, the (neighbour, direction, side) slots of the
    // elements whose limiter reads it (as lg_adjoint.cu builds the map)
    void reverse_neighbours()
    {
        using namespace lg;
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
        revStart.assign(E + 1, 0);
        for (int k = 0; k < E; ++k) {
            revStart[k + 1] = revStart[k] + (int)lists[k].size();
            revEntry.insert(revEntry.end(), lists[k].begin(), lists[k].end());
        }
        if (revEntry.empty()) revEntry.push_back(0);
    }

    // reverse sweep over the tape's cycles; dts[c] is cycle c's time step;
    // returns dJ/dhgcoef
    double backward(Tape &t, const double *dts)
    {
        using namespace lg::adj;
        double hgb = 0.;
        for (int c = t.ncyc - 1; c >= 0; --c) {
            A.s0 = t.snap(c);
            A.s1 = t.snap(c + 1);
            for (int k = 0; k < 8; ++k) A.tc.t[k] = &t.temps[(c * 8 + k) * (size_t)E];
            A.dt = dts[c];
            for (int k = 0; k < E; ++k) adj_material(s, A, k);
            for (int k = 0; k < E; ++k) adj_qslots(s, A, k);
            for (int k = 0; k < E; ++k) adj_kinematics(s, A, k);
            for (int n = 0; n < N; ++n) adj_nodes(s, A, n);
            for (int k = 0; k < E; ++k) hgb += adj_forces(s, A, k);
            for (int n = 0; n < N; ++n) adj_gather(s, A, n);
        }
        return hgb;
    }
};

}  // namespace hostadj
