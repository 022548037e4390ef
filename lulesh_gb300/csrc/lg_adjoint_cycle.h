// lg_adjoint_cycle.h -- one cycle's adjoint, item by item (host and device).
//
// The bodies of the adjoint kernels of lg_adjoint.cu: each function handles
// one element or node; the kernels map threads onto them, and the host
// adjoint check in the tests maps a loop onto them.  The forward values come
// from the stored states S_c, S_{c+1} and the cycle's temporaries.
#pragma once

#include <cstddef>

#include "lg_adjoint_math.h"
#include "lg_device.h"

namespace lg {
namespace adj {

// fields of a state snapshot: node x y z xd yd zd, then element e p q v ss
struct Snap {
    double *n[6];
    double *el[5];
};
// per-cycle temporaries: vnew vdov delx_xi delx_eta delx_zeta delv_xi delv_eta delv_zeta
struct Temps {
    double *t[8];
};

struct AdjArgs {
    Snap s0, s1;  // S_c, S_{c+1}
    Temps tc;     // temporaries of cycle c
    double dt, hg;
    // adjoint of S_{c+1} on entry, of S_c on exit
    double *nb[6];
    double *eb, *pb, *qb, *vb, *ssb;
    // adjoint temporaries
    double *vnewb, *delxb[3], *delvb[3], *slot, *corner, *fb, *hgPart;
    const int *revStart, *revEntry;
};


LG_HD void limiter_sources(const DevState &s, const double *dv, int k,
                                                int bc, int mmask, int msymm, int mfree,
                                                int pmask, int psymm, int pfree, int nbm, int nbp,
                                                double &sm, int &km, double &sp, int &kp)
{
    const int bm = bc & mmask, bp = bc & pmask;
    if (bm == msymm) { sm = dv[k]; km = 1; }
    else if (bm == mfree) { sm = 0.; km = 2; }
    else if (bm == 0 || bm == (mmask & ~(msymm | mfree))) { sm = dv[nbm]; km = 0; }
    else { sm = 0.; km = 2; }
    if (bp == psymm) { sp = dv[k]; kp = 1; }
    else if (bp == pfree) { sp = 0.; kp = 2; }
    else if (bp == 0 || bp == (pmask & ~(psymm | pfree))) { sp = dv[nbp]; kp = 0; }
    else { sp = 0.; kp = 2; }
}

// EOS + limiter adjoint of one element (lulesh.cc:1761-1921, 2014-2427)
LG_HD void adj_material(const DevState &s, const AdjArgs &a, const int k)
{
    const Params &P = s.prm;
    const int E = s.E;
    const double vnew = a.tc.t[0][k], vdov = a.tc.t[1][k], v0 = a.s0.el[3][k];
    double vnewb = a.vb[k];  // v = vnew (the v_cut snap passes the derivative)
    double vc = vnew;
    bool clamped = false;
    if (P.eosvmin != 0. && vc < P.eosvmin) { vc = P.eosvmin; clamped = true; }
    if (P.eosvmax != 0. && vc > P.eosvmax) { vc = P.eosvmax; clamped = true; }
    const double delv = vnew - v0;

    // limiter forward
    const int bc = s.elemBC[k];
    const double *dvs[3] = {a.tc.t[5], a.tc.t[6], a.tc.t[7]};
    double self[3], delx[3], sm[3], sp[3];
    int km[3], kp[3];
    const int nbm[3] = {s.lxim[k], s.letam[k], s.lzetam[k]};
    const int nbp[3] = {s.lxip[k], s.letap[k], s.lzetap[k]};
    const int mm[3] = {XI_M, ETA_M, ZETA_M}, ms[3] = {XI_M_SYMM, ETA_M_SYMM, ZETA_M_SYMM},
              mf[3] = {XI_M_FREE, ETA_M_FREE, ZETA_M_FREE};
    const int pm[3] = {XI_P, ETA_P, ZETA_P}, ps[3] = {XI_P_SYMM, ETA_P_SYMM, ZETA_P_SYMM},
              pf_[3] = {XI_P_FREE, ETA_P_FREE, ZETA_P_FREE};
    adj::PhiFwd pf[3];
    double phi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        self[d] = dvs[d][k];
        delx[d] = a.tc.t[2 + d][k];
        limiter_sources(s, dvs[d], k, bc, mm[d], ms[d], mf[d], pm[d], ps[d], pf_[d], nbm[d],
                        nbp[d], sm[d], km[d], sp[d], kp[d]);
        pf[d] = adj::phi_forward(self[d], sm[d], sp[d], P.monoq_limiter_mult, P.monoq_max_slope);
        phi[d] = pf[d].phi;
    }
    const bool qact = !(vdov > 0.);
    double ql = 0., qq = 0., rho = 0.;
    if (qact) {
        double dxx[3];
        for (int d = 0; d < 3; ++d) {
            dxx[d] = self[d] * delx[d];
            if (dxx[d] > 0.) dxx[d] = 0.;
        }
        rho = s.elemMass[k] / (s.volo[k] * vnew);
        ql = -P.qlc_monoq * rho *
             (dxx[0] * (1. - phi[0]) + dxx[1] * (1. - phi[1]) + dxx[2] * (1. - phi[2]));
        qq = P.qqc_monoq * rho *
             (dxx[0] * dxx[0] * (1. - phi[0] * phi[0]) + dxx[1] * dxx[1] * (1. - phi[1] * phi[1]) +
              dxx[2] * dxx[2] * (1. - phi[2] * phi[2]));
    }
    // EOS
    const EosConst K = {P.e_cut, P.p_cut, P.q_cut, P.eosvmin, P.eosvmax, P.pmin, P.emin, P.refdens};
    const double e0 = a.s0.el[0][k], p0 = a.s0.el[1][k], q0 = a.s0.el[2][k];
    const adj::EosFwd f = adj::eos_forward(K, e0, delv, p0, q0, qq, ql, vc);
    const adj::EosAdj ea = adj::eos_vjp(K, f, e0, delv, p0, q0, qq, ql, vc, a.pb[k], a.eb[k],
                                        a.qb[k], a.ssb[k]);
    if (!clamped) vnewb += ea.vcb;
    vnewb += ea.delvcb;
    const double v0b = -ea.delvcb;
    // limiter adjoint
    double dvb[3] = {0., 0., 0.}, dxb[3] = {0., 0., 0.};
    double slot_m[3] = {0., 0., 0.}, slot_p[3] = {0., 0., 0.};
    if (qact) {
        double phib[3], rhob;
        adj::qlq_vjp(self, delx, phi, rho, P.qlc_monoq, P.qqc_monoq, ea.qlb, ea.qqb, dvb, dxb,
                     phib, rhob);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double smb, spb;
            adj::phi_vjp(pf[d], sm[d], sp[d], P.monoq_limiter_mult, phib[d], dvb[d], smb, spb);
            if (km[d] == 0) slot_m[d] = smb;
            else if (km[d] == 1) dvb[d] += smb;
            if (kp[d] == 0) slot_p[d] = spb;
            else if (kp[d] == 1) dvb[d] += spb;
        }
        vnewb += rhob * (-rho / vnew);
    }
    a.eb[k] = ea.e_oldb;
    a.pb[k] = ea.p_oldb;
    a.qb[k] = ea.q_oldb;
    a.vb[k] = v0b;
    a.ssb[k] = 0.;
    a.vnewb[k] = vnewb;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        a.delxb[d][k] = dxb[d];
        a.delvb[d][k] = dvb[d];
        a.slot[(size_t)(2 * d) * E + k] = slot_m[d];
        a.slot[(size_t)(2 * d + 1) * E + k] = slot_p[d];
    }
}

// neighbour reads of the limiter, gathered: entry j*6 + 2d + side
LG_HD void adj_qslots(const DevState &s, const AdjArgs &a, const int k)
{
    const int E = s.E;
    double add[3] = {0., 0., 0.};
    for (int i = a.revStart[k]; i < a.revStart[k + 1]; ++i) {
        const int en = a.revEntry[i];
        const int j = en / 6, r = en % 6;
        add[r >> 1] += a.slot[(size_t)r * E + j];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) a.delvb[d][k] += add[d];
}

// Q gradients + volume (lulesh.cc:1504-1757) at the updated positions
LG_HD void adj_kinematics(const DevState &s, const AdjArgs &a, const int k)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    int nd[8];
    double x[8], y[8], z[8], xd[8], yd[8], zd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        nd[j] = s.nodelistT[(size_t)j * E + k];
        x[j] = a.s1.n[0][nd[j]];
        y[j] = a.s1.n[1][nd[j]];
        z[j] = a.s1.n[2][nd[j]];
        xd[j] = a.s1.n[3][nd[j]];
        yd[j] = a.s1.n[4][nd[j]];
        zd[j] = a.s1.n[5][nd[j]];
    }
    double xb[8], yb[8], zb[8], xdb[8], ydb[8], zdb[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) xb[j] = yb[j] = zb[j] = xdb[j] = ydb[j] = zdb[j] = 0.;
    const double dxb[3] = {a.delxb[0][k], a.delxb[1][k], a.delxb[2][k]};
    const double dvb[3] = {a.delvb[0][k], a.delvb[1][k], a.delvb[2][k]};
    const double volo = s.volo[k], vnew = a.tc.t[0][k];
    const double vnewb = a.vnewb[k] + adj::qgrad_vjp(x, y, z, xd, yd, zd, volo, vnew, dxb, dvb, xb,
                                                     yb, zb, xdb, ydb, zdb);
    // vnew = V(x) / volo, dV/dx = CalcElemVolumeDerivative
    const double Vb = vnewb * (1.0 / volo);  // vnewb is 0 for most elements
    double dvdx[8], dvdy[8], dvdz[8];
    geom::volume_derivative(x, y, z, dvdx, dvdy, dvdz);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        a.corner[0 * E8 + (size_t)j * E + k] = xb[j] + Vb * dvdx[j];
        a.corner[1 * E8 + (size_t)j * E + k] = yb[j] + Vb * dvdy[j];
        a.corner[2 * E8 + (size_t)j * E + k] = zb[j] + Vb * dvdz[j];
        a.corner[3 * E8 + (size_t)j * E + k] = xdb[j];
        a.corner[4 * E8 + (size_t)j * E + k] = ydb[j];
        a.corner[5 * E8 + (size_t)j * E + k] = zdb[j];
    }
}

LG_HD void corner_sums(const DevState &s, const AdjArgs &a, int n,
                                            double out[6])
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
#pragma unroll
    for (int c = 0; c < 6; ++c) out[c] = 0.;
    for (int i = s.nodeElemStart[n]; i < s.nodeElemStart[n + 1]; ++i) {
        const int cr = s.nodeElemCornerList[i];
        const size_t idx = (size_t)(cr & 7) * E + (cr >> 3);
#pragma unroll
        for (int c = 0; c < 6; ++c) out[c] += a.corner[c * E8 + idx];
    }
}

// position / velocity update and a = F / m (lulesh.cc:1139-1219)
LG_HD void adj_nodes(const DevState &s, const AdjArgs &a, const int n)
{
    double cs[6];
    corner_sums(s, a, n, cs);
    const int sym = s.symm[n];
    const double m = s.nodalMass[n];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double Xb1 = a.nb[c][n] + cs[c];       // adjoint of the new position
        double Ub1 = a.nb[3 + c][n] + cs[3 + c];    // adjoint of the new velocity
        Ub1 += Xb1 * a.dt;                          // x' = x + u' dt
        const double Ub = Ub1;                      // u' = u + a dt (u_cut passes)
        const double ab = Ub1 * a.dt;
        const double Fb = (sym & (1 << c)) ? 0. : ab / m;  // a = F / m, zero on symmetry planes
        a.nb[c][n] = Xb1;
        a.nb[3 + c][n] = Ub;
        a.fb[3 * (size_t)n + c] = Fb;
    }
}

// stress + FB hourglass forces (lulesh.cc:273-1057)
// returns this element's share of the hourglass-coefficient adjoint
LG_HD double adj_forces(const DevState &s, const AdjArgs &a, const int k)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    double hgb = 0.;
    {
        int nd[8];
        double x[8], y[8], z[8], xd[8], yd[8], zd[8], fb[3][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            nd[j] = s.nodelistT[(size_t)j * E + k];
            x[j] = a.s0.n[0][nd[j]];
            y[j] = a.s0.n[1][nd[j]];
            z[j] = a.s0.n[2][nd[j]];
            xd[j] = a.s0.n[3][nd[j]];
            yd[j] = a.s0.n[4][nd[j]];
            zd[j] = a.s0.n[5][nd[j]];
            fb[0][j] = a.fb[3 * (size_t)nd[j] + 0];
            fb[1][j] = a.fb[3 * (size_t)nd[j] + 1];
            fb[2][j] = a.fb[3 * (size_t)nd[j] + 2];
        }
        double xb[8], yb[8], zb[8], xdb[8], ydb[8], zdb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) xb[j] = yb[j] = zb[j] = xdb[j] = ydb[j] = zdb[j] = 0.;
        adj::ForceAdj o = {0., 0., 0., 0., 0.};
        adj::forces_vjp(x, y, z, xd, yd, zd, a.s0.el[1][k], a.s0.el[2][k], a.s0.el[3][k],
                        s.volo[k], a.s0.el[4][k], s.elemMass[k], a.hg, fb, xb, yb, zb, xdb, ydb,
                        zdb, o);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            a.corner[0 * E8 + (size_t)j * E + k] = xb[j];
            a.corner[1 * E8 + (size_t)j * E + k] = yb[j];
            a.corner[2 * E8 + (size_t)j * E + k] = zb[j];
            a.corner[3 * E8 + (size_t)j * E + k] = xdb[j];
            a.corner[4 * E8 + (size_t)j * E + k] = ydb[j];
            a.corner[5 * E8 + (size_t)j * E + k] = zdb[j];
        }
        a.pb[k] += o.pb;
        a.qb[k] += o.qb;
        a.vb[k] += o.vb;
        a.ssb[k] += o.ssb;
        hgb = o.hgb;
    }
    return hgb;
}

// the element -> node corner sums of the forces adjoint
LG_HD void adj_gather(const DevState &s, const AdjArgs &a, const int n)
{
    double cs[6];
    corner_sums(s, a, n, cs);
    for (int c = 0; c < 6; ++c) a.nb[c][n] += cs[c];
}

}  // namespace adj
}  // namespace lg
