// lg_adjoint_math.h -- element-local vector-Jacobian products of the
// leap-frog cycle (reverse mode, FP64), usable on the device and the host.
//
// Each function recomputes the forward values it needs from the same inputs
// the forward kernel read and accumulates the adjoints (suffix "b") of those
// inputs from the adjoints of its outputs.  Non-smooth operations: the
// physical clamps and switches (emin, pmin, eosvmin/eosvmax, the monotonic
// limiter's min/max and its vdov > 0 switch, the sound-speed floor) take the
// derivative of the branch the forward took (zero when they fire); the
// numerical noise cut-offs (|e| < e_cut, |p| < p_cut, |q| < q_cut, and in
// the node and volume updates u_cut and v_cut), which zero values within
// ~1e-7 of zero, pass the derivative through -- the derivative of the map
// without its noise suppressor, which is what finite differences of any
// resolvable step see.  The time step is an input (frozen), so the
// Courant/hydro constraints and everything only they read (arealg, vdov's
// value) have no
// adjoint.  Forward formulas: lulesh.cc lines cited at each function.
#pragma once

#include "lg_geometry.cuh"

namespace lg {
namespace adj {

using geom::gam;

struct V3 {
    double x, y, z;
};
LG_HD V3 cross(const V3 &a, const V3 &b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
LG_HD double dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ---------------------------------------------------------------------------
// CalcElemNodeNormals (lulesh.cc:381-474): pf = sum over faces of
// 0.25 * b0 x b1, b0/b1 the face bisectors.  pfb -> xb, yb, zb.
// ---------------------------------------------------------------------------
LG_HD void face_normal_vjp(const double *x, const double *y, const double *z, int a, int b, int c,
                           int d, const double *pbx, const double *pby, const double *pbz,
                           double *xb, double *yb, double *zb)
{
    const V3 b0 = {0.5 * (x[d] + x[c] - x[b] - x[a]), 0.5 * (y[d] + y[c] - y[b] - y[a]),
                   0.5 * (z[d] + z[c] - z[b] - z[a])};
    const V3 b1 = {0.5 * (x[c] + x[b] - x[d] - x[a]), 0.5 * (y[c] + y[b] - y[d] - y[a]),
                   0.5 * (z[c] + z[b] - z[d] - z[a])};
    const V3 A = {pbx[a] + pbx[b] + pbx[c] + pbx[d], pby[a] + pby[b] + pby[c] + pby[d],
                  pbz[a] + pbz[b] + pbz[c] + pbz[d]};
    const V3 c0 = cross(b1, A), c1 = cross(A, b0);  // d(b0 x b1).A = db0.(b1 x A) + db1.(A x b0)
    const V3 g0 = {0.25 * c0.x, 0.25 * c0.y, 0.25 * c0.z};
    const V3 g1 = {0.25 * c1.x, 0.25 * c1.y, 0.25 * c1.z};
    xb[d] += 0.5 * (g0.x - g1.x); yb[d] += 0.5 * (g0.y - g1.y); zb[d] += 0.5 * (g0.z - g1.z);
    xb[c] += 0.5 * (g0.x + g1.x); yb[c] += 0.5 * (g0.y + g1.y); zb[c] += 0.5 * (g0.z + g1.z);
    xb[b] += 0.5 * (g1.x - g0.x); yb[b] += 0.5 * (g1.y - g0.y); zb[b] += 0.5 * (g1.z - g0.z);
    xb[a] -= 0.5 * (g0.x + g1.x); yb[a] -= 0.5 * (g0.y + g1.y); zb[a] -= 0.5 * (g0.z + g1.z);
}

LG_HD void node_normals_vjp(const double *x, const double *y, const double *z, const double *pbx,
                            const double *pby, const double *pbz, double *xb, double *yb,
                            double *zb)
{
    face_normal_vjp(x, y, z, 0, 1, 2, 3, pbx, pby, pbz, xb, yb, zb);
    face_normal_vjp(x, y, z, 0, 4, 5, 1, pbx, pby, pbz, xb, yb, zb);
    face_normal_vjp(x, y, z, 1, 5, 6, 2, pbx, pby, pbz, xb, yb, zb);
    face_normal_vjp(x, y, z, 2, 6, 7, 3, pbx, pby, pbz, xb, yb, zb);
    face_normal_vjp(x, y, z, 3, 7, 4, 0, pbx, pby, pbz, xb, yb, zb);
    face_normal_vjp(x, y, z, 4, 7, 6, 5, pbx, pby, pbz, xb, yb, zb);
}

// ---------------------------------------------------------------------------
// VoluDer / CalcElemVolumeDerivative (lulesh.cc:591-663).  With pair sums
// U[P] = u[P.first] + u[P.second] over the six neighbour nodes m0..m5:
//   dvdx =  t * sum_i S_i Y[P_i] Z[Q_i]
//   dvdy = -t * sum_i S_i X[P_i] Z[Q_i]
//   dvdz = -t * sum_i S_i Y[P_i] X[Q_i],   t = 1/12,
// P = {12,01,04,34,25,35}, Q = {01,12,34,04,35,25}, S = {+,-,+,-,-,+}.
// ---------------------------------------------------------------------------
LG_HD void volu_der_vjp(const double *x, const double *y, const double *z, const int m[6],
                        double a, double b, double c, double *xb, double *yb, double *zb)
{
    const int P[6][2] = {{1, 2}, {0, 1}, {0, 4}, {3, 4}, {2, 5}, {3, 5}};
    const int Q[6][2] = {{0, 1}, {1, 2}, {3, 4}, {0, 4}, {3, 5}, {2, 5}};
    const double S[6] = {1., -1., 1., -1., -1., 1.};
    const double t = 1.0 / 12.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const int p0 = m[P[i][0]], p1 = m[P[i][1]], q0 = m[Q[i][0]], q1 = m[Q[i][1]];
        const double Xp = x[p0] + x[p1], Yp = y[p0] + y[p1];
        const double Xq = x[q0] + x[q1], Zq = z[q0] + z[q1];
        const double ts = t * S[i];
        const double gYp = ts * (a * Zq - c * Xq);
        const double gZq = ts * (a * Yp - b * Xp);
        const double gXp = -ts * b * Zq;
        const double gXq = -ts * c * Yp;
        yb[p0] += gYp; yb[p1] += gYp;
        zb[q0] += gZq; zb[q1] += gZq;
        xb[p0] += gXp; xb[p1] += gXp;
        xb[q0] += gXq; xb[q1] += gXq;
    }
}

// neighbour nodes of each corner, CalcElemVolumeDerivative (lulesh.cc:631-662)
LG_HD void corner_neighbours(int k, int m[6])
{
    const int T[8][6] = {{1, 2, 3, 4, 5, 7}, {2, 3, 0, 5, 6, 4}, {3, 0, 1, 6, 7, 5},
                         {0, 1, 2, 7, 4, 6}, {7, 6, 5, 0, 3, 1}, {4, 7, 6, 1, 0, 2},
                         {5, 4, 7, 2, 1, 3}, {6, 5, 4, 3, 2, 0}};
    for (int i = 0; i < 6; ++i) m[i] = T[k][i];
}

LG_HD void volume_derivative_vjp(const double *x, const double *y, const double *z,
                                 const double *dxb, const double *dyb, const double *dzb,
                                 double *xb, double *yb, double *zb)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int m[6];
        corner_neighbours(k, m);
        volu_der_vjp(x, y, z, m, dxb[k], dyb[k], dzb[k], xb, yb, zb);
    }
}

// ---------------------------------------------------------------------------
// Element forces (lulesh.cc:273-286, 494-587, 710-1057): stress forces
// -sig * normals, sig = -p - q, plus the FB hourglass forces
//   f_c[i] = coef * sum_m hourgam[i][m] * hxx_c[m],
//   hxx_c[m] = sum_j hourgam[j][m] u_c[j],
//   hourgam[i][m] = gamma[m][i] - volinv * (dvd(i) . hourmod(m)),
//   coef = -hg 0.01 ss mass / cbrt(volo v).
// fb[c][i]: adjoint of the corner force component c at corner i (stress and
// hourglass parts are summed into the same node force, so they share it).
// ---------------------------------------------------------------------------
struct ForceAdj {
    double pb, qb, vb, ssb, hgb;
};

LG_HD void forces_vjp(const double *x, const double *y, const double *z, const double *xd,
                      const double *yd, const double *zd, double p, double q, double v, double volo,
                      double ss, double mass, double hg, const double (*fb)[8], double *xb,
                      double *yb, double *zb, double *xdb, double *ydb, double *zdb, ForceAdj &o)
{
    // stress part
    {
        const double sig = -p - q;
        double pfx[8], pfy[8], pfz[8];
        geom::node_normals(pfx, pfy, pfz, x, y, z);
        double pbx[8], pby[8], pbz[8], sigb = 0.0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            pbx[j] = -sig * fb[0][j];
            pby[j] = -sig * fb[1][j];
            pbz[j] = -sig * fb[2][j];
            sigb -= fb[0][j] * pfx[j] + fb[1][j] * pfy[j] + fb[2][j] * pfz[j];
        }
        o.pb -= sigb;
        o.qb -= sigb;
        node_normals_vjp(x, y, z, pbx, pby, pbz, xb, yb, zb);
    }
    if (!(hg > 0.)) return;
    // hourglass part: forward recompute
    double dvdx[8], dvdy[8], dvdz[8];
    geom::volume_derivative(x, y, z, dvdx, dvdy, dvdz);
    const double vol = volo * v;
    const double volinv = 1.0 / vol;
    double hm[4][3];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        double a = 0., b = 0., c = 0.;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            a += x[j] * gam(m, j);
            b += y[j] * gam(m, j);
            c += z[j] * gam(m, j);
        }
        hm[m][0] = a;
        hm[m][1] = b;
        hm[m][2] = c;
    }
    double hg_[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int m = 0; m < 4; ++m)
            hg_[i][m] = gam(m, i) - volinv * (dvdx[i] * hm[m][0] + dvdy[i] * hm[m][1] +
                                               dvdz[i] * hm[m][2]);
    const double cr = cbrt(vol);
    const double coef = -hg * 0.01 * ss * mass / cr;
    const double *vel[3] = {xd, yd, zd};
    double *velb[3] = {xdb, ydb, zdb};
    double G[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int m = 0; m < 4; ++m) G[i][m] = 0.0;
    double coefb = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double *u = vel[c];
        double hxx[4], hxxb[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            double h = 0.;
#pragma unroll
            for (int j = 0; j < 8; ++j) h += hg_[j][m] * u[j];
            hxx[m] = h;
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            double h = 0.;
#pragma unroll
            for (int i = 0; i < 8; ++i) h += fb[c][i] * hg_[i][m];
            hxxb[m] = coef * h;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            double t = 0.;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                t += hg_[i][m] * hxx[m];
                G[i][m] += coef * fb[c][i] * hxx[m] + hxxb[m] * u[i];
            }
            coefb += fb[c][i] * t;
            double ub = 0.;
#pragma unroll
            for (int m = 0; m < 4; ++m) ub += hxxb[m] * hg_[i][m];
            velb[c][i] += ub;
        }
    }
    // hourgam = gamma - volinv * (dvd . hm)
    double volinvb = 0.0, dvdxb[8], dvdyb[8], dvdzb[8], hmb[4][3];
#pragma unroll
    for (int m = 0; m < 4; ++m) hmb[m][0] = hmb[m][1] = hmb[m][2] = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        double a = 0., b = 0., c = 0.;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const double g = G[i][m];
            volinvb -= g * (dvdx[i] * hm[m][0] + dvdy[i] * hm[m][1] + dvdz[i] * hm[m][2]);
            a -= volinv * g * hm[m][0];
            b -= volinv * g * hm[m][1];
            c -= volinv * g * hm[m][2];
            hmb[m][0] -= volinv * g * dvdx[i];
            hmb[m][1] -= volinv * g * dvdy[i];
            hmb[m][2] -= volinv * g * dvdz[i];
        }
        dvdxb[i] = a;
        dvdyb[i] = b;
        dvdzb[i] = c;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        double a = 0., b = 0., c = 0.;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            a += hmb[m][0] * gam(m, j);
            b += hmb[m][1] * gam(m, j);
            c += hmb[m][2] * gam(m, j);
        }
        xb[j] += a;
        yb[j] += b;
        zb[j] += c;
    }
    volume_derivative_vjp(x, y, z, dvdxb, dvdyb, dvdzb, xb, yb, zb);
    // coef = -hg 0.01 ss mass vol^(-1/3); volinv = 1 / vol; vol = volo v
    o.hgb += coefb * (-0.01 * ss * mass / cr);
    o.ssb += coefb * (-hg * 0.01 * mass / cr);
    // the divisions take forward values: an adjoint dividend is 0 for most
    // elements, and a zero dividend takes division's special-operand path
    double volb = coefb * (coef * (-1.0 / 3.0) / vol);
    volb -= volinvb * volinv * volinv;
    o.vb += volb * volo;
}

// ---------------------------------------------------------------------------
// CalcMonotonicQGradientsForElems (lulesh.cc:1613-1757).  Per direction
// (zeta: a = Di x Dj, xi: a = Dj x Dk, eta: a = Dk x Di):
//   delx = vol / sqrt(|a|^2 + ptiny),  delv = norm * (a . V),
//   vol = volo vnew, norm = 1 / (vol + ptiny).
// In: node positions/velocities, volo, vnew and the adjoints of
// delx[3], delv[3] (order xi, eta, zeta).  Accumulates node adjoints and
// returns the adjoint of vnew.
// ---------------------------------------------------------------------------
LG_HD void pattern_i(const double *u, double &s) { s = 0.25 * ((u[1] + u[2] + u[6] + u[5]) - (u[0] + u[3] + u[7] + u[4])); }
LG_HD void pattern_j(const double *u, double &s) { s = -0.25 * ((u[0] + u[1] + u[5] + u[4]) - (u[3] + u[2] + u[6] + u[7])); }
LG_HD void pattern_k(const double *u, double &s) { s = 0.25 * ((u[4] + u[5] + u[6] + u[7]) - (u[0] + u[1] + u[2] + u[3])); }
LG_HD void pattern_i_vjp(double g, double *ub)
{
    ub[1] += 0.25 * g; ub[2] += 0.25 * g; ub[6] += 0.25 * g; ub[5] += 0.25 * g;
    ub[0] -= 0.25 * g; ub[3] -= 0.25 * g; ub[7] -= 0.25 * g; ub[4] -= 0.25 * g;
}
LG_HD void pattern_j_vjp(double g, double *ub)
{
    ub[0] -= 0.25 * g; ub[1] -= 0.25 * g; ub[5] -= 0.25 * g; ub[4] -= 0.25 * g;
    ub[3] += 0.25 * g; ub[2] += 0.25 * g; ub[6] += 0.25 * g; ub[7] += 0.25 * g;
}
LG_HD void pattern_k_vjp(double g, double *ub)
{
    ub[4] += 0.25 * g; ub[5] += 0.25 * g; ub[6] += 0.25 * g; ub[7] += 0.25 * g;
    ub[0] -= 0.25 * g; ub[1] -= 0.25 * g; ub[2] -= 0.25 * g; ub[3] -= 0.25 * g;
}

LG_HD V3 pat(void (*f)(const double *, double &), const double *x, const double *y,
             const double *z)
{
    V3 r;
    f(x, r.x);
    f(y, r.y);
    f(z, r.z);
    return r;
}

LG_HD double qgrad_vjp(const double *x, const double *y, const double *z, const double *xd,
                       const double *yd, const double *zd, double volo, double vnew,
                       const double delxb[3], const double delvb[3], double *xb, double *yb,
                       double *zb, double *xdb, double *ydb, double *zdb)
{
    const double ptiny = 1.e-36;
    const double vol = volo * vnew;
    const double norm = 1.0 / (vol + ptiny);
    const V3 Di = pat(pattern_i, x, y, z), Dj = pat(pattern_j, x, y, z), Dk = pat(pattern_k, x, y, z);
    const V3 Vi = pat(pattern_i, xd, yd, zd), Vj = pat(pattern_j, xd, yd, zd),
             Vk = pat(pattern_k, xd, yd, zd);
    V3 Dib = {0, 0, 0}, Djb = {0, 0, 0}, Dkb = {0, 0, 0}, Vib = {0, 0, 0}, Vjb = {0, 0, 0},
       Vkb = {0, 0, 0};
    double volb = 0.0, normb = 0.0;
    // (P, Q, V, adjoint index) for xi, eta, zeta
    const V3 *Ps[3] = {&Dj, &Dk, &Di}, *Qs[3] = {&Dk, &Di, &Dj}, *Vs[3] = {&Vi, &Vj, &Vk};
    V3 *Pb[3] = {&Djb, &Dkb, &Dib}, *Qb[3] = {&Dkb, &Dib, &Djb}, *Vb[3] = {&Vib, &Vjb, &Vkb};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const V3 a = cross(*Ps[d], *Qs[d]);
        const double s = sqrt(dot(a, a) + ptiny);
        const double gx = delxb[d], gv = delvb[d];
        const double rs = 1.0 / s;  // gx, an adjoint, is 0 for most elements
        volb += gx * rs;
        const double ka = -gx * (vol * (rs * rs * rs));
        V3 ab = {ka * a.x + gv * norm * Vs[d]->x, ka * a.y + gv * norm * Vs[d]->y,
                 ka * a.z + gv * norm * Vs[d]->z};
        normb += gv * dot(a, *Vs[d]);
        Vb[d]->x += gv * norm * a.x;
        Vb[d]->y += gv * norm * a.y;
        Vb[d]->z += gv * norm * a.z;
        const V3 pb = cross(*Qs[d], ab), qb = cross(ab, *Ps[d]);
        Pb[d]->x += pb.x; Pb[d]->y += pb.y; Pb[d]->z += pb.z;
        Qb[d]->x += qb.x; Qb[d]->y += qb.y; Qb[d]->z += qb.z;
    }
    pattern_i_vjp(Dib.x, xb); pattern_i_vjp(Dib.y, yb); pattern_i_vjp(Dib.z, zb);
    pattern_j_vjp(Djb.x, xb); pattern_j_vjp(Djb.y, yb); pattern_j_vjp(Djb.z, zb);
    pattern_k_vjp(Dkb.x, xb); pattern_k_vjp(Dkb.y, yb); pattern_k_vjp(Dkb.z, zb);
    pattern_i_vjp(Vib.x, xdb); pattern_i_vjp(Vib.y, ydb); pattern_i_vjp(Vib.z, zdb);
    pattern_j_vjp(Vjb.x, xdb); pattern_j_vjp(Vjb.y, ydb); pattern_j_vjp(Vjb.z, zdb);
    pattern_k_vjp(Vkb.x, xdb); pattern_k_vjp(Vkb.y, ydb); pattern_k_vjp(Vkb.z, zdb);
    volb -= normb * norm * norm;
    return volb * volo;  // adjoint of vnew
}

// ---------------------------------------------------------------------------
// One direction of the monotonic limiter (lulesh.cc:1778-1813).  kind_m /
// kind_p: 0 neighbour value, 1 own value (symmetry), 2 zero (free).
// Forward phi; reverse from phib: adjoint of the own value (selfb) and of the
// neighbour values (nbmb, nbpb).
// ---------------------------------------------------------------------------
struct PhiFwd {
    double phi, norm, m, p;
    int branch;  // 0 average, 1 2m, 2 2p, 3 zero, 4 max slope
};

LG_HD PhiFwd phi_forward(double self, double src_m, double src_p, double lim, double maxs)
{
    const double ptiny = 1.e-36;
    PhiFwd f;
    f.norm = 1. / (self + ptiny);
    f.m = src_m * f.norm;
    f.p = src_p * f.norm;
    double phi = .5 * (f.m + f.p);
    int br = 0;
    const double m2 = f.m * lim, p2 = f.p * lim;
    if (m2 < phi) { phi = m2; br = 1; }
    if (p2 < phi) { phi = p2; br = 2; }
    if (phi < 0.) { phi = 0.; br = 3; }
    if (phi > maxs) { phi = maxs; br = 4; }
    f.phi = phi;
    f.branch = br;
    return f;
}

LG_HD void phi_vjp(const PhiFwd &f, double src_m, double src_p, double lim, double phib,
                   double &selfb, double &srcmb, double &srcpb)
{
    double mb = 0., pb = 0.;
    if (f.branch == 0) { mb = .5 * phib; pb = .5 * phib; }
    else if (f.branch == 1) mb = lim * phib;
    else if (f.branch == 2) pb = lim * phib;
    srcmb = mb * f.norm;
    srcpb = pb * f.norm;
    const double normb = mb * src_m + pb * src_p;
    selfb -= normb * f.norm * f.norm;
}

// qlin / qquad of CalcMonotonicQRegionForElems (lulesh.cc:1892-1916) for an
// element with vdov <= 0.  In: delv[3], delx[3], phi[3], rho; adjoints of
// qlin, qquad.  Out: adjoints of delv, delx, phi, rho.
LG_HD void qlq_vjp(const double delv[3], const double delx[3], const double phi[3], double rho,
                   double qlc, double qqc, double qlb, double qqb, double delvb[3],
                   double delxb[3], double phib[3], double &rhob)
{
    double dx[3];
    bool clip[3];
    double S1 = 0., S2 = 0.;
    for (int d = 0; d < 3; ++d) {
        dx[d] = delv[d] * delx[d];
        clip[d] = dx[d] > 0.;
        if (clip[d]) dx[d] = 0.;
        S1 += dx[d] * (1. - phi[d]);
        S2 += dx[d] * dx[d] * (1. - phi[d] * phi[d]);
    }
    rhob = qlb * (-qlc) * S1 + qqb * qqc * S2;
    for (int d = 0; d < 3; ++d) {
        const double dxb = qlb * (-qlc * rho) * (1. - phi[d]) +
                           qqb * (qqc * rho) * 2. * dx[d] * (1. - phi[d] * phi[d]);
        phib[d] = qlb * (-qlc * rho) * (-dx[d]) + qqb * (qqc * rho) * dx[d] * dx[d] * (-2. * phi[d]);
        delvb[d] = clip[d] ? 0. : dxb * delx[d];
        delxb[d] = clip[d] ? 0. : dxb * delv[d];
    }
}

// ---------------------------------------------------------------------------
// EOS of one element, one repetition (EvalEOSForElems / CalcEnergyForElems /
// CalcPressureForElems / CalcSoundSpeedForElems, lulesh.cc:2014-2324; the
// repetitions recompute identical values, so one pass is the function).
// ---------------------------------------------------------------------------
struct EosConst {
    double e_cut, p_cut, q_cut, eosvmin, eosvmax, pmin, emin, rho0;
};

struct EosFwd {
    double comp, chs, vhalf, bvcH, e1, pH, sscH, qn1, e2, e3, bvc, pn1, sscT, qt, e4, pn2, sscF,
        qn2, ss;
    bool vmin, vmax, e1clamp, pHkeep, sscHsqrt, e3keep, pn1keep, sscTsqrt, e4keep, pn2keep,
        sscFsqrt, qn2keep, sssqrt, comp_gt;
};

// Keeps the compiler from moving the computation of v out of the branch it
// sits in (on the device; nothing on the host).  A hoisted square root or
// division runs for every element, and an element at rest gives it the
// operands of the special-operand path (a zero numerator).
LG_HD void adj_fence(double &v)
{
#ifdef __CUDA_ARCH__
    asm volatile("" : "+d"(v));
#else
    (void)v;
#endif
}

// The sound-speed term; kUnitRho (refdens == 1, decided once by the caller)
// skips x / 1.0, which is x.
template <bool kUnitRho>
LG_HD double ssc_val(double num, double rho0, bool &took_sqrt)
{
    double ssc = kUnitRho ? num : num / rho0;
    took_sqrt = !(ssc <= .1111111e-36);
    if (!took_sqrt) return .3333333e-18;
    adj_fence(ssc);
    return sqrt(ssc);
}

// pressure with its cut-off and clamps; keep = the derivative passes (the
// p_cut noise cut-off keeps it, the eosvmax and pmin clamps do not)
LG_HD double p_eval(const EosConst &K, double bvc, double e, double vc, bool &keep)
{
    double p = bvc * e;
    keep = true;
    if (fabs(p) < K.p_cut) p = 0.0;
    if (vc >= K.eosvmax) { p = 0.0; keep = false; }
    if (p < K.pmin) { p = K.pmin; keep = false; }
    return p;
}

template <bool kUnitRho>
LG_HD EosFwd eos_forward_rho(const EosConst &K, double e_old, double delvc, double p_old,
                             double q_old, double qq, double ql, double vc)
{
    EosFwd f;
    const double c1s = 2.0 / 3.0, sixth = 1.0 / 6.0;
    f.comp = 1. / vc - 1.;
    const double vchalf = vc - delvc * .5;
    f.chs = 1. / vchalf - 1.;
    f.vmin = (K.eosvmin != 0. && vc <= K.eosvmin);
    if (f.vmin) f.chs = f.comp;
    f.vmax = (K.eosvmax != 0. && vc >= K.eosvmax);
    if (f.vmax) { p_old = 0.; f.comp = 0.; f.chs = 0.; }
    f.e1 = e_old - .5 * delvc * (p_old + q_old);
    f.e1clamp = f.e1 < K.emin;
    if (f.e1clamp) f.e1 = K.emin;
    f.bvcH = c1s * (f.chs + 1.);
    f.pH = p_eval(K, f.bvcH, f.e1, vc, f.pHkeep);
    f.vhalf = 1. / (1. + f.chs);
    f.comp_gt = delvc > 0.;
    if (f.comp_gt) {
        f.qn1 = 0.;
        f.sscH = 0.;
        f.sscHsqrt = false;
    } else {
        f.sscH = ssc_val<kUnitRho>(c1s * f.e1 + f.vhalf * f.vhalf * f.bvcH * f.pH, K.rho0, f.sscHsqrt);
        f.qn1 = f.sscH * ql + qq;
    }
    f.e2 = f.e1 + .5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (f.pH + f.qn1));
    f.e3 = f.e2;
    f.e3keep = true;
    if (fabs(f.e3) < K.e_cut) f.e3 = 0.;
    if (f.e3 < K.emin) { f.e3 = K.emin; f.e3keep = false; }
    f.bvc = c1s * (f.comp + 1.);
    f.pn1 = p_eval(K, f.bvc, f.e3, vc, f.pn1keep);
    if (f.comp_gt) {
        f.qt = 0.;
        f.sscT = 0.;
        f.sscTsqrt = false;
    } else {
        f.sscT = ssc_val<kUnitRho>(c1s * f.e3 + vc * vc * f.bvc * f.pn1, K.rho0, f.sscTsqrt);
        f.qt = f.sscT * ql + qq;
    }
    f.e4 = f.e3 - (7.0 * (p_old + q_old) - 8.0 * (f.pH + f.qn1) + (f.pn1 + f.qt)) * delvc * sixth;
    f.e4keep = true;
    if (fabs(f.e4) < K.e_cut) f.e4 = 0.;
    if (f.e4 < K.emin) { f.e4 = K.emin; f.e4keep = false; }
    f.pn2 = p_eval(K, f.bvc, f.e4, vc, f.pn2keep);
    f.qn2 = f.qn1;
    f.qn2keep = false;
    f.sscF = 0.;
    f.sscFsqrt = false;
    if (!f.comp_gt) {
        f.sscF = ssc_val<kUnitRho>(c1s * f.e4 + vc * vc * f.bvc * f.pn2, K.rho0, f.sscFsqrt);
        f.qn2 = f.sscF * ql + qq;
        f.qn2keep = true;
        if (fabs(f.qn2) < K.q_cut) f.qn2 = 0.;
    }
    f.ss = ssc_val<kUnitRho>(c1s * f.e4 + vc * vc * f.bvc * f.pn2, K.rho0, f.sssqrt);
    return f;
}

LG_HD EosFwd eos_forward(const EosConst &K, double e_old, double delvc, double p_old,
                         double q_old, double qq, double ql, double vc)
{
    if (K.rho0 == 1.0) return eos_forward_rho<true>(K, e_old, delvc, p_old, q_old, qq, ql, vc);
    return eos_forward_rho<false>(K, e_old, delvc, p_old, q_old, qq, ql, vc);
}

struct EosAdj {
    double e_oldb, delvcb, p_oldb, q_oldb, qqb, qlb, vcb;
};

// From the adjoints of (p_new = pn2, e_new = e4, q_new, ss).
LG_HD EosAdj eos_vjp(const EosConst &K, const EosFwd &f, double e_old, double delvc,
                     double p_old_in, double q_old, double qq, double ql, double vc, double pb,
                     double eb, double qb, double ssb)
{
    (void)e_old;
    (void)qq;
    const double c1s = 2.0 / 3.0, sixth = 1.0 / 6.0, r0 = K.rho0;
    const double p_old = f.vmax ? 0. : p_old_in;
    EosAdj a = {0, 0, 0, 0, 0, 0, 0};
    double e4b = eb, pn2b = pb, bvcb = 0.;
    // ss = sqrt((c1s e4 + vc^2 bvc pn2) / rho0)
    if (f.sssqrt) {
        const double nb = ssb * (1.0 / (2. * f.ss * r0));
        e4b += nb * c1s;
        a.vcb += nb * 2. * vc * f.bvc * f.pn2;
        bvcb += nb * vc * vc * f.pn2;
        pn2b += nb * vc * vc * f.bvc;
    }
    // q_new
    if (!f.comp_gt && f.qn2keep) {
        const double sb = qb * ql;
        a.qlb += qb * f.sscF;
        a.qqb += qb;
        if (f.sscFsqrt) {
            const double nb = sb * (1.0 / (2. * f.sscF * r0));
            e4b += nb * c1s;
            a.vcb += nb * 2. * vc * f.bvc * f.pn2;
            bvcb += nb * vc * vc * f.pn2;
            pn2b += nb * vc * vc * f.bvc;
        }
    }
    double qn1b = 0.;  // q_new = qn1 when delvc > 0 (then qn1 = 0: no flow)
    // pn2 = bvc e4
    if (f.pn2keep) {
        bvcb += pn2b * f.e4;
        e4b += pn2b * f.bvc;
    }
    // e4 = e3 - W delvc / 6
    double e3b = 0., pHb = 0., pn1b = 0., qtb = 0.;
    if (f.e4keep) {
        const double W = 7.0 * (p_old + q_old) - 8.0 * (f.pH + f.qn1) + (f.pn1 + f.qt);
        e3b += e4b;
        const double Wb = -e4b * delvc * sixth;
        a.delvcb += -e4b * W * sixth;
        a.p_oldb += 7. * Wb;
        a.q_oldb += 7. * Wb;
        pHb += -8. * Wb;
        qn1b += -8. * Wb;
        pn1b += Wb;
        qtb += Wb;
    }
    // qt = sscT ql + qq
    if (!f.comp_gt) {
        a.qlb += qtb * f.sscT;
        a.qqb += qtb;
        if (f.sscTsqrt) {
            const double nb = qtb * ql * (1.0 / (2. * f.sscT * r0));
            e3b += nb * c1s;
            a.vcb += nb * 2. * vc * f.bvc * f.pn1;
            bvcb += nb * vc * vc * f.pn1;
            pn1b += nb * vc * vc * f.bvc;
        }
    }
    if (f.pn1keep) {
        bvcb += pn1b * f.e3;
        e3b += pn1b * f.bvc;
    }
    // e3 = e2 (cut-offs)
    const double e2b = f.e3keep ? e3b : 0.;
    // e2 = e1 + 0.5 delvc (3 (p_old + q_old) - 4 (pH + qn1))
    double e1b = e2b, bvcHb = 0., vhalfb = 0.;
    {
        const double G = .5 * delvc * e2b;
        a.delvcb += e2b * .5 * (3.0 * (p_old + q_old) - 4.0 * (f.pH + f.qn1));
        a.p_oldb += 3. * G;
        a.q_oldb += 3. * G;
        pHb += -4. * G;
        qn1b += -4. * G;
    }
    // qn1 = sscH ql + qq
    if (!f.comp_gt) {
        a.qlb += qn1b * f.sscH;
        a.qqb += qn1b;
        if (f.sscHsqrt) {
            const double nb = qn1b * ql * (1.0 / (2. * f.sscH * r0));
            e1b += nb * c1s;
            vhalfb += nb * 2. * f.vhalf * f.bvcH * f.pH;
            bvcHb += nb * f.vhalf * f.vhalf * f.pH;
            pHb += nb * f.vhalf * f.vhalf * f.bvcH;
        }
    }
    double chsb = -vhalfb * f.vhalf * f.vhalf;
    if (f.pHkeep) {
        bvcHb += pHb * f.e1;
        e1b += pHb * f.bvcH;
    }
    chsb += bvcHb * c1s;
    // e1 = e_old - 0.5 delvc (p_old + q_old)
    if (!f.e1clamp) {
        a.e_oldb += e1b;
        a.delvcb += -.5 * e1b * (p_old + q_old);
        a.p_oldb += -.5 * delvc * e1b;
        a.q_oldb += -.5 * delvc * e1b;
    }
    double compb = bvcb * c1s;
    if (f.vmax) {
        a.p_oldb = 0.;  // p_old, compression, compHalfStep were set to zero
        compb = 0.;
        chsb = 0.;
    }
    if (f.vmin) {
        compb += chsb;  // compHalfStep = compression
        chsb = 0.;
    }
    // chs = 1 / (vc - 0.5 delvc) - 1; comp = 1 / vc - 1.  By reciprocals:
    // at rest chsb and compb are 0, and a zero dividend would send a division
    // down its special-operand path.
    const double vchalf = vc - delvc * .5;
    const double vchb = -chsb * (1.0 / (vchalf * vchalf));
    a.vcb += vchb;
    a.delvcb += -.5 * vchb;
    a.vcb += -compb * (1.0 / (vc * vc));
    return a;
}

}  // namespace adj
}  // namespace lg
