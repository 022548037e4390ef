// adjoint_selftest.cc -- host check of the element-local vector-Jacobian
// products in lulesh_gb300/csrc/lg_adjoint_math.h against central finite
// differences of the forward formulas (compiled and run by
// tests/test_adjoint_math.py).  For random inputs x, output weights w and
// directions d it compares <VJP(w), d> with (w.f(x+hd) - w.f(x-hd)) / 2h and
// prints one line per function: name, worst relative error.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "lg_adjoint_math.h"

using namespace lg;

static std::mt19937_64 rng(7);
static double U(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

struct Elem {
    double x[8], y[8], z[8], xd[8], yd[8], zd[8];
};

static Elem random_elem()
{
    static const double cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                        cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    Elem e;
    const double h = 0.02;
    for (int j = 0; j < 8; ++j) {
        e.x[j] = 0.3 + h * cx[j] + U(-0.15, 0.15) * h;
        e.y[j] = 0.2 + h * cy[j] + U(-0.15, 0.15) * h;
        e.z[j] = 0.1 + h * cz[j] + U(-0.15, 0.15) * h;
        e.xd[j] = U(-1, 1);
        e.yd[j] = U(-1, 1);
        e.zd[j] = U(-1, 1);
    }
    return e;
}

static double worst = 0.0;
static double check(const char *name, double ad, double fd)
{
    const double err = std::fabs(ad - fd) / std::max(std::fabs(fd), 1e-12 + 1e-6 * std::fabs(ad));
    printf("  %-14s adjoint % .12e  fd % .12e  rel %.2e\n", name, ad, fd, err);
    return err;
}

// forces of one element (the forward kernel's formulas)
static void forces_fwd(const Elem &e, double p, double q, double v, double volo, double ss,
                       double mass, double hg, double f[3][8])
{
    const double sig = -p - q;
    double pfx[8], pfy[8], pfz[8];
    geom::node_normals(pfx, pfy, pfz, e.x, e.y, e.z);
    for (int j = 0; j < 8; ++j) {
        f[0][j] = -(sig * pfx[j]);
        f[1][j] = -(sig * pfy[j]);
        f[2][j] = -(sig * pfz[j]);
    }
    double dvdx[8], dvdy[8], dvdz[8];
    geom::volume_derivative(e.x, e.y, e.z, dvdx, dvdy, dvdz);
    const double determ = volo * v, volinv = 1.0 / determ;
    double hourgam[8][4];
    for (int i1 = 0; i1 < 4; ++i1) {
        double hx = 0, hy = 0, hz = 0;
        for (int j = 0; j < 8; ++j) {
            hx += e.x[j] * geom::gam(i1, j);
            hy += e.y[j] * geom::gam(i1, j);
            hz += e.z[j] * geom::gam(i1, j);
        }
        for (int k = 0; k < 8; ++k)
            hourgam[k][i1] = geom::gam(i1, k) - volinv * (dvdx[k] * hx + dvdy[k] * hy + dvdz[k] * hz);
    }
    const double coef = -hg * 0.01 * ss * mass / cbrt(determ);
    const double *vel[3] = {e.xd, e.yd, e.zd};
    for (int c = 0; c < 3; ++c) {
        double hxx[4];
        for (int i = 0; i < 4; ++i) {
            hxx[i] = 0;
            for (int j = 0; j < 8; ++j) hxx[i] += hourgam[j][i] * vel[c][j];
        }
        for (int i = 0; i < 8; ++i)
            f[c][i] += coef * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                               hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
    }
}

static void qgrad_fwd(const Elem &e, double volo, double vnew, double delx[3], double delv[3])
{
    using adj::V3;
    const double ptiny = 1.e-36, vol = volo * vnew, norm = 1.0 / (vol + ptiny);
    const V3 Di = adj::pat(adj::pattern_i, e.x, e.y, e.z), Dj = adj::pat(adj::pattern_j, e.x, e.y, e.z),
             Dk = adj::pat(adj::pattern_k, e.x, e.y, e.z);
    const V3 Vi = adj::pat(adj::pattern_i, e.xd, e.yd, e.zd),
             Vj = adj::pat(adj::pattern_j, e.xd, e.yd, e.zd),
             Vk = adj::pat(adj::pattern_k, e.xd, e.yd, e.zd);
    const V3 P[3] = {Dj, Dk, Di}, Q[3] = {Dk, Di, Dj}, V[3] = {Vi, Vj, Vk};
    for (int d = 0; d < 3; ++d) {
        const V3 a = adj::cross(P[d], Q[d]);
        delx[d] = vol / sqrt(adj::dot(a, a) + ptiny);
        delv[d] = norm * adj::dot(a, V[d]);
    }
}

int main()
{
    double worst_all = 0.0;
    for (int trial = 0; trial < 6; ++trial) {
        printf("trial %d\n", trial);
        const Elem e = random_elem();
        std::vector<double> d(48);
        for (auto &v : d) v = U(-1, 1);
        auto perturbed = [&](double h) {
            Elem p = e;
            for (int j = 0; j < 8; ++j) {
                p.x[j] += h * d[j];
                p.y[j] += h * d[8 + j];
                p.z[j] += h * d[16 + j];
                p.xd[j] += h * d[24 + j];
                p.yd[j] += h * d[32 + j];
                p.zd[j] += h * d[40 + j];
            }
            return p;
        };
        // node normals
        {
            double w[3][8];
            for (auto &r : w) for (auto &v : r) v = U(-1, 1);
            double xb[8] = {0}, yb[8] = {0}, zb[8] = {0};
            adj::node_normals_vjp(e.x, e.y, e.z, w[0], w[1], w[2], xb, yb, zb);
            double ad = 0;
            for (int j = 0; j < 8; ++j) ad += xb[j] * d[j] + yb[j] * d[8 + j] + zb[j] * d[16 + j];
            const double h = 1e-7;
            auto F = [&](const Elem &p) {
                double a[8], b[8], c[8];
                geom::node_normals(a, b, c, p.x, p.y, p.z);
                double s = 0;
                for (int j = 0; j < 8; ++j) s += w[0][j] * a[j] + w[1][j] * b[j] + w[2][j] * c[j];
                return s;
            };
            worst_all = std::max(worst_all, check("node_normals", ad, (F(perturbed(h)) - F(perturbed(-h))) / (2 * h)));
        }
        // volume derivative, and volume gradient == volume derivative
        {
            double w[3][8];
            for (auto &r : w) for (auto &v : r) v = U(-1, 1);
            double xb[8] = {0}, yb[8] = {0}, zb[8] = {0};
            adj::volume_derivative_vjp(e.x, e.y, e.z, w[0], w[1], w[2], xb, yb, zb);
            double ad = 0;
            for (int j = 0; j < 8; ++j) ad += xb[j] * d[j] + yb[j] * d[8 + j] + zb[j] * d[16 + j];
            const double h = 1e-7;
            auto F = [&](const Elem &p) {
                double a[8], b[8], c[8];
                geom::volume_derivative(p.x, p.y, p.z, a, b, c);
                double s = 0;
                for (int j = 0; j < 8; ++j) s += w[0][j] * a[j] + w[1][j] * b[j] + w[2][j] * c[j];
                return s;
            };
            worst_all = std::max(worst_all, check("volume_deriv", ad, (F(perturbed(h)) - F(perturbed(-h))) / (2 * h)));
            double dx[8], dy[8], dz[8];
            geom::volume_derivative(e.x, e.y, e.z, dx, dy, dz);
            double g = 0;
            for (int j = 0; j < 8; ++j) g += dx[j] * d[j] + dy[j] * d[8 + j] + dz[j] * d[16 + j];
            const Elem a = perturbed(1e-6), b = perturbed(-1e-6);
            worst_all = std::max(worst_all, check("volume_grad", g,
                (geom::elem_volume(a.x, a.y, a.z) - geom::elem_volume(b.x, b.y, b.z)) / 2e-6));
        }
        // element forces (positions, velocities and the scalars)
        {
            const double p = U(1e3, 1e5), q = U(0, 1e4), v = U(0.8, 1.2), volo = 8e-6,
                         ss = U(10, 300), mass = 8e-6, hg = U(1, 3);
            double w[3][8];
            for (auto &r : w) for (auto &vv : r) vv = U(-1, 1);
            double xb[8] = {0}, yb[8] = {0}, zb[8] = {0}, xdb[8] = {0}, ydb[8] = {0}, zdb[8] = {0};
            adj::ForceAdj o = {0, 0, 0, 0, 0};
            adj::forces_vjp(e.x, e.y, e.z, e.xd, e.yd, e.zd, p, q, v, volo, ss, mass, hg, w, xb,
                            yb, zb, xdb, ydb, zdb, o);
            const double sp = U(-1, 1), sq = U(-1, 1), sv = U(-1, 1), sss = U(-1, 1), shg = U(-1, 1);
            double ad = o.pb * sp * p + o.qb * sq * q + o.vb * sv * v + o.ssb * sss * ss + o.hgb * shg * hg;
            for (int j = 0; j < 8; ++j)
                ad += xb[j] * d[j] + yb[j] * d[8 + j] + zb[j] * d[16 + j] + xdb[j] * d[24 + j] +
                      ydb[j] * d[32 + j] + zdb[j] * d[40 + j];
            auto F = [&](double h) {
                const Elem el = perturbed(h);
                double f[3][8];
                forces_fwd(el, p * (1 + h * sp), q * (1 + h * sq), v * (1 + h * sv), volo,
                           ss * (1 + h * sss), mass, hg * (1 + h * shg), f);
                double s = 0;
                for (int c = 0; c < 3; ++c) for (int j = 0; j < 8; ++j) s += w[c][j] * f[c][j];
                return s;
            };
            const double h = 1e-7;
            worst_all = std::max(worst_all, check("forces", ad, (F(h) - F(-h)) / (2 * h)));
        }
        // monotonic-Q gradients
        {
            const double volo = 8e-6, vnew = U(0.8, 1.2);
            double wx[3], wv[3];
            for (int i = 0; i < 3; ++i) { wx[i] = U(-1, 1) * 1e2; wv[i] = U(-1, 1); }
            double xb[8] = {0}, yb[8] = {0}, zb[8] = {0}, xdb[8] = {0}, ydb[8] = {0}, zdb[8] = {0};
            const double vnb = adj::qgrad_vjp(e.x, e.y, e.z, e.xd, e.yd, e.zd, volo, vnew, wx, wv, xb, yb, zb, xdb, ydb, zdb);
            const double sv = U(-1, 1);
            double ad = vnb * sv * vnew;
            for (int j = 0; j < 8; ++j)
                ad += xb[j] * d[j] + yb[j] * d[8 + j] + zb[j] * d[16 + j] + xdb[j] * d[24 + j] +
                      ydb[j] * d[32 + j] + zdb[j] * d[40 + j];
            auto F = [&](double h) {
                double dx[3], dv[3];
                qgrad_fwd(perturbed(h), volo, vnew * (1 + h * sv), dx, dv);
                double s = 0;
                for (int i = 0; i < 3; ++i) s += wx[i] * dx[i] + wv[i] * dv[i];
                return s;
            };
            const double h = 1e-7;
            worst_all = std::max(worst_all, check("qgrad", ad, (F(h) - F(-h)) / (2 * h)));
        }
        // limiter + qlin/qquad, all branches through random inputs
        for (int rep = 0; rep < 4; ++rep) {
            const double lim = 2.0, maxs = 1.0, qlc = 0.5, qqc = 2.0 / 3.0;
            double self[3], sm[3], sp[3], delx[3];
            for (int i = 0; i < 3; ++i) {
                self[i] = -U(0.5, 2.0);
                sm[i] = self[i] * U(0.2, 1.8);
                sp[i] = self[i] * U(0.2, 1.8);
                delx[i] = U(0.01, 0.03);
            }
            const double rho = U(0.5, 3), wl = U(-1, 1), wq = U(-1, 1);
            auto Fq = [&](const double *se, const double *m_, const double *p_, const double *dx_,
                          double r) {
                double phi[3];
                for (int i = 0; i < 3; ++i) phi[i] = adj::phi_forward(se[i], m_[i], p_[i], lim, maxs).phi;
                double s1 = 0, s2 = 0;
                for (int i = 0; i < 3; ++i) {
                    double dxv = se[i] * dx_[i];
                    if (dxv > 0.) dxv = 0.;
                    s1 += dxv * (1. - phi[i]);
                    s2 += dxv * dxv * (1. - phi[i] * phi[i]);
                }
                return wl * (-qlc * r * s1) + wq * (qqc * r * s2);
            };
            double phi[3], delvb[3], delxb[3], phib[3], rhob;
            adj::PhiFwd pf[3];
            for (int i = 0; i < 3; ++i) { pf[i] = adj::phi_forward(self[i], sm[i], sp[i], lim, maxs); phi[i] = pf[i].phi; }
            adj::qlq_vjp(self, delx, phi, rho, qlc, qqc, wl, wq, delvb, delxb, phib, rhob);
            double selfb[3], smb[3], spb[3];
            for (int i = 0; i < 3; ++i) {
                selfb[i] = delvb[i];
                adj::phi_vjp(pf[i], sm[i], sp[i], lim, phib[i], selfb[i], smb[i], spb[i]);
            }
            double ds[3], dm[3], dp[3], dx[3];
            for (int i = 0; i < 3; ++i) { ds[i] = U(-1, 1); dm[i] = U(-1, 1); dp[i] = U(-1, 1); dx[i] = U(-1, 1); }
            const double dr = U(-1, 1);
            double ad = rhob * dr;
            for (int i = 0; i < 3; ++i) ad += selfb[i] * ds[i] + smb[i] * dm[i] + spb[i] * dp[i] + delxb[i] * dx[i];
            auto F = [&](double h) {
                double se[3], m_[3], p_[3], dx_[3];
                for (int i = 0; i < 3; ++i) { se[i] = self[i] + h * ds[i]; m_[i] = sm[i] + h * dm[i]; p_[i] = sp[i] + h * dp[i]; dx_[i] = delx[i] + h * dx[i]; }
                return Fq(se, m_, p_, dx_, rho + h * dr);
            };
            const double h = 1e-7;
            worst_all = std::max(worst_all, check("qlimiter", ad, (F(h) - F(-h)) / (2 * h)));
        }
        // EOS, compression and expansion
        for (int sgn = 0; sgn < 2; ++sgn) {
            adj::EosConst K = {1e-7, 1e-7, 1e-7, 1e-9, 1e9, 0., -1e15, 1.};
            const double e_old = U(1e3, 1e5), delvc = (sgn ? 1 : -1) * U(1e-4, 1e-2),
                         p_old = U(1e2, 1e4), q_old = U(0, 1e3), qq = U(0, 1e2), ql = U(0, 1e-1),
                         vc = U(0.7, 1.3);
            const adj::EosFwd f = adj::eos_forward(K, e_old, delvc, p_old, q_old, qq, ql, vc);
            const double wp = U(-1, 1), we = U(-1, 1), wq = U(-1, 1), ws = U(-1, 1) * 1e2;
            const adj::EosAdj a = adj::eos_vjp(K, f, e_old, delvc, p_old, q_old, qq, ql, vc, wp, we, wq, ws);
            double dd[7];
            for (auto &v : dd) v = U(-1, 1);
            const double sc[7] = {e_old, 1e-3, p_old, q_old, qq, ql, vc};
            const double ad = a.e_oldb * dd[0] * sc[0] + a.delvcb * dd[1] * sc[1] + a.p_oldb * dd[2] * sc[2] +
                              a.q_oldb * dd[3] * sc[3] + a.qqb * dd[4] * sc[4] + a.qlb * dd[5] * sc[5] +
                              a.vcb * dd[6] * sc[6];
            auto F = [&](double h) {
                const adj::EosFwd g = adj::eos_forward(K, e_old + h * dd[0] * sc[0], delvc + h * dd[1] * sc[1],
                                                        p_old + h * dd[2] * sc[2], q_old + h * dd[3] * sc[3],
                                                        qq + h * dd[4] * sc[4], ql + h * dd[5] * sc[5],
                                                        vc + h * dd[6] * sc[6]);
                return wp * g.pn2 + we * g.e4 + wq * g.qn2 + ws * g.ss;
            };
            const double h = 1e-7;
            worst_all = std::max(worst_all, check(sgn ? "eos_expand" : "eos_compress", ad, (F(h) - F(-h)) / (2 * h)));
        }
    }
    printf("WORST %.3e\n", worst_all);
    return worst_all < 1e-6 ? 0 : 1;
}
