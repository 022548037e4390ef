// geometry_selftest.cc -- the element geometry of lg_geometry.cuh, compiled
// for the host without contraction, against the oracle's functions
// (geometry_ref_shim.c) on random hexahedra.  Where lg_geometry.cuh applies
// the reference's power-of-two factors once (face areas, Jacobian, the
// half-step B matrix and the monotonic-Q gradients), the results must be
// the same bits.  Prints the number of mismatches; exits 1 if any.
//
// geometry_selftest N plant: the oracle's values of the reassociated forms
// are scaled by 1 + 1e-8 before the comparison, and every form's check must
// then report elements beyond its tolerance (the tolerances are tight enough
// to see an error of that size).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <string>

#include "lg_geometry.cuh"
#include "lulesh_oracle.h"

extern "C" {
void geo_ref_shape(const double *x, const double *y, const double *z, double *b24, double *det);
void geo_ref_normals(const double *x, const double *y, const double *z, double *pfx, double *pfy,
                     double *pfz);
void geo_ref_volume_derivative(const double *x, const double *y, const double *z, double *dvdx,
                               double *dvdy, double *dvdz);
double geo_ref_volume(const double *x, const double *y, const double *z);
double geo_ref_char_length(const double *x, const double *y, const double *z, double volume);
void geo_ref_monoq_gradients(orc_domain *d);
}

using namespace lg::geom;

static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }

static long g_bad = 0;
static void check(const char *what, double want, double got)
{
    if (!same(want, got)) {
        if (g_bad < 10) std::printf("mismatch %s: %.17g vs %.17g\n", what, want, got);
        ++g_bad;
    }
}

// one half of the kinematics' velocity-gradient trace: inv_detJ * (B . dv)
static double grad(double inv, const double *b, const double *v)
{
    return inv * (b[0] * (v[0] - v[6]) + b[1] * (v[1] - v[7]) + b[2] * (v[2] - v[4]) +
                  b[3] * (v[3] - v[5]));
}

// reassociated forms: |want - got| <= tol, want being the oracle's value
// (scaled by 1 + g_plant in plant mode)
static long g_far = 0;
static double g_plant = 0.0;
static std::map<std::string, long> g_far_by;
static void near(const char *what, double want, double got, double tol)
{
    want *= 1.0 + g_plant;
    long &far = g_far_by[what];
    if (!(std::fabs(want - got) <= tol)) {
        if (g_far < 10 && g_plant == 0.0)
            std::printf("beyond tolerance %s: %.17g vs %.17g (tol %.3g)\n", what, want, got, tol);
        ++g_far;
        ++far;
    }
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 200000;
    if (argc > 2 && std::strcmp(argv[2], "plant") == 0) g_plant = 1e-8;
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0), sc(1e-4, 10.0);
    const double cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                 cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    for (long it = 0; it < n; ++it) {
        const double h = sc(g), jit = (it % 3 == 0) ? 0.4 : (it % 3 == 1 ? 1e-3 : 0.0);
        const double o[3] = {10 * u(g), 10 * u(g), 10 * u(g)};
        double x[8], y[8], z[8], xv[8], yv[8], zv[8];
        for (int j = 0; j < 8; ++j) {
            x[j] = o[0] + h * (cx[j] + jit * u(g));
            y[j] = o[1] + h * (cy[j] + jit * u(g));
            z[j] = o[2] + h * (cz[j] + jit * u(g));
            xv[j] = u(g);
            yv[j] = u(g);
            zv[j] = u(g);
        }
        double b[24], det;
        geo_ref_shape(x, y, z, b, &det);
        check("jacobian_det", det, jacobian_det(x, y, z));
        double bx[4], by[4], bz[4];
        const double inv = 1.0 / det, inv64 = 1.0 / shape_derivs_x64(x, y, z, bx, by, bz);
        check("dxx", grad(inv, b, xv), grad(inv64, bx, xv));
        check("dyy", grad(inv, b + 8, yv), grad(inv64, by, yv));
        check("dzz", grad(inv, b + 16, zv), grad(inv64, bz, zv));
        double rx[8], ry[8], rz[8], px[8], py[8], pz[8];
        geo_ref_normals(x, y, z, rx, ry, rz);
        node_normals(px, py, pz, x, y, z);
        for (int j = 0; j < 8; ++j) {
            check("normal x", rx[j], px[j]);
            check("normal y", ry[j], py[j]);
            check("normal z", rz[j], pz[j]);
        }
        geo_ref_volume_derivative(x, y, z, rx, ry, rz);
        volume_derivative(x, y, z, px, py, pz);
        for (int j = 0; j < 8; ++j) {
            check("dvdx", rx[j], px[j]);
            check("dvdy", ry[j], py[j]);
            check("dvdz", rz[j], pz[j]);
        }
        const double vol = geo_ref_volume(x, y, z);
        check("volume", vol, elem_volume(x, y, z));
        check("char_length", geo_ref_char_length(x, y, z, vol), char_length(x, y, z, vol));

        // the FMA build's reassociated forms: equal in exact arithmetic,
        // within the reference expressions' own rounding (their bisectors
        // sum coordinates of magnitude |o| + h before differencing)
        geo_ref_normals(x, y, z, rx, ry, rz);
        node_normals_x8(px, py, pz, x, y, z);
        const double omax = std::fabs(o[0]) + std::fabs(o[1]) + std::fabs(o[2]) + 2 * h;
        const double tol_n = 64 * 2.220446049250313e-16 * omax * h * 3;
        for (int j = 0; j < 8; ++j) {
            near("normal x from diagonals", rx[j], 0.125 * px[j], tol_n);
            near("normal y from diagonals", ry[j], 0.125 * py[j], tol_n);
            near("normal z from diagonals", rz[j], 0.125 * pz[j], tol_n);
        }
        const double cl = geo_ref_char_length(x, y, z, vol);
        near("char_length from diagonals", cl, char_length<double, true>(x, y, z, vol),
             1e-12 * std::fabs(cl));

        // the normals from the twelve differences are node_normals_x8's
        // operations; the volume gradient from them is the reference's
        // CalcElemVolumeDerivative within its rounding
        {
            double dX[12], dY[12], dZ[12], qx[8], qy[8], qz[8];
            elem_differences(x, dX);
            elem_differences(y, dY);
            elem_differences(z, dZ);
            node_normals_x8(px, py, pz, x, y, z);
            node_normals_x8_diff(qx, qy, qz, dX, dY, dZ);
            for (int j = 0; j < 8; ++j) {
                check("normals from the differences x", px[j], qx[j]);
                check("normals from the differences y", py[j], qy[j]);
                check("normals from the differences z", pz[j], qz[j]);
            }
            geo_ref_volume_derivative(x, y, z, rx, ry, rz);
            volume_gradient_x12_diff(dX, dY, dZ, qx, qy, qz);
            // VoluDer multiplies sums of absolute coordinates (size |r|^2)
            // that cancel to a result of size h^2: its own error is ~eps |r|^2
            const double tol_v = 64 * 2.220446049250313e-16 * omax * omax;
            for (int j = 0; j < 8; ++j) {
                near("volume gradient x", rx[j], qx[j] / 12.0, tol_v);
                near("volume gradient y", ry[j], qy[j] / 12.0, tol_v);
                near("volume gradient z", rz[j], qz[j] / 12.0, tol_v);
            }
        }

        // the velocity gradient from the body diagonals (at dt = 0 the
        // half-step diagonals are the coordinates' own)
        double Dx[4], Dy[4], Dz[4], Ex[4], Ey[4], Ez[4];
        body_diagonals(x, Dx);
        body_diagonals(y, Dy);
        body_diagonals(z, Dz);
        body_diagonals(xv, Ex);
        body_diagonals(yv, Ey);
        body_diagonals(zv, Ez);
        double fxi, fxe, fxz, fyi, fye, fyz, fzi, fze, fzz;
        diag_directions(Dx, fxi, fxe, fxz);
        diag_directions(Dy, fyi, fye, fyz);
        diag_directions(Dz, fzi, fze, fzz);
        const double invd =
            1.0 / shape_derivs_x64_jac(fxi, fxe, fxz, fyi, fye, fyz, fzi, fze, fzz, bx, by, bz);
        const double cond = omax / h;  // the reference's node sums lose this factor
        const double tol_g = 256 * 2.220446049250313e-16 * cond * cond / h;
        near("dxx from diagonals", grad(inv, b, xv),
             -invd * (bx[0] * Ex[0] + bx[1] * Ex[2] + bx[2] * Ex[3] + bx[3] * Ex[1]), tol_g);
        near("dyy from diagonals", grad(inv, b + 8, yv),
             -invd * (by[0] * Ey[0] + by[1] * Ey[2] + by[2] * Ey[3] + by[3] * Ey[1]), tol_g);
        near("dzz from diagonals", grad(inv, b + 16, zv),
             -invd * (bz[0] * Ez[0] + bz[1] * Ez[2] + bz[2] * Ez[3] + bz[3] * Ez[1]), tol_g);

        // the trace from the xi, eta, zeta differences at a half step
        // x - dt2 v (the velocities are O(1), so the step moves a node by up
        // to 5 % of h), against the reference's B matrix at those coordinates
        {
            const double dt2 = 0.05 * h * std::fabs(u(g));
            double xh[8], yh[8], zh[8], bh[24], deth;
            for (int j = 0; j < 8; ++j) {
                xh[j] = x[j] - dt2 * xv[j];
                yh[j] = y[j] - dt2 * yv[j];
                zh[j] = z[j] - dt2 * zv[j];
            }
            geo_ref_shape(xh, yh, zh, bh, &deth);
            const double invh = 1.0 / deth;
            const double tr_ref = grad(invh, bh, xv) + grad(invh, bh + 8, yv) + grad(invh, bh + 16, zv);
            double P[9], V[9];
            directions3(Dx, Dy, Dz, P);
            directions3(Ex, Ey, Ez, V);
            near("velocity trace from directions", tr_ref, velocity_trace_dirs(P, V, dt2),
                 3 * tol_g);
        }

        // the monotonic-Q gradients from the body diagonals
        double gref[6], gdia[6];
        monoq_gradients<double, false>(x, y, z, xv, yv, zv, vol, gref);
        monoq_gradients_diag(Dx, Dy, Dz, Ex, Ey, Ez, vol, gdia);
        for (int c = 0; c < 3; ++c)
            near("delx from diagonals", gref[c], gdia[c], 256 * 2.220446049250313e-16 * cond * h);
        for (int c = 3; c < 6; ++c)
            near("delv from diagonals", gref[c], gdia[c], 256 * 2.220446049250313e-16 * cond * cond);
    }

    // the FP32 sign filter of the Jacobian determinant: it may only claim
    // "positive" where the FP64 determinant is positive.  Elements: unit
    // cubes at offsets up to 1e3 with sizes from 1e-6 to 10 (large offsets
    // against small sizes push the coordinate rounding), jittered, flattened
    // toward a plane, collapsed toward a node, and inverted (two nodes
    // swapped).
    long certain = 0, shaped = 0, claimed_wrong = 0;
    std::uniform_real_distribution<double> lsz(-6.0, 1.0), loff(-3.0, 3.0);
    for (long it = 0; it < 4 * n; ++it) {
        const double h = std::pow(10.0, lsz(g)), off = std::pow(10.0, loff(g));
        const int kind = (int)(it % 5);
        const double o[3] = {off * u(g), off * u(g), off * u(g)};
        double x[8], y[8], z[8];
        for (int j = 0; j < 8; ++j) {
            const double jit = kind == 1 ? 0.3 : 0.0;
            x[j] = o[0] + h * (cx[j] + jit * u(g));
            y[j] = o[1] + h * (cy[j] + jit * u(g));
            z[j] = o[2] + h * (cz[j] + jit * u(g));
            if (kind == 2) z[j] = o[2] + h * std::pow(10.0, -8.0 * std::fabs(u(g))) * cz[j];
        }
        if (kind == 3) {  // node 6 collapsed onto node 0, nearly
            const double t = std::pow(10.0, -10.0 * std::fabs(u(g)));
            x[6] = x[0] + t * (x[6] - x[0]);
            y[6] = y[0] + t * (y[6] - y[0]);
            z[6] = z[0] + t * (z[6] - z[0]);
        }
        if (kind == 4) {  // inverted: nodes 0 and 6 swapped
            std::swap(x[0], x[6]);
            std::swap(y[0], y[6]);
            std::swap(z[0], z[6]);
        }
        const bool sure = jacobian_certainly_positive(x, y, z);
        const double det = jacobian_det(x, y, z);
        if (sure && !(det > 0.0)) {
            if (claimed_wrong < 10)
                std::printf("filter claimed a positive determinant: %.17g (kind %d)\n", det, kind);
            ++claimed_wrong;
        }
        if (kind == 0 && off < 1e3 * h) {  // coordinates up to 1e3 element sizes, as s <= 1000
            ++shaped;
            certain += sure;
        }
    }
    g_bad += claimed_wrong;
    std::printf("jacobian filter: %ld wrong claims; certain for %ld of %ld cubes\n", claimed_wrong,
                certain, shaped);
    if (certain < shaped) {
        std::printf("filter undecided on a well-shaped cube\n");
        ++g_bad;
    }

    // monotonic-Q gradients: the oracle's domain-level loop on a jittered
    // mesh with random velocities and relative volumes
    orc_domain *d = orc_create(6, 11, 1, 1);
    size_t N = 0, E = 0, L = 0;
    double *X = orc_field_f64(d, "x", &N), *Y = orc_field_f64(d, "y", nullptr),
           *Z = orc_field_f64(d, "z", nullptr), *XD = orc_field_f64(d, "xd", nullptr),
           *YD = orc_field_f64(d, "yd", nullptr), *ZD = orc_field_f64(d, "zd", nullptr);
    double *vnew = orc_field_f64(d, "vnew", &E), *volo = orc_field_f64(d, "volo", nullptr);
    const int *nl = orc_field_i32(d, "nodelist", &L);
    for (size_t i = 0; i < N; ++i) {
        X[i] += 0.02 * u(g);
        Y[i] += 0.02 * u(g);
        Z[i] += 0.02 * u(g);
        XD[i] = u(g);
        YD[i] = u(g);
        ZD[i] = u(g);
    }
    for (size_t k = 0; k < E; ++k) vnew[k] = 1.0 + 0.3 * u(g);
    geo_ref_monoq_gradients(d);
    const char *names[6] = {"delx_xi", "delx_eta", "delx_zeta", "delv_xi", "delv_eta", "delv_zeta"};
    const double *want[6];
    for (int c = 0; c < 6; ++c) want[c] = orc_field_f64(d, names[c], nullptr);
    for (size_t k = 0; k < E; ++k) {
        double x[8], y[8], z[8], xv[8], yv[8], zv[8], out[6];
        for (int j = 0; j < 8; ++j) {
            const int m = nl[8 * k + j];
            x[j] = X[m]; y[j] = Y[m]; z[j] = Z[m];
            xv[j] = XD[m]; yv[j] = YD[m]; zv[j] = ZD[m];
        }
        monoq_gradients<double, true>(x, y, z, xv, yv, zv, volo[k] * vnew[k], out);
        for (int c = 0; c < 6; ++c) check(names[c], want[c][k], out[c]);
        monoq_gradients<double, false>(x, y, z, xv, yv, zv, volo[k] * vnew[k], out);
        for (int c = 0; c < 6; ++c) check(names[c], want[c][k], out[c]);
    }
    orc_destroy(d);
    if (g_plant != 0.0)
        for (const auto &kv : g_far_by)
            std::printf("planted %s: %ld beyond tolerance\n", kv.first.c_str(), kv.second);
    std::printf("reassociated forms beyond tolerance %ld\n", g_far);
    std::printf("%ld random elements, %zu mesh elements, mismatches %ld\n", n, E, g_bad + g_far);
    return (g_bad + g_far) != 0;
}
