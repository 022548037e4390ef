// lg_kernels_mixed.cu -- the mixed-precision cycle (same four kernels).
//
// FP32, on element-relative coordinates (node positions minus node 0's,
// differenced in FP64 and then converted): stress and hourglass forces, the
// per-corner force scratch (one summed stress + hourglass force per corner
// and component) and its per-node sums, the characteristic length,
// the velocity gradient and the monotonic-Q gradients and limiter.
// FP64: node coordinates and velocities and their update, the element volume
// and relative volume (CalcElemVolume differences nearly equal coordinates),
// the EOS predictor-corrector with all its repetitions, the sound speed and
// the Courant/hydro reduction -- with the reciprocal, square root and
// comparisons of lg_fastmath.cuh.
#define LG_NS mixed
#define LG_NS_NAME "mixed"
#include "lg_cycle_common.cuh"
#include "lg_fastmath.cuh"
#include "lg_geometry.cuh"

namespace lg {
namespace mixed {

using namespace ::lg::geom;
using ::lg::fast::FastOps;
using ::lg::fast::rcp_nr;
using ::lg::fast::sqrt_nr;
using ::lg::fast::to_f32;
using ::lg::fast::to_f64;

__device__ __forceinline__ float *fview(double *p) { return reinterpret_cast<float *>(p); }

// element-relative FP32 coordinates of the 8 corners
__device__ __forceinline__ void relative_coords(const DevState &s, const int nd[8], float *x,
                                                float *y, float *z)
{
    const double x0 = s.x[nd[0]], y0 = s.y[nd[0]], z0 = s.z[nd[0]];
    x[0] = y[0] = z[0] = 0.f;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        x[j] = to_f32(s.x[nd[j]] - x0);
        y[j] = to_f32(s.y[nd[j]] - y0);
        z[j] = to_f32(s.z[nd[j]] - z0);
    }
}

// CalcVolumeForceForElems (lulesh.cc:1062-1100) in FP32
__device__ __forceinline__ void forces_element(const DevState &s, const int k, Ctl *ctl,
                                               const double hg64)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    float *const cs = fview(s.corner);
    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = __ldg(&s.nodelistT[(size_t)j * E + k]);
    float x[8], y[8], z[8];
    relative_coords(s, nd, x, y, z);
    // stress corner forces, kept until the hourglass forces are added: one
    // summed force per corner and component goes to the scratch
    float fs[3][8];
    {
        const float sig = to_f32(-s.p[k] - s.q[k]);
        const float determ = jacobian_det(x, y, z);
        node_normals(fs[0], fs[1], fs[2], x, y, z);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            fs[0][j] = -(sig * fs[0][j]);
            fs[1][j] = -(sig * fs[1][j]);
            fs[2][j] = -(sig * fs[2][j]);
        }
        if (determ <= 0.f) raise_status(ctl, -1);
    }
    const double vk = s.v[k];
    if (vk <= 0.0) raise_status(ctl, -1);
    if (!(hg64 > 0.)) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int j = 0; j < 8; ++j) cs[c * E8 + (size_t)j * E + k] = fs[c][j];
        return;
    }
    const float determ = to_f32(s.volo[k]) * to_f32(vk);
    float hourgam[8][4];
    {
        float dvdx[8], dvdy[8], dvdz[8];
        volume_derivative(x, y, z, dvdx, dvdy, dvdz);
        const float volinv = 1.f / determ;
#pragma unroll
        for (int i1 = 0; i1 < 4; ++i1) {
            float hmx = 0.f, hmy = 0.f, hmz = 0.f;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                hmx += x[j] * gam<float>(i1, j);
                hmy += y[j] * gam<float>(i1, j);
                hmz += z[j] * gam<float>(i1, j);
            }
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                hourgam[kk][i1] =
                    gam<float>(i1, kk) - volinv * (dvdx[kk] * hmx + dvdy[kk] * hmy + dvdz[kk] * hmz);
        }
    }
    const float coefficient = -to_f32(hg64) * 0.01f * to_f32(s.ss[k]) *
                              to_f32(s.elemMass[k]) / cbrtf(determ);
    const double *vel[3] = {s.xd, s.yd, s.zd};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float u[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) u[j] = to_f32(__ldg(&vel[c][nd[j]]));
        float hxx[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float h = 0.f;
#pragma unroll
            for (int j = 0; j < 8; ++j) h += hourgam[j][i] * u[j];
            hxx[i] = h;
        }
#pragma unroll
        for (int i = 0; i < 8; i++)
            cs[c * E8 + (size_t)i * E + k] =
                fs[c][i] + coefficient * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                                          hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
    }
}

template <bool BATCHED, int BS>
__global__ void __launch_bounds__(BS) k_forces(DevState s)
{
    if (!BATCHED && !cycle_live(s.ctl)) return;
    for (int k = blockIdx.x * BS + threadIdx.x; k < s.E; k += gridDim.x * BS) {
        const int pid = BATCHED ? s.elemProb[k] : 0;
        Ctl *ctl = s.ctl + pid;
        if (BATCHED && !cycle_live(ctl)) continue;
        forces_element(s, k, ctl, BATCHED ? s.hgcoefs[pid] : s.prm.hgcoef);
    }
}

// ordered FP32 gather of the corners' summed stress + hourglass forces,
// then LagrangeNodal's FP64 node update (lulesh.cc:1139-1219)
__device__ __forceinline__ void nodes_node(const DevState &s, const int n, const Ctl *ctl)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    const float *cs = fview(s.corner);
    const int b = s.nodeElemStart[n], e = s.nodeElemStart[n + 1];
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int i = b; i < e; ++i) {
        const int c = s.nodeElemCornerList[i];
        const size_t idx = (size_t)(c & 7) * E + (c >> 3);
        fx += cs[0 * E8 + idx];
        fy += cs[1 * E8 + idx];
        fz += cs[2 * E8 + idx];
    }
    const double Fx = to_f64(fx), Fy = to_f64(fy), Fz = to_f64(fz);
    s.fx[n] = Fx;
    s.fy[n] = Fy;
    s.fz[n] = Fz;
    const double im = s.invMass[n];
    double xdd = Fx * im, ydd = Fy * im, zdd = Fz * im;
    const int sym = s.symm[n];
    if (sym & 1) xdd = 0.0;
    if (sym & 2) ydd = 0.0;
    if (sym & 4) zdd = 0.0;
    s.xdd[n] = xdd;
    s.ydd[n] = ydd;
    s.zdd[n] = zdd;
    const double dt = ctl->deltatime;
    const double u_cut = s.prm.u_cut;
    double xd = s.xd[n] + xdd * dt;
    if (FastOps::abs_lt(xd, u_cut)) xd = 0.0;
    double yd = s.yd[n] + ydd * dt;
    if (FastOps::abs_lt(yd, u_cut)) yd = 0.0;
    double zd = s.zd[n] + zdd * dt;
    if (FastOps::abs_lt(zd, u_cut)) zd = 0.0;
    s.xd[n] = xd;
    s.yd[n] = yd;
    s.zd[n] = zd;
    s.x[n] += xd * dt;
    s.y[n] += yd * dt;
    s.z[n] += zd * dt;
}

template <bool BATCHED, int BS>
__global__ void __launch_bounds__(BS) k_nodes(DevState s)
{
    if (!BATCHED && !cycle_live(s.ctl)) return;
    for (int n = blockIdx.x * BS + threadIdx.x; n < s.N; n += gridDim.x * BS) {
        const int pid = BATCHED ? s.nodeProb[n] : 0;
        const Ctl *ctl = s.ctl + pid;
        if (BATCHED && !cycle_live(ctl)) continue;
        nodes_node(s, n, ctl);
    }
}

// CalcKinematicsForElems + CalcMonotonicQGradientsForElems
// (lulesh.cc:1504-1757): FP64 volume, FP32 the rest
__device__ __forceinline__ void kinematics_element(const DevState &s, const int k, Ctl *ctl)
{
    const int E = s.E;
    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = __ldg(&s.nodelistT[(size_t)j * E + k]);
    double xa[8], ya[8], za[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        xa[j] = s.x[nd[j]];
        ya[j] = s.y[nd[j]];
        za[j] = s.z[nd[j]];
    }
    const double volo = s.volo[k];
    const double volume = elem_volume(xa, ya, za);
    const double relativeVolume = FastOps::div(volume, volo);
    s.vnew[k] = relativeVolume;
    s.delv[k] = relativeVolume - s.v[k];

    float x[8], y[8], z[8], xv[8], yv[8], zv[8];
    x[0] = y[0] = z[0] = 0.f;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        x[j] = to_f32(xa[j] - xa[0]);
        y[j] = to_f32(ya[j] - ya[0]);
        z[j] = to_f32(za[j] - za[0]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        xv[j] = to_f32(s.xd[nd[j]]);
        yv[j] = to_f32(s.yd[nd[j]]);
        zv[j] = to_f32(s.zd[nd[j]]);
    }
    const float vol32 = to_f32(volume);
    s.arealg[k] = to_f64(char_length(x, y, z, vol32));
    {
        const float dt2 = to_f32(0.5 * ctl->deltatime);
        float xh[8], yh[8], zh[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            xh[j] = x[j] - dt2 * xv[j];
            yh[j] = y[j] - dt2 * yv[j];
            zh[j] = z[j] - dt2 * zv[j];
        }
        float bx[4], by[4], bz[4];
        const float detJ = shape_derivs(xh, yh, zh, bx, by, bz);
        const float inv_detJ = 1.f / detJ;
        const float dxx = inv_detJ * (bx[0] * (xv[0] - xv[6]) + bx[1] * (xv[1] - xv[7]) +
                                      bx[2] * (xv[2] - xv[4]) + bx[3] * (xv[3] - xv[5]));
        const float dyy = inv_detJ * (by[0] * (yv[0] - yv[6]) + by[1] * (yv[1] - yv[7]) +
                                      by[2] * (yv[2] - yv[4]) + by[3] * (yv[3] - yv[5]));
        const float dzz = inv_detJ * (bz[0] * (zv[0] - zv[6]) + bz[1] * (zv[1] - zv[7]) +
                                      bz[2] * (zv[2] - zv[4]) + bz[3] * (zv[3] - zv[5]));
        s.vdov[k] = to_f64(dxx + dyy + dzz);
    }
    if (relativeVolume <= 0.0) raise_status(ctl, -1);

    const float ptiny = 1.e-36f;
    float ax, ay, az, dxv, dyv, dzv;
    const float vol = to_f32(volo) * to_f32(relativeVolume);
    const float norm = 1.f / (vol + ptiny);
#define S4(A, a, b, c, d) (A[a] + A[b] + A[c] + A[d])
    const float dxj = -0.25f * (S4(x, 0, 1, 5, 4) - S4(x, 3, 2, 6, 7));
    const float dyj = -0.25f * (S4(y, 0, 1, 5, 4) - S4(y, 3, 2, 6, 7));
    const float dzj = -0.25f * (S4(z, 0, 1, 5, 4) - S4(z, 3, 2, 6, 7));
    const float dxi = 0.25f * (S4(x, 1, 2, 6, 5) - S4(x, 0, 3, 7, 4));
    const float dyi = 0.25f * (S4(y, 1, 2, 6, 5) - S4(y, 0, 3, 7, 4));
    const float dzi = 0.25f * (S4(z, 1, 2, 6, 5) - S4(z, 0, 3, 7, 4));
    const float dxk = 0.25f * (S4(x, 4, 5, 6, 7) - S4(x, 0, 1, 2, 3));
    const float dyk = 0.25f * (S4(y, 4, 5, 6, 7) - S4(y, 0, 1, 2, 3));
    const float dzk = 0.25f * (S4(z, 4, 5, 6, 7) - S4(z, 0, 1, 2, 3));
    float *const gxz = fview(s.delx_zeta), *const gvz = fview(s.delv_zeta);
    float *const gxx = fview(s.delx_xi), *const gvx = fview(s.delv_xi);
    float *const gxe = fview(s.delx_eta), *const gve = fview(s.delv_eta);

    ax = dyi * dzj - dzi * dyj;
    ay = dzi * dxj - dxi * dzj;
    az = dxi * dyj - dyi * dxj;
    gxz[k] = vol / sqrtf(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = 0.25f * (S4(xv, 4, 5, 6, 7) - S4(xv, 0, 1, 2, 3));
    dyv = 0.25f * (S4(yv, 4, 5, 6, 7) - S4(yv, 0, 1, 2, 3));
    dzv = 0.25f * (S4(zv, 4, 5, 6, 7) - S4(zv, 0, 1, 2, 3));
    gvz[k] = ax * dxv + ay * dyv + az * dzv;

    ax = dyj * dzk - dzj * dyk;
    ay = dzj * dxk - dxj * dzk;
    az = dxj * dyk - dyj * dxk;
    gxx[k] = vol / sqrtf(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = 0.25f * (S4(xv, 1, 2, 6, 5) - S4(xv, 0, 3, 7, 4));
    dyv = 0.25f * (S4(yv, 1, 2, 6, 5) - S4(yv, 0, 3, 7, 4));
    dzv = 0.25f * (S4(zv, 1, 2, 6, 5) - S4(zv, 0, 3, 7, 4));
    gvx[k] = ax * dxv + ay * dyv + az * dzv;

    ax = dyk * dzi - dzk * dyi;
    ay = dzk * dxi - dxk * dzi;
    az = dxk * dyi - dyk * dxi;
    gxe[k] = vol / sqrtf(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = -0.25f * (S4(xv, 0, 1, 5, 4) - S4(xv, 3, 2, 6, 7));
    dyv = -0.25f * (S4(yv, 0, 1, 5, 4) - S4(yv, 3, 2, 6, 7));
    dzv = -0.25f * (S4(zv, 0, 1, 5, 4) - S4(zv, 3, 2, 6, 7));
    gve[k] = ax * dxv + ay * dyv + az * dzv;
#undef S4
}

template <bool BATCHED, int BS>
__global__ void __launch_bounds__(BS) k_kinematics(DevState s)
{
    if (!BATCHED && !cycle_live(s.ctl)) return;
    for (int k = blockIdx.x * BS + threadIdx.x; k < s.E; k += gridDim.x * BS) {
        Ctl *ctl = s.ctl + (BATCHED ? s.elemProb[k] : 0);
        if (BATCHED && !cycle_live(ctl)) continue;
        kinematics_element(s, k, ctl);
    }
}

// Q limiter (FP32) + material update (FP64 EOS) + time constraints (FP64)
// for one element at region-order position t holding all its repetitions
// (nItems == E, and the batched kernel); MODE as in the FP64 kernels.  Kept
// beside the two-phase form: it measures 1.5 % faster when no element is
// shared.
template <int MODE>
__device__ __forceinline__ void material_element(const DevState &s, const int t, Ctl *ctl,
                                                 double &dtc, double &dth)
{
    const Params &P = s.prm;
    const int ielem = s.regPerm[t];
    if (MODE != 1) {
        const float lm = to_f32(P.monoq_limiter_mult), ms = to_f32(P.monoq_max_slope);
        const float *gvx = fview(s.delv_xi), *gve = fview(s.delv_eta),
                    *gvz = fview(s.delv_zeta);
        const int bc = s.elemBC[ielem];
        const float phixi = monoq_phi(lm, ms, gvx, ielem, bc, XI_M_SYMM, XI_M_FREE, XI_M,
                                      XI_P_SYMM, XI_P_FREE, XI_P, s.lxim[ielem],
                                      s.lxip[ielem]);
        const float phieta = monoq_phi(lm, ms, gve, ielem, bc, ETA_M_SYMM, ETA_M_FREE,
                                       ETA_M, ETA_P_SYMM, ETA_P_FREE, ETA_P, s.letam[ielem],
                                       s.letap[ielem]);
        const float phizeta = monoq_phi(lm, ms, gvz, ielem, bc, ZETA_M_SYMM, ZETA_M_FREE,
                                        ZETA_M, ZETA_P_SYMM, ZETA_P_FREE, ZETA_P,
                                        s.lzetam[ielem], s.lzetap[ielem]);
        const double vnew = s.vnew[ielem];
        const double vdov = s.vdov[ielem];
        double qlin, qquad;
        if (FastOps::lt(0.0, vdov)) {
            qlin = 0.;
            qquad = 0.;
        } else {
            float dxxi = gvx[ielem] * fview(s.delx_xi)[ielem];
            float dxeta = gve[ielem] * fview(s.delx_eta)[ielem];
            float dxzeta = gvz[ielem] * fview(s.delx_zeta)[ielem];
            if (dxxi > 0.f) dxxi = 0.f;
            if (dxeta > 0.f) dxeta = 0.f;
            if (dxzeta > 0.f) dxzeta = 0.f;
            const float rho = to_f32(s.elemMass[ielem]) /
                              (to_f32(s.volo[ielem]) * to_f32(vnew));
            qlin = to_f64(-to_f32(P.qlc_monoq) * rho *
                          (dxxi * (1.f - phixi) + dxeta * (1.f - phieta) +
                           dxzeta * (1.f - phizeta)));
            qquad = to_f64(to_f32(P.qqc_monoq) * rho *
                           (dxxi * dxxi * (1.f - phixi * phixi) +
                            dxeta * dxeta * (1.f - phieta * phieta) +
                            dxzeta * dxzeta * (1.f - phizeta * phizeta)));
        }
        s.qq[ielem] = qquad;
        s.ql[ielem] = qlin;

        const double q_old = s.q[ielem];
        if (FastOps::lt(P.qstop, q_old)) ctl->err_qstop = 1;

        double vnewc = vnew;
        if (P.eosvmin != 0. && FastOps::lt(vnewc, P.eosvmin)) vnewc = P.eosvmin;
        if (P.eosvmax != 0. && FastOps::lt(P.eosvmax, vnewc)) vnewc = P.eosvmax;
        double vc = s.v[ielem];
        if (P.eosvmin != 0. && FastOps::lt(vc, P.eosvmin)) vc = P.eosvmin;
        if (P.eosvmax != 0. && FastOps::lt(P.eosvmax, vc)) vc = P.eosvmax;
        if (FastOps::le(vc, 0.)) ctl->err_matvol = 1;

        double p_new, e_new, q_new, ss_new;
        eval_eos<FastOps>(P, s.e[ielem], s.delv[ielem], s.p[ielem], q_old, qquad, qlin,
                          vnewc, s.regRep[t], p_new, e_new, q_new, ss_new);
        s.p[ielem] = p_new;
        s.e[ielem] = e_new;
        s.q[ielem] = q_new;
        s.ss[ielem] = ss_new;

        double tmpV = vnew;
        if (FastOps::abs_lt(tmpV - 1.0, P.v_cut)) tmpV = 1.0;
        s.v[ielem] = tmpV;
    }
    if (MODE != 0) {
        // Only elements with vdov != 0 constrain dt; a warp of elements at
        // rest skips the FP64 square root and reciprocals altogether.
        double vdov = s.vdov[ielem];
        const bool moving = ((unsigned long long)__double_as_longlong(vdov) << 1) != 0ull;
        if (__any_sync(__activemask(), moving) && moving) {
            const double qqc2 = 64.0 * P.qqc * P.qqc;
            double ssv = s.ss[ielem];
            double arealg = s.arealg[ielem];
            opaque(vdov); opaque(ssv); opaque(arealg);
            double dtf = ssv * ssv;
            if (FastOps::lt(vdov, 0.)) dtf = dtf + qqc2 * arealg * arealg * vdov * vdov;
            dtf = arealg * rcp_nr(sqrt_nr(dtf));
            if (dtf < dtc) dtc = dtf;
            const double dtdvov = P.dvovmax * rcp_nr(fabs(vdov) + 1.e-20);
            if (dth > dtdvov) dth = dtdvov;
        }
    }
}

// An element of the split material phase (k_material_inputs / _finish): its
// limiter results, clamped volumes and EOS inputs (MatItem of the FP64
// kernels; reps and writer are unused here).
struct MatItem {
    int ielem, reps;
    bool writer;
    double qlin, qquad, q_old, vnewc, vnew, e, delv, p;
};

// The element part of phase 1, reads only: Q limiter (FP32), qstop check and
// material clamps of element ielem.
__device__ __forceinline__ void material_inputs(const DevState &s, const int ielem, Ctl *ctl,
                                                MatItem &m)
{
    const Params &P = s.prm;
    const float lm = to_f32(P.monoq_limiter_mult), ms = to_f32(P.monoq_max_slope);
    const float *gvx = fview(s.delv_xi), *gve = fview(s.delv_eta),
                *gvz = fview(s.delv_zeta);
    const int bc = s.elemBC[ielem];
    const float phixi = monoq_phi(lm, ms, gvx, ielem, bc, XI_M_SYMM, XI_M_FREE, XI_M,
                                  XI_P_SYMM, XI_P_FREE, XI_P, s.lxim[ielem],
                                  s.lxip[ielem]);
    const float phieta = monoq_phi(lm, ms, gve, ielem, bc, ETA_M_SYMM, ETA_M_FREE,
                                   ETA_M, ETA_P_SYMM, ETA_P_FREE, ETA_P, s.letam[ielem],
                                   s.letap[ielem]);
    const float phizeta = monoq_phi(lm, ms, gvz, ielem, bc, ZETA_M_SYMM, ZETA_M_FREE,
                                    ZETA_M, ZETA_P_SYMM, ZETA_P_FREE, ZETA_P,
                                    s.lzetam[ielem], s.lzetap[ielem]);
    const double vnew = s.vnew[ielem];
    const double vdov = s.vdov[ielem];
    double qlin, qquad;
    if (FastOps::lt(0.0, vdov)) {
        qlin = 0.;
        qquad = 0.;
    } else {
        float dxxi = gvx[ielem] * fview(s.delx_xi)[ielem];
        float dxeta = gve[ielem] * fview(s.delx_eta)[ielem];
        float dxzeta = gvz[ielem] * fview(s.delx_zeta)[ielem];
        if (dxxi > 0.f) dxxi = 0.f;
        if (dxeta > 0.f) dxeta = 0.f;
        if (dxzeta > 0.f) dxzeta = 0.f;
        const float rho = to_f32(s.elemMass[ielem]) /
                          (to_f32(s.volo[ielem]) * to_f32(vnew));
        qlin = to_f64(-to_f32(P.qlc_monoq) * rho *
                      (dxxi * (1.f - phixi) + dxeta * (1.f - phieta) +
                       dxzeta * (1.f - phizeta)));
        qquad = to_f64(to_f32(P.qqc_monoq) * rho *
                       (dxxi * dxxi * (1.f - phixi * phixi) +
                        dxeta * dxeta * (1.f - phieta * phieta) +
                        dxzeta * dxzeta * (1.f - phizeta * phizeta)));
    }
    m.qlin = qlin;
    m.qquad = qquad;

    m.q_old = s.q[ielem];
    if (FastOps::lt(P.qstop, m.q_old)) ctl->err_qstop = 1;

    double vnewc = vnew;
    if (P.eosvmin != 0. && FastOps::lt(vnewc, P.eosvmin)) vnewc = P.eosvmin;
    if (P.eosvmax != 0. && FastOps::lt(P.eosvmax, vnewc)) vnewc = P.eosvmax;
    double vc = s.v[ielem];
    if (P.eosvmin != 0. && FastOps::lt(vc, P.eosvmin)) vc = P.eosvmin;
    if (P.eosvmax != 0. && FastOps::lt(P.eosvmax, vc)) vc = P.eosvmax;
    if (FastOps::le(vc, 0.)) ctl->err_matvol = 1;
    m.vnewc = vnewc;
    m.vnew = vnew;
    m.e = s.e[ielem];
    m.delv = s.delv[ielem];
    m.p = s.p[ielem];
}

// The writer's part of phase 2: the element's update from the results o of
// its FP64 repetitions (MODE != 1) and its FP64 Courant/hydro candidates
// (MODE != 0).
template <int MODE>
__device__ __forceinline__ void material_finish(const DevState &s, const MatItem &m,
                                                const EosOut &o, double &dtc, double &dth)
{
    const Params &P = s.prm;
    const int ielem = m.ielem;
    if (MODE != 1) {
        s.qq[ielem] = m.qquad;
        s.ql[ielem] = m.qlin;
        s.p[ielem] = o.p;
        s.e[ielem] = o.e;
        s.q[ielem] = o.q;
        s.ss[ielem] = eos_sound_speed<FastOps>(P, o, m.vnewc);

        double tmpV = m.vnew;
        if (FastOps::abs_lt(tmpV - 1.0, P.v_cut)) tmpV = 1.0;
        s.v[ielem] = tmpV;
    }
    if (MODE != 0) {
        // Only elements with vdov != 0 constrain dt; a warp of elements at
        // rest skips the FP64 square root and reciprocals altogether.
        double vdov = s.vdov[ielem];
        const bool moving = ((unsigned long long)__double_as_longlong(vdov) << 1) != 0ull;
        if (__any_sync(__activemask(), moving) && moving) {
            const double qqc2 = 64.0 * P.qqc * P.qqc;
            double ssv = s.ss[ielem];
            double arealg = s.arealg[ielem];
            opaque(vdov); opaque(ssv); opaque(arealg);
            double dtf = ssv * ssv;
            if (FastOps::lt(vdov, 0.)) dtf = dtf + qqc2 * arealg * arealg * vdov * vdov;
            dtf = arealg * rcp_nr(sqrt_nr(dtf));
            if (dtf < dtc) dtc = dtf;
            const double dtdvov = P.dvovmax * rcp_nr(fabs(vdov) + 1.e-20);
            if (dth > dtdvov) dth = dtdvov;
        }
    }
}

// The split material phase (DevState::matSplit, small meshes): three
// kernels instead of one, so that every FP64 instruction runs with full
// warps.  k_material_inputs (one thread per element, natural order): the
// monotonic-Q limiter, qstop check and clamps, staging the EOS inputs;
// k_material_eos (one thread per repetition item, equal shares per warp):
// the item's share of the EOS repetitions, the writer staging the results;
// k_material_finish (one thread per element): sound speed, stores, volume
// update, Courant/hydro candidates and the block reduction whose last block
// runs the next TimeIncrement.  The staging area is the per-corner scratch,
// which k_nodes has consumed and the next k_forces overwrites: eight inputs
// and five results per element, SoA.  Each element's arithmetic is that of
// the one-kernel path.
namespace matstage {
enum { E_OLD, DELV, P_OLD, Q_OLD, QQ, QL, VNEWC, VNEW, N_IN };
enum { P_NEW = N_IN, E_NEW, Q_NEW, BVC, PBVC, N_ALL };
}  // namespace matstage

template <int MODE, int BS>
__global__ void __launch_bounds__(BS) k_material_inputs(DevState s)
{
    if (!cycle_live(s.ctl)) return;
    const int k = blockIdx.x * BS + threadIdx.x;
    if (k >= s.E) return;
    MatItem m;
    material_inputs(s, k, s.ctl, m);
    double *st = s.corner;
    const size_t E = (size_t)s.E;
    st[matstage::E_OLD * E + k] = m.e;
    st[matstage::DELV * E + k] = m.delv;
    st[matstage::P_OLD * E + k] = m.p;
    st[matstage::Q_OLD * E + k] = m.q_old;
    st[matstage::QQ * E + k] = m.qquad;
    st[matstage::QL * E + k] = m.qlin;
    st[matstage::VNEWC * E + k] = m.vnewc;
    st[matstage::VNEW * E + k] = m.vnew;
}

template <int BS>
__global__ void __launch_bounds__(BS) k_material_eos(DevState s)
{
    if (!cycle_live(s.ctl)) return;
    const int t = blockIdx.x * BS + threadIdx.x;
    if (t >= s.nItems) return;
    const int k = s.regPerm[t], r = s.regRep[t];
    double *st = s.corner;
    const size_t E = (size_t)s.E;
    const EosOut o = eos_reps<FastOps>(s.prm, st[matstage::E_OLD * E + k], st[matstage::DELV * E + k],
                              st[matstage::P_OLD * E + k], st[matstage::Q_OLD * E + k],
                              st[matstage::QQ * E + k], st[matstage::QL * E + k],
                              st[matstage::VNEWC * E + k], r > 0 ? r : -r);
    if (r > 0) {
        st[matstage::P_NEW * E + k] = o.p;
        st[matstage::E_NEW * E + k] = o.e;
        st[matstage::Q_NEW * E + k] = o.q;
        st[matstage::BVC * E + k] = o.bvc;
        st[matstage::PBVC * E + k] = o.pbvc;
    }
}

template <int MODE, int BS>
__global__ void __launch_bounds__(BS) k_material_finish(DevState s)
{
    if (!cycle_live(s.ctl)) return;
    double dtc = 1.0e+20, dth = 1.0e+20;
    const int k = blockIdx.x * BS + threadIdx.x;
    if (k < s.E) {
        MatItem m;
        m.ielem = k;
        m.writer = true;
        EosOut o{};
        if (MODE != 1) {
            const double *st = s.corner;
            const size_t E = (size_t)s.E;
            m.qquad = st[matstage::QQ * E + k];
            m.qlin = st[matstage::QL * E + k];
            m.vnewc = st[matstage::VNEWC * E + k];
            m.vnew = st[matstage::VNEW * E + k];
            o = {st[matstage::P_NEW * E + k], st[matstage::E_NEW * E + k],
                 st[matstage::Q_NEW * E + k], st[matstage::BVC * E + k],
                 st[matstage::PBVC * E + k]};
        }
        material_finish<MODE>(s, m, o, dtc, dth);
    }
    if (MODE != 0)
        finish_dt<BS>(s, dtc, dth, MODE == 2);
    else
        finish_material_flags(s);
}

template <int MODE, bool BATCHED, int BS>
__global__ void __launch_bounds__(BS) k_material(DevState s)
{
    if (!BATCHED && !cycle_live(s.ctl)) return;
    double dtc = 1.0e+20, dth = 1.0e+20;
    if (!BATCHED) {
        // one item per element (nItems == E); small meshes run the split
        // kernels above
        const int t = blockIdx.x * BS + threadIdx.x;
        if (t < s.E) material_element<MODE>(s, t, s.ctl, dtc, dth);
        if (MODE != 0)
            finish_dt<BS>(s, dtc, dth, MODE == 2);
        else
            finish_material_flags(s);
        return;
    }
    for (int t0 = blockIdx.x * BS; t0 < s.E; t0 += gridDim.x * BS) {
        const int t = t0 + threadIdx.x;
        int pid = -1;
        dtc = 1.0e+20;
        dth = 1.0e+20;
        if (t < s.E) {
            pid = s.elemProb[s.regPerm[t]];
            Ctl *ctl = s.ctl + pid;
            if (cycle_live(ctl)) material_element<2>(s, t, ctl, dtc, dth);
        }
        batched_dt_candidates(s, pid, dtc, dth);
    }
    finish_batched(s);
}

}  // namespace mixed
}  // namespace lg

#include "lg_kernelset.inc"
namespace lg {
const KernelSet *kernels_mixed() { return &mixed::kKernelSet; }
}
