// lg_kernels.cuh -- FP64 kernels of the leap-frog cycle (one cycle = 4 launches).
//
// Included by lg_kernels_fp64.cu (compiled with --fmad=false: every operation
// rounds exactly as the reference's -ffp-contract=off build) and by
// lg_kernels_fma.cu (--fmad=true).  LG_NS names the namespace of each copy.
//
//   k_forces      per element: stress (IntegrateStressForElems) and
//                 Flanagan-Belytschko hourglass forces (CalcHourglassControl/
//                 CalcFBHourglassForceForElems) into the per-corner scratch
//   k_nodes       per node: ordered corner gather, a = F/m, symmetry BC,
//                 velocity with u_cut, position (LagrangeNodal)
//   k_kinematics  per element: volume, vnew, delv, arealg, vdov
//                 (CalcKinematicsForElems) and the monotonic-Q gradients
//                 (CalcMonotonicQGradientsForElems)
//   k_material    per element in region order: monotonic-Q limiter, qstop
//                 check, EOS with its repetitions, sound speed, volume
//                 update, Courant/hydro constraints with a block reduction;
//                 its last block finishes the reduction and runs the next
//                 cycle's TimeIncrement.  Small meshes run the same work as
//                 k_material_inputs (per element), k_material_eos (per
//                 repetition item) and k_material_finish (per element)
//
// Every arithmetic expression keeps the reference's operand order (see the
// oracle's lulesh_oracle.c for the line-by-line correspondence), with two
// kinds of exception.  Exact ones, in both builds: power-of-two factors
// applied once (lg_geometry.cuh) and comparisons of doubles on the integer
// pipe (dlt and friends); the strict build's results stay those of the
// reference's operation order bit for bit.  Rounding ones, in the FMA build
// only: the regrouped sums under LG_REASSOC.  Work the reference does and
// then discards (the shape-function B matrix that CalcElemNodeNormals
// overwrites, the off-diagonal velocity gradient terms, the deviatoric
// strains, the Courant dt of elements with vdov == 0) is not computed;
// division by refdens is skipped when refdens == 1 (x / 1.0 == x exactly).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "lg_device.h"
#include "lg_geometry.cuh"
#include "lg_cycle_common.cuh"

#ifndef LG_NS
#error "define LG_NS"
#endif
// LG_REASSOC (the FMA build): algebraically equal forms that save FP64
// instructions.  k_forces: node normals and the volume gradient from the
// element's twelve edge differences (node_normals_x8_diff,
// volume_gradient_x12_diff), the hourglass_modes butterfly, the 1/12 and
// 1/volume factors applied once per mode, and the hourglass coefficient by
// the reciprocal cube root applied to the four mode sums.  k_kinematics: face
// areas from the faces' diagonals (area_face_cross), the velocity-gradient
// trace and the monotonic-Q gradients from the xi/eta/zeta differences of
// the coordinates and velocities (velocity_trace_dirs, monoq_gradients_dirs),
// lengths by reciprocal square roots.  The rounding differs from the
// reference's operand order, as FMA contraction's does; the parity bar
// covers both.
#ifndef LG_REASSOC
#define LG_REASSOC 0
#endif

namespace lg {
namespace LG_NS {

// element geometry: lg_geometry.cuh
using namespace ::lg::geom;

// ---------------------------------------------------------------------------
// k_forces: CalcVolumeForceForElems (lulesh.cc:1062-1100)
// ---------------------------------------------------------------------------
// one element; hourg is the element's problem's hourglass coefficient
__device__ __forceinline__ void forces_element(const DevState &s, const int k, Ctl *ctl,
                                               const double hourg)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    double *const cs = s.corner;

    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = __ldg(&s.nodelistT[(size_t)j * E + k]);
#if LG_REASSOC
    double gvx[8], gvy[8], gvz[8];  // 12 x the volume gradient (hourglass part)
#endif
    double x[8], y[8], z[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        x[j] = __ldg(&s.x[nd[j]]);
        y[j] = __ldg(&s.y[nd[j]]);
        z[j] = __ldg(&s.z[nd[j]]);
    }

    // InitStressTermsForElems (273-286) + IntegrateStressForElems (494-587)
    {
        double pfx[8], pfy[8], pfz[8];
#if LG_REASSOC
        // 8 x the normals from the twelve differences, which also give the
        // volume gradient of the hourglass part below; the 1/8 goes into sig
        // (exact)
        const double sig = (-s.p[k] - s.q[k]) * 0.125;
        {
            double dX[12], dY[12], dZ[12];
            elem_differences(x, dX);
            elem_differences(y, dY);
            elem_differences(z, dZ);
            node_normals_x8_diff(pfx, pfy, pfz, dX, dY, dZ);
            volume_gradient_x12_diff(dX, dY, dZ, gvx, gvy, gvz);
        }
#else
        const double sig = -s.p[k] - s.q[k];
        node_normals(pfx, pfy, pfz, x, y, z);
#endif
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            cs[0 * E8 + (size_t)j * E + k] = -(sig * pfx[j]);
            cs[1 * E8 + (size_t)j * E + k] = -(sig * pfy[j]);
            cs[2 * E8 + (size_t)j * E + k] = -(sig * pfz[j]);
        }
        // lulesh.cc:1082-1091 uses the Jacobian determinant only for its
        // sign: an FP32 filter with a rigorous error bound settles it, and
        // the FP64 determinant is evaluated only in a warp with an element
        // the filter cannot settle (none on a valid mesh)
        const bool sure = jacobian_certainly_positive(x, y, z);
        if (__any_sync(__activemask(), !sure) && !sure && jacobian_det(x, y, z) <= 0.0)
            raise_status(ctl, -1);
    }

    // CalcHourglassControlForElems (995-1057)
    const double vk = s.v[k];
    const double determ = s.volo[k] * vk;
    if (dle(vk, 0.0)) raise_status(ctl, -1);  // lulesh.cc:1034-1040
    if (!(hourg > 0.)) return;

    // CalcFBHourglassForceForElems (710-991), CalcElemFBHourglassForce (667-706)
    double hourgam[8][4];
#if LG_REASSOC
    {
        // 12 x dV/dx (from the twelve differences, above), with 1/(12 volume)
        // folded into the four mode sums
        const double *dvdx = gvx, *dvdy = gvy, *dvdz = gvz;
        const double volinv12 = (1.0 / determ) * (1.0 / 12.0);
        double hmx[4], hmy[4], hmz[4];
        hourglass_modes(x, hmx);
        hourglass_modes(y, hmy);
        hourglass_modes(z, hmz);
#pragma unroll
        for (int i1 = 0; i1 < 4; ++i1) {
            const double hx = volinv12 * hmx[i1], hy = volinv12 * hmy[i1],
                         hz = volinv12 * hmz[i1];
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                hourgam[kk][i1] = gam(i1, kk) - dvdx[kk] * hx - dvdy[kk] * hy - dvdz[kk] * hz;
        }
    }
#else
    {
        double dvdx[8], dvdy[8], dvdz[8];
        volume_derivative(x, y, z, dvdx, dvdy, dvdz);
        const double volinv = 1.0 / determ;
#pragma unroll
        for (int i1 = 0; i1 < 4; ++i1) {
            const double hourmodx = x[0] * gam(i1, 0) + x[1] * gam(i1, 1) + x[2] * gam(i1, 2) +
                                    x[3] * gam(i1, 3) + x[4] * gam(i1, 4) + x[5] * gam(i1, 5) +
                                    x[6] * gam(i1, 6) + x[7] * gam(i1, 7);
            const double hourmody = y[0] * gam(i1, 0) + y[1] * gam(i1, 1) + y[2] * gam(i1, 2) +
                                    y[3] * gam(i1, 3) + y[4] * gam(i1, 4) + y[5] * gam(i1, 5) +
                                    y[6] * gam(i1, 6) + y[7] * gam(i1, 7);
            const double hourmodz = z[0] * gam(i1, 0) + z[1] * gam(i1, 1) + z[2] * gam(i1, 2) +
                                    z[3] * gam(i1, 3) + z[4] * gam(i1, 4) + z[5] * gam(i1, 5) +
                                    z[6] * gam(i1, 6) + z[7] * gam(i1, 7);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                hourgam[kk][i1] = gam(i1, kk) - volinv * (dvdx[kk] * hourmodx +
                                                          dvdy[kk] * hourmody +
                                                          dvdz[kk] * hourmodz);
        }
    }
#endif
    const double ss1 = s.ss[k];
    const double mass1 = s.elemMass[k];
#if LG_REASSOC
    // the reciprocal cube root in place of cbrt and a quotient; the
    // coefficient goes into the four mode sums hxx (4 products, not 8)
    const double coefficient = (-hourg * 0.01 * ss1 * mass1) * rcbrt(determ);
#else
    const double volume13 = cbrt(determ);
    const double coefficient = -hourg * 0.01 * ss1 * mass1 / volume13;
#endif
    const double *vel[3] = {s.xd, s.yd, s.zd};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double u[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) u[j] = __ldg(&vel[c][nd[j]]);
        double hxx[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
            hxx[i] = hourgam[0][i] * u[0] + hourgam[1][i] * u[1] + hourgam[2][i] * u[2] +
                     hourgam[3][i] * u[3] + hourgam[4][i] * u[4] + hourgam[5][i] * u[5] +
                     hourgam[6][i] * u[6] + hourgam[7][i] * u[7];
#if LG_REASSOC
#pragma unroll
        for (int i = 0; i < 4; i++) hxx[i] *= coefficient;
#pragma unroll
        for (int i = 0; i < 8; i++)
            cs[(3 + c) * E8 + (size_t)i * E + k] =
                hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] + hourgam[i][2] * hxx[2] +
                hourgam[i][3] * hxx[3];
#else
#pragma unroll
        for (int i = 0; i < 8; i++)
            cs[(3 + c) * E8 + (size_t)i * E + k] =
                coefficient * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                               hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
#endif
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

// f / m, rounded as the IEEE quotient, from rm = RN(1 / m) (the set-up's
// invMass, constant over the run) by Markstein's residual correction
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990): q0 = RN(f rm), the exact
// residual f - m q0 by one FMA, q = RN(q0 + residual rm).  Three FP64
// instructions instead of a division; equal to f / m for operands in the
// normal range whose residual does not underflow.  An exact q0 (zero
// residual) is returned as is, which keeps the sign of a zero quotient.
__device__ __forceinline__ double div_by_mass(double f, double m, double rm)
{
    const double q0 = __dmul_rn(f, rm);
    const double res = __fma_rn(-m, q0, f);
    return dnz(res) ? __fma_rn(res, rm, q0) : q0;
}

// ---------------------------------------------------------------------------
// k_nodes: corner gather (lulesh.cc:565-582, 969-986), CalcAccelerationForNodes
// (1139-1149), ApplyAccelerationBoundaryConditionsForNodes (1153-1179),
// CalcVelocityForNodes (1183-1205), CalcPositionForNodes (1209-1219)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void nodes_node(const DevState &s, const int n, const Ctl *ctl,
                                           const bool hg)
{
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    const double *cs = s.corner;
    const int b = s.nodeElemStart[n], e = s.nodeElemStart[n + 1];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    double hx = 0.0, hy = 0.0, hz = 0.0;
    for (int i = b; i < e; ++i) {
        const int c = s.nodeElemCornerList[i];
        const size_t idx = (size_t)(c & 7) * E + (c >> 3);
        fx += cs[0 * E8 + idx];
        fy += cs[1 * E8 + idx];
        fz += cs[2 * E8 + idx];
        if (hg) {
            hx += cs[3 * E8 + idx];
            hy += cs[4 * E8 + idx];
            hz += cs[5 * E8 + idx];
        }
    }
    if (hg) {
        fx += hx;
        fy += hy;
        fz += hz;
    }
    s.fx[n] = fx;
    s.fy[n] = fy;
    s.fz[n] = fz;
    const double m = s.nodalMass[n], rm = s.invMass[n];
    double xdd = div_by_mass(fx, m, rm), ydd = div_by_mass(fy, m, rm),
           zdd = div_by_mass(fz, m, rm);
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
    if (dabs_lt(xd, u_cut)) xd = 0.0;
    double yd = s.yd[n] + ydd * dt;
    if (dabs_lt(yd, u_cut)) yd = 0.0;
    double zd = s.zd[n] + zdd * dt;
    if (dabs_lt(zd, u_cut)) zd = 0.0;
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
        nodes_node(s, n, ctl, (BATCHED ? s.hgcoefs[pid] : s.prm.hgcoef) > 0.);
    }
}

// ---------------------------------------------------------------------------
// k_kinematics: CalcKinematicsForElems (lulesh.cc:1504-1568), the strain loop
// of CalcLagrangeElements (1584-1606) and CalcMonotonicQGradientsForElems
// (1613-1757)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void kinematics_element(const DevState &s, const int k, Ctl *ctl)
{
    const int E = s.E;
    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = __ldg(&s.nodelistT[(size_t)j * E + k]);
    double x[8], y[8], z[8], xv[8], yv[8], zv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        x[j] = s.x[nd[j]];
        y[j] = s.y[nd[j]];
        z[j] = s.z[nd[j]];
        xv[j] = s.xd[nd[j]];
        yv[j] = s.yd[nd[j]];
        zv[j] = s.zd[nd[j]];
    }
    const double volo = s.volo[k];
    const double volume = elem_volume(x, y, z);
    const double relativeVolume = volume / volo;
    s.vnew[k] = relativeVolume;
    s.delv[k] = relativeVolume - s.v[k];
    s.arealg[k] = char_length<double, LG_REASSOC != 0>(x, y, z, volume);
#if LG_REASSOC
    // The velocity gradient's trace and the monotonic-Q gradients from the
    // xi, eta, zeta differences of the coordinates (P) and velocities (V),
    // formed once from the element's body diagonals: the half-step Jacobian
    // is P - dt/2 V (velocity_trace_dirs).
    double P[9], V[9];
    {
        double Dx[4], Dy[4], Dz[4];
        body_diagonals(x, Dx);
        body_diagonals(y, Dy);
        body_diagonals(z, Dz);
        directions3(Dx, Dy, Dz, P);
        body_diagonals(xv, Dx);
        body_diagonals(yv, Dy);
        body_diagonals(zv, Dz);
        directions3(Dx, Dy, Dz, V);
    }
    s.vdov[k] = velocity_trace_dirs(P, V, 0.5 * ctl->deltatime);
    if (dle(relativeVolume, 0.0)) raise_status(ctl, -1);  // lulesh.cc:1598-1605

    // CalcMonotonicQGradientsForElems
    double g[6];
    monoq_gradients_dirs(P, V, volo * relativeVolume, g);
#else
    {
        const double dt2 = 0.5 * ctl->deltatime;
        double xh[8], yh[8], zh[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            xh[j] = x[j] - dt2 * xv[j];
            yh[j] = y[j] - dt2 * yv[j];
            zh[j] = z[j] - dt2 * zv[j];
        }
        // 64 x the determinant and 64 x B, whose factors cancel exactly in
        // inv_detJ * (B . v)
        double bx[4], by[4], bz[4];
        const double inv_detJ = 1.0 / shape_derivs_x64(xh, yh, zh, bx, by, bz);
        const double dxx = inv_detJ * (bx[0] * (xv[0] - xv[6]) + bx[1] * (xv[1] - xv[7]) +
                                       bx[2] * (xv[2] - xv[4]) + bx[3] * (xv[3] - xv[5]));
        const double dyy = inv_detJ * (by[0] * (yv[0] - yv[6]) + by[1] * (yv[1] - yv[7]) +
                                       by[2] * (yv[2] - yv[4]) + by[3] * (yv[3] - yv[5]));
        const double dzz = inv_detJ * (bz[0] * (zv[0] - zv[6]) + bz[1] * (zv[1] - zv[7]) +
                                       bz[2] * (zv[2] - zv[4]) + bz[3] * (zv[3] - zv[5]));
        s.vdov[k] = dxx + dyy + dzz;
    }
    if (dle(relativeVolume, 0.0)) raise_status(ctl, -1);  // lulesh.cc:1598-1605

    // CalcMonotonicQGradientsForElems
    double g[6];
    monoq_gradients<double, true>(x, y, z, xv, yv, zv, volo * relativeVolume, g);
#endif
    s.delx_xi[k] = g[0];
    s.delx_eta[k] = g[1];
    s.delx_zeta[k] = g[2];
    s.delv_xi[k] = g[3];
    s.delv_eta[k] = g[4];
    s.delv_zeta[k] = g[5];
}

// The FMA build's k_kinematics runs three blocks of 128 threads per SM (at
// most 168 registers, a few values spilled to L1) instead of the two its
// 184 registers allow: 2.4 % faster at s=150 with the same results bit for
// bit.
#if LG_REASSOC
#define LG_KIN_MIN_BLOCKS(BS) ((BS) <= 384 ? 384 / (BS) : 1)
#else
#define LG_KIN_MIN_BLOCKS(BS) 1
#endif
template <bool BATCHED, int BS>
__global__ void __launch_bounds__(BS, LG_KIN_MIN_BLOCKS(BS)) k_kinematics(DevState s)
{
    if (!BATCHED && !cycle_live(s.ctl)) return;
    for (int k = blockIdx.x * BS + threadIdx.x; k < s.E; k += gridDim.x * BS) {
        Ctl *ctl = s.ctl + (BATCHED ? s.elemProb[k] : 0);
        if (BATCHED && !cycle_live(ctl)) continue;
        kinematics_element(s, k, ctl);
    }
}

// One element of the material phase: its id and EOS repetitions (work item
// t of k_material, region order: regPerm[t], regRep[t]; every such item is
// its element's writer), its limiter results, clamped volumes and EOS
// inputs.  Every repetition computes the same values from the same inputs,
// so any repetition's results are the update; the split kernels for small
// meshes rely on that too.
struct MatItem {
    int ielem, reps;
    bool writer;
    double qlin, qquad, q_old, vnewc, vnew, e, delv, p;
};

// The element part of phase 1, reads only: monotonic-Q limiter, qstop check
// and the material clamps of element ielem.
__device__ __forceinline__ void material_inputs(const DevState &s, const int ielem, Ctl *ctl,
                                                MatItem &m)
{
    const Params &P = s.prm;
    // CalcMonotonicQRegionForElems, lulesh.cc:1761-1921
    const int bc = s.elemBC[ielem];
    const double phixi = monoq_phi(P.monoq_limiter_mult, P.monoq_max_slope, s.delv_xi, ielem, bc, XI_M_SYMM, XI_M_FREE,
                                   XI_M, XI_P_SYMM, XI_P_FREE, XI_P, s.lxim[ielem],
                                   s.lxip[ielem]);
    const double phieta = monoq_phi(P.monoq_limiter_mult, P.monoq_max_slope, s.delv_eta, ielem, bc, ETA_M_SYMM, ETA_M_FREE,
                                    ETA_M, ETA_P_SYMM, ETA_P_FREE, ETA_P,
                                    s.letam[ielem], s.letap[ielem]);
    const double phizeta = monoq_phi(P.monoq_limiter_mult, P.monoq_max_slope, s.delv_zeta, ielem, bc, ZETA_M_SYMM,
                                     ZETA_M_FREE, ZETA_M, ZETA_P_SYMM, ZETA_P_FREE,
                                     ZETA_P, s.lzetam[ielem], s.lzetap[ielem]);
    const double vnew = s.vnew[ielem];
    const double vdov = s.vdov[ielem];
    double qlin, qquad;
    if (dlt(0., vdov)) {
        qlin = 0.;
        qquad = 0.;
    } else {
        double delvxxi = s.delv_xi[ielem] * s.delx_xi[ielem];
        double delvxeta = s.delv_eta[ielem] * s.delx_eta[ielem];
        double delvxzeta = s.delv_zeta[ielem] * s.delx_zeta[ielem];
        if (dlt(0., delvxxi)) delvxxi = 0.;
        if (dlt(0., delvxeta)) delvxeta = 0.;
        if (dlt(0., delvxzeta)) delvxzeta = 0.;
        const double rho = s.elemMass[ielem] / (s.volo[ielem] * vnew);
        qlin = -P.qlc_monoq * rho *
               (delvxxi * (1. - phixi) + delvxeta * (1. - phieta) +
                delvxzeta * (1. - phizeta));
        qquad = P.qqc_monoq * rho *
                (delvxxi * delvxxi * (1. - phixi * phixi) +
                 delvxeta * delvxeta * (1. - phieta * phieta) +
                 delvxzeta * delvxzeta * (1. - phizeta * phizeta));
    }
    m.qlin = qlin;
    m.qquad = qquad;

    // qstop check on the previous cycle's q, lulesh.cc:1993-2008
    m.q_old = s.q[ielem];
    if (dlt(P.qstop, m.q_old)) ctl->err_qstop = 1;

    // ApplyMaterialPropertiesForElems, lulesh.cc:2328-2406
    double vnewc = vnew;
    if (dnz(P.eosvmin) && dlt(vnewc, P.eosvmin)) vnewc = P.eosvmin;
    if (dnz(P.eosvmax) && dlt(P.eosvmax, vnewc)) vnewc = P.eosvmax;
    double vc = s.v[ielem];
    if (dnz(P.eosvmin) && dlt(vc, P.eosvmin)) vc = P.eosvmin;
    if (dnz(P.eosvmax) && dlt(P.eosvmax, vc)) vc = P.eosvmax;
    if (dle(vc, 0.)) ctl->err_matvol = 1;
    m.vnewc = vnewc;
    m.vnew = vnew;
    m.e = s.e[ielem];
    m.delv = s.delv[ielem];
    m.p = s.p[ielem];
}

// Phase 1 of item t: its element, repetitions and role, and (MODE != 1) the
// element's inputs.  False for an item without an element.
template <int MODE>
__device__ __forceinline__ bool material_load(const DevState &s, const int t, Ctl *ctl,
                                              MatItem &m)
{
    const int ielem = s.regPerm[t];
    if (ielem < 0) return false;
    const int r = s.regRep[t];
    m.ielem = ielem;
    m.writer = r > 0;
    m.reps = r > 0 ? r : -r;
    if (MODE != 1) material_inputs(s, ielem, ctl, m);
    return true;
}

// The writer's part of phase 2: the element's update from the results o of
// its repetitions (MODE != 1) and its Courant/hydro candidates (MODE != 0).
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
        s.ss[ielem] = eos_sound_speed(P, o, m.vnewc);

        // UpdateVolumesForElems, lulesh.cc:2410-2427
        double tmpV = m.vnew;
        if (dabs_lt(tmpV - 1.0, P.v_cut)) tmpV = 1.0;
        s.v[ielem] = tmpV;
    }
    if (MODE != 0) {
        // CalcCourantConstraintForElems (2447-2513) and
        // CalcHydroConstraintForElems (2517-2572) for one element.  The
        // reference evaluates the Courant dt of every element but keeps it
        // only where vdov != 0; a warp of elements at rest skips it (the
        // barriers keep the compiler from hoisting that work above the vote).
        double vdov = s.vdov[ielem];
        const bool moving = dnz(vdov);
        if (__any_sync(__activemask(), moving) && moving) {
            const double qqc2 = 64.0 * P.qqc * P.qqc;
            double ssv = s.ss[ielem];
            double arealg = s.arealg[ielem];
            opaque(vdov); opaque(ssv); opaque(arealg);
            double dtf = ssv * ssv;
            if (dlt(vdov, 0.)) dtf = dtf + qqc2 * arealg * arealg * vdov * vdov;
            dtf = sqrt(dtf);
            dtf = arealg / dtf;
            if (dlt(dtf, dtc)) dtc = dtf;
            const double dtdvov = P.dvovmax / (fabs(vdov) + 1.e-20);
            if (dlt(dtdvov, dth)) dth = dtdvov;
        }
    }
}

// Phase 2: the item's EOS repetitions (MODE != 1); the writer finishes the
// element.
template <int MODE>
__device__ __forceinline__ void material_update(const DevState &s, const MatItem &m,
                                                double &dtc, double &dth)
{
    EosOut o{};
    if (MODE != 1)
        o = eos_reps(s.prm, m.e, m.delv, m.p, m.q_old, m.qquad, m.qlin, m.vnewc, m.reps);
    if (m.writer) material_finish<MODE>(s, m, o, dtc, dth);
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
    const EosOut o = eos_reps(s.prm, st[matstage::E_OLD * E + k], st[matstage::DELV * E + k],
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
        finish_dt<BS, true>(s, dtc, dth, MODE == 2);
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
        MatItem m;
        if (t < s.nItems && material_load<MODE>(s, t, s.ctl, m))
            material_update<MODE>(s, m, dtc, dth);
        if (MODE != 0)
            finish_dt<BS, true>(s, dtc, dth, MODE == 2);
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
            MatItem m;
            if (cycle_live(ctl) && material_load<2>(s, t, ctl, m))
                material_update<2>(s, m, dtc, dth);
        }
        batched_dt_candidates(s, pid, dtc, dth);
    }
    finish_batched(s);
}

}  // namespace LG_NS
}  // namespace lg
