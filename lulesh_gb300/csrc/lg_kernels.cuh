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
//                 cycle's TimeIncrement
//
// Every arithmetic expression keeps the reference's operand order (see the
// oracle's lulesh_oracle.c for the line-by-line correspondence).  Work the
// reference does and then discards (the shape-function B matrix that
// CalcElemNodeNormals overwrites, the off-diagonal velocity gradient terms,
// the deviatoric strains) is not computed; division by refdens is skipped
// when refdens == 1 (x / 1.0 == x exactly).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "lg_device.h"

#ifndef LG_NS
#error "define LG_NS"
#endif

namespace lg {
namespace LG_NS {

constexpr int kBlock = 128;

// Keeps the compiler from treating a value as loop-invariant, so that every
// EOS repetition the reference performs is evaluated.
__device__ __forceinline__ void opaque(double &v) { asm volatile("" : "+d"(v)); }

__device__ __forceinline__ void raise_status(Ctl *c, int code) { atomicCAS(&c->status, 0, code); }

// TimeIncrement, lulesh.cc:166-222
__device__ __forceinline__ void time_increment(Ctl *c)
{
    double targetdt = c->stoptime - c->time;
    if ((c->dtfixed <= 0.0) && (c->cycle != 0)) {
        double ratio;
        const double olddt = c->deltatime;
        double gnewdt = 1.0e+20;
        double newdt;
        if (c->dtcourant < gnewdt) gnewdt = c->dtcourant / 2.0;
        if (c->dthydro < gnewdt) gnewdt = c->dthydro * 2.0 / 3.0;
        newdt = gnewdt;
        ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < c->dtmultlb)
                newdt = olddt;
            else if (ratio > c->dtmultub)
                newdt = olddt * c->dtmultub;
        }
        if (newdt > c->dtmax) newdt = c->dtmax;
        c->deltatime = newdt;
    }
    if ((targetdt > c->deltatime) && (targetdt < (4.0 * c->deltatime / 3.0)))
        targetdt = 2.0 * c->deltatime / 3.0;
    if (targetdt < c->deltatime) c->deltatime = targetdt;
    c->time += c->deltatime;
    ++c->cycle;
}

// Loop condition of lulesh.cc:2745 followed by TimeIncrement.
__device__ __forceinline__ void begin_cycle(Ctl *c)
{
    if (c->status == 0 && c->time < c->stoptime && c->cycle < c->cycle_limit) {
        time_increment(c);
        c->active = 1;
    } else {
        c->active = 0;
    }
}

__global__ void k_begin(Ctl *c) { begin_cycle(c); }
__global__ void k_time_increment(Ctl *c)
{
    time_increment(c);
    c->active = 1;
}
__global__ void k_set_active(Ctl *c) { c->active = 1; }

__device__ __forceinline__ bool cycle_live(const Ctl *c) { return c->active && c->status == 0; }

// ---------------------------------------------------------------------------
// element geometry (lulesh.cc:290-474, 591-663, 1273-1435)
// ---------------------------------------------------------------------------

// Jacobian determinant of CalcElemShapeFunctionDerivatives (lulesh.cc:319-376)
__device__ __forceinline__ double jacobian_det(const double *x, const double *y, const double *z)
{
    const double fjxxi = .125 * ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    const double fjxet = .125 * ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    const double fjxze = .125 * ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    const double fjyxi = .125 * ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    const double fjyet = .125 * ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    const double fjyze = .125 * ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    const double fjzxi = .125 * ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    const double fjzet = .125 * ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    const double fjzze = .125 * ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    const double cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    const double cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    const double cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    return 8. * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

// CalcElemShapeFunctionDerivatives rows 0..3 of B (rows 4..7 are their
// negatives) and the determinant, lulesh.cc:290-377
__device__ __forceinline__ double shape_derivs(const double *x, const double *y, const double *z,
                                               double bx[4], double by[4], double bz[4])
{
    const double fjxxi = .125 * ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    const double fjxet = .125 * ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    const double fjxze = .125 * ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    const double fjyxi = .125 * ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    const double fjyet = .125 * ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    const double fjyze = .125 * ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    const double fjzxi = .125 * ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    const double fjzet = .125 * ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    const double fjzze = .125 * ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    const double cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
    const double cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    const double cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
    const double cjyxi = -(fjxet * fjzze) + (fjzet * fjxze);
    const double cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    const double cjyze = -(fjxxi * fjzet) + (fjzxi * fjxet);
    const double cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
    const double cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    const double cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);
    bx[0] = -cjxxi - cjxet - cjxze;
    bx[1] = cjxxi - cjxet - cjxze;
    bx[2] = cjxxi + cjxet - cjxze;
    bx[3] = -cjxxi + cjxet - cjxze;
    by[0] = -cjyxi - cjyet - cjyze;
    by[1] = cjyxi - cjyet - cjyze;
    by[2] = cjyxi + cjyet - cjyze;
    by[3] = -cjyxi + cjyet - cjyze;
    bz[0] = -cjzxi - cjzet - cjzze;
    bz[1] = cjzxi - cjzet - cjzze;
    bz[2] = cjzxi + cjzet - cjzze;
    bz[3] = -cjzxi + cjzet - cjzze;
    return 8. * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

// SumElemFaceNormal, lulesh.cc:381-415 (the four corners a,b,c,d of a face)
__device__ __forceinline__ void face_normal(double *nx, double *ny, double *nz, const double *x,
                                            const double *y, const double *z, int a, int b, int c,
                                            int d)
{
    const double bisectX0 = 0.5 * (x[d] + x[c] - x[b] - x[a]);
    const double bisectY0 = 0.5 * (y[d] + y[c] - y[b] - y[a]);
    const double bisectZ0 = 0.5 * (z[d] + z[c] - z[b] - z[a]);
    const double bisectX1 = 0.5 * (x[c] + x[b] - x[d] - x[a]);
    const double bisectY1 = 0.5 * (y[c] + y[b] - y[d] - y[a]);
    const double bisectZ1 = 0.5 * (z[c] + z[b] - z[d] - z[a]);
    const double areaX = 0.25 * (bisectY0 * bisectZ1 - bisectZ0 * bisectY1);
    const double areaY = 0.25 * (bisectZ0 * bisectX1 - bisectX0 * bisectZ1);
    const double areaZ = 0.25 * (bisectX0 * bisectY1 - bisectY0 * bisectX1);
    nx[a] += areaX; nx[b] += areaX; nx[c] += areaX; nx[d] += areaX;
    ny[a] += areaY; ny[b] += areaY; ny[c] += areaY; ny[d] += areaY;
    nz[a] += areaZ; nz[b] += areaZ; nz[c] += areaZ; nz[d] += areaZ;
}

// CalcElemNodeNormals, lulesh.cc:419-474
__device__ __forceinline__ void node_normals(double *pfx, double *pfy, double *pfz,
                                             const double *x, const double *y, const double *z)
{
#pragma unroll
    for (int i = 0; i < 8; ++i) pfx[i] = pfy[i] = pfz[i] = 0.0;
    face_normal(pfx, pfy, pfz, x, y, z, 0, 1, 2, 3);
    face_normal(pfx, pfy, pfz, x, y, z, 0, 4, 5, 1);
    face_normal(pfx, pfy, pfz, x, y, z, 1, 5, 6, 2);
    face_normal(pfx, pfy, pfz, x, y, z, 2, 6, 7, 3);
    face_normal(pfx, pfy, pfz, x, y, z, 3, 7, 4, 0);
    face_normal(pfx, pfy, pfz, x, y, z, 4, 7, 6, 5);
}

// VoluDer, lulesh.cc:591-619, for corner k of CalcElemVolumeDerivative
// (lulesh.cc:623-663) with neighbour nodes m0..m5
__device__ __forceinline__ void volu_der(const double *x, const double *y, const double *z, int m0,
                                         int m1, int m2, int m3, int m4, int m5, double &dvdx,
                                         double &dvdy, double &dvdz)
{
    const double twelfth = 1.0 / 12.0;
    const double x0 = x[m0], x1 = x[m1], x2 = x[m2], x3 = x[m3], x4 = x[m4], x5 = x[m5];
    const double y0 = y[m0], y1 = y[m1], y2 = y[m2], y3 = y[m3], y4 = y[m4], y5 = y[m5];
    const double z0 = z[m0], z1 = z[m1], z2 = z[m2], z3 = z[m3], z4 = z[m4], z5 = z[m5];
    dvdx = (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) + (y0 + y4) * (z3 + z4) -
           (y3 + y4) * (z0 + z4) - (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    dvdy = -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) - (x0 + x4) * (z3 + z4) +
           (x3 + x4) * (z0 + z4) + (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    dvdz = -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) - (y0 + y4) * (x3 + x4) +
           (y3 + y4) * (x0 + x4) + (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
    dvdx *= twelfth;
    dvdy *= twelfth;
    dvdz *= twelfth;
}

__device__ __forceinline__ void volume_derivative(const double *x, const double *y,
                                                  const double *z, double *dvdx, double *dvdy,
                                                  double *dvdz)
{
    volu_der(x, y, z, 1, 2, 3, 4, 5, 7, dvdx[0], dvdy[0], dvdz[0]);
    volu_der(x, y, z, 0, 1, 2, 7, 4, 6, dvdx[3], dvdy[3], dvdz[3]);
    volu_der(x, y, z, 3, 0, 1, 6, 7, 5, dvdx[2], dvdy[2], dvdz[2]);
    volu_der(x, y, z, 2, 3, 0, 5, 6, 4, dvdx[1], dvdy[1], dvdz[1]);
    volu_der(x, y, z, 7, 6, 5, 0, 3, 1, dvdx[4], dvdy[4], dvdz[4]);
    volu_der(x, y, z, 4, 7, 6, 1, 0, 2, dvdx[5], dvdy[5], dvdz[5]);
    volu_der(x, y, z, 5, 4, 7, 2, 1, 3, dvdx[6], dvdy[6], dvdz[6]);
    volu_der(x, y, z, 6, 5, 4, 3, 2, 0, dvdx[7], dvdy[7], dvdz[7]);
}

// CalcElemVolume, lulesh.cc:1273-1356
__device__ __forceinline__ double elem_volume(const double *x, const double *y, const double *z)
{
    const double twelveth = 1.0 / 12.0;
    const double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    const double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    const double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    const double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    const double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    const double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    const double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    const double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    const double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    const double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    const double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    const double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
#define LG_TP(a1, b1, c1, a2, b2, c2, a3, b3, c3) \
    ((a1) * ((b2) * (c3) - (c2) * (b3)) + (a2) * ((c1) * (b3) - (b1) * (c3)) + \
     (a3) * ((b1) * (c2) - (c1) * (b2)))
    double volume =
        LG_TP(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
        LG_TP(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
        LG_TP(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
#undef LG_TP
    volume *= twelveth;
    return volume;
}

// AreaFace, lulesh.cc:1370-1390
__device__ __forceinline__ double area_face(const double *x, const double *y, const double *z,
                                            int a, int b, int c, int d)
{
    const double fx = (x[c] - x[a]) - (x[d] - x[b]);
    const double fy = (y[c] - y[a]) - (y[d] - y[b]);
    const double fz = (z[c] - z[a]) - (z[d] - z[b]);
    const double gx = (x[c] - x[a]) + (x[d] - x[b]);
    const double gy = (y[c] - y[a]) + (y[d] - y[b]);
    const double gz = (z[c] - z[a]) + (z[d] - z[b]);
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) -
           (fx * gx + fy * gy + fz * gz) * (fx * gx + fy * gy + fz * gz);
}

// CalcElemCharacteristicLength, lulesh.cc:1394-1435 (std::max(a,b) is
// (a < b) ? b : a)
__device__ __forceinline__ double char_length(const double *x, const double *y, const double *z,
                                              double volume)
{
    double cl = 0.0, a;
    a = area_face(x, y, z, 0, 1, 2, 3); cl = (a < cl) ? cl : a;
    a = area_face(x, y, z, 4, 5, 6, 7); cl = (a < cl) ? cl : a;
    a = area_face(x, y, z, 0, 1, 5, 4); cl = (a < cl) ? cl : a;
    a = area_face(x, y, z, 1, 2, 6, 5); cl = (a < cl) ? cl : a;
    a = area_face(x, y, z, 2, 3, 7, 6); cl = (a < cl) ? cl : a;
    a = area_face(x, y, z, 3, 0, 4, 7); cl = (a < cl) ? cl : a;
    return 4.0 * volume / sqrt(cl);
}

// hourglass base vectors, lulesh.cc:743-776
__device__ __forceinline__ constexpr double gam(int mode, int k)
{
    constexpr signed char G[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1},
                                     {1, -1, -1, 1, -1, 1, 1, -1},
                                     {1, -1, 1, -1, 1, -1, 1, -1},
                                     {-1, 1, -1, 1, 1, -1, 1, -1}};
    return (double)G[mode][k];
}

// ---------------------------------------------------------------------------
// k_forces: CalcVolumeForceForElems (lulesh.cc:1062-1100)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_forces(DevState s)
{
    Ctl *ctl = s.ctl;
    if (!cycle_live(ctl)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int E = s.E;
    if (k >= E) return;
    const size_t E8 = 8 * (size_t)E;
    double *const cs = s.corner;

    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = __ldg(&s.nodelistT[(size_t)j * E + k]);
    double x[8], y[8], z[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        x[j] = __ldg(&s.x[nd[j]]);
        y[j] = __ldg(&s.y[nd[j]]);
        z[j] = __ldg(&s.z[nd[j]]);
    }

    // InitStressTermsForElems (273-286) + IntegrateStressForElems (494-587)
    {
        const double sig = -s.p[k] - s.q[k];
        const double determ = jacobian_det(x, y, z);
        double pfx[8], pfy[8], pfz[8];
        node_normals(pfx, pfy, pfz, x, y, z);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            cs[0 * E8 + (size_t)j * E + k] = -(sig * pfx[j]);
            cs[1 * E8 + (size_t)j * E + k] = -(sig * pfy[j]);
            cs[2 * E8 + (size_t)j * E + k] = -(sig * pfz[j]);
        }
        if (determ <= 0.0) raise_status(ctl, -1);  // lulesh.cc:1082-1091
    }

    // CalcHourglassControlForElems (995-1057)
    const double vk = s.v[k];
    const double determ = s.volo[k] * vk;
    if (vk <= 0.0) raise_status(ctl, -1);  // lulesh.cc:1034-1040
    const double hourg = s.prm.hgcoef;
    if (!(hourg > 0.)) return;

    // CalcFBHourglassForceForElems (710-991), CalcElemFBHourglassForce (667-706)
    double hourgam[8][4];
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
    const double ss1 = s.ss[k];
    const double mass1 = s.elemMass[k];
    const double volume13 = cbrt(determ);
    const double coefficient = -hourg * 0.01 * ss1 * mass1 / volume13;
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
#pragma unroll
        for (int i = 0; i < 8; i++)
            cs[(3 + c) * E8 + (size_t)i * E + k] =
                coefficient * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                               hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
    }
}

// ---------------------------------------------------------------------------
// k_nodes: corner gather (lulesh.cc:565-582, 969-986), CalcAccelerationForNodes
// (1139-1149), ApplyAccelerationBoundaryConditionsForNodes (1153-1179),
// CalcVelocityForNodes (1183-1205), CalcPositionForNodes (1209-1219)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_nodes(DevState s)
{
    Ctl *ctl = s.ctl;
    if (!cycle_live(ctl)) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= s.N) return;
    const int E = s.E;
    const size_t E8 = 8 * (size_t)E;
    const double *cs = s.corner;
    const int b = s.nodeElemStart[n], e = s.nodeElemStart[n + 1];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    double hx = 0.0, hy = 0.0, hz = 0.0;
    const bool hg = s.prm.hgcoef > 0.;
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
    const double m = s.nodalMass[n];
    double xdd = fx / m, ydd = fy / m, zdd = fz / m;
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
    if (fabs(xd) < u_cut) xd = 0.0;
    double yd = s.yd[n] + ydd * dt;
    if (fabs(yd) < u_cut) yd = 0.0;
    double zd = s.zd[n] + zdd * dt;
    if (fabs(zd) < u_cut) zd = 0.0;
    s.xd[n] = xd;
    s.yd[n] = yd;
    s.zd[n] = zd;
    s.x[n] += xd * dt;
    s.y[n] += yd * dt;
    s.z[n] += zd * dt;
}

// ---------------------------------------------------------------------------
// k_kinematics: CalcKinematicsForElems (lulesh.cc:1504-1568), the strain loop
// of CalcLagrangeElements (1584-1606) and CalcMonotonicQGradientsForElems
// (1613-1757)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_kinematics(DevState s)
{
    Ctl *ctl = s.ctl;
    if (!cycle_live(ctl)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int E = s.E;
    if (k >= E) return;
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
    s.arealg[k] = char_length(x, y, z, volume);
    {
        const double dt2 = 0.5 * ctl->deltatime;
        double xh[8], yh[8], zh[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            xh[j] = x[j] - dt2 * xv[j];
            yh[j] = y[j] - dt2 * yv[j];
            zh[j] = z[j] - dt2 * zv[j];
        }
        double bx[4], by[4], bz[4];
        const double detJ = shape_derivs(xh, yh, zh, bx, by, bz);
        const double inv_detJ = 1.0 / detJ;
        const double dxx = inv_detJ * (bx[0] * (xv[0] - xv[6]) + bx[1] * (xv[1] - xv[7]) +
                                       bx[2] * (xv[2] - xv[4]) + bx[3] * (xv[3] - xv[5]));
        const double dyy = inv_detJ * (by[0] * (yv[0] - yv[6]) + by[1] * (yv[1] - yv[7]) +
                                       by[2] * (yv[2] - yv[4]) + by[3] * (yv[3] - yv[5]));
        const double dzz = inv_detJ * (bz[0] * (zv[0] - zv[6]) + bz[1] * (zv[1] - zv[7]) +
                                       bz[2] * (zv[2] - zv[4]) + bz[3] * (zv[3] - zv[5]));
        s.vdov[k] = dxx + dyy + dzz;
    }
    if (relativeVolume <= 0.0) raise_status(ctl, -1);  // lulesh.cc:1598-1605

    // CalcMonotonicQGradientsForElems
    const double ptiny = 1.e-36;
    double ax, ay, az, dxv, dyv, dzv;
    const double vol = volo * relativeVolume;
    const double norm = 1.0 / (vol + ptiny);
#define S4(A, a, b, c, d) (A[a] + A[b] + A[c] + A[d])
    const double dxj = -0.25 * (S4(x, 0, 1, 5, 4) - S4(x, 3, 2, 6, 7));
    const double dyj = -0.25 * (S4(y, 0, 1, 5, 4) - S4(y, 3, 2, 6, 7));
    const double dzj = -0.25 * (S4(z, 0, 1, 5, 4) - S4(z, 3, 2, 6, 7));
    const double dxi = 0.25 * (S4(x, 1, 2, 6, 5) - S4(x, 0, 3, 7, 4));
    const double dyi = 0.25 * (S4(y, 1, 2, 6, 5) - S4(y, 0, 3, 7, 4));
    const double dzi = 0.25 * (S4(z, 1, 2, 6, 5) - S4(z, 0, 3, 7, 4));
    const double dxk = 0.25 * (S4(x, 4, 5, 6, 7) - S4(x, 0, 1, 2, 3));
    const double dyk = 0.25 * (S4(y, 4, 5, 6, 7) - S4(y, 0, 1, 2, 3));
    const double dzk = 0.25 * (S4(z, 4, 5, 6, 7) - S4(z, 0, 1, 2, 3));

    ax = dyi * dzj - dzi * dyj;
    ay = dzi * dxj - dxi * dzj;
    az = dxi * dyj - dyi * dxj;
    s.delx_zeta[k] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = 0.25 * (S4(xv, 4, 5, 6, 7) - S4(xv, 0, 1, 2, 3));
    dyv = 0.25 * (S4(yv, 4, 5, 6, 7) - S4(yv, 0, 1, 2, 3));
    dzv = 0.25 * (S4(zv, 4, 5, 6, 7) - S4(zv, 0, 1, 2, 3));
    s.delv_zeta[k] = ax * dxv + ay * dyv + az * dzv;

    ax = dyj * dzk - dzj * dyk;
    ay = dzj * dxk - dxj * dzk;
    az = dxj * dyk - dyj * dxk;
    s.delx_xi[k] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = 0.25 * (S4(xv, 1, 2, 6, 5) - S4(xv, 0, 3, 7, 4));
    dyv = 0.25 * (S4(yv, 1, 2, 6, 5) - S4(yv, 0, 3, 7, 4));
    dzv = 0.25 * (S4(zv, 1, 2, 6, 5) - S4(zv, 0, 3, 7, 4));
    s.delv_xi[k] = ax * dxv + ay * dyv + az * dzv;

    ax = dyk * dzi - dzk * dyi;
    ay = dzk * dxi - dxk * dzi;
    az = dxk * dyi - dyk * dxi;
    s.delx_eta[k] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = -0.25 * (S4(xv, 0, 1, 5, 4) - S4(xv, 3, 2, 6, 7));
    dyv = -0.25 * (S4(yv, 0, 1, 5, 4) - S4(yv, 3, 2, 6, 7));
    dzv = -0.25 * (S4(zv, 0, 1, 5, 4) - S4(zv, 3, 2, 6, 7));
    s.delv_eta[k] = ax * dxv + ay * dyv + az * dzv;
#undef S4
}

// ---------------------------------------------------------------------------
// k_material
// ---------------------------------------------------------------------------

// one direction of CalcMonotonicQRegionForElems, lulesh.cc:1778-1813
__device__ __forceinline__ double monoq_phi(const Params &P, const double *dv, int ielem, int bc,
                                            int msymm, int mfree, int mmask, int psymm,
                                            int pfree, int pmask, int nbm, int nbp)
{
    const double ptiny = 1.e-36;
    double delvm, delvp;
    const double self = dv[ielem];
    const double norm = 1. / (self + ptiny);
    const int bm = bc & mmask, bp = bc & pmask;
    if (bm == msymm)
        delvm = self;
    else if (bm == mfree)
        delvm = 0.0;
    else if (bm == 0 || bm == (mmask & ~(msymm | mfree)))
        delvm = dv[nbm];
    else
        delvm = 0;
    if (bp == psymm)
        delvp = self;
    else if (bp == pfree)
        delvp = 0.0;
    else if (bp == 0 || bp == (pmask & ~(psymm | pfree)))
        delvp = dv[nbp];
    else
        delvp = 0;
    delvm = delvm * norm;
    delvp = delvp * norm;
    double phi = .5 * (delvm + delvp);
    delvm *= P.monoq_limiter_mult;
    delvp *= P.monoq_limiter_mult;
    if (delvm < phi) phi = delvm;
    if (delvp < phi) phi = delvp;
    if (phi < 0.) phi = 0.;
    if (phi > P.monoq_max_slope) phi = P.monoq_max_slope;
    return phi;
}

// sound-speed term of lulesh.cc:2083-2090, 2126-2133, 2158-2165, 2190-2197
__device__ __forceinline__ double ssc_of(double num, double rho0)
{
    double ssc = (rho0 == 1.0) ? num : num / rho0;
    if (ssc <= .1111111e-36)
        ssc = .3333333e-18;
    else
        ssc = sqrt(ssc);
    return ssc;
}

// CalcPressureForElems for one element, lulesh.cc:2014-2044
__device__ __forceinline__ double pressure(const Params &P, double &bvc, double &pbvc,
                                           double e_old, double compression, double vnewc)
{
    const double c1s = 2.0 / 3.0;
    bvc = c1s * (compression + 1.);
    pbvc = c1s;
    double p_new = bvc * e_old;
    if (fabs(p_new) < P.p_cut) p_new = 0.0;
    if (vnewc >= P.eosvmax) p_new = 0.0;
    if (p_new < P.pmin) p_new = P.pmin;
    return p_new;
}

// EvalEOSForElems for one element (lulesh.cc:2204-2324) with
// CalcEnergyForElems (2048-2176) and CalcSoundSpeedForElems (2180-2200).
// All rep repetitions are evaluated, as in the reference.
__device__ __forceinline__ void eval_eos(const Params &P, double e_in, double delv_in,
                                         double p_in, double q_in, double qq_in, double ql_in,
                                         double vnewc, int rep, double &p_out, double &e_out,
                                         double &q_out, double &ss_out)
{
    const double rho0 = P.refdens;
    double p_new = 0., e_new = 0., q_new = 0., bvc = 0., pbvc = 0.;
    for (int j = 0; j < rep; j++) {
        double e_old = e_in, delvc = delv_in, p_old = p_in, q_old = q_in, qq_old = qq_in,
               ql_old = ql_in, vc = vnewc;
        opaque(e_old); opaque(delvc); opaque(p_old); opaque(q_old);
        opaque(qq_old); opaque(ql_old); opaque(vc);
        double compression = 1. / vc - 1.;
        const double vchalf = vc - delvc * .5;
        double compHalfStep = 1. / vchalf - 1.;
        if (P.eosvmin != 0. && vc <= P.eosvmin) compHalfStep = compression;
        if (P.eosvmax != 0. && vc >= P.eosvmax) {
            p_old = 0.;
            compression = 0.;
            compHalfStep = 0.;
        }
        const double work = 0.;

        e_new = e_old - .5 * delvc * (p_old + q_old) + .5 * work;
        if (e_new < P.emin) e_new = P.emin;

        const double pHalfStep = pressure(P, bvc, pbvc, e_new, compHalfStep, vc);
        const double vhalf = 1. / (1. + compHalfStep);
        if (delvc > 0.) {
            q_new = 0.;
        } else {
            const double ssc = ssc_of(pbvc * e_new + vhalf * vhalf * bvc * pHalfStep, rho0);
            q_new = (ssc * ql_old + qq_old);
        }
        e_new = e_new + .5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (pHalfStep + q_new));

        e_new += .5 * work;
        if (fabs(e_new) < P.e_cut) e_new = 0.;
        if (e_new < P.emin) e_new = P.emin;

        p_new = pressure(P, bvc, pbvc, e_new, compression, vc);
        {
            const double sixth = 1.0 / 6.0;
            double q_tilde;
            if (delvc > 0.) {
                q_tilde = 0.;
            } else {
                const double ssc = ssc_of(pbvc * e_new + vc * vc * bvc * p_new, rho0);
                q_tilde = (ssc * ql_old + qq_old);
            }
            e_new = e_new - (7.0 * (p_old + q_old) - 8.0 * (pHalfStep + q_new) +
                             (p_new + q_tilde)) * delvc * sixth;
            if (fabs(e_new) < P.e_cut) e_new = 0.;
            if (e_new < P.emin) e_new = P.emin;
        }

        p_new = pressure(P, bvc, pbvc, e_new, compression, vc);
        if (delvc <= 0.) {
            const double ssc = ssc_of(pbvc * e_new + vc * vc * bvc * p_new, rho0);
            q_new = (ssc * ql_old + qq_old);
            if (fabs(q_new) < P.q_cut) q_new = 0.;
        }
    }
    p_out = p_new;
    e_out = e_new;
    q_out = q_new;
    ss_out = ssc_of(pbvc * e_new + vnewc * vnewc * bvc * p_new, rho0);
}

__device__ __forceinline__ double dmin_sel(double a, double b) { return (b < a) ? b : a; }

// Reduces (dtc, dth) over the block; the last block of the grid reduces the
// per-block results into ctl->dtcourant/dthydro, merges error flags and, if
// advance, evaluates the loop condition and TimeIncrement of the next cycle.
__device__ __forceinline__ void finish_dt(DevState &s, double dtc, double dth, bool advance)
{
    __shared__ double red[2][kBlock / 32];
    __shared__ bool am_last;
    Ctl *ctl = s.ctl;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dtc = dmin_sel(dtc, __shfl_down_sync(0xffffffffu, dtc, off));
        dth = dmin_sel(dth, __shfl_down_sync(0xffffffffu, dth, off));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][warp] = dtc;
        red[1][warp] = dth;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bc = red[0][0], bh = red[1][0];
        for (int w = 1; w < kBlock / 32; ++w) {
            bc = dmin_sel(bc, red[0][w]);
            bh = dmin_sel(bh, red[1][w]);
        }
        s.dt_partial[2 * blockIdx.x] = bc;
        s.dt_partial[2 * blockIdx.x + 1] = bh;
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->blocks_done, 1u);
        am_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    double c = 1.0e+20, h = 1.0e+20;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        c = dmin_sel(c, __ldcg(&s.dt_partial[2 * i]));
        h = dmin_sel(h, __ldcg(&s.dt_partial[2 * i + 1]));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        c = dmin_sel(c, __shfl_down_sync(0xffffffffu, c, off));
        h = dmin_sel(h, __shfl_down_sync(0xffffffffu, h, off));
    }
    __syncthreads();
    if (lane == 0) {
        red[0][warp] = c;
        red[1][warp] = h;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kBlock / 32; ++w) {
            red[0][0] = dmin_sel(red[0][0], red[0][w]);
            red[1][0] = dmin_sel(red[1][0], red[1][w]);
        }
        ctl->dtcourant = red[0][0];
        ctl->dthydro = red[1][0];
        ctl->blocks_done = 0;
        if (ctl->status == 0) {
            if (ctl->err_qstop)
                ctl->status = -2;
            else if (ctl->err_matvol)
                ctl->status = -1;
        }
        ctl->err_qstop = 0;
        ctl->err_matvol = 0;
        if (advance) begin_cycle(ctl);
    }
}

// MODE 0: Q limiter + qstop + EOS + sound speed + volume update (the part of
//         LagrangeElements after the kinematics)
// MODE 1: time constraints only (CalcTimeConstraintsForElems)
// MODE 2: both, then the next cycle's TimeIncrement (the fused main loop)
template <int MODE>
__global__ void __launch_bounds__(kBlock) k_material(DevState s)
{
    Ctl *ctl = s.ctl;
    if (!cycle_live(ctl)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < s.E;
    const Params &P = s.prm;
    double dtc = 1.0e+20, dth = 1.0e+20;
    if (valid) {
        const int ielem = s.regPerm[t];
        if (MODE != 1) {
            // CalcMonotonicQRegionForElems, lulesh.cc:1761-1921
            const int bc = s.elemBC[ielem];
            const double phixi = monoq_phi(P, s.delv_xi, ielem, bc, XI_M_SYMM, XI_M_FREE,
                                           XI_M, XI_P_SYMM, XI_P_FREE, XI_P, s.lxim[ielem],
                                           s.lxip[ielem]);
            const double phieta = monoq_phi(P, s.delv_eta, ielem, bc, ETA_M_SYMM, ETA_M_FREE,
                                            ETA_M, ETA_P_SYMM, ETA_P_FREE, ETA_P,
                                            s.letam[ielem], s.letap[ielem]);
            const double phizeta = monoq_phi(P, s.delv_zeta, ielem, bc, ZETA_M_SYMM,
                                             ZETA_M_FREE, ZETA_M, ZETA_P_SYMM, ZETA_P_FREE,
                                             ZETA_P, s.lzetam[ielem], s.lzetap[ielem]);
            const double vnew = s.vnew[ielem];
            const double vdov = s.vdov[ielem];
            double qlin, qquad;
            if (vdov > 0.) {
                qlin = 0.;
                qquad = 0.;
            } else {
                double delvxxi = s.delv_xi[ielem] * s.delx_xi[ielem];
                double delvxeta = s.delv_eta[ielem] * s.delx_eta[ielem];
                double delvxzeta = s.delv_zeta[ielem] * s.delx_zeta[ielem];
                if (delvxxi > 0.) delvxxi = 0.;
                if (delvxeta > 0.) delvxeta = 0.;
                if (delvxzeta > 0.) delvxzeta = 0.;
                const double rho = s.elemMass[ielem] / (s.volo[ielem] * vnew);
                qlin = -P.qlc_monoq * rho *
                       (delvxxi * (1. - phixi) + delvxeta * (1. - phieta) +
                        delvxzeta * (1. - phizeta));
                qquad = P.qqc_monoq * rho *
                        (delvxxi * delvxxi * (1. - phixi * phixi) +
                         delvxeta * delvxeta * (1. - phieta * phieta) +
                         delvxzeta * delvxzeta * (1. - phizeta * phizeta));
            }
            s.qq[ielem] = qquad;
            s.ql[ielem] = qlin;

            // qstop check on the previous cycle's q, lulesh.cc:1993-2008
            const double q_old = s.q[ielem];
            if (q_old > P.qstop) ctl->err_qstop = 1;

            // ApplyMaterialPropertiesForElems, lulesh.cc:2328-2406
            double vnewc = vnew;
            if (P.eosvmin != 0. && vnewc < P.eosvmin) vnewc = P.eosvmin;
            if (P.eosvmax != 0. && vnewc > P.eosvmax) vnewc = P.eosvmax;
            double vc = s.v[ielem];
            if (P.eosvmin != 0. && vc < P.eosvmin) vc = P.eosvmin;
            if (P.eosvmax != 0. && vc > P.eosvmax) vc = P.eosvmax;
            if (vc <= 0.) ctl->err_matvol = 1;

            double p_new, e_new, q_new, ss_new;
            eval_eos(P, s.e[ielem], s.delv[ielem], s.p[ielem], q_old, qquad, qlin, vnewc,
                     s.regRep[t], p_new, e_new, q_new, ss_new);
            s.p[ielem] = p_new;
            s.e[ielem] = e_new;
            s.q[ielem] = q_new;
            s.ss[ielem] = ss_new;

            // UpdateVolumesForElems, lulesh.cc:2410-2427
            double tmpV = vnew;
            if (fabs(tmpV - 1.0) < P.v_cut) tmpV = 1.0;
            s.v[ielem] = tmpV;
        }
        if (MODE != 0) {
            // CalcCourantConstraintForElems (2447-2513) and
            // CalcHydroConstraintForElems (2517-2572) for one element
            const double qqc2 = 64.0 * P.qqc * P.qqc;
            const double ssv = s.ss[ielem];
            const double vdov = s.vdov[ielem];
            const double arealg = s.arealg[ielem];
            double dtf = ssv * ssv;
            if (vdov < 0.) dtf = dtf + qqc2 * arealg * arealg * vdov * vdov;
            dtf = sqrt(dtf);
            dtf = arealg / dtf;
            if (vdov != 0.) {
                if (dtf < dtc) dtc = dtf;
                const double dtdvov = P.dvovmax / (fabs(vdov) + 1.e-20);
                if (dth > dtdvov) dth = dtdvov;
            }
        }
    }
    if (MODE != 0) {
        finish_dt(s, dtc, dth, MODE == 2);
    } else {
        // merge the material-phase error flags once every block is done
        __shared__ bool am_last;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned prev = atomicAdd(&ctl->blocks_done, 1u);
            am_last = (prev == gridDim.x - 1);
        }
        __syncthreads();
        if (am_last && threadIdx.x == 0) {
            __threadfence();
            ctl->blocks_done = 0;
            if (ctl->status == 0) {
                if (ctl->err_qstop)
                    ctl->status = -2;
                else if (ctl->err_matvol)
                    ctl->status = -1;
            }
            ctl->err_qstop = 0;
            ctl->err_matvol = 0;
        }
    }
}

}  // namespace LG_NS
}  // namespace lg
