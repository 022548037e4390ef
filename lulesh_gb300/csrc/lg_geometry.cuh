// lg_geometry.cuh -- hex-element geometry of the reference, generic in the
// arithmetic type (double for the FP64 paths, float for the FP32 parts of the
// mixed path).  Every expression keeps the reference's operand order.  Where
// the reference scales by powers of two, some functions apply the product of
// those factors once (each says so); a power of two scales a rounded result
// exactly, so with R = double and no contraction the values are the
// reference's bit for bit.  node_normals_x8 / node_normals_x8_diff,
// volume_gradient_x12_diff, area_face_cross and rsqrt_fast (through
// char_length<R, true>), body_diagonals / diag_directions /
// monoq_gradients_diag / monoq_gradients_dirs / velocity_trace_dirs and
// hourglass_modes are algebraically equal reformulations that round
// differently; only the FMA build uses them.
#pragma once

#ifdef __CUDACC__
#include <cuda_runtime.h>
#include <cstring>
#define LG_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#include <cstring>
#define LG_HD inline
#include <math.h>
using std::sqrt;
#endif

namespace lg {
namespace geom {

// a < b.  Device code compares doubles through an order-preserving integer
// key (-0 and +0 equal), which equals the IEEE comparison for non-NaN
// operands and keeps it off GB300's FP64 pipe.
template <typename R>
LG_HD bool lt(R a, R b)
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(R) == 8) {
        const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
        const long long sa = ba >> 63, sb = bb >> 63;
        return ((ba ^ (sa & 0x7fffffffffffffffLL)) - sa) < ((bb ^ (sb & 0x7fffffffffffffffLL)) - sb);
    }
#endif
    return a < b;
}

// ---------------------------------------------------------------------------
// element geometry (lulesh.cc:290-474, 591-663, 1273-1435)
// ---------------------------------------------------------------------------

// Jacobian determinant of CalcElemShapeFunctionDerivatives (lulesh.cc:319-376).
// The reference scales each of the nine sums by 0.125 and the triple
// product by 8; those powers of two combine to one factor 2^-6.  Scaling by a
// power of two is exact, so the value is the reference's bit for bit (for
// coordinates far from the underflow range).
template <typename R>
LG_HD R jacobian_det(const R *x, const R *y, const R *z)
{
    const R fjxxi = ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxet = ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxze = ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    const R fjyxi = ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyet = ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyze = ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    const R fjzxi = ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzet = ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzze = ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    const R cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    const R cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    const R cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    return R(0.015625) * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

// Bits of a double, and a float from its bits, on host and device.
LG_HD unsigned long long bits_of(double v)
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(v);
#else
    unsigned long long b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}
LG_HD float float_of(unsigned u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}

// double -> float toward zero by re-biasing the exponent on the integer pipe
// (off GB300's FP64 pipe): |error| <= 2^-23 |v|; magnitudes below 2^-126
// become zero, above the float range infinity.
LG_HD float f32_trunc(double v)
{
    const unsigned long long b = bits_of(v);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0) return float_of(sign);
    if (e >= 255) return float_of(sign | 0x7f800000u);
    return float_of(sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// True when jacobian_det(x, y, z) in FP64 is certainly positive, decided in
// FP32 with an a-priori error bound; false means "evaluate it in FP64".  The
// reference uses that determinant only for its sign (the VolumeError test of
// CalcVolumeForceForElems, lulesh.cc:1082-1091), so the filter changes no
// result.  Bound, with u = 2^-24 and X the largest coordinate magnitude:
//   * each converted coordinate is off by at most 2u X (+ 2^-126 flushed);
//     each of the nine sums fj (7 roundings of partial sums bounded by 8X)
//     is then off by at most Delta = 80 u X + 2^-120;
//   * the determinant is a sum of six signed triple products of the fj, so
//     input errors move it by at most 18 G^2 Delta (G = max |fj| + Delta),
//     and its FP32 evaluation (with or without contraction) adds at most
//     32 u G^3;
// twice that bound, times the 2^-6 scale, is compared with the FP32 value.
// The FP64 value's own error (~1e-16 relative) is far inside the factor 2.
// NaN or out-of-range inputs give false.
LG_HD bool jacobian_certainly_positive(const double *x, const double *y, const double *z)
{
    float xf[8], yf[8], zf[8];
    float X = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        xf[j] = f32_trunc(x[j]);
        yf[j] = f32_trunc(y[j]);
        zf[j] = f32_trunc(z[j]);
        X = fmaxf(X, fmaxf(fabsf(xf[j]), fmaxf(fabsf(yf[j]), fabsf(zf[j]))));
    }
    const float a = jacobian_det(xf, yf, zf);  // includes the 2^-6 scale
    const float fx0 = (xf[6] - xf[0]) + (xf[5] - xf[3]) - (xf[7] - xf[1]) - (xf[4] - xf[2]);
    const float fx1 = (xf[6] - xf[0]) - (xf[5] - xf[3]) + (xf[7] - xf[1]) - (xf[4] - xf[2]);
    const float fx2 = (xf[6] - xf[0]) + (xf[5] - xf[3]) + (xf[7] - xf[1]) + (xf[4] - xf[2]);
    const float fy0 = (yf[6] - yf[0]) + (yf[5] - yf[3]) - (yf[7] - yf[1]) - (yf[4] - yf[2]);
    const float fy1 = (yf[6] - yf[0]) - (yf[5] - yf[3]) + (yf[7] - yf[1]) - (yf[4] - yf[2]);
    const float fy2 = (yf[6] - yf[0]) + (yf[5] - yf[3]) + (yf[7] - yf[1]) + (yf[4] - yf[2]);
    const float fz0 = (zf[6] - zf[0]) + (zf[5] - zf[3]) - (zf[7] - zf[1]) - (zf[4] - zf[2]);
    const float fz1 = (zf[6] - zf[0]) - (zf[5] - zf[3]) + (zf[7] - zf[1]) - (zf[4] - zf[2]);
    const float fz2 = (zf[6] - zf[0]) + (zf[5] - zf[3]) + (zf[7] - zf[1]) + (zf[4] - zf[2]);
    const float F = fmaxf(fmaxf(fmaxf(fabsf(fx0), fabsf(fx1)), fmaxf(fabsf(fx2), fabsf(fy0))),
                          fmaxf(fmaxf(fabsf(fy1), fabsf(fy2)),
                                fmaxf(fabsf(fz0), fmaxf(fabsf(fz1), fabsf(fz2)))));
    const float u = 5.9604645e-8f;  // 2^-24
    const float delta = 80.f * u * X + 7.5231638e-37f;  // + 2^-120
    const float G = F + delta;
    const float bound = 2.f * 0.015625f * (18.f * G * G * delta + 32.f * u * G * G * G);
    return a > bound;  // false for NaN
}

// CalcElemShapeFunctionDerivatives rows 0..3 of B (rows 4..7 are their
// negatives) and the determinant, lulesh.cc:290-377
template <typename R>
LG_HD R shape_derivs(const R *x, const R *y, const R *z, R bx[4], R by[4],
                                          R bz[4])
{
    const R fjxxi = R(.125) * ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxet = R(.125) * ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxze = R(.125) * ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    const R fjyxi = R(.125) * ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyet = R(.125) * ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyze = R(.125) * ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    const R fjzxi = R(.125) * ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzet = R(.125) * ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzze = R(.125) * ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    const R cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
    const R cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    const R cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
    const R cjyxi = -(fjxet * fjzze) + (fjzet * fjxze);
    const R cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    const R cjyze = -(fjxxi * fjzet) + (fjzxi * fjxet);
    const R cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
    const R cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    const R cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);
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
    return R(8.) * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

// shape_derivs without the reference's power-of-two factors: returns 64 x the
// determinant and fills 64 x rows 0..3 of B.  A velocity gradient formed as
// (1 / det) * (B . v) from these equals the one formed from shape_derivs bit
// for bit, since only powers of two were dropped and they cancel exactly.
// The cofactor part of shape_derivs_x64 from 8 x the Jacobian's columns.
template <typename R>
LG_HD R shape_derivs_x64_jac(R fjxxi, R fjxet, R fjxze, R fjyxi, R fjyet, R fjyze, R fjzxi,
                             R fjzet, R fjzze, R bx[4], R by[4], R bz[4])
{
    const R cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
    const R cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    const R cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
    const R cjyxi = -(fjxet * fjzze) + (fjzet * fjxze);
    const R cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    const R cjyze = -(fjxxi * fjzet) + (fjzxi * fjxet);
    const R cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
    const R cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    const R cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);
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
    return fjxet * cjxet + fjyet * cjyet + fjzet * cjzet;
}

template <typename R>
LG_HD R shape_derivs_x64(const R *x, const R *y, const R *z, R bx[4], R by[4], R bz[4])
{
    const R fjxxi = ((x[6] - x[0]) + (x[5] - x[3]) - (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxet = ((x[6] - x[0]) - (x[5] - x[3]) + (x[7] - x[1]) - (x[4] - x[2]));
    const R fjxze = ((x[6] - x[0]) + (x[5] - x[3]) + (x[7] - x[1]) + (x[4] - x[2]));
    const R fjyxi = ((y[6] - y[0]) + (y[5] - y[3]) - (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyet = ((y[6] - y[0]) - (y[5] - y[3]) + (y[7] - y[1]) - (y[4] - y[2]));
    const R fjyze = ((y[6] - y[0]) + (y[5] - y[3]) + (y[7] - y[1]) + (y[4] - y[2]));
    const R fjzxi = ((z[6] - z[0]) + (z[5] - z[3]) - (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzet = ((z[6] - z[0]) - (z[5] - z[3]) + (z[7] - z[1]) - (z[4] - z[2]));
    const R fjzze = ((z[6] - z[0]) + (z[5] - z[3]) + (z[7] - z[1]) + (z[4] - z[2]));
    return shape_derivs_x64_jac(fjxxi, fjxet, fjxze, fjyxi, fjyet, fjyze, fjzxi, fjzet, fjzze,
                                bx, by, bz);
}

// Area vector of SumElemFaceNormal, lulesh.cc:381-415 (the four corners
// a,b,c,d of a face).  Twice the reference's bisectors are formed; its
// factors 0.5 (each bisector) and 0.25 (the area) are applied once as
// 0.0625.  Powers of two scale exactly, so the area vector is the
// reference's bit for bit.
template <typename R>
LG_HD void face_area(const R *x, const R *y, const R *z, int a, int b, int c, int d, R &areaX,
                     R &areaY, R &areaZ)
{
    const R bisectX0 = (x[d] + x[c] - x[b] - x[a]);
    const R bisectY0 = (y[d] + y[c] - y[b] - y[a]);
    const R bisectZ0 = (z[d] + z[c] - z[b] - z[a]);
    const R bisectX1 = (x[c] + x[b] - x[d] - x[a]);
    const R bisectY1 = (y[c] + y[b] - y[d] - y[a]);
    const R bisectZ1 = (z[c] + z[b] - z[d] - z[a]);
    areaX = R(0.0625) * (bisectY0 * bisectZ1 - bisectZ0 * bisectY1);
    areaY = R(0.0625) * (bisectZ0 * bisectX1 - bisectX0 * bisectZ1);
    areaZ = R(0.0625) * (bisectX0 * bisectY1 - bisectY0 * bisectX1);
}

// SumElemFaceNormal, lulesh.cc:381-415
template <typename R>
LG_HD void face_normal(R *nx, R *ny, R *nz, const R *x, const R *y,
                                            const R *z, int a, int b, int c, int d)
{
    R areaX, areaY, areaZ;
    face_area(x, y, z, a, b, c, d, areaX, areaY, areaZ);
    nx[a] += areaX; nx[b] += areaX; nx[c] += areaX; nx[d] += areaX;
    ny[a] += areaY; ny[b] += areaY; ny[c] += areaY; ny[d] += areaY;
    nz[a] += areaZ; nz[b] += areaZ; nz[c] += areaZ; nz[d] += areaZ;
}

// CalcElemNodeNormals, lulesh.cc:419-474
template <typename R>
LG_HD void node_normals(R *pfx, R *pfy, R *pfz, const R *x, const R *y,
                                             const R *z)
{
#pragma unroll
    for (int i = 0; i < 8; ++i) pfx[i] = pfy[i] = pfz[i] = R(0.0);
    face_normal(pfx, pfy, pfz, x, y, z, 0, 1, 2, 3);
    face_normal(pfx, pfy, pfz, x, y, z, 0, 4, 5, 1);
    face_normal(pfx, pfy, pfz, x, y, z, 1, 5, 6, 2);
    face_normal(pfx, pfy, pfz, x, y, z, 2, 6, 7, 3);
    face_normal(pfx, pfy, pfz, x, y, z, 3, 7, 4, 0);
    face_normal(pfx, pfy, pfz, x, y, z, 4, 7, 6, 5);
}

// 1 / sqrt(a): the device's reciprocal square root (within an ulp or two;
// not the correctly rounded 1 / sqrt(a), so only the FMA build's
// reformulated forms use it), the quotient on the host.
LG_HD double rsqrt_fast(double a)
{
#ifdef __CUDA_ARCH__
    return rsqrt(a);
#else
    return 1.0 / sqrt(a);
#endif
}
LG_HD float rsqrt_fast(float a)
{
#ifdef __CUDA_ARCH__
    return rsqrtf(a);
#else
    return 1.0f / sqrtf(a);
#endif
}

// Body diagonals r6 - r0, r5 - r3, r7 - r1, r4 - r2 of one coordinate.
template <typename R>
LG_HD void body_diagonals(const R *a, R D[4])
{
    D[0] = a[6] - a[0];
    D[1] = a[5] - a[3];
    D[2] = a[7] - a[1];
    D[3] = a[4] - a[2];
}

// An element's xi, eta and zeta differences of one coordinate from its body
// diagonals D: 8 x a column of CalcElemShapeFunctionDerivatives' Jacobian
// (lulesh.cc:304-316 without the factor 1/8) and 4 x the differences of
// CalcMonotonicQGradientsForElems (lulesh.cc:1650-1706 without the 1/4),
// xi = D0 + D1 - D2 - D3, eta = D0 - D1 + D2 - D3, zeta = D0 + D1 + D2 + D3.
// 7 operations for the three, where the node sums take 21; the rounding
// differs from the reference's sums.
template <typename R>
LG_HD void diag_directions(const R D[4], R &xi, R &et, R &ze)
{
    const R s = D[0] + D[1], t = D[2] + D[3], u = D[0] - D[1], w = D[2] - D[3];
    xi = s - t;
    et = u + w;
    ze = s + t;
}

// CalcMonotonicQGradientsForElems for one element from the xi, eta and zeta
// differences of its coordinates (P) and velocities (V), 4 x the reference's
// (diag_directions of the body diagonals; P[3c..3c+2] and V[3c..3c+2] are
// coordinate c's xi, eta, zeta), with the powers of two folded as in
// monoq_gradients<R, true>.
template <typename R>
LG_HD void monoq_gradients_dirs(const R P[9], const R V[9], R vol, R out[6])
{
    const R ptiny_s = R(256.e-36);
    const R norm = (R(1.0) / (vol + R(1.e-36))) * R(0.015625);
    const R vol_s = R(16.0) * vol;
    const R dxi = P[0], dxj = P[1], dxk = P[2], dyi = P[3], dyj = P[4], dyk = P[5];
    const R dzi = P[6], dzj = P[7], dzk = P[8];
    const R vxi = V[0], vxj = V[1], vxk = V[2], vyi = V[3], vyj = V[4], vyk = V[5];
    const R vzi = V[6], vzj = V[7], vzk = V[8];
    // vol / sqrt(|a|^2) by the reciprocal square root, and norm applied to
    // the dot product once
    R ax, ay, az;
    ax = dyi * dzj - dzi * dyj;
    ay = dzi * dxj - dxi * dzj;
    az = dxi * dyj - dyi * dxj;
    out[2] = vol_s * rsqrt_fast(ax * ax + ay * ay + az * az + ptiny_s);
    out[5] = norm * (ax * vxk + ay * vyk + az * vzk);
    ax = dyj * dzk - dzj * dyk;
    ay = dzj * dxk - dxj * dzk;
    az = dxj * dyk - dyj * dxk;
    out[0] = vol_s * rsqrt_fast(ax * ax + ay * ay + az * az + ptiny_s);
    out[3] = norm * (ax * vxi + ay * vyi + az * vzi);
    ax = dyk * dzi - dzk * dyi;
    ay = dzk * dxi - dxk * dzi;
    az = dxk * dyi - dyk * dxi;
    out[1] = vol_s * rsqrt_fast(ax * ax + ay * ay + az * az + ptiny_s);
    out[4] = norm * (ax * vxj + ay * vyj + az * vzj);
}

// The xi, eta, zeta differences of the three coordinates from their body
// diagonals, in monoq_gradients_dirs' layout.
template <typename R>
LG_HD void directions3(const R *Dx, const R *Dy, const R *Dz, R P[9])
{
    diag_directions(Dx, P[0], P[1], P[2]);
    diag_directions(Dy, P[3], P[4], P[5]);
    diag_directions(Dz, P[6], P[7], P[8]);
}

// CalcMonotonicQGradientsForElems for one element from the body diagonals of
// its coordinates (Dx, Dy, Dz) and velocities (Ex, Ey, Ez).
template <typename R>
LG_HD void monoq_gradients_diag(const R *Dx, const R *Dy, const R *Dz, const R *Ex, const R *Ey,
                                const R *Ez, R vol, R out[6])
{
    R P[9], V[9];
    directions3(Dx, Dy, Dz, P);
    directions3(Ex, Ey, Ez, V);
    monoq_gradients_dirs(P, V, vol, out);
}

// dxx + dyy + dzz of CalcElemVelocityGradient (lulesh.cc:1437-1500) with the
// B matrix and determinant of CalcElemShapeFunctionDerivatives (290-377) at
// the half-step coordinates x - dt2 v (CalcKinematicsForElems, 1540-1556),
// from the xi, eta, zeta differences P of the coordinates and V of the
// velocities (monoq_gradients_dirs' layout):
// * diag_directions is linear, so 8 x the half-step Jacobian is P - dt2 V;
// * a row of B is the Jacobian's cofactor row c times the shape functions'
//   sign pattern, and summed against the velocity differences
//   v0 - v6, v1 - v7, v2 - v4, v3 - v5 that pattern gives the velocity's own
//   xi, eta, zeta differences: dxx = (c_x . V_x) / detJ, and so on.
// The cofactors are 64 x and the determinant 512 x the reference's (which is
// 8 x det J); the factor 64 cancels in the quotient.  Equal to the
// reference's trace in exact arithmetic; the rounding differs.
template <typename R>
LG_HD R velocity_trace_dirs(const R P[9], const R V[9], R dt2)
{
    const R fxi = P[0] - dt2 * V[0], fxe = P[1] - dt2 * V[1], fxz = P[2] - dt2 * V[2];
    const R fyi = P[3] - dt2 * V[3], fye = P[4] - dt2 * V[4], fyz = P[5] - dt2 * V[5];
    const R fzi = P[6] - dt2 * V[6], fze = P[7] - dt2 * V[7], fzz = P[8] - dt2 * V[8];
    const R cxi = (fye * fzz) - (fze * fyz);
    const R cxe = -(fyi * fzz) + (fzi * fyz);
    const R cxz = (fyi * fze) - (fzi * fye);
    const R cyi = -(fxe * fzz) + (fze * fxz);
    const R cye = (fxi * fzz) - (fzi * fxz);
    const R cyz = -(fxi * fze) + (fzi * fxe);
    const R czi = (fxe * fyz) - (fye * fxz);
    const R cze = -(fxi * fyz) + (fyi * fxz);
    const R czz = (fxi * fye) - (fyi * fxe);
    const R det = fxe * cxe + fye * cye + fze * cze;
    const R tr = (cxi * V[0] + cxe * V[1] + cxz * V[2]) + (cyi * V[3] + cye * V[4] + cyz * V[5]) +
                 (czi * V[6] + cze * V[7] + czz * V[8]);
    // the reciprocal, not tr / det: tr is 0 for an element at rest, and a
    // zero dividend takes the quotient's slow special-operand path
    return tr * (R(1.0) / det);
}

// 8 x the node normals of CalcElemNodeNormals from the faces' diagonals: the
// reference's bisectors of face (a, b, c, d) are (p + q) / 2 and (p - q) / 2
// for p = r_c - r_a, q = r_d - r_b, so its area vector
// 0.25 (p + q)/2 x (p - q)/2 equals (q x p) / 8 in exact arithmetic.  Each
// node sums its three faces' q x p in the reference's face order, starting
// from the first face instead of from 0.0 (equal but for the sign of an
// all-zero sum); the caller
// applies the factor 1/8 (an exact power of two) once.  12 operations per
// face instead of 27; the rounding differs from the reference's.
template <typename R>
LG_HD void node_normals_x8(R *pfx, R *pfy, R *pfz, const R *x, const R *y, const R *z)
{
    R ax[6], ay[6], az[6];
    constexpr int F[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                             {2, 6, 7, 3}, {3, 7, 4, 0}, {4, 7, 6, 5}};
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const int a = F[f][0], b = F[f][1], c = F[f][2], d = F[f][3];
        const R px = x[c] - x[a], py = y[c] - y[a], pz = z[c] - z[a];
        const R qx = x[d] - x[b], qy = y[d] - y[b], qz = z[d] - z[b];
        ax[f] = qy * pz - qz * py;
        ay[f] = qz * px - qx * pz;
        az[f] = qx * py - qy * px;
    }
#define LG_NN(P, A)                                 \
    P[0] = (A[0] + A[1]) + A[4];                    \
    P[1] = (A[0] + A[1]) + A[2];                    \
    P[2] = (A[0] + A[2]) + A[3];                    \
    P[3] = (A[0] + A[3]) + A[4];                    \
    P[4] = (A[1] + A[4]) + A[5];                    \
    P[5] = (A[1] + A[2]) + A[5];                    \
    P[6] = (A[2] + A[3]) + A[5];                    \
    P[7] = (A[3] + A[4]) + A[5];
    LG_NN(pfx, ax)
    LG_NN(pfy, ay)
    LG_NN(pfz, az)
#undef LG_NN
}

// The twelve differences of CalcElemVolume (lulesh.cc:1274-1356) for one
// coordinate; they are also the element's twelve face diagonals.  Order:
// 0 d20, 1 d31, 2 d50, 3 d14, 4 d61, 5 d25, 6 d72, 7 d63, 8 d43, 9 d70,
// 10 d64, 11 d57 (dab = r_a - r_b).
template <typename R>
LG_HD void elem_differences(const R *a, R d[12])
{
    d[0] = a[2] - a[0];
    d[1] = a[3] - a[1];
    d[2] = a[5] - a[0];
    d[3] = a[1] - a[4];
    d[4] = a[6] - a[1];
    d[5] = a[2] - a[5];
    d[6] = a[7] - a[2];
    d[7] = a[6] - a[3];
    d[8] = a[4] - a[3];
    d[9] = a[7] - a[0];
    d[10] = a[6] - a[4];
    d[11] = a[5] - a[7];
}

// node_normals_x8 from elem_differences: face (a, b, c, d) has area vector
// 8 (q x p) with p = r_c - r_a, q = r_d - r_b, which are (up to sign) two of
// the twelve differences.  The same operations as node_normals_x8.
template <typename R>
LG_HD void node_normals_x8_diff(R *pfx, R *pfy, R *pfz, const R *dx, const R *dy, const R *dz)
{
    // (q, p) per face; q x p = p x (-q) where q is the negated difference
    constexpr int Q[6] = {1, 3, 5, 6, 8, 11}, P[6] = {0, 2, 4, 7, 9, 10};
    R ax[6], ay[6], az[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        const int q = Q[f], p = P[f];
        ax[f] = dy[q] * dz[p] - dz[q] * dy[p];
        ay[f] = dz[q] * dx[p] - dx[q] * dz[p];
        az[f] = dx[q] * dy[p] - dy[q] * dx[p];
    }
#define LG_NN(P_, A)                                \
    P_[0] = (A[0] + A[1]) + A[4];                   \
    P_[1] = (A[0] + A[1]) + A[2];                   \
    P_[2] = (A[0] + A[2]) + A[3];                   \
    P_[3] = (A[0] + A[3]) + A[4];                   \
    P_[4] = (A[1] + A[4]) + A[5];                   \
    P_[5] = (A[1] + A[2]) + A[5];                   \
    P_[6] = (A[2] + A[3]) + A[5];                   \
    P_[7] = (A[3] + A[4]) + A[5];
    LG_NN(pfx, ax)
    LG_NN(pfy, ay)
    LG_NN(pfz, az)
#undef LG_NN
}

// 12 x the volume gradient (CalcElemVolumeDerivative without its 1/12,
// lulesh.cc:591-663) from elem_differences.  CalcElemVolume is
// (1/12) sum_k a_k . (b_k x c_k) with (a, b, c) = (d31 + d72, d63, d20),
// (d43 + d57, d64, d70), (d14 + d25, d61, d50); its gradient is, per node,
// a signed sum of X_k = b_k x c_k, Y_k = c_k x a_k and Z_k = a_k x b_k:
// nine cross products where the reference's VoluDer forms 24.  Equal to
// volume_derivative<R, false> in exact arithmetic; the rounding differs.
template <typename R>
LG_HD void volume_gradient_x12_diff(const R *dx, const R *dy, const R *dz, R *gx, R *gy, R *gz)
{
    const R a1x = dx[1] + dx[6], a1y = dy[1] + dy[6], a1z = dz[1] + dz[6];
    const R a2x = dx[8] + dx[11], a2y = dy[8] + dy[11], a2z = dz[8] + dz[11];
    const R a3x = dx[3] + dx[5], a3y = dy[3] + dy[5], a3z = dz[3] + dz[5];
#define LG_CR(N, ux, uy, uz, vx, vy, vz)                                             \
    const R N##x = (uy) * (vz) - (uz) * (vy), N##y = (uz) * (vx) - (ux) * (vz),      \
            N##z = (ux) * (vy) - (uy) * (vx);
    // k = 1: b = d63 (7), c = d20 (0)
    LG_CR(X1, dx[7], dy[7], dz[7], dx[0], dy[0], dz[0])
    LG_CR(Y1, dx[0], dy[0], dz[0], a1x, a1y, a1z)
    LG_CR(Z1, a1x, a1y, a1z, dx[7], dy[7], dz[7])
    // k = 2: b = d64 (10), c = d70 (9)
    LG_CR(X2, dx[10], dy[10], dz[10], dx[9], dy[9], dz[9])
    LG_CR(Y2, dx[9], dy[9], dz[9], a2x, a2y, a2z)
    LG_CR(Z2, a2x, a2y, a2z, dx[10], dy[10], dz[10])
    // k = 3: b = d61 (4), c = d50 (2)
    LG_CR(X3, dx[4], dy[4], dz[4], dx[2], dy[2], dz[2])
    LG_CR(Y3, dx[2], dy[2], dz[2], a3x, a3y, a3z)
    LG_CR(Z3, a3x, a3y, a3z, dx[4], dy[4], dz[4])
#undef LG_CR
#define LG_G(C)                                     \
    g##C[0] = -Z1##C - Z2##C - Z3##C;               \
    g##C[1] = -X1##C + X3##C - Y3##C;               \
    g##C[2] = -X1##C + Z1##C + X3##C;               \
    g##C[3] = X1##C - Y1##C - X2##C;                \
    g##C[4] = X2##C - Y2##C - X3##C;                \
    g##C[5] = X2##C - X3##C + Z3##C;                \
    g##C[6] = Y1##C + Y2##C + Y3##C;                \
    g##C[7] = X1##C - X2##C + Z2##C;
    LG_G(x)
    LG_G(y)
    LG_G(z)
#undef LG_G
}

// The four hourglass mode sums sum_k gam(m, k) * v[k] of CalcFBHourglassForceForElems
// (lulesh.cc:894-920) by a pairwise butterfly: 18 additions instead of 28.
// The FMA build uses it; it rounds differently from the left-to-right sums.
template <typename R>
LG_HD void hourglass_modes(const R *v, R m[4])
{
    const R s01 = v[0] + v[1], d01 = v[0] - v[1];
    const R s23 = v[2] + v[3], d23 = v[2] - v[3];
    const R s45 = v[4] + v[5], d45 = v[4] - v[5];
    const R s67 = v[6] + v[7], d67 = v[6] - v[7];
    const R a = d01 + d67, b = d23 + d45;
    m[0] = (s01 + s67) - (s23 + s45);
    m[1] = a - b;
    m[2] = a + b;
    m[3] = (d45 + d67) - (d01 + d23);
}

// VoluDer, lulesh.cc:591-619, for corner k of CalcElemVolumeDerivative
// (lulesh.cc:623-663) with neighbour nodes m0..m5
// (kScale = false leaves out the final factor 1/12: 12 x dV/dx)
template <typename R, bool kScale = true>
LG_HD void volu_der(const R *x, const R *y, const R *z, int m0, int m1, int m2,
                                         int m3, int m4, int m5, R &dvdx, R &dvdy, R &dvdz)
{
    const R twelfth = R(1.0) / R(12.0);
    const R x0 = x[m0], x1 = x[m1], x2 = x[m2], x3 = x[m3], x4 = x[m4], x5 = x[m5];
    const R y0 = y[m0], y1 = y[m1], y2 = y[m2], y3 = y[m3], y4 = y[m4], y5 = y[m5];
    const R z0 = z[m0], z1 = z[m1], z2 = z[m2], z3 = z[m3], z4 = z[m4], z5 = z[m5];
    dvdx = (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) + (y0 + y4) * (z3 + z4) -
           (y3 + y4) * (z0 + z4) - (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    dvdy = -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) - (x0 + x4) * (z3 + z4) +
           (x3 + x4) * (z0 + z4) + (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    dvdz = -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) - (y0 + y4) * (x3 + x4) +
           (y3 + y4) * (x0 + x4) + (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
    if (kScale) {
        dvdx *= twelfth;
        dvdy *= twelfth;
        dvdz *= twelfth;
    }
}

template <typename R, bool kScale = true>
LG_HD void volume_derivative(const R *x, const R *y, const R *z, R *dvdx,
                                                  R *dvdy, R *dvdz)
{
    volu_der<R, kScale>(x, y, z, 1, 2, 3, 4, 5, 7, dvdx[0], dvdy[0], dvdz[0]);
    volu_der<R, kScale>(x, y, z, 0, 1, 2, 7, 4, 6, dvdx[3], dvdy[3], dvdz[3]);
    volu_der<R, kScale>(x, y, z, 3, 0, 1, 6, 7, 5, dvdx[2], dvdy[2], dvdz[2]);
    volu_der<R, kScale>(x, y, z, 2, 3, 0, 5, 6, 4, dvdx[1], dvdy[1], dvdz[1]);
    volu_der<R, kScale>(x, y, z, 7, 6, 5, 0, 3, 1, dvdx[4], dvdy[4], dvdz[4]);
    volu_der<R, kScale>(x, y, z, 4, 7, 6, 1, 0, 2, dvdx[5], dvdy[5], dvdz[5]);
    volu_der<R, kScale>(x, y, z, 5, 4, 7, 2, 1, 3, dvdx[6], dvdy[6], dvdz[6]);
    volu_der<R, kScale>(x, y, z, 6, 5, 4, 3, 2, 0, dvdx[7], dvdy[7], dvdz[7]);
}

// CalcElemVolume, lulesh.cc:1273-1356
template <typename R>
LG_HD R elem_volume(const R *x, const R *y, const R *z)
{
    const R twelveth = R(1.0) / R(12.0);
    const R dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    const R dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    const R dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    const R dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    const R dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    const R dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    const R dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    const R dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    const R dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    const R dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    const R dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    const R dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
#define LG_TP(a1, b1, c1, a2, b2, c2, a3, b3, c3) \
    ((a1) * ((b2) * (c3) - (c2) * (b3)) + (a2) * ((c1) * (b3) - (b1) * (c3)) + \
     (a3) * ((b1) * (c2) - (c1) * (b2)))
    R volume =
        LG_TP(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
        LG_TP(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
        LG_TP(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
#undef LG_TP
    volume *= twelveth;
    return volume;
}

// AreaFace, lulesh.cc:1370-1390
template <typename R>
LG_HD R area_face(const R *x, const R *y, const R *z, int a, int b, int c,
                                       int d)
{
    const R fx = (x[c] - x[a]) - (x[d] - x[b]);
    const R fy = (y[c] - y[a]) - (y[d] - y[b]);
    const R fz = (z[c] - z[a]) - (z[d] - z[b]);
    const R gx = (x[c] - x[a]) + (x[d] - x[b]);
    const R gy = (y[c] - y[a]) + (y[d] - y[b]);
    const R gz = (z[c] - z[a]) + (z[d] - z[b]);
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) -
           (fx * gx + fy * gy + fz * gz) * (fx * gx + fy * gy + fz * gz);
}

// A quarter of AreaFace from the face's diagonals p = r_c - r_a and
// q = r_d - r_b: with f = p - q and g = p + q, |f|^2 |g|^2 - (f.g)^2 equals
// 4 |p x q|^2 in exact arithmetic.  15 operations instead of 23; the
// rounding differs from the reference's expression.
template <typename R>
LG_HD R area_face_cross(const R *x, const R *y, const R *z, int a, int b, int c, int d)
{
    const R px = x[c] - x[a], py = y[c] - y[a], pz = z[c] - z[a];
    const R qx = x[d] - x[b], qy = y[d] - y[b], qz = z[d] - z[b];
    const R cx = py * qz - pz * qy, cy = pz * qx - px * qz, cz = px * qy - py * qx;
    return cx * cx + cy * cy + cz * cz;
}

// CalcElemCharacteristicLength, lulesh.cc:1394-1435 (std::max(a,b) is
// (a < b) ? b : a).  kCross (the FMA build) takes the face areas from
// area_face_cross: the maximum of a quarter of each area, and
// 4 v / sqrt(4 m) = 2 v / sqrt(m), the factor 4 only shifting exponents,
// evaluated as 2 v rsqrt(m).  Three faces are walked in the opposite sense
// (4,7,6,5 for 4,5,6,7; 0,4,5,1 for 0,1,5,4; 1,5,6,2 for 1,2,6,5), which
// negates one diagonal and leaves |p x q|^2 unchanged bit for bit: every
// diagonal is then one of elem_volume's differences with its sign, and
// the compiler shares them.
template <typename R, bool kCross = false>
LG_HD R char_length(const R *x, const R *y, const R *z, R volume)
{
    if (kCross) {
        R m = R(0.0), a;
        a = area_face_cross(x, y, z, 0, 1, 2, 3); m = lt(a, m) ? m : a;
        a = area_face_cross(x, y, z, 4, 7, 6, 5); m = lt(a, m) ? m : a;
        a = area_face_cross(x, y, z, 0, 4, 5, 1); m = lt(a, m) ? m : a;
        a = area_face_cross(x, y, z, 1, 5, 6, 2); m = lt(a, m) ? m : a;
        a = area_face_cross(x, y, z, 2, 3, 7, 6); m = lt(a, m) ? m : a;
        a = area_face_cross(x, y, z, 3, 0, 4, 7); m = lt(a, m) ? m : a;
        return R(2.0) * volume * rsqrt_fast(m);
    }
    R cl = R(0.0), a;
    a = area_face(x, y, z, 0, 1, 2, 3); cl = lt(a, cl) ? cl : a;
    a = area_face(x, y, z, 4, 5, 6, 7); cl = lt(a, cl) ? cl : a;
    a = area_face(x, y, z, 0, 1, 5, 4); cl = lt(a, cl) ? cl : a;
    a = area_face(x, y, z, 1, 2, 6, 5); cl = lt(a, cl) ? cl : a;
    a = area_face(x, y, z, 2, 3, 7, 6); cl = lt(a, cl) ? cl : a;
    a = area_face(x, y, z, 3, 0, 4, 7); cl = lt(a, cl) ? cl : a;
    return R(4.0) * volume / sqrt(cl);
}

// CalcMonotonicQGradientsForElems for one element (lulesh.cc:1613-1757):
// out = {delx_xi, delx_eta, delx_zeta, delv_xi, delv_eta, delv_zeta}.
// kFold drops the reference's factors 0.25 on the eighteen coordinate and
// velocity differences and compensates with exact powers of two (16 on the
// length numerator with 256 x ptiny under the root, 1/64 on norm): without
// contraction every output is the reference's bit for bit.  kFold = false is
// the reference's formulation.
template <typename R, bool kFold>
LG_HD void monoq_gradients(const R *x, const R *y, const R *z, const R *xv, const R *yv,
                           const R *zv, R vol, R out[6])
{
    const R q = kFold ? R(1) : R(.25);
    const R ptiny_s = kFold ? R(256.e-36) : R(1.e-36);
    const R norm = kFold ? (R(1.0) / (vol + R(1.e-36))) * R(0.015625) : R(1.0) / (vol + R(1.e-36));
    const R vol_s = kFold ? R(16.0) * vol : vol;
#define S4(A, a, b, c, d) (A[a] + A[b] + A[c] + A[d])
#define SC(e) (kFold ? (e) : q * (e))
    const R dxj = SC(-(S4(x, 0, 1, 5, 4) - S4(x, 3, 2, 6, 7)));
    const R dyj = SC(-(S4(y, 0, 1, 5, 4) - S4(y, 3, 2, 6, 7)));
    const R dzj = SC(-(S4(z, 0, 1, 5, 4) - S4(z, 3, 2, 6, 7)));
    const R dxi = SC((S4(x, 1, 2, 6, 5) - S4(x, 0, 3, 7, 4)));
    const R dyi = SC((S4(y, 1, 2, 6, 5) - S4(y, 0, 3, 7, 4)));
    const R dzi = SC((S4(z, 1, 2, 6, 5) - S4(z, 0, 3, 7, 4)));
    const R dxk = SC((S4(x, 4, 5, 6, 7) - S4(x, 0, 1, 2, 3)));
    const R dyk = SC((S4(y, 4, 5, 6, 7) - S4(y, 0, 1, 2, 3)));
    const R dzk = SC((S4(z, 4, 5, 6, 7) - S4(z, 0, 1, 2, 3)));
    R ax, ay, az, dxv, dyv, dzv;

    ax = dyi * dzj - dzi * dyj;
    ay = dzi * dxj - dxi * dzj;
    az = dxi * dyj - dyi * dxj;
    out[2] = vol_s / sqrt(ax * ax + ay * ay + az * az + ptiny_s);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = SC((S4(xv, 4, 5, 6, 7) - S4(xv, 0, 1, 2, 3)));
    dyv = SC((S4(yv, 4, 5, 6, 7) - S4(yv, 0, 1, 2, 3)));
    dzv = SC((S4(zv, 4, 5, 6, 7) - S4(zv, 0, 1, 2, 3)));
    out[5] = ax * dxv + ay * dyv + az * dzv;

    ax = dyj * dzk - dzj * dyk;
    ay = dzj * dxk - dxj * dzk;
    az = dxj * dyk - dyj * dxk;
    out[0] = vol_s / sqrt(ax * ax + ay * ay + az * az + ptiny_s);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = SC((S4(xv, 1, 2, 6, 5) - S4(xv, 0, 3, 7, 4)));
    dyv = SC((S4(yv, 1, 2, 6, 5) - S4(yv, 0, 3, 7, 4)));
    dzv = SC((S4(zv, 1, 2, 6, 5) - S4(zv, 0, 3, 7, 4)));
    out[3] = ax * dxv + ay * dyv + az * dzv;

    ax = dyk * dzi - dzk * dyi;
    ay = dzk * dxi - dxk * dzi;
    az = dxk * dyi - dyk * dxi;
    out[1] = vol_s / sqrt(ax * ax + ay * ay + az * az + ptiny_s);
    ax *= norm;
    ay *= norm;
    az *= norm;
    dxv = SC(-(S4(xv, 0, 1, 5, 4) - S4(xv, 3, 2, 6, 7)));
    dyv = SC(-(S4(yv, 0, 1, 5, 4) - S4(yv, 3, 2, 6, 7)));
    dzv = SC(-(S4(zv, 0, 1, 5, 4) - S4(zv, 3, 2, 6, 7)));
    out[4] = ax * dxv + ay * dyv + az * dzv;
#undef SC
#undef S4
}

// hourglass base vectors, lulesh.cc:743-776
template <typename R = double>
LG_HD constexpr R gam(int mode, int k)
{
    constexpr signed char G[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1},
                                     {1, -1, -1, 1, -1, 1, 1, -1},
                                     {1, -1, 1, -1, 1, -1, 1, -1},
                                     {-1, 1, -1, 1, 1, -1, 1, -1}};
    return (R)G[mode][k];
}

}  // namespace geom
}  // namespace lg
