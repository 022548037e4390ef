// lg_cycle_common.cuh -- the cycle's control logic and the per-element EOS,
// shared by the FP64 and mixed kernel sets.  Included once per kernel
// translation unit inside namespace lg::LG_NS (each unit is compiled with its
// own FMA setting).
#pragma once

#include <cuda_runtime.h>

#include "lg_device.h"

#ifndef LG_NS
#error "define LG_NS"
#endif

namespace lg {
namespace LG_NS {

constexpr int kBlock = 128;
// k_material's block when it runs one item per element (the dt partials are
// sized for blocks of kBlock, so kMatBlock must not be smaller)
constexpr int kMatBlock = 256;

// Keeps the compiler from treating a value as loop-invariant, so that every
// EOS repetition the reference performs is evaluated.
__device__ __forceinline__ void opaque(double &v) { asm volatile("" : "+d"(v)); }

__device__ __forceinline__ void raise_status(Ctl *c, int code) { atomicCAS(&c->status, 0, code); }

// TimeIncrement, lulesh.cc:166-222 (or the frozen step of this cycle)
__device__ __forceinline__ void time_increment(Ctl *c)
{
    if (c->dt_frozen && c->cycle < c->dt_frozen_len) {
        c->deltatime = c->dt_frozen[c->cycle];
        c->time += c->deltatime;
        ++c->cycle;
        return;
    }
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
    if (c->dt_record && c->cycle < c->dt_record_len) c->dt_record[c->cycle] = c->deltatime;
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
// k_material
// ---------------------------------------------------------------------------

// Exact comparisons of doubles on the integer pipe.  On GB300 an FP64
// comparison occupies the FP64 pipe like an FMA, and the FP64 pipe bounds
// every FP64 kernel here.  The results equal IEEE comparisons for operands
// that are not NaN (the cycle stops on a volume error before a NaN can
// form).  dkey() maps a double to a signed integer of the same order, with
// -0 and +0 both at 0 since they compare equal.
__device__ __forceinline__ long long dkey(double v)
{
    const long long b = __double_as_longlong(v);
    const long long sgn = b >> 63;  // 0 or -1
    return (b ^ (sgn & 0x7fffffffffffffffLL)) - sgn;
}
__device__ __forceinline__ bool dlt(double a, double b) { return dkey(a) < dkey(b); }
// a + 0.0 for a not NaN: a, except -0 -> +0
__device__ __forceinline__ double plus_zero(double a)
{
    return __double_as_longlong(a) == (long long)0x8000000000000000ULL ? 0.0 : a;
}
__device__ __forceinline__ bool dle(double a, double b) { return dkey(a) <= dkey(b); }
// |a| < b for b >= +0: the magnitude bits order like the magnitudes
__device__ __forceinline__ bool dabs_lt(double a, double b)
{
    return (__double_as_longlong(a) & 0x7fffffffffffffffLL) < __double_as_longlong(b);
}
// a != 0 (true for NaN, as in IEEE)
__device__ __forceinline__ bool dnz(double a)
{
    return ((unsigned long long)__double_as_longlong(a) << 1) != 0ull;
}
// a < b in the arithmetic type of the limiter
__device__ __forceinline__ bool less(float a, float b) { return a < b; }
__device__ __forceinline__ bool less(double a, double b) { return dlt(a, b); }

// one direction of CalcMonotonicQRegionForElems, lulesh.cc:1778-1813
template <typename R>
__device__ __forceinline__ R monoq_phi(R limiter_mult, R max_slope, const R *dv, int ielem, int bc,
                                       int msymm, int mfree, int mmask, int psymm, int pfree,
                                       int pmask, int nbm, int nbp)
{
    const R ptiny = R(1.e-36);
    R delvm, delvp;
    const R self = dv[ielem];
    const R norm = R(1.) / (self + ptiny);
    const int bm = bc & mmask, bp = bc & pmask;
    if (bm == msymm)
        delvm = self;
    else if (bm == mfree)
        delvm = R(0.0);
    else if (bm == 0 || bm == (mmask & ~(msymm | mfree)))
        delvm = dv[nbm];
    else
        delvm = R(0);
    if (bp == psymm)
        delvp = self;
    else if (bp == pfree)
        delvp = R(0.0);
    else if (bp == 0 || bp == (pmask & ~(psymm | pfree)))
        delvp = dv[nbp];
    else
        delvp = R(0);
    delvm = delvm * norm;
    delvp = delvp * norm;
    R phi = R(.5) * (delvm + delvp);
    delvm *= limiter_mult;
    delvp *= limiter_mult;
    if (less(delvm, phi)) phi = delvm;
    if (less(delvp, phi)) phi = delvp;
    if (less(phi, R(0.))) phi = R(0.);
    if (less(max_slope, phi)) phi = max_slope;
    return phi;
}

// The FP64 builds' arithmetic for the EOS: IEEE division and square root, and
// comparisons on the integer pipe (dlt, dle, dabs_lt; the IEEE results for
// every non-NaN operand).  lg_fastmath.cuh has the mixed path's variant with
// the same interface.
struct IeeeOps {
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }
    static __device__ __forceinline__ bool lt(double a, double b) { return dlt(a, b); }
    static __device__ __forceinline__ bool le(double a, double b) { return dle(a, b); }
    // |a| < b for b >= +0
    static __device__ __forceinline__ bool abs_lt(double a, double b) { return dabs_lt(a, b); }
    // the sound-speed numerator of CalcSoundSpeedForElems (lulesh.cc:2190),
    // in the reference's operation order (contracted only by the FMA build)
    static __device__ __forceinline__ double ss_num(double pbvc, double e, double v, double bvc,
                                                    double p)
    {
        return pbvc * e + v * v * bvc * p;
    }
};

// refdens == 1 exactly (every problem the reference sets up): x / refdens
// is then x, and the sound-speed terms skip the division.  The decision is
// taken once, outside the repetitions: a per-term select let the compiler
// evaluate the quotient anyway, and for elements at rest (numerator 0) that
// quotient takes the division's long special-operand path.
__device__ __forceinline__ bool unit_refdens(const Params &P)
{
    return __double_as_longlong(P.refdens) == 0x3ff0000000000000LL;
}

// sound-speed term of lulesh.cc:2083-2090, 2126-2133, 2158-2165, 2190-2197
template <class M = IeeeOps, bool kUnitRho = false>
__device__ __forceinline__ double ssc_of(double num, double rho0)
{
    const double ssc = kUnitRho ? num : M::div(num, rho0);
    // Elements at rest take the floor.  A predicated square root would still
    // occupy the FP64 pipe for a warp of them, so the sequence runs only when
    // a converged lane of the warp needs it.  The barrier on its operand keeps
    // the compiler from hoisting the root above the vote, where it would run
    // for every warp.
    const bool floor = M::le(ssc, .1111111e-36);
    double r = .3333333e-18;
    if (__any_sync(__activemask(), !floor)) {
        double a = floor ? 1.0 : ssc;
        opaque(a);
        const double t = M::sqrt_(a);
        if (!floor) r = t;
    }
    return r;
}

// CalcPressureForElems for one element, lulesh.cc:2014-2044
template <class M = IeeeOps>
__device__ __forceinline__ double pressure(const Params &P, double &bvc, double &pbvc,
                                           double e_old, double compression, double vnewc)
{
    const double c1s = 2.0 / 3.0;
    bvc = c1s * (compression + 1.);
    pbvc = c1s;
    double p_new = bvc * e_old;
    if (M::abs_lt(p_new, P.p_cut)) p_new = 0.0;
    if (M::le(P.eosvmax, vnewc)) p_new = 0.0;  // vnewc >= eosvmax
    if (M::lt(p_new, P.pmin)) p_new = P.pmin;
    return p_new;
}

// The results of an element's EOS repetitions: the last repetition's
// pressure, energy and viscosity, and the bulk-viscosity terms bvc, pbvc the
// sound speed is computed from.
struct EosOut {
    double p, e, q, bvc, pbvc;
};

// The rep repetitions of CalcEnergyForElems (lulesh.cc:2048-2176) with
// CalcPressureForElems (2014-2044), as EvalEOSForElems runs them for one
// element (2204-2324).  Every repetition is evaluated, as in the reference.
template <class M, bool kUnitRho>
__device__ __forceinline__ EosOut eos_reps_rho(const Params &P, double e_in, double delv_in,
                                               double p_in, double q_in, double qq_in,
                                               double ql_in, double vnewc, int rep)
{
    const double rho0 = P.refdens;
    double p_new = 0., e_new = 0., q_new = 0., bvc = 0., pbvc = 0.;
    for (int j = 0; j < rep; j++) {
        double e_old = e_in, delvc = delv_in, p_old = p_in, q_old = q_in, qq_old = qq_in,
               ql_old = ql_in, vc = vnewc;
        opaque(e_old); opaque(delvc); opaque(p_old); opaque(q_old);
        opaque(qq_old); opaque(ql_old); opaque(vc);
        double compression = M::div(1., vc) - 1.;
        const double vchalf = vc - delvc * .5;
        double compHalfStep = M::div(1., vchalf) - 1.;
        if (dnz(P.eosvmin) && M::le(vc, P.eosvmin)) compHalfStep = compression;
        if (dnz(P.eosvmax) && M::le(P.eosvmax, vc)) {
            p_old = 0.;
            compression = 0.;
            compHalfStep = 0.;
        }
        // The reference adds .5 * work with work = 0 (lulesh.cc:2065, 2103, 2286):
        // x + 0.0 is x except that -0 becomes +0, which plus_zero does on the
        // integer pipe.
        e_new = plus_zero(e_old - .5 * delvc * (p_old + q_old));
        if (M::lt(e_new, P.emin)) e_new = P.emin;

        const double pHalfStep = pressure<M>(P, bvc, pbvc, e_new, compHalfStep, vc);
        const double vhalf = M::div(1., 1. + compHalfStep);
        if (M::lt(0., delvc)) {
            q_new = 0.;
        } else {
            const double ssc = ssc_of<M, kUnitRho>(pbvc * e_new + vhalf * vhalf * bvc * pHalfStep, rho0);
            q_new = (ssc * ql_old + qq_old);
        }
        e_new = e_new + .5 * delvc * (3.0 * (p_old + q_old) - 4.0 * (pHalfStep + q_new));

        e_new = plus_zero(e_new);
        if (M::abs_lt(e_new, P.e_cut)) e_new = 0.;
        if (M::lt(e_new, P.emin)) e_new = P.emin;

        p_new = pressure<M>(P, bvc, pbvc, e_new, compression, vc);
        {
            const double sixth = 1.0 / 6.0;
            double q_tilde;
            if (M::lt(0., delvc)) {
                q_tilde = 0.;
            } else {
                const double ssc = ssc_of<M, kUnitRho>(pbvc * e_new + vc * vc * bvc * p_new, rho0);
                q_tilde = (ssc * ql_old + qq_old);
            }
            e_new = e_new - (7.0 * (p_old + q_old) - 8.0 * (pHalfStep + q_new) +
                             (p_new + q_tilde)) * delvc * sixth;
            if (M::abs_lt(e_new, P.e_cut)) e_new = 0.;
            if (M::lt(e_new, P.emin)) e_new = P.emin;
        }

        p_new = pressure<M>(P, bvc, pbvc, e_new, compression, vc);
        if (M::le(delvc, 0.)) {
            const double ssc = ssc_of<M, kUnitRho>(pbvc * e_new + vc * vc * bvc * p_new, rho0);
            q_new = (ssc * ql_old + qq_old);
            if (M::abs_lt(q_new, P.q_cut)) q_new = 0.;
        }
    }
    return {p_new, e_new, q_new, bvc, pbvc};
}

template <class M = IeeeOps>
__device__ __forceinline__ EosOut eos_reps(const Params &P, double e_in, double delv_in,
                                           double p_in, double q_in, double qq_in,
                                           double ql_in, double vnewc, int rep)
{
    if (unit_refdens(P))
        return eos_reps_rho<M, true>(P, e_in, delv_in, p_in, q_in, qq_in, ql_in, vnewc, rep);
    return eos_reps_rho<M, false>(P, e_in, delv_in, p_in, q_in, qq_in, ql_in, vnewc, rep);
}

// CalcSoundSpeedForElems for one element (lulesh.cc:2180-2200).
template <class M = IeeeOps>
__device__ __forceinline__ double eos_sound_speed(const Params &P, const EosOut &o, double vnewc)
{
    const double num = M::ss_num(o.pbvc, o.e, vnewc, o.bvc, o.p);
    if (unit_refdens(P)) return ssc_of<M, true>(num, P.refdens);
    return ssc_of<M, false>(num, P.refdens);
}

// EvalEOSForElems for one element (lulesh.cc:2204-2324): the repetitions,
// then the sound speed when need_ss.
template <class M = IeeeOps>
__device__ __forceinline__ void eval_eos(const Params &P, double e_in, double delv_in,
                                         double p_in, double q_in, double qq_in, double ql_in,
                                         double vnewc, int rep, double &p_out, double &e_out,
                                         double &q_out, double &ss_out, bool need_ss = true)
{
    const EosOut o = eos_reps<M>(P, e_in, delv_in, p_in, q_in, qq_in, ql_in, vnewc, rep);
    p_out = o.p;
    e_out = o.e;
    q_out = o.q;
    ss_out = need_ss ? eos_sound_speed<M>(P, o, vnewc) : 0.0;
}

// min(a, b) as (b < a) ? b : a, the comparison on the integer pipe (dlt): the
// block and grid reductions of the dt candidates run it ten times per thread
__device__ __forceinline__ double dmin_sel(double a, double b) { return dlt(b, a) ? b : a; }

// Reduces (dtc, dth) over the block; the last block of the grid reduces the
// per-block results into ctl->dtcourant/dthydro, merges error flags and, if
// advance, evaluates the loop condition and TimeIncrement of the next cycle.
template <int BS, bool kUnrolledFold = false>
__device__ __forceinline__ void finish_dt(const DevState &s, double dtc, double dth, bool advance)
{
    __shared__ double red[2][BS / 32];
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
        for (int w = 1; w < BS / 32; ++w) {
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
    const int nb = (int)gridDim.x;
    constexpr int kLanes = 8;
    if (kUnrolledFold && nb >= 4 * kLanes * BS) {
        // A large grid: eight independent minima per thread, so that the
        // loads of the partials overlap instead of waiting one after another
        // (the minimum of exact values does not depend on the order).  Only
        // the FP64 kernels take it: in the mixed path's k_material the same
        // fold measured 1.5 ms slower per launch at s=192, for a cause not
        // found, while it saves 64 us in the FP64 one at s=150.
        double cu[kLanes], hu[kLanes];
#pragma unroll
        for (int u = 0; u < kLanes; ++u) cu[u] = hu[u] = 1.0e+20;
        for (int i0 = threadIdx.x; i0 < nb; i0 += kLanes * BS) {
#pragma unroll
            for (int u = 0; u < kLanes; ++u) {
                const int i = i0 + u * BS;
                if (i < nb) {
                    cu[u] = dmin_sel(cu[u], __ldcg(&s.dt_partial[2 * i]));
                    hu[u] = dmin_sel(hu[u], __ldcg(&s.dt_partial[2 * i + 1]));
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kLanes; ++u) {
            c = dmin_sel(c, cu[u]);
            h = dmin_sel(h, hu[u]);
        }
    } else {
        for (int i = threadIdx.x; i < nb; i += BS) {
            c = dmin_sel(c, __ldcg(&s.dt_partial[2 * i]));
            h = dmin_sel(h, __ldcg(&s.dt_partial[2 * i + 1]));
        }
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
        for (int w = 1; w < BS / 32; ++w) {
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


// Merges the material phase's error flags once every block is done (the
// qstop test precedes the material volume test, lulesh.cc:1993-2008, 2377).
__device__ __forceinline__ void finish_material_flags(const DevState &s)
{
    __shared__ bool am_last;
    Ctl *ctl = s.ctl;
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

// ---------------------------------------------------------------------------
// batched problems: per-problem minima and the grid-wide end of the cycle
// ---------------------------------------------------------------------------

// Loop test + TimeIncrement of every problem (start of an ensemble step).
__global__ void k_begin_all(Ctl *c, int n)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) begin_cycle(c + p);
}

// Folds this warp's Courant/hydro candidates into the per-problem slots.
// Positive doubles order like their bit patterns, so an integer atomicMin is
// an exact, order-independent minimum.  A warp inside one problem reduces
// first and issues one atomic per slot.  pid < 0: no element.
__device__ __forceinline__ void batched_dt_candidates(const DevState &s, int pid, double dtc,
                                                      double dth)
{
    const unsigned full = 0xffffffffu;
    unsigned long long c = (unsigned long long)__double_as_longlong(dtc);
    unsigned long long h = (unsigned long long)__double_as_longlong(dth);
    const unsigned long long big = (unsigned long long)__double_as_longlong(1.0e+20);
    const int pid0 = __shfl_sync(full, pid, 0);
    if (__all_sync(full, pid == pid0)) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long oc = __shfl_down_sync(full, c, off);
            const unsigned long long oh = __shfl_down_sync(full, h, off);
            c = oc < c ? oc : c;
            h = oh < h ? oh : h;
        }
        if ((threadIdx.x & 31) == 0 && pid0 >= 0) {
            if (c < big) atomicMin(&s.dtSlots[2 * pid0], c);
            if (h < big) atomicMin(&s.dtSlots[2 * pid0 + 1], h);
        }
    } else if (pid >= 0) {
        if (c < big) atomicMin(&s.dtSlots[2 * pid], c);
        if (h < big) atomicMin(&s.dtSlots[2 * pid + 1], h);
    }
}

// After every block of the batched material kernel: the last block takes each
// live problem's minima (resetting the slots), merges its error flags and runs
// its loop test and TimeIncrement for the next cycle.
__device__ __forceinline__ void finish_batched(const DevState &s)
{
    __shared__ bool am_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(s.gridCounter, 1u);
        am_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    const unsigned long long big = (unsigned long long)__double_as_longlong(1.0e+20);
    for (int p = threadIdx.x; p < s.nprob; p += blockDim.x) {
        Ctl *c = s.ctl + p;
        if (!c->active) continue;
        c->dtcourant = __longlong_as_double((long long)atomicExch(&s.dtSlots[2 * p], big));
        c->dthydro = __longlong_as_double((long long)atomicExch(&s.dtSlots[2 * p + 1], big));
        volatile int *vq = &c->err_qstop, *vm = &c->err_matvol;
        if (c->status == 0) {
            if (*vq)
                c->status = -2;
            else if (*vm)
                c->status = -1;
        }
        *vq = 0;
        *vm = 0;
        begin_cycle(c);
    }
    __syncthreads();
    if (threadIdx.x == 0) *s.gridCounter = 0;
}

}  // namespace LG_NS
}  // namespace lg
