// eos_paths_selftest.cu -- the EOS's unit-density path against its general
// path (lulesh_gb300/csrc/lg_cycle_common.cuh), and fixed kernels for an ncu
// count of what the EOS's parts cost on the FP64 pipe.
//
// `eos_paths_selftest` (check): with refdens == 1 the EOS repetitions and the
// sound speed through the unit-density path (eos_reps_rho<IeeeOps, true>: the
// x / refdens of the sound-speed terms skipped) must equal those through the
// general path (eos_reps_rho<IeeeOps, false>, x / 1.0) on elements at rest,
// compressing and expanding, at 1 to 3 repetitions.  Prints the number of
// differing results and the largest relative difference; exits 1 on a
// mismatch.  Built without contraction the two paths must agree bit for bit;
// with contraction the compiler may fuse the numerator differently in each
// (build with -DEOS_SELFTEST_STRICT=1 and --fmad=false for the bitwise check).
//
// `eos_paths_selftest costs`: launches, in this order, each kernel once with
// 1 and once with 11 iterations (the difference over 10 is the cost of one
// iteration), 1M threads each:
//   0-1 EOS repetitions of elements at rest, unit path
//   2-3 EOS repetitions of compressing elements, unit path
//   4-5 EOS repetitions of elements at rest, general path (x / 1.0)
//   6-7 sound-speed term of a zero numerator, unit path
//   8-9 sound-speed term of a zero numerator, general path
//   10-11 sound-speed term of a positive numerator, unit path
//   12-13 0.0 / 1.0        14-15 1.3 / 0.7        16-17 1.0 / 0.7
//   18-19 sqrt(2.0)        20-21 the empty loop (one add per iteration)
#define LG_NS eos_selftest
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "lg_device.h"
#include "lg_cycle_common.cuh"

using namespace lg::eos_selftest;

namespace {

lg::Params reference_params()
{
    // the Domain constructor's constants, lulesh-init.cc:20-38 (refdens = 1)
    lg::Params P{};
    P.e_cut = 1e-7; P.p_cut = 1e-7; P.q_cut = 1e-7; P.v_cut = 1e-10; P.u_cut = 1e-7;
    P.hgcoef = 3.0; P.ss4o3 = 4.0 / 3.0; P.qstop = 1e12; P.monoq_max_slope = 1.0;
    P.monoq_limiter_mult = 2.0; P.qlc_monoq = 0.5; P.qqc_monoq = 2.0 / 3.0; P.qqc = 2.0;
    P.eosvmax = 1e9; P.eosvmin = 1e-9; P.pmin = 0.0; P.emin = -1e15; P.dvovmax = 0.1;
    P.refdens = 1.0;
    return P;
}

constexpr int kIn = 7;   // e, delv, p, q, qq, ql, vnewc
constexpr int kOut = 6;  // p, e, q, bvc, pbvc, ss

template <bool kUnit>
__global__ void k_eos(lg::Params P, const double *in, const int *reps, double *out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *a = in + kIn * (size_t)i;
    const EosOut o =
        eos_reps_rho<IeeeOps, kUnit>(P, a[0], a[1], a[2], a[3], a[4], a[5], a[6], reps[i]);
    const double num = IeeeOps::ss_num(o.pbvc, o.e, a[6], o.bvc, o.p);
    double *r = out + kOut * (size_t)i;
    r[0] = o.p; r[1] = o.e; r[2] = o.q; r[3] = o.bvc; r[4] = o.pbvc;
    r[5] = ssc_of<IeeeOps, kUnit>(num, P.refdens);
}

// ---- cost kernels: every iteration recomputes from barrier-fenced operands
template <bool kUnit>
__global__ void c_eos(lg::Params P, double e, double delv, double p, double vnewc, double *out,
                      int n, int rep)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const EosOut o = eos_reps_rho<IeeeOps, kUnit>(P, e, delv, p, 0.1 * p, 0.01 * p, 0.02 * p,
                                                  vnewc, rep);
    out[i] = o.p + o.e + o.q;
}
template <bool kUnit>
__global__ void c_ssc(double num0, double *out, int n, int iters)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double num = num0, acc = 0.;
    for (int k = 0; k < iters; ++k) {
        opaque(num);
        acc = acc + ssc_of<IeeeOps, kUnit>(num, 1.0);
    }
    out[i] = acc;
}
__global__ void c_div(double a0, double b0, double *out, int n, int iters)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = a0, b = b0, acc = 0.;
    for (int k = 0; k < iters; ++k) {
        opaque(a); opaque(b);
        acc = acc + a / b;
    }
    out[i] = acc;
}
__global__ void c_sqrt(double a0, double *out, int n, int iters)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = a0, acc = 0.;
    for (int k = 0; k < iters; ++k) {
        opaque(a);
        acc = acc + sqrt(a);
    }
    out[i] = acc;
}
__global__ void c_empty(double *out, int n, int iters)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = 1.5, acc = 0.;
    for (int k = 0; k < iters; ++k) {
        opaque(a);
        acc = acc + a;
    }
    out[i] = acc;
}

unsigned long long mix64(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
double unit(unsigned long long &s) { return (double)((s = mix64(s)) >> 11) * 0x1.0p-53; }

int run_costs()
{
    const int n = 1 << 20, B = 128, G = (n + B - 1) / B;
    const lg::Params P = reference_params();
    double *d_out = nullptr;
    if (cudaMalloc(&d_out, n * sizeof(double)) != cudaSuccess) return 1;
    for (int it : {1, 11}) c_eos<true><<<G, B>>>(P, 0.0, 0.0, 0.0, 1.0, d_out, n, it);
    for (int it : {1, 11}) c_eos<true><<<G, B>>>(P, 5e2, -1e-3, 10.0, 0.999, d_out, n, it);
    for (int it : {1, 11}) c_eos<false><<<G, B>>>(P, 0.0, 0.0, 0.0, 1.0, d_out, n, it);
    for (int it : {1, 11}) c_ssc<true><<<G, B>>>(0.0, d_out, n, it);
    for (int it : {1, 11}) c_ssc<false><<<G, B>>>(0.0, d_out, n, it);
    for (int it : {1, 11}) c_ssc<true><<<G, B>>>(2.0, d_out, n, it);
    for (int it : {1, 11}) c_div<<<G, B>>>(0.0, 1.0, d_out, n, it);
    for (int it : {1, 11}) c_div<<<G, B>>>(1.3, 0.7, d_out, n, it);
    for (int it : {1, 11}) c_div<<<G, B>>>(1.0, 0.7, d_out, n, it);
    for (int it : {1, 11}) c_sqrt<<<G, B>>>(2.0, d_out, n, it);
    for (int it : {1, 11}) c_empty<<<G, B>>>(d_out, n, it);
    const cudaError_t e = cudaDeviceSynchronize();
    printf("cost kernels: 22 launches, status %s\n", cudaGetErrorString(e));
    cudaFree(d_out);
    return e != cudaSuccess;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc > 1 && !strcmp(argv[1], "costs")) return run_costs();

    const int n = 1 << 20;
    std::vector<double> in((size_t)kIn * n);
    std::vector<int> reps(n);
    unsigned long long s = 20250611ull;
    for (int i = 0; i < n; ++i) {
        double *a = &in[(size_t)kIn * i];
        const int kind = i % 4;  // at rest, compressing, expanding, mixed zeros
        const double u = unit(s);
        a[0] = kind == 0 ? 0.0 : 1e4 * unit(s);              // e
        a[1] = kind == 0 ? 0.0 : (kind == 2 ? 1e-3 : -1e-3) * unit(s);  // delv
        a[2] = kind == 0 ? 0.0 : 1e3 * unit(s);              // p
        a[3] = kind == 0 ? 0.0 : 10.0 * unit(s);             // q
        a[4] = kind == 0 ? 0.0 : unit(s);                    // qq
        a[5] = kind == 0 ? 0.0 : unit(s);                    // ql
        a[6] = kind == 0 ? 1.0 : 0.5 + u;                    // vnewc
        if (kind == 3) {
            for (int k = 0; k < 6; ++k)
                if (unit(s) < 0.5) a[k] = 0.0;
        }
        reps[i] = 1 + i % 3;
    }
    double *d_in = nullptr, *d_a = nullptr, *d_b = nullptr;
    int *d_reps = nullptr;
    const size_t nin = in.size() * sizeof(double), nout = (size_t)kOut * n * sizeof(double);
    if (cudaMalloc(&d_in, nin) != cudaSuccess || cudaMalloc(&d_a, nout) != cudaSuccess ||
        cudaMalloc(&d_b, nout) != cudaSuccess || cudaMalloc(&d_reps, n * sizeof(int)) != cudaSuccess)
        return 1;
    cudaMemcpy(d_in, in.data(), nin, cudaMemcpyHostToDevice);
    cudaMemcpy(d_reps, reps.data(), n * sizeof(int), cudaMemcpyHostToDevice);
    const lg::Params P = reference_params();
    const int B = 128, G = (n + B - 1) / B;
    k_eos<true><<<G, B>>>(P, d_in, d_reps, d_a, n);
    k_eos<false><<<G, B>>>(P, d_in, d_reps, d_b, n);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("CUDA error %s\n", cudaGetErrorString(e));
        return 1;
    }
    std::vector<double> a((size_t)kOut * n), b((size_t)kOut * n);
    cudaMemcpy(a.data(), d_a, nout, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), d_b, nout, cudaMemcpyDeviceToHost);
    long long bad = 0;
    double worst = 0.0;
    for (size_t k = 0; k < a.size(); ++k) {
        unsigned long long x, y;
        memcpy(&x, &a[k], 8);
        memcpy(&y, &b[k], 8);
        if (x != y) {
            ++bad;
            const double rel = std::fabs(a[k] - b[k]) / std::fmax(std::fabs(b[k]), 1e-300);
            if (rel > worst) worst = rel;
        }
    }
    printf("unit vs general path: %d elements x %d results, differing %lld, "
           "largest relative difference %.3e\n", n, kOut, bad, worst);
    cudaFree(d_in); cudaFree(d_a); cudaFree(d_b); cudaFree(d_reps);
#if EOS_SELFTEST_STRICT
    return bad != 0;
#else
    return worst > 1e-13;
#endif
}
