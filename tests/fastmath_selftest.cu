// fastmath_selftest.cu -- the mixed path's integer-pipe conversions
// (lulesh_gb300/csrc/lg_fastmath.cuh) against the hardware conversions:
// to_f32 must equal __double2float_rn for every input that is zero or at
// least the smallest normal float (smaller ones it flushes to zero by
// design), including rounding up to infinity, and
// to_f64 must equal the exact widening of every normal float.  Inputs:
// random doubles across and beyond the float range, exact rounding ties (the
// 29 dropped mantissa bits equal to one half), one-ulp neighbours of ties,
// and the edges of the float range.  Prints the number of mismatches and
// exits 1 if any.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

#include "lg_fastmath.cuh"

__global__ void k_check(int n, const double *in, unsigned *bad, double *first_bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = in[i];
    const float want = __double2float_rn(v);
    const float got = lg::fast::to_f32(v);
    const float a = fabsf(want);
    // inputs at or above the smallest normal float (or zero): below it the
    // conversion flushes to zero by design
    const bool comparable = v == 0.0 || fabs(v) >= 1.1754943508222875e-38;
    if (comparable && __float_as_uint(got) != __float_as_uint(want)) {
        if (atomicAdd(bad, 1u) == 0u) *first_bad = v;
    }
    // widening of a normal float is exact
    if (a >= 1.17549435e-38f && a <= 3.40282347e+38f) {
        const double w = lg::fast::to_f64(want);
        if (__double_as_longlong(w) != __double_as_longlong((double)want)) atomicAdd(bad + 1, 1u);
    }
}

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next()
{
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double from_bits(uint64_t b)
{
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

int main()
{
    std::vector<double> v;
    for (int i = 0; i < 4000000; ++i) {
        // exponent within +-140 of 1.0: across, below and above the float range
        const uint64_t e = 1023 - 140 + next() % 281;
        const uint64_t m = next() & 0xfffffffffffffull;
        const uint64_t s = next() & 1;
        const uint64_t b = (s << 63) | (e << 52) | m;
        v.push_back(from_bits(b));
        // an exact tie on the same float mantissa, and its neighbours
        const uint64_t tie = (b & ~0x1fffffffull) | 0x10000000ull;
        v.push_back(from_bits(tie));
        v.push_back(from_bits(tie + 1));
        v.push_back(from_bits(tie - 1));
    }
    const double edges[] = {3.4028234663852886e+38, 3.4028235677973366e+38, 3.40282357e+38,
                            1.1754943508222875e-38, 1.1754942e-38, 1.0, -1.0, 0.0, -0.0,
                            1.0 + 0x1p-24, 1.0 + 0x1p-23 + 0x1p-24, 6.5e4, 1e300, -1e-300};
    for (double e : edges) v.push_back(e);
    const int n = (int)v.size();
    double *d_in, *d_first;
    unsigned *d_bad;
    cudaMalloc(&d_in, n * sizeof(double));
    cudaMalloc(&d_bad, 2 * sizeof(unsigned));
    cudaMalloc(&d_first, sizeof(double));
    cudaMemcpy(d_in, v.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, 2 * sizeof(unsigned));
    k_check<<<(n + 255) / 256, 256>>>(n, d_in, d_bad, d_first);
    unsigned bad[2] = {0, 0};
    double first = 0;
    if (cudaMemcpy(bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost) != cudaSuccess) {
        std::printf("CUDA error\n");
        return 2;
    }
    cudaMemcpy(&first, d_first, sizeof first, cudaMemcpyDeviceToHost);
    std::printf("values %d, to_f32 mismatches %u, to_f64 mismatches %u\n", n, bad[0], bad[1]);
    if (bad[0]) std::printf("first mismatch at %.17g\n", first);
    return bad[0] || bad[1] ? 1 : 0;
}
