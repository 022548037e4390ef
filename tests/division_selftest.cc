// division_selftest.cc -- the nodal-acceleration quotient of the FP64
// kernels (div_by_mass in lg_kernels.cuh): q0 = RN(f * RN(1/m)), the exact
// residual f - m q0 by FMA, q = RN(q0 + residual * RN(1/m)), with q0 kept
// when the residual is zero.  Markstein's correction makes q the IEEE
// quotient f / m; this restatement checks that on the host, whose division
// and fma are IEEE too, over random operands with adversarial mantissas.
// Prints the number of mismatches; exits 1 if any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }
static double from_bits(uint64_t u)
{
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
}

static double div_by_mass(double f, double m, double rm)
{
    const double q0 = f * rm;
    const double res = std::fma(-m, q0, f);
    return res != 0.0 ? std::fma(res, rm, q0) : q0;
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 10000000;
    std::mt19937_64 g(7);
    long bad = 0;
    for (long i = 0; i < n; ++i) {
        const uint64_t r1 = g(), r2 = g();
        const int cls = (int)(i & 3);
        const int ea = 1023 + (int)(r1 >> 58) - 32, eb = 1023 + (int)(r2 >> 58) - 32;
        uint64_t ma = r1 & 0xfffffffffffffull, mb = r2 & 0xfffffffffffffull;
        if (cls == 1) mb |= 0xffffffffff000ull;  // long runs of ones in the mass
        if (cls == 2) mb &= 0xff00000000000ull;  // short mass mantissas
        if (cls == 3) ma = mb ^ (r1 & 0xff);     // force close to the mass
        const double f = from_bits((uint64_t)ea << 52 | ma) * ((r1 & 1) ? -1.0 : 1.0);
        const double m = from_bits((uint64_t)eb << 52 | mb);
        const double q = div_by_mass(f, m, 1.0 / m);
        if (!same(q, f / m)) {
            if (bad < 10) std::printf("f=%a m=%a got %a want %a\n", f, m, q, f / m);
            ++bad;
        }
    }
    const double z = div_by_mass(0.0, 3.0, 1.0 / 3.0), nz = div_by_mass(-0.0, 3.0, 1.0 / 3.0);
    if (!same(z, 0.0 / 3.0) || !same(nz, -0.0 / 3.0)) ++bad;
    std::printf("%ld quotients, mismatches %ld\n", n, bad);
    return bad != 0;
}
