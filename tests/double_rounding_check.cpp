// Host check of bepuphysics1_gb300/csrc/double_rounding.cuh: for seeded random
// arguments, every result the double-float path decides, and every result of
// the routines with their double fallback, equals the float the double
// expression rounds to.  Prints one line per routine: name, arguments,
// fast-path decisions, mismatches (and for pow the typical arguments, dt = 1/60
// and c >= 2^-20, and their fast-path decisions).  Built and run by
// tests/test_double_rounding.py.
#include <cmath>
#include <cstdio>
#include <random>

#include "../bepuphysics1_gb300/csrc/double_rounding.cuh"

using namespace bepugpu::dr;

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 rng(20261204);
    std::uniform_real_distribution<double> U(0, 1);
    {  // kind 0: (float)(1 / Math.Sqrt(x)) over 2^-95 .. 2^95 and the unit range
        long fast = 0, bad = 0;
        for (long i = 0; i < n; i++) {
            float x = (i & 1) ? (float)(U(rng) * 4) : (float)std::ldexp(U(rng) + 0.5, (int)(U(rng) * 190) - 95);
            float r;
            if (TryInvSqrt(x, r)) {
                fast++;
                if (r != (float)(1.0 / std::sqrt((double)x))) bad++;
            }
            if (InvSqrtAsDouble(x) != (float)(1.0 / std::sqrt((double)x))) bad++;
        }
        std::printf("invsqrt %ld %ld %ld\n", n, fast, bad);
    }
    {  // kind 1: (float)(Math.Sqrt(e) / y), the boost's energies and other scales
        long fast = 0, bad = 0;
        for (long i = 0; i < n; i++) {
            float e = (i & 1) ? (float)(U(rng) * 0.0676) : (float)std::ldexp(U(rng) + 0.5, (int)(U(rng) * 190) - 95);
            float y = (i % 3) ? 0.52f : (float)std::ldexp(U(rng) + 0.5, (int)(U(rng) * 110) - 55);
            float r;
            const float want = (float)(std::sqrt((double)e) / (double)y);
            if (TrySqrtQuotient(e, y, r)) {
                fast++;
                if (r != want) bad++;
            }
            if (SqrtQuotientAsDouble(e, y) != want) bad++;
        }
        std::printf("sqrtquotient %ld %ld %ld\n", n, fast, bad);
    }
    {  // kind 2: (float)Math.Pow(c, dt), c in [0, 1], dt = 1/60 or up to 16
        long fast = 0, bad = 0, typical = 0, typicalFast = 0;  // typical: dt = 1/60, c >= 2^-20
        for (long i = 0; i < n; i++) {
            float c = (i % 3 == 0) ? (float)std::pow(U(rng), 20.0) : (float)U(rng);
            float dt = (i % 4 == 0) ? (float)(U(rng) * 16) : 1.f / 60;
            if (i % 97 == 0) c = (i % 2) ? 0.f : 1.f;
            float r;
            const float want = (float)std::pow((double)c, (double)dt);
            const bool isTypical = dt == 1.f / 60 && c >= 0x1p-20f;
            typical += isTypical;
            if (TryPow(c, dt, r)) {
                fast++;
                typicalFast += isTypical;
                if (r != want) bad++;
            }
            if (PowAsDouble(c, dt) != want) bad++;
        }
        std::printf("pow %ld %ld %ld %ld %ld\n", n, fast, bad, typical, typicalFast);
    }
    return 0;
}
