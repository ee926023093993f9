// Host check of gbivf::add_norms_rn (mestrado_gb300/csrc/exact_round.cuh):
// random, near-midpoint and edge inputs against (float)(D + (double)f).
// Build with -ffp-contract=off. Prints the number of mismatches.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "exact_round.cuh"

static float ref(double D, float f) { return (float)(D + (double)f); }

int main(int argc, char** argv) {
    long n = argc > 1 ? atol(argv[1]) : 2000000;
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long bad = 0, tested = 0;
    auto check = [&](double D, float f) {
        if (!(D >= 0) || !(f >= 0)) return;
        float hi, lo;
        gbivf::split_norm(D, &hi, &lo);
        float a = gbivf::add_norms_rn(&D, hi, lo, f), b = ref(D, f);
        uint32_t ua, ub;
        memcpy(&ua, &a, 4);
        memcpy(&ub, &b, 4);
        tested++;
        if (ua != ub) {
            if (bad < 10) printf("mismatch D=%.17g f=%.9g got %.9g want %.9g\n", D, f, a, b);
            bad++;
        }
    };
    for (long i = 0; i < n; i++) {
        int e = (int)(U(g) * 40) - 20;
        // random magnitudes
        double D = std::ldexp(1.0 + U(g), e) * (U(g) < 0.5 ? 1.0 : U(g));
        float f = (float)std::ldexp(1.0 + U(g), e + (int)(U(g) * 8) - 4);
        check(D, f);
        // integer-like norms (byte-valued vectors)
        check(std::floor(U(g) * 2e6), (float)std::floor(U(g) * 2e6));
        // near a float midpoint of the sum
        float S = (float)std::ldexp(1.0 + U(g), e);
        uint32_t sb;
        memcpy(&sb, &S, 4);
        float Sn;
        uint32_t sn = sb + 1;
        memcpy(&Sn, &sn, 4);
        double mid = 0.5 * ((double)S + (double)Sn);
        float ff = (float)(mid * U(g));
        int k = (int)(U(g) * 17) - 8;
        double target = mid + k * std::ldexp(mid, -60);
        check(target - (double)ff, ff);
        check(std::nextafter(target - (double)ff, 0.0), ff);
        check(std::nextafter(target - (double)ff, 1e300), ff);
        // exact float sums, zeros, powers of two
        check((double)S, 0.0f);
        check(0.0, S);
        check(std::ldexp(1.0, e), (float)std::ldexp(1.0, e - 30));
    }
    printf("tested %ld mismatches %ld\n", tested, bad);
    return bad != 0;
}
