// Host check of the double-word operations in pansfem2_gb300/csrc/psf_dw.cuh (the same
// source the kernels use, compiled for the host): random operands spanning the ranges the
// MMA / CONLIN kernels see, every result against long double arithmetic.  Prints the
// worst relative error of each operation; exits 1 if any exceeds 2^-44.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "psf_dw.cuh"

using namespace psf;

static long double val(dw::D a) { return (long double)a.h + (long double)a.l; }

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> mant(1.0, 2.0), expo(-20.0, 20.0), sgn(-1.0, 1.0);
    auto draw = [&]() {
        double m = mant(rng) * std::pow(2.0, std::floor(expo(rng)));
        return sgn(rng) < 0 ? -m : m;
    };
    const double bound = std::ldexp(1.0, -44);
    double worst[6] = {0, 0, 0, 0, 0, 0};
    const char *names[6] = {"from_double", "add", "mul", "mulf", "rcp", "add (cancelling)"};
    for (int it = 0; it < 200000; it++) {
        const double a = draw(), b = draw();
        const dw::D A = dw::from_double(a), B = dw::from_double(b);
        const long double la = val(A), lb = val(B);
        auto rel = [](long double got, long double ref) {
            return (double)(ref == 0 ? fabsl(got) : fabsl((got - ref) / ref));
        };
        double e[6];
        e[0] = rel(la, (long double)a);
        e[1] = rel(val(dw::add(A, B)), la + lb);
        e[2] = rel(val(dw::mul(A, B)), la * lb);
        e[3] = rel(val(dw::mulf(A, B.h)), la * (long double)B.h);
        e[4] = rel(val(dw::rcp(A)), 1.0L / la);
        // x - y with y within a few percent of x: the cancellation the kernels meet in U - x, x - L
        const dw::D C = dw::from_double(a * (1.0 + 0.03 * sgn(rng)));
        const long double ref = la - val(C);
        e[5] = ref == 0 ? 0.0 : rel(val(dw::sub(A, C)), ref);
        for (int k = 0; k < 6; k++)
            if (e[k] > worst[k]) worst[k] = e[k];
    }
    int bad = 0;
    for (int k = 0; k < 6; k++) {
        printf("%-18s worst relative error %.3e (2^%.1f)\n", names[k], worst[k],
               worst[k] > 0 ? std::log2(worst[k]) : -999.0);
        if (worst[k] > bound) bad = 1;
    }
    // ordering, min/max on ties
    const dw::D x = dw::make(1.0f, 1e-9f), y = dw::make(1.0f, -1e-9f);
    if (!dw::lt(y, x) || dw::lt(x, y) || dw::max(x, y).l != x.l || dw::min(x, y).l != y.l) {
        printf("ordering wrong\n");
        bad = 1;
    }
    return bad;
}
