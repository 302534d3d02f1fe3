// Accuracy of fvm::pow_pos (csrc/fvm_pow.h) against long double powl: prints the largest error
// in units of the last place over seeded random arguments for the exponents the step control
// uses (7/100 and 2/25) and a few others in [-1, 1].
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>

#include "fvm_pow.h"

static double ulp_err(double got, long double ref) {
    const double r = (double)ref;
    const double u = std::nextafter(std::fabs(r), INFINITY) - std::fabs(r);
    return (double)(std::fabs((long double)got - ref) / u);
}

int main() {
    fvm::PowTables T;
    fvm::pow_build_tables(T);
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> lg(-300.0, 300.0);
    const double ys[] = {7.0 / 100.0, 2.0 / 25.0, 0.5, -0.3, 1.0, 1e-3};
    double worst = 0.0;
    for (double y : ys) {
        for (int t = 0; t < 200000; ++t) {
            double x = std::exp2(lg(rng));
            if (t < 64) x = std::ldexp(1.0 + t / 64.0, -1060 + t);  // subnormal and tiny arguments
            if (std::fabs(y * std::log2(x)) >= 1000.0) continue;     // outside the stated domain
            const double got = fvm::pow_pos(x, y, T);
            const long double ref = std::pow((long double)x, (long double)y);
            const double e = ulp_err(got, ref);
            if (e > worst) worst = e;
        }
    }
    std::printf("max_ulp %.3f\n", worst);
    return 0;
}
