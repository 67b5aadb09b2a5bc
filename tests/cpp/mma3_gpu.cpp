// The optimiser test program src/Optimize/Solver/test_MMA_3.cpp (n = 2, m = 2, per-variable
// bounds) on the mirrored API: MMA<double> with the reference's constructor runs on the device.
// Prints the iterates in the reference program's format.
#include <cmath>
#include <cstdio>
#include <vector>

#include "pansfem2_gb300.hpp"

using PANSFEM2_GB300::MMA;

int main() {
    const double C1 = 1.0, C2 = 0.124;
    std::vector<double> s = {1.5, 0.5};
    MMA<double> optimizer(2, 2, 1.0, {0.0, 0.0}, {1000.0, 1000.0}, {1.0, 1.0}, {0.2, 0.1}, {4.0, 1.6});
    optimizer.SetParameters(1.0e-5, 0.1, 0.5, 0.5, 0.7, 1.2, 1.0e-5);
    for (int k = 0; k < 100; k++) {
        const double q = std::sqrt(1.0 + s[1] * s[1]);
        const double f = C1 * s[0] * q;
        std::vector<double> df = {C1 * q, C1 * s[0] * s[1] / q};
        std::vector<double> g = {C2 * q * (8.0 / s[0] + 1.0 / (s[0] * s[1])) - 1.0,
                                 C2 * q * (8.0 / s[0] - 1.0 / (s[0] * s[1])) - 1.0};
        std::vector<std::vector<double> > dg = {
            {C2 * q * (-8.0 / (s[0] * s[0]) - 1.0 / (s[0] * s[0] * s[1])),
             C2 * s[1] / q * (8.0 / s[0] + 1.0 / (s[0] * s[1])) + C2 * q * (-1.0 / (s[0] * s[1] * s[1]))},
            {C2 * q * (-8.0 / (s[0] * s[0]) + 1.0 / (s[0] * s[0] * s[1])),
             C2 * s[1] / q * (8.0 / s[0] - 1.0 / (s[0] * s[1])) + C2 * q * (1.0 / (s[0] * s[1] * s[1]))}};
        std::printf("k = %d\t%.6g\t%.6g\n", k, s[0], s[1]);
        if (optimizer.IsConvergence(f)) break;
        optimizer.UpdateVariables(s, f, df, g, dg);
    }
    return 0;
}
