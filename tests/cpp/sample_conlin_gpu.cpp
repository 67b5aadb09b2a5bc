// The CONLIN sample loop (sample/optimize/sample_optimize_density_CONLIN.cpp:23-206)
// written against the GPU library's C++ mirror of the reference API: the cantilever
// with the sample's material and scaling, the HeavisideFilter with beta doubled every
// 40 iterations, and CONLIN(n, 1, 1, {0}, {10000}, {0}, 0.01, 1) with
// SetParameters(0.2, 1e-6).  Prints the objective of every iteration and a checksum
// of the final design.   usage: sample_conlin_gpu nx ny iters
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pansfem2_gb300.hpp"

using namespace PANSFEM2_GB300;

int main(int argc, char **argv) {
    const int nx = argc > 1 ? atoi(argv[1]) : 60, ny = argc > 2 ? atoi(argv[2]) : 40;
    const int iters = argc > 3 ? atoi(argv[3]) : 5;
    const double E0 = 0.0001, E1 = 210000.0, p = 3.0, weightlimit = 0.5, scale0 = 1.0e5, scale1 = 1.0;
    Problem prob(PSF_Q4_PLANE_STRAIN, nx, ny, 0, nx, ny, 0.0, 0.3, 1.0);
    const int ne = nx * ny;
    // GenerateFixedlist order: nodes i-major, dofs in list order; the load at (lx, ly/2)
    std::vector<std::pair<std::pair<int, int>, double> > ufixed, qfixed;
    for (int j = 0; j <= ny; j++) {
        ufixed.push_back({{j, 0}, 0.0});
        ufixed.push_back({{j, 1}, 0.0});
    }
    qfixed.push_back({{(ny + 1) * nx + ny / 2, 1}, -1.0});
    prob.SetDirichlet(ufixed);
    prob.SetLoads(qfixed);
    HeavisideFilter<double> filter(prob, 1.5);
    std::vector<double> s(ne, 0.5);
    double beta = 0.5;
    CONLIN<double> optimizer(prob, ne, 1, 1.0, {0.0}, {10000.0}, {0.0}, std::vector<double>(ne, 0.01),
                             std::vector<double>(ne, 1.0));
    optimizer.SetParameters(0.2, 1.0e-6);
    for (int k = 0; k < iters; k++) {
        if (k % 40 == 0) {
            beta *= 2.0;
            filter.UpdateBeta(beta);
        }
        std::vector<double> rho = filter.GetFilteredVariables(s);
        double g = 0.0;
        std::vector<double> dgdrho(ne, 0.0);
        for (int i = 0; i < ne; i++) {
            g += scale1 * rho[i] / (weightlimit * ne);
            dgdrho[i] = scale1 / (weightlimit * ne);
        }
        g -= 1.0 * scale1;
        std::vector<double> E(ne);
        for (int i = 0; i < ne; i++) E[i] = E1 * pow(rho[i], p) + E0 * (1.0 - pow(rho[i], p));
        prob.Assemble(E);
        prob.Solve(PSF_SOLVE_CSR_JACOBI_F64, 100000, 1.0e-10);
        std::vector<double> dfdrho;
        const double f = prob.ComplianceSensitivity(rho, E1, E0, p, scale0, dfdrho);
        std::vector<double> dfds = filter.GetFilteredSensitivitis(s, dfdrho);
        std::vector<double> dgds = filter.GetFilteredSensitivitis(s, dgdrho);
        printf("k %d f %.15e g %.15e\n", k, f, g);
        if (optimizer.IsConvergence(f)) break;
        optimizer.UpdateVariables(s, f, dfds, {g}, {dgds});
    }
    double cs = 0.0;
    for (double v : s) cs += v;
    printf("checksum %.15e\n", cs);
    return 0;
}
