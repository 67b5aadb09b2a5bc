// The Krylov solvers of CG.h through the mirrored API (include/pansfem2_gb300.hpp) on a system read
// from a text file (rows nnz / indptr / indices / values / rhs); prints each solution on a line.
#include <cstdio>
#include <fstream>
#include <vector>

#include "pansfem2_gb300.hpp"

using namespace PANSFEM2_GB300;

static void print(const char *name, const std::vector<double> &x) {
    std::printf("%s", name);
    for (double v : x) std::printf(" %.17g", v);
    std::printf("\n");
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::ifstream in(argv[1]);
    int n, nnz;
    in >> n >> nnz;
    std::vector<int32_t> ip(n + 1), ix(nnz);
    std::vector<double> a(nnz), b(n);
    for (auto &v : ip) in >> v;
    for (auto &v : ix) in >> v;
    for (auto &v : a) in >> v;
    for (auto &v : b) in >> v;
    CSR<double> A(n, n, ip, ix, a);
    print("BiCGSTAB", BiCGSTAB(A, b, 100000, 1.0e-10));
    print("ScalingBiCGSTAB", ScalingBiCGSTAB(A, b, 100000, 1.0e-10));
    print("BiCGSTAB2", BiCGSTAB2(A, b, 100000, 1.0e-10));
    CSR<double> M = ILU0(A);
    print("ILU0CG", ILU0CG(A, M, b, 100000, 1.0e-10));
    print("ILU0BiCGSTAB", ILU0BiCGSTAB(A, M, b, 100000, 1.0e-10));
    return 0;
}
