// sample/solid/sample_linear.cpp of the reference written against pansfem2_gb300.hpp: an H8
// mesh and its boundary conditions read from CSV files, SolidLinearIsotropicElastic
// (E = 210000, nu = 0.3) assembled for every element, the point loads, CSR, ScalingCG to
// 1e-10 and Disassembling -- on the device.  Prints "u <node> <ux> <uy> <uz>" per node.
#include <cstdio>
#include <string>
#include <vector>

#include "pansfem2_gb300.hpp"

using namespace PANSFEM2_GB300;

int main(int argc, char **argv) {
    std::string model_path = argc > 1 ? std::string(argv[1]) + "/" : "sample/solid/";
    std::vector<std::vector<double> > x;
    ImportNodesFromCSV(x, model_path + "Node.csv");
    std::vector<std::vector<int> > elements;
    ImportElementsFromCSV(elements, model_path + "Element.csv");
    std::vector<std::pair<std::pair<int, int>, double> > ufixed;
    ImportDirichletFromCSV(ufixed, model_path + "Dirichlet.csv");
    std::vector<std::pair<std::pair<int, int>, double> > qfixed;
    ImportNeumannFromCSV(qfixed, model_path + "Neumann.csv");

    FemMesh mesh(PSF_H8_SOLID, x, elements);
    int KDEGREE = mesh.SetDirichlet(ufixed);
    mesh.SetLoads(qfixed);
    mesh.Assemble(std::vector<double>(elements.size(), 210000.0), 0.3, 1.0);
    psf_solve_info info;
    std::vector<double> u = mesh.Solve(PSF_SOLVE_CSR_JACOBI_F64, 100000, 1.0e-10, &info);
    printf("KDEGREE %d iterations %d\n", KDEGREE, info.iterations);
    for (size_t i = 0; i < x.size(); i++)
        printf("u %zu %.17g %.17g %.17g\n", i, u[3 * i], u[3 * i + 1], u[3 * i + 2]);
    return 0;
}
