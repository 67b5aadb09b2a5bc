// ref_driver.cpp -- runs the PANSFEM2 reference itself (its headers, compiled
// here with g++) on the SIMP configurations and dumps full-precision results,
// so the C oracle and the GPU library can be pinned against the real thing.
//
// TEST INFRASTRUCTURE: built by oracle/build_ref.sh into oracle/_ref/ only where
// the reference source tree is present; the outputs become the committed
// fixtures under tests/golden/.
//
// The SIMP loop is the call sequence of
// sample/optimize/sample_optimize_density_oc.cpp:93-207 (OC) and
// sample/optimize/sample_optimize_density_mma.cpp:98-203 (MMA) and
// sample/optimize/sample_optimize_density_CONLIN.cpp:75-206 (CONLIN, opt=2), with the
// configuration's parameters in place of the sample's literals, the linear
// DensityFilter (or the sample's HeavisideFilter with heaviside=1); with
// vtk=<file> iteration 0 is also written by the reference's VTK writer.  Usage:  ref_driver <mode> out=<file> key=value ...
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>
#include <algorithm>
#include <numeric>
#include <cassert>
#include <sstream>

// CSR keeps indptr/indices/data private (CSR.h:71-74); the harness reads them
// through an access-only remap while compiling the unmodified headers.
#define private public
#include "src/LinearAlgebra/Models/Vector.h"
#include "src/FEM/Equation/PlaneStrain.h"
#include "src/FEM/Equation/HeatTransfer.h"
#include "src/FEM/Equation/Solid.h"
#include "src/FEM/Controller/ShapeFunction.h"
#include "src/FEM/Controller/GaussIntegration.h"
#include "src/FEM/Controller/BoundaryCondition.h"
#include "src/FEM/Controller/Assembling.h"
#include "src/PrePost/Import/ImportFromCSV.h"
#include "src/LinearAlgebra/Solvers/CG.h"
#include "src/Optimize/Solver/OC.h"
#include "src/PrePost/Export/ExportToVTK.h"
#include "src/Optimize/Solver/MMA.h"
#include "src/Optimize/Solver/CONLIN.h"
#include "src/Optimize/Filter/DensityFilter.h"
#include "src/Optimize/Filter/HeavisideFilter.h"
#include "src/PrePost/Mesher/SquareMesh.h"
#include "src/FEM/Equation/General.h"

using namespace PANSFEM2;

// ---------------- tiny binary container: [namelen][name][type][count][data] ----------------
struct Dump {
    FILE* f;
    explicit Dump(const std::string& path) { f = fopen(path.c_str(), "wb"); if (!f) { perror("open"); exit(2); } }
    ~Dump() { fclose(f); }
    void put(const std::string& name, int type, long long count, const void* data, size_t elem) {
        int nl = (int)name.size();
        fwrite(&nl, 4, 1, f); fwrite(name.data(), 1, nl, f);
        fwrite(&type, 4, 1, f); fwrite(&count, 8, 1, f);
        if (count) fwrite(data, elem, (size_t)count, f);
    }
    void d(const std::string& n, const std::vector<double>& v) { put(n, 0, (long long)v.size(), v.data(), 8); }
    void i(const std::string& n, const std::vector<int>& v) { put(n, 1, (long long)v.size(), v.data(), 4); }
};

static std::map<std::string, std::string> g_args;
static double argd(const char* k, double dflt) { auto it = g_args.find(k); return it == g_args.end() ? dflt : atof(it->second.c_str()); }
static int argi(const char* k, int dflt) { auto it = g_args.find(k); return it == g_args.end() ? dflt : atoi(it->second.c_str()); }
static std::string args(const char* k, const char* dflt) { auto it = g_args.find(k); return it == g_args.end() ? dflt : it->second; }

// 3D structured grid in the SquareMesh i-major convention (no 3D mesher exists in the reference)
static void grid3d(double lx, double ly, double lz, int nx, int ny, int nz, std::vector<Vector<double> >& x,
                   std::vector<std::vector<int> >& el) {
    auto nid = [&](int i, int j, int k) { return ((ny + 1) * i + j) * (nz + 1) + k; };
    x.assign((size_t)(nx + 1) * (ny + 1) * (nz + 1), Vector<double>(3));
    for (int i = 0; i <= nx; i++) for (int j = 0; j <= ny; j++) for (int k = 0; k <= nz; k++)
        x[nid(i, j, k)] = {lx * (i / (double)nx), ly * (j / (double)ny), lz * (k / (double)nz)};
    el.assign((size_t)nx * ny * nz, std::vector<int>());
    for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) for (int k = 0; k < nz; k++)
        el[(ny * i + j) * nz + k] = {nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                                     nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
}

typedef std::vector<std::pair<std::pair<int, int>, double> > BCList;

static void element_matrix(int kind, Matrix<double>& Ke, std::vector<std::vector<std::pair<int, int> > >& n2e,
                           const std::vector<int>& el, std::vector<Vector<double> >& x, double E, double V, double t) {
    if (kind == 0) PlaneStrainStiffness<double, ShapeFunction4Square, Gauss4Square>(Ke, n2e, el, {0, 1}, x, E, V, t);
    else if (kind == 1) HeatTransfer<double, ShapeFunction4Square, Gauss4Square>(Ke, n2e, el, {0}, x, E, t);
    else SolidLinearIsotropicElastic<double, ShapeFunction8Cubic, Gauss8Cubic>(Ke, n2e, el, {0, 1, 2}, x, E, V);
}

// ------------------------------- SIMP -------------------------------
static int run_simp() {
    int kind = argi("kind", 0), nx = argi("nx", 12), ny = argi("ny", 6), nz = argi("nz", 0);
    double lx = argd("lx", nx), ly = argd("ly", ny), lz = argd("lz", nz);
    double V = argd("V", 0.3), t = argd("t", 1.0), E1 = argd("E1", 1.0), E0 = argd("E0", 1e-9), p = argd("p", 3.0);
    double vf = argd("vf", 0.5), R = argd("R", 1.5), scale0 = argd("scale0", 1.0), scale1 = argd("scale1", 1.0);
    double rho0 = argd("rho0", vf);
    int optimizer = argi("opt", 0), iters = argi("iters", 5), heav = argi("heaviside", 0);
    double move = argd("move", 0.2), cg_eps = argd("cg_eps", 1e-10);
    int cg_itmax = argi("cg_itmax", 100000);
    std::string bc = args("bc", "cantilever");
    int ndof = kind == 0 ? 2 : (kind == 1 ? 1 : 3);

    std::vector<Vector<double> > x;
    std::vector<std::vector<int> > elements;
    BCList ufixed, qfixed;
    if (kind != 2) {
        SquareMesh<double> mesh(lx, ly, nx, ny);
        x = mesh.GenerateNodes();
        elements = mesh.GenerateElements();
        if (bc == "cantilever") {
            std::vector<int> dl = kind == 0 ? std::vector<int>{0, 1} : std::vector<int>{0};
            ufixed = mesh.GenerateFixedlist(dl, [](Vector<double> _x) { return std::abs(_x(0)) < 1.0e-5; });
            qfixed = mesh.GenerateFixedlist({kind == 0 ? 1 : 0}, [&](Vector<double> _x) {
                return std::abs(_x(0) - lx) < 1.0e-5 && std::abs(_x(1) - 0.5 * ly) < 1.0e-5; });
            for (auto& q : qfixed) q.second = -1.0;
        } else if (bc == "mbb") {
            ufixed = mesh.GenerateFixedlist({0}, [](Vector<double> _x) { return std::abs(_x(0)) < 1.0e-5; });
            BCList u2 = mesh.GenerateFixedlist({1}, [&](Vector<double> _x) {
                return std::abs(_x(0) - lx) < 1.0e-5 && std::abs(_x(1)) < 1.0e-5; });
            ufixed.insert(ufixed.end(), u2.begin(), u2.end());
            qfixed = mesh.GenerateFixedlist({1}, [&](Vector<double> _x) {
                return std::abs(_x(0)) < 1.0e-5 && std::abs(_x(1) - ly) < 1.0e-5; });
            for (auto& q : qfixed) q.second = -1.0;
        } else if (bc == "heatsink") {
            // zero temperature on a patch of the bottom edge; uniform unit source as nodal loads
            int w = argi("patch_w", std::max(1, nx / 10)), p0 = argi("patch_i0", (nx - w) / 2);
            for (int i = p0; i <= p0 + w; i++) ufixed.push_back({{(ny + 1) * i + 0, 0}, 0.0});
            double h2 = (lx / nx) * (ly / ny) * 0.25;
            for (int i = 0; i <= nx; i++) for (int j = 0; j <= ny; j++) {
                int c = (i > 0 && j > 0) + (i < nx && j > 0) + (i > 0 && j < ny) + (i < nx && j < ny);
                qfixed.push_back({{(ny + 1) * i + j, 0}, c * h2});
            }
        }
    } else {
        grid3d(lx, ly, lz, nx, ny, nz, x, elements);
        for (int j = 0; j <= ny; j++) for (int k = 0; k <= nz; k++)
            for (int d = 0; d < 3; d++) ufixed.push_back({{(ny + 1) * 0 * (nz + 1) + j * (nz + 1) + k, d}, 0.0});
        for (int j = 0; j <= ny; j++) qfixed.push_back({{((ny + 1) * nx + j) * (nz + 1) + 0, 2}, -1.0 / (ny + 1)});
    }
    int dim = kind == 2 ? 3 : 2;

    // neighbour lists exactly as sample_optimize_density_oc.cpp:43-60 (all pairs)
    std::vector<Vector<double> > cg(elements.size());
    for (size_t i = 0; i < elements.size(); i++) cg[i] = CenterOfGravity(x, elements[i]);
    std::vector<std::vector<int> > neighbors(elements.size());
    std::vector<std::vector<double> > w(elements.size());
    for (size_t i = 0; i < elements.size(); i++)
        for (size_t j = 0; j < elements.size(); j++)
            if ((cg[i] - cg[j]).Norm() <= R) {
                neighbors[i].push_back((int)j);
                w[i].push_back((R - (cg[i] - cg[j]).Norm()) / R);
            }
    DensityFilter<double> dfilter(elements.size(), neighbors, w);
    HeavisideFilter<double> hfilter(elements.size(), neighbors, w);
    double beta = 0.5;

    std::vector<double> s(elements.size(), rho0);
    OC<double> oc(s.size(), argd("iota", 0.5), argd("lmin", 0.0), argd("lmax", 1.0e4), argd("leps", 1.0e-3), move,
                  std::vector<double>(s.size(), 0.01), std::vector<double>(s.size(), 1.0));
    MMA<double> mma(s.size(), 1, argd("a0", 1.0), std::vector<double>(1, 0.0), std::vector<double>(1, argd("mma_c", 10000.0)),
                    std::vector<double>(1, 0.0), std::vector<double>(s.size(), argd("xmin", 0.01)),
                    std::vector<double>(s.size(), argd("xmax", 1.0)));
    mma.SetParameters(argd("raa0", 1.0e-5), argd("albefa", 0.1), move, argd("asyinit", 0.5), argd("asydecr", 0.7),
                      argd("asyincr", 1.2), argd("mma_eps", 1.0e-6));
    CONLIN<double> conlin(s.size(), 1, argd("a0", 1.0), std::vector<double>(1, 0.0),
                          std::vector<double>(1, argd("mma_c", 10000.0)), std::vector<double>(1, 0.0),
                          std::vector<double>(s.size(), argd("xmin", 0.01)), std::vector<double>(s.size(), argd("xmax", 1.0)));
    conlin.SetParameters(move, argd("mma_eps", 1.0e-6));

    Dump out(args("out", "ref.bin"));
    {
        std::vector<int> nfix, dfix, nl, dl; std::vector<double> vl;
        for (auto& u : ufixed) { nfix.push_back(u.first.first); dfix.push_back(u.first.second); }
        for (auto& q : qfixed) { nl.push_back(q.first.first); dl.push_back(q.first.second); vl.push_back(q.second); }
        out.i("fix_node", nfix); out.i("fix_dof", dfix); out.i("load_node", nl); out.i("load_dof", dl); out.d("load_val", vl);
        std::vector<int> nptr(1, 0), nidx; std::vector<double> nw;
        for (size_t i = 0; i < neighbors.size(); i++) {
            nidx.insert(nidx.end(), neighbors[i].begin(), neighbors[i].end());
            nw.insert(nw.end(), w[i].begin(), w[i].end());
            nptr.push_back((int)nidx.size());
        }
        out.i("nb_ptr", nptr); out.i("nb_idx", nidx); out.d("nb_w", nw);
        std::vector<double> xc, cgc;
        for (auto& xi : x) for (int k = 0; k < dim; k++) xc.push_back(xi(k));
        for (auto& ci : cg) for (int k = 0; k < dim; k++) cgc.push_back(ci(k));
        out.d("coords", xc); out.d("centroids", cgc);
        std::vector<int> conn;
        for (auto& e : elements) conn.insert(conn.end(), e.begin(), e.end());
        out.i("conn", conn);
        Matrix<double> Ke; std::vector<std::vector<std::pair<int, int> > > n2e;
        element_matrix(kind, Ke, n2e, elements[0], x, 1.0, V, t);
        std::vector<double> kv;
        for (int a = 0; a < Ke.ROW(); a++) for (int b = 0; b < Ke.COL(); b++) kv.push_back(Ke(a, b));
        out.d("Ke0", kv);
        element_matrix(kind, Ke, n2e, elements.back(), x, 0.37, V, t);
        kv.clear();
        for (int a = 0; a < Ke.ROW(); a++) for (int b = 0; b < Ke.COL(); b++) kv.push_back(Ke(a, b));
        out.d("Ke_last_E037", kv);
    }
    std::vector<double> F_hist, f_hist, g_hist, rho_hist, dfdrho_hist, dfds_hist, s_hist, u_hist, r_hist;
    for (int k = 0; k < iters; k++) {
        if (heav && k % 40 == 0) { beta *= 2.0; hfilter.UpdateBeta(beta); }
        std::vector<double> rho = heav ? hfilter.GetFilteredVariables(s) : dfilter.GetFilteredVariables(s);
        double g = 0.0;
        std::vector<double> dgdrho(s.size(), 0.0);
        for (size_t i = 0; i < elements.size(); i++) {
            g += scale1 * rho[i] / (vf * elements.size());
            dgdrho[i] = scale1 / (vf * elements.size());
        }
        g -= 1.0 * scale1;

        std::vector<Vector<double> > u(x.size(), Vector<double>(ndof));
        std::vector<std::vector<int> > nodetoglobal(x.size(), std::vector<int>(ndof, 0));
        SetDirichlet(u, nodetoglobal, ufixed);
        int KDEGREE = Renumbering(nodetoglobal);
        LILCSR<double> K(KDEGREE, KDEGREE);
        std::vector<double> F(KDEGREE, 0.0);
        for (size_t i = 0; i < elements.size(); i++) {
            double E = E1 * pow(rho[i], p) + E0 * (1.0 - pow(rho[i], p));
            std::vector<std::vector<std::pair<int, int> > > nodetoelement;
            Matrix<double> Ke;
            element_matrix(kind, Ke, nodetoelement, elements[i], x, E, V, t);
            Assembling(K, F, u, Ke, nodetoglobal, nodetoelement, elements[i]);
        }
        Assembling(F, qfixed, nodetoglobal);
        CSR<double> Kmod(K);
        if (k == 0) {
            std::vector<int> n2g;
            for (auto& nd : nodetoglobal) n2g.insert(n2g.end(), nd.begin(), nd.end());
            out.i("n2g", n2g);
            out.i("indptr", Kmod.indptr);
            out.i("indices", Kmod.indices);
            out.d("data", Kmod.data);
            out.d("F0", F);
        }
        if (k == 0 && argi("solvers", 0)) {
            // the other Krylov solvers and ILU(0) of CG.h on the first system
            out.d("sol_cg", CG(Kmod, F, cg_itmax, cg_eps));
            out.d("sol_bicgstab", BiCGSTAB(Kmod, F, cg_itmax, cg_eps));
            out.d("sol_bicgstab2", BiCGSTAB2(Kmod, F, cg_itmax, cg_eps));
            CSR<double> M = ILU0(Kmod);
            out.i("ilu_indptr", M.indptr);
            out.i("ilu_indices", M.indices);
            out.d("ilu_data", M.data);
            std::vector<double> Fc = F;
            out.d("ilu_apply_F", PreILU0(M, Fc));
            out.d("sol_ilu0cg", ILU0CG(Kmod, M, F, cg_itmax, cg_eps));
            out.d("sol_scalingbicgstab", ScalingBiCGSTAB(Kmod, F, cg_itmax, cg_eps));
            out.d("sol_ilu0bicgstab", ILU0BiCGSTAB(Kmod, M, F, cg_itmax, cg_eps));
        }
        std::vector<double> result = ScalingCG(Kmod, F, cg_itmax, cg_eps);
        Disassembling(u, result, nodetoglobal);
        if (k == 0) out.d("result0", result);

        RemoveBoundaryConditions(nodetoglobal);
        KDEGREE = Renumbering(nodetoglobal);
        std::vector<double> RF(KDEGREE, 0.0);
        std::vector<Vector<double> > r(x.size(), Vector<double>(ndof));
        for (size_t i = 0; i < elements.size(); i++) {
            double E = E1 * pow(rho[i], p) + E0 * (1.0 - pow(rho[i], p));
            std::vector<std::vector<std::pair<int, int> > > nodetoelement;
            Matrix<double> Ke;
            element_matrix(kind, Ke, nodetoelement, elements[i], x, E, V, t);
            Vector<double> Keue = Ke * ElementVector(u, nodetoelement, elements[i]);
            Assembling(RF, Keue, nodetoglobal, nodetoelement, elements[i]);
        }
        Disassembling(r, RF, nodetoglobal);
        double f = scale0 * std::inner_product(u.begin(), u.end(), r.begin(), 0.0);
        std::vector<double> dfdrho(s.size(), 0.0);
        for (size_t i = 0; i < elements.size(); i++) {
            std::vector<std::vector<std::pair<int, int> > > nodetoelement;
            Matrix<double> Ke;
            element_matrix(kind, Ke, nodetoelement, elements[i], x, 1.0, V, t);
            Vector<double> ue = ElementVector(u, nodetoelement, elements[i]);
            dfdrho[i] = -scale0 * p * (-E0 + E1) * pow(rho[i], p - 1.0) * (ue * (Ke * ue));
        }
        std::vector<double> dfds = heav ? hfilter.GetFilteredSensitivitis(s, dfdrho) : dfilter.GetFilteredSensitivitis(s, dfdrho);
        std::vector<double> dgds = heav ? hfilter.GetFilteredSensitivitis(s, dgdrho) : dfilter.GetFilteredSensitivitis(s, dgdrho);

        f_hist.push_back(f); g_hist.push_back(g);
        rho_hist.insert(rho_hist.end(), rho.begin(), rho.end());
        dfdrho_hist.insert(dfdrho_hist.end(), dfdrho.begin(), dfdrho.end());
        dfds_hist.insert(dfds_hist.end(), dfds.begin(), dfds.end());
        for (auto& ui : u) for (int d = 0; d < ndof; d++) u_hist.push_back(ui(d));
        if (k == 0) for (auto& ri : r) for (int d = 0; d < ndof; d++) r_hist.push_back(ri(d));
        // vtk=<path>: iteration 0 written by the reference's own writer in the sample's order
        if (k == 0 && !args("vtk", "").empty()) {
            std::ofstream fout(args("vtk", ""));
            MakeHeadderToVTK(fout);
            AddPointsToVTK(x, fout);
            AddElementToVTK(elements, fout);
            AddElementTypes(std::vector<int>(elements.size(), kind == 2 ? 12 : 9), fout);
            AddPointVectors(u, "u", fout, true);
            AddPointVectors(r, "r", fout, false);
            AddElementScalers(rho, "s", fout, true);
            fout.close();
        }

        if (optimizer == 1) {
            mma.UpdateVariables(s, f, dfds, {g}, {dgds});
        } else if (optimizer == 2) {
            conlin.UpdateVariables(s, f, dfds, {g}, {dgds});
        } else {
            oc.UpdateVariables(s, f, dfds, g, dgds, [&](std::vector<double> _xkp1) {
                double gg = 0.0;
                std::vector<double> rr = heav ? hfilter.GetFilteredVariables(_xkp1) : dfilter.GetFilteredVariables(_xkp1);
                for (size_t i = 0; i < elements.size(); i++) gg += scale1 * rr[i] / (vf * elements.size());
                return gg - 1.0 * scale1;
            });
        }
        s_hist.insert(s_hist.end(), s.begin(), s.end());
    }
    out.d("f", f_hist); out.d("g", g_hist); out.d("rho", rho_hist); out.d("dfdrho", dfdrho_hist);
    out.d("dfds", dfds_hist); out.d("s_after", s_hist); out.d("u", u_hist); out.d("r0", r_hist);
    return 0;
}

// ------------------------------- CONLIN on the optimiser test problems -------------------------------
// The objective/constraint functions of src/Optimize/Solver/test_MMA.cpp (problem=mma),
// test_MMA_3.cpp (problem=mma3) and test_MMA_TOY2.cpp (problem=toy2), driven through
// CONLIN<double> with the tests' constructor arguments and move = 0.5.  Every iteration's
// inputs (x, f, df, g, dg) and the design CONLIN returns are dumped, so each update can
// be replayed one step at a time.
static void eval_problem(const std::string& pb, const std::vector<double>& s, double& f, std::vector<double>& df,
                         std::vector<double>& g, std::vector<std::vector<double> >& dg) {
    if (pb == "mma") {
        const double C1 = 0.0624, C2 = 1.0, cf[5] = {61.0, 37.0, 19.0, 7.0, 1.0};
        f = C1 * (s[0] + s[1] + s[2] + s[3] + s[4]);
        df.assign(5, C1);
        double gg = 0.0;
        for (int j = 0; j < 5; j++) gg += cf[j] * pow(s[j], -3.0);
        g.assign(1, gg - C2);
        dg.assign(1, std::vector<double>(5));
        for (int j = 0; j < 5; j++) dg[0][j] = -3.0 * cf[j] * pow(s[j], -4.0);
    } else if (pb == "mma3") {
        const double C1 = 1.0, C2 = 0.124, q = sqrt(1.0 + pow(s[1], 2.0));
        f = C1 * s[0] * q;
        df = {C1 * q, C1 * s[0] * s[1] / q};
        g = {C2 * q * (8.0 / s[0] + 1.0 / (s[0] * s[1])) - 1.0, C2 * q * (8.0 / s[0] - 1.0 / (s[0] * s[1])) - 1.0};
        dg = {{C2 * q * (-8.0 / (s[0] * s[0]) - 1.0 / (s[0] * s[0] * s[1])),
               C2 * s[1] / q * (8.0 / s[0] + 1.0 / (s[0] * s[1])) - C2 * q / (s[0] * s[1] * s[1])},
              {C2 * q * (-8.0 / (s[0] * s[0]) + 1.0 / (s[0] * s[0] * s[1])),
               C2 * s[1] / q * (8.0 / s[0] - 1.0 / (s[0] * s[1])) + C2 * q / (s[0] * s[1] * s[1])}};
    } else {
        f = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
        df = {2.0 * s[0], 2.0 * s[1], 2.0 * s[2]};
        g = {pow(s[0] - 5.0, 2.0) + pow(s[1] - 2.0, 2.0) + pow(s[2] - 1.0, 2.0) - 9.0,
             pow(s[0] - 3.0, 2.0) + pow(s[1] - 4.0, 2.0) + pow(s[2] - 3.0, 2.0) - 9.0};
        dg = {{2.0 * (s[0] - 5.0), 2.0 * (s[1] - 2.0), 2.0 * (s[2] - 1.0)},
              {2.0 * (s[0] - 3.0), 2.0 * (s[1] - 4.0), 2.0 * (s[2] - 3.0)}};
    }
}

static int run_conlin() {
    std::string pb = args("problem", "mma");
    int iters = argi("iters", 10);
    std::vector<double> s, xmin, xmax;
    int m;
    if (pb == "mma") { s.assign(5, 5.0); xmin.assign(5, 1.0); xmax.assign(5, 10.0); m = 1; }
    else if (pb == "mma3") { s = {1.5, 0.5}; xmin = {0.2, 0.1}; xmax = {4.0, 1.6}; m = 2; }
    else { s = {4.0, 3.0, 2.0}; xmin.assign(3, 0.0); xmax.assign(3, 5.0); m = 2; }
    const int n = (int)s.size();
    CONLIN<double> opt(n, m, 1.0, std::vector<double>(m, 0.0), std::vector<double>(m, 1000.0),
                       std::vector<double>(m, 1.0), xmin, xmax);
    opt.SetParameters(argd("move", 0.5), 1.0e-5);
    std::vector<double> xin, fs, dfs, gs, dgs, xout;
    for (int k = 0; k < iters; k++) {
        double f;
        std::vector<double> df, g;
        std::vector<std::vector<double> > dg;
        eval_problem(pb, s, f, df, g, dg);
        bool finite = std::isfinite(f);
        for (int j = 0; j < n; j++) finite = finite && std::isfinite(s[j]);
        if (!finite || opt.IsConvergence(f)) break;
        xin.insert(xin.end(), s.begin(), s.end());
        fs.push_back(f);
        dfs.insert(dfs.end(), df.begin(), df.end());
        gs.insert(gs.end(), g.begin(), g.end());
        for (auto& r : dg) dgs.insert(dgs.end(), r.begin(), r.end());
        opt.UpdateVariables(s, f, df, g, dg);
        xout.insert(xout.end(), s.begin(), s.end());
    }
    Dump out(args("out", "ref.bin"));
    out.i("nm", {n, m});
    out.d("xmin", xmin); out.d("xmax", xmax);
    out.d("xin", xin); out.d("f", fs); out.d("df", dfs); out.d("g", gs); out.d("dg", dgs); out.d("xout", xout);
    return 0;
}

// ------------------------------- explicit meshes -------------------------------
// mesh=<file>: "kind nnodes nelem nen", coordinates, connectivity, E per element, "V t",
// "nfix" + (node dof value) lines, "nload" + (node dof value) lines, optionally
// "hasbody fx fy nedge tx ty" + (node node) edge lines.  The call sequence of
// sample/planestrain/sample_planestrain.cpp:26-77 (SetDirichlet, Renumbering, element loop
// with Assembling, point loads, CSR, the solve, Disassembling, the reaction by
// RemoveBoundaryConditions + Renumbering + Assembling of Ke*ElementVector) with ScalingCG
// (solver=cg: CG, as that sample uses) to cg_eps.
static void fem_element(int kind, Matrix<double>& Ke, std::vector<std::vector<std::pair<int, int> > >& n2e,
                        const std::vector<int>& el, std::vector<Vector<double> >& x, double E, double V, double t) {
    if (kind == 0) PlaneStrainStiffness<double, ShapeFunction4Square, Gauss4Square>(Ke, n2e, el, {0, 1}, x, E, V, t);
    else if (kind == 3) PlaneStrainStiffness<double, ShapeFunction3Triangle, Gauss1Triangle>(Ke, n2e, el, {0, 1}, x, E, V, t);
    else if (kind == 1) HeatTransfer<double, ShapeFunction4Square, Gauss4Square>(Ke, n2e, el, {0}, x, E, t);
    else SolidLinearIsotropicElastic<double, ShapeFunction8Cubic, Gauss8Cubic>(Ke, n2e, el, {0, 1, 2}, x, E, V);
}

// csvread csvdir=<dir> nd=<dofs per node>: the six ImportFromCSV.h readers on Node.csv,
// Element.csv, Dirichlet.csv, Neumann.csv, Initial.csv (into zero vectors of nd entries per
// node) and Periodic.csv; ragged rows are flattened with their lengths
static int run_csvread() {
    const std::string dir = args("csvdir", ".");
    const int nd = (int)argd("nd", 2);
    std::vector<Vector<double> > x;
    std::vector<std::vector<int> > elements;
    BCList ufixed, qfixed;
    std::vector<std::pair<int, int> > periodic;
    if (!ImportNodesFromCSV(x, dir + "/Node.csv") || !ImportElementsFromCSV(elements, dir + "/Element.csv") ||
        !ImportDirichletFromCSV(ufixed, dir + "/Dirichlet.csv") || !ImportNeumannFromCSV(qfixed, dir + "/Neumann.csv") ||
        !ImportPeriodicFromCSV(periodic, dir + "/Periodic.csv"))
        return 2;
    std::vector<Vector<double> > u(x.size(), Vector<double>(nd));
    if (!ImportInitialFromCSV(u, dir + "/Initial.csv")) return 2;
    std::vector<double> xs, fixv, loadv, us;
    std::vector<int> xlen, cs, clen, fixi, loadi, per;
    for (auto& xi : x) { xlen.push_back(xi.SIZE()); for (int d = 0; d < xi.SIZE(); d++) xs.push_back(xi(d)); }
    for (auto& el : elements) { clen.push_back((int)el.size()); cs.insert(cs.end(), el.begin(), el.end()); }
    for (auto& f : ufixed) { fixi.push_back(f.first.first); fixi.push_back(f.first.second); fixv.push_back(f.second); }
    for (auto& f : qfixed) { loadi.push_back(f.first.first); loadi.push_back(f.first.second); loadv.push_back(f.second); }
    for (auto& pr : periodic) { per.push_back(pr.first); per.push_back(pr.second); }
    for (auto& ui : u) for (int d = 0; d < nd; d++) us.push_back(ui(d));
    Dump out(args("out", "ref.bin"));
    out.d("nodes", xs); out.i("node_len", xlen); out.i("conn", cs); out.i("conn_len", clen);
    out.i("fix", fixi); out.d("fixval", fixv); out.i("load", loadi); out.d("loadval", loadv);
    out.i("periodic", per); out.d("initial", us);
    return 0;
}

static int run_fem() {
    int kind, nn, ne, nen;
    std::vector<Vector<double> > x;
    std::vector<std::vector<int> > elements;
    std::vector<double> Ee;
    double V, t;
    BCList ufixed, qfixed;
    int hasbody = 0, nedge = 0;
    double bfx = 0.0, bfy = 0.0, etx = 0.0, ety = 0.0;
    std::vector<std::vector<int> > edges;
    if (g_args.count("csvdir")) {
        // csvdir=<dir> kind=<k> E=<E> V=<V> t=<t>: Node.csv, Element.csv, Dirichlet.csv and
        // Neumann.csv through the reference's ImportFromCSV.h, as sample/solid/sample_linear.cpp
        const std::string dir = args("csvdir", ".");
        if (!ImportNodesFromCSV(x, dir + "/Node.csv") || !ImportElementsFromCSV(elements, dir + "/Element.csv") ||
            !ImportDirichletFromCSV(ufixed, dir + "/Dirichlet.csv") || !ImportNeumannFromCSV(qfixed, dir + "/Neumann.csv"))
            return 2;
        kind = (int)argd("kind", 2);
        nn = (int)x.size();
        ne = (int)elements.size();
        nen = (int)elements[0].size();
        Ee.assign(ne, argd("E", 210000.0));
        V = argd("V", 0.3);
        t = argd("t", 1.0);
    } else {
        std::ifstream in(args("mesh", "mesh.txt"));
        if (!in) { fprintf(stderr, "cannot read mesh\n"); return 2; }
        in >> kind >> nn >> ne >> nen;
        const int dim = kind == 2 ? 3 : 2;
        x.assign(nn, Vector<double>(dim));
        for (int i = 0; i < nn; i++)
            for (int d = 0; d < dim; d++) in >> x[i](d);
        elements.assign(ne, std::vector<int>(nen));
        for (int e = 0; e < ne; e++)
            for (int q = 0; q < nen; q++) in >> elements[e][q];
        Ee.resize(ne);
        for (int e = 0; e < ne; e++) in >> Ee[e];
        in >> V >> t;
        int nfix, nload;
        in >> nfix;
        for (int k = 0; k < nfix; k++) { int n, d; double v; in >> n >> d >> v; ufixed.push_back({{n, d}, v}); }
        in >> nload;
        for (int k = 0; k < nload; k++) { int n, d; double v; in >> n >> d >> v; qfixed.push_back({{n, d}, v}); }
        if (in >> hasbody >> bfx >> bfy >> nedge >> etx >> ety) {
            for (int k = 0; k < nedge; k++) { int a0, a1; in >> a0 >> a1; edges.push_back({a0, a1}); }
        } else {
            hasbody = 0;
            nedge = 0;
        }
    }
    const int nd = kind == 1 ? 1 : (kind == 2 ? 3 : 2);
    std::vector<Vector<double> > u(nn, Vector<double>(nd)), r(nn, Vector<double>(nd));
    std::vector<std::vector<int> > nodetoglobal(nn, std::vector<int>(nd, 0));
    SetDirichlet(u, nodetoglobal, ufixed);
    int KDEGREE = Renumbering(nodetoglobal);
    LILCSR<double> K(KDEGREE, KDEGREE);
    std::vector<double> F(KDEGREE, 0.0);
    for (int e = 0; e < ne; e++) {
        std::vector<std::vector<std::pair<int, int> > > n2e;
        Matrix<double> Ke;
        fem_element(kind, Ke, n2e, elements[e], x, Ee[e], V, t);
        Assembling(K, F, u, Ke, nodetoglobal, n2e, elements[e]);
        if (hasbody) {   // sample_planestrain.cpp:42-47: uniform body force per element
            Vector<double> Fe;
            auto fb = [&](Vector<double>) { Vector<double> f = {bfx, bfy}; return f; };
            if (kind == 3)
                PlaneStrainBodyForce<double, ShapeFunction3Triangle, Gauss1Triangle>(Fe, n2e, elements[e], {0, 1}, x, fb, t);
            else
                PlaneStrainBodyForce<double, ShapeFunction4Square, Gauss4Square>(Fe, n2e, elements[e], {0, 1}, x, fb, t);
            Assembling(F, Fe, nodetoglobal, n2e, elements[e]);
        }
    }
    Assembling(F, qfixed, nodetoglobal);
    for (auto& edge : edges) {   // sample_planestrain.cpp:51-60: uniform traction per edge
        std::vector<std::vector<std::pair<int, int> > > n2e;
        Vector<double> Fe;
        auto fs = [&](Vector<double>) { Vector<double> f = {etx, ety}; return f; };
        PlaneStrainSurfaceForce<double, ShapeFunction2Line, Gauss1Line>(Fe, n2e, edge, {0, 1}, x, fs, t);
        Assembling(F, Fe, nodetoglobal, n2e, edge);
    }
    CSR<double> Kmod(K);
    Dump out(args("out", "ref.bin"));
    {   // what was read: the mesh and the boundary lists in the order they were given
        std::vector<double> xs, fixv, loadv;
        std::vector<int> cs, fixi, loadi;
        for (auto& xi : x) for (int d = 0; d < xi.SIZE(); d++) xs.push_back(xi(d));
        for (auto& el : elements) cs.insert(cs.end(), el.begin(), el.end());
        for (auto& f : ufixed) { fixi.push_back(f.first.first); fixi.push_back(f.first.second); fixv.push_back(f.second); }
        for (auto& f : qfixed) { loadi.push_back(f.first.first); loadi.push_back(f.first.second); loadv.push_back(f.second); }
        out.d("read_coords", xs); out.i("read_conn", cs);
        out.i("read_fix", fixi); out.d("read_fixval", fixv);
        out.i("read_load", loadi); out.d("read_loadval", loadv);
    }
    std::vector<int> n2g;
    for (auto& nd2 : nodetoglobal) n2g.insert(n2g.end(), nd2.begin(), nd2.end());
    out.i("n2g", n2g);
    out.i("indptr", Kmod.indptr);
    out.i("indices", Kmod.indices);
    out.d("data", Kmod.data);
    out.d("F", F);
    const double eps = argd("cg_eps", 1e-10);
    std::vector<double> result = args("solver", "scaling_cg") == std::string("cg") ? CG(Kmod, F, 100000, eps)
                                                                                  : ScalingCG(Kmod, F, 100000, eps);
    Disassembling(u, result, nodetoglobal);
    out.d("result", result);
    RemoveBoundaryConditions(nodetoglobal);
    KDEGREE = Renumbering(nodetoglobal);
    std::vector<double> R(KDEGREE, 0.0);
    for (int e = 0; e < ne; e++) {
        std::vector<std::vector<std::pair<int, int> > > n2e;
        Matrix<double> Ke;
        fem_element(kind, Ke, n2e, elements[e], x, Ee[e], V, t);
        Vector<double> Keue = Ke * ElementVector(u, n2e, elements[e]);
        Assembling(R, Keue, nodetoglobal, n2e, elements[e]);
    }
    Disassembling(r, R, nodetoglobal);
    std::vector<double> uh, rh;
    for (auto& ui : u) for (int d = 0; d < nd; d++) uh.push_back(ui(d));
    for (auto& ri : r) for (int d = 0; d < nd; d++) rh.push_back(ri(d));
    out.d("u", uh);
    out.d("r", rh);
    {
        std::vector<std::vector<std::pair<int, int> > > n2e;
        Matrix<double> Ke;
        fem_element(kind, Ke, n2e, elements[0], x, Ee[0], V, t);
        std::vector<double> kv;
        for (int a = 0; a < Ke.ROW(); a++) for (int b = 0; b < Ke.COL(); b++) kv.push_back(Ke(a, b));
        out.d("Ke0", kv);
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_driver <simp|...> key=value ...\n"); return 2; }
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        size_t eq = a.find('=');
        if (eq != std::string::npos) g_args[a.substr(0, eq)] = a.substr(eq + 1);
    }
    std::string mode = argv[1];
    if (mode == "simp") return run_simp();
    if (mode == "conlin") return run_conlin();
    if (mode == "fem") return run_fem();
    if (mode == "csvread") return run_csvread();
    fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
