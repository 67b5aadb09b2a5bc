// pansfem2_gb300.hpp -- the reference's C++ template API for the SIMP path,
// backed by the GB300 library through its C ABI (pansfem2_gpu.h).
//
// A driver written against PANSFEM2's headers (sample/optimize/
// sample_optimize_density_{oc,mma}.cpp) switches to the GPU by including this
// header instead and using namespace PANSFEM2_GB300: the class and function
// names, argument order and meaning, and the error behaviour (return the last
// iterate when a solver hits itrmax) are the reference's.  Differences, all
// forced by the device boundary, are listed where they occur:
//   * OC::UpdateVariables takes the samples' volume constraint as a
//     VolumeConstraint value instead of a host callable, because the
//     bisection runs on the device (a host callable cannot run there).
//   * Structured grids: Problem owns the device context of a SquareMesh-style
//     grid (or its 3D analogue); the matrix-free and multigrid solvers and the
//     whole-iteration driver SimpLoop work on it.
//   * Explicit meshes: FemMesh takes the node and element lists the
//     Import*FromCSV readers fill and replaces the element loop of
//     Assembling calls; nodes are std::vector<T> rows (or any type built from
//     one, such as the reference's Vector<T>).
// Every call throws std::runtime_error with psf_last_error() on a device or
// input error; nothing falls back to the CPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pansfem2_gpu.h"

namespace PANSFEM2_GB300 {

inline psf_status check(psf_status s, bool allow_not_converged = true) {
    if (s == PSF_OK || (allow_not_converged && (s == PSF_NOT_CONVERGED || s == PSF_FELL_BACK))) return s;
    throw std::runtime_error(std::string("pansfem2_gb300: ") + psf_last_error());
}

// ------------------------------------------------------------------ LILCSR / CSR (LILCSR.h, CSR.h)
template <class T>
class CSR;

// LILCSR<T> (LILCSR.h:24-63): rows of (column, value) pairs in first-touch order
template <class T>
class LILCSR {
public:
    LILCSR(int rows, int cols) : ROWS(rows), COLS(cols), data(rows) {}
    const int ROWS;
    const int COLS;
    bool set(int row, int col, T v) {
        for (auto &d : data[row])
            if (d.first == col) { d.second = v; return true; }
        data[row].push_back({col, v});
        return false;
    }
    T get(int row, int col) const {
        for (const auto &d : data[row])
            if (d.first == col) return d.second;
        return T();
    }
    template <class F>
    friend class CSR;

private:
    std::vector<std::vector<std::pair<int, T> > > data;
};

// CSR<T> (CSR.h:25-75): host arrays; operator* runs on the GPU
template <class T>
class CSR {
public:
    CSR(int rows, int cols) : ROWS(rows), COLS(cols), indptr(rows + 1, 0) {}
    // CSR(LILCSR&) (CSR.h:92-105): row sizes, per-row column sort, concatenation
    explicit CSR(LILCSR<T> &m) : ROWS(m.ROWS), COLS(m.COLS), indptr(m.ROWS + 1, 0) {
        for (int i = 0; i < ROWS; i++) {
            auto row = m.data[i];
            std::sort(row.begin(), row.end());
            indptr[i + 1] = indptr[i] + (int)row.size();
            for (auto &e : row) { indices.push_back(e.first); values.push_back(e.second); }
        }
    }
    CSR(int rows, int cols, std::vector<int32_t> p, std::vector<int32_t> idx, std::vector<T> v)
        : ROWS(rows), COLS(cols), indptr(std::move(p)), indices(std::move(idx)), values(std::move(v)) {}
    const int ROWS;
    const int COLS;
    const std::vector<T> operator*(const std::vector<T> &x) {
        std::vector<T> y(ROWS);
        check(psf_csr_spmv(ROWS, indptr.data(), indices.data(), values.data(), x.data(), y.data()), false);
        return y;
    }
    T get(int row, int col) const {
        auto b = indices.begin() + indptr[row], e = indices.begin() + indptr[row + 1];
        auto it = std::lower_bound(b, e, col);
        return (it != e && *it == col) ? values[it - indices.begin()] : T();
    }
    const std::vector<int32_t> &Indptr() const { return indptr; }
    const std::vector<int32_t> &Indices() const { return indices; }
    const std::vector<T> &Data() const { return values; }

private:
    std::vector<int32_t> indptr, indices;
    std::vector<T> values;
};

namespace detail {
template <class T>
std::vector<T> csr_solve(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps, int solver) {
    static_assert(sizeof(T) == sizeof(double), "the GPU solvers take double");
    std::vector<T> x(b.size());
    psf_solve_info info;
    psf_status s = psf_csr_solve(A.ROWS, A.Indptr().data(), A.Indices().data(), A.Data().data(), b.data(), solver,
                                 itrmax, eps, x.data(), &info);
    check(s);
    return x;   // last iterate on PSF_NOT_CONVERGED, as CG.h:451-452
}
}  // namespace detail

// ScalingCG (CG.h:419-453)
template <class T>
std::vector<T> ScalingCG(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps) {
    return detail::csr_solve(A, b, itrmax, eps, PSF_SOLVE_CSR_JACOBI_F64);
}
// CG (CG.h:123-154)
template <class T>
std::vector<T> CG(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps) {
    return detail::csr_solve(A, b, itrmax, eps, PSF_SOLVE_CSR_CG_F64);
}
// BiCGSTAB (CG.h:158-193)
template <class T>
std::vector<T> BiCGSTAB(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps) {
    return detail::csr_solve(A, b, itrmax, eps, PSF_SOLVE_CSR_BICGSTAB_F64);
}
// BiCGSTAB2 (CG.h:196-253)
template <class T>
std::vector<T> BiCGSTAB2(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps) {
    return detail::csr_solve(A, b, itrmax, eps, PSF_SOLVE_CSR_BICGSTAB2_F64);
}
// ScalingBiCGSTAB (CG.h:457-495)
template <class T>
std::vector<T> ScalingBiCGSTAB(CSR<T> &A, const std::vector<T> &b, int itrmax, T eps) {
    return detail::csr_solve(A, b, itrmax, eps, PSF_SOLVE_CSR_SCALING_BICGSTAB_F64);
}
// ILU0 (CG.h:257-284): the factor on A's pattern, computed on the GPU
template <class T>
CSR<T> ILU0(CSR<T> &A) {
    std::vector<T> m(A.Data().size());
    check(psf_csr_ilu0(A.ROWS, A.Indptr().data(), A.Indices().data(), A.Data().data(), nullptr, nullptr, m.data(),
                       nullptr), false);
    return CSR<T>(A.ROWS, A.COLS, A.Indptr(), A.Indices(), m);
}
// PreILU0 (CG.h:288-315): U^-1 L^-1 b with the factor M
template <class T>
std::vector<T> PreILU0(CSR<T> &M, std::vector<T> &b) {
    std::vector<T> v(b.size());
    check(psf_csr_ilu0(M.ROWS, M.Indptr().data(), M.Indices().data(), M.Data().data(), M.Data().data(), b.data(),
                       nullptr, v.data()), false);
    return v;
}
// ILU0CG (CG.h:319-352) and ILU0BiCGSTAB (CG.h:356-391) with the factor M of ILU0(A)
template <class T>
std::vector<T> ILU0CG(CSR<T> &A, CSR<T> &M, const std::vector<T> &b, int itrmax, T eps) {
    std::vector<T> x(b.size());
    psf_solve_info info;
    check(psf_csr_solve_ilu0(A.ROWS, A.Indptr().data(), A.Indices().data(), A.Data().data(), M.Data().data(),
                             b.data(), PSF_SOLVE_CSR_ILU0_CG_F64, itrmax, eps, x.data(), &info));
    return x;
}
template <class T>
std::vector<T> ILU0BiCGSTAB(CSR<T> &A, CSR<T> &M, std::vector<T> &b, int itrmax, T eps) {
    std::vector<T> x(b.size());
    psf_solve_info info;
    check(psf_csr_solve_ilu0(A.ROWS, A.Indptr().data(), A.Indices().data(), A.Data().data(), M.Data().data(),
                             b.data(), PSF_SOLVE_CSR_ILU0_BICGSTAB_F64, itrmax, eps, x.data(), &info));
    return x;
}

// ------------------------------------------------------------------ structured-grid problem
// SquareMesh<T>(lx, ly, nx, ny) (SquareMesh.h:19-45) or its 3D analogue, with
// the element routine of `kind` (psf_element_kind); owns the device context.
class Problem {
public:
    Problem(int kind, int nx, int ny, int nz, double lx, double ly, double lz, double V = 0.3, double t = 1.0) {
        check(psf_create(&ctx_, kind, nx, ny, nz, lx, ly, lz, V, t), false);
        int64_t ne, nn, nf, nz2;
        int nd;
        check(psf_sizes(ctx_, &ne, &nn, &nd, &nf, &nz2), false);
        ne_ = ne; nnodes_ = nn; ndof_ = nd;
    }
    ~Problem() { psf_destroy(ctx_); }
    Problem(const Problem &) = delete;
    Problem &operator=(const Problem &) = delete;
    psf_ctx *ctx() const { return ctx_; }
    long long ne() const { return ne_; }
    long long nnodes() const { return nnodes_; }
    int ndof() const { return ndof_; }

    // SetDirichlet + Renumbering (BoundaryCondition.h:19-25, Assembling.h:175-186): the
    // samples' ufixed list of ((node, dof), value); returns KDEGREE
    int SetDirichlet(const std::vector<std::pair<std::pair<int, int>, double> > &ufixed) {
        std::vector<int> n, d;
        std::vector<double> v;
        for (auto &u : ufixed) { n.push_back(u.first.first); d.push_back(u.first.second); v.push_back(u.second); }
        check(psf_set_dirichlet(ctx_, (int)n.size(), n.data(), d.data(), v.data(), nullptr), false);
        int64_t nf;
        check(psf_sizes(ctx_, nullptr, nullptr, nullptr, &nf, nullptr), false);
        return (int)nf;
    }
    // Assembling(F, qfixed, nodetoglobal) (Assembling.h:151-158)
    void SetLoads(const std::vector<std::pair<std::pair<int, int>, double> > &qfixed) {
        std::vector<int> n, d;
        std::vector<double> v;
        for (auto &q : qfixed) { n.push_back(q.first.first); d.push_back(q.first.second); v.push_back(q.second); }
        check(psf_set_loads(ctx_, (int)n.size(), n.data(), d.data(), v.data()), false);
    }
    // the element loop of the samples (PlaneStrainStiffness + Assembling for every
    // element with modulus E_e, then CSR(LILCSR&)), assembled on the device
    void Assemble(const std::vector<double> &E) { check(psf_assemble(ctx_, E.data(), nullptr, nullptr), false); }
    // ScalingCG(Kmod, F, itrmax, eps) on the assembled system (solver
    // PSF_SOLVE_CSR_JACOBI_F64), or any other psf_solver; returns the reduced u
    std::vector<double> Solve(int solver, int itrmax, double eps, psf_solve_info *info = nullptr) {
        int64_t nf;
        check(psf_sizes(ctx_, nullptr, nullptr, nullptr, &nf, nullptr), false);
        std::vector<double> u(nf);
        psf_solve_info tmp;
        check(psf_solve(ctx_, solver, itrmax, eps, u.data(), info ? info : &tmp));
        return u;
    }
    // compliance and dfdrho of the samples' reaction/sensitivity loops
    // (sample_optimize_density_oc.cpp:136-162) for the last solution
    double ComplianceSensitivity(const std::vector<double> &rho, double E1, double E0, double p, double scale0,
                                 std::vector<double> &dfdrho) {
        double f = 0.0;
        dfdrho.resize(rho.size());
        check(psf_compliance_sensitivity(ctx_, rho.data(), E1, E0, p, scale0, &f, dfdrho.data()), false);
        return f;
    }

private:
    psf_ctx *ctx_ = nullptr;
    long long ne_ = 0, nnodes_ = 0;
    int ndof_ = 0;
};

// ------------------------------------------------------------------ DensityFilter (DensityFilter.h:16-71)
template <class T>
class DensityFilter {
public:
    // the reference's constructor: explicit neighbour lists and weights
    DensityFilter(int n, std::vector<std::vector<int> > neighbors, std::vector<std::vector<T> > w) : n_(n) {
        ptr_.push_back(0);
        for (int i = 0; i < n; i++) {
            for (size_t k = 0; k < neighbors[i].size(); k++) { idx_.push_back(neighbors[i][k]); w_.push_back(w[i][k]); }
            ptr_.push_back((int32_t)idx_.size());
        }
    }
    // structured grid: the lists of radius R are the clipped stencil, built on the device
    DensityFilter(Problem &p, double R) : n_((int)p.ne()), prob_(&p) { check(psf_filter_setup(p.ctx(), R), false); }
    std::vector<T> GetFilteredVariables(std::vector<T> s) {
        std::vector<T> out(n_);
        if (prob_) check(psf_filter_forward(prob_->ctx(), s.data(), out.data()), false);
        else check(psf_list_filter(n_, ptr_.data(), idx_.data(), w_.data(), s.data(), out.data()), false);
        return out;
    }
    // normalised by wsum_i, as DensityFilter.h:68 does
    std::vector<T> GetFilteredSensitivitis(std::vector<T> s, std::vector<T> dfdrho) {
        (void)s;
        std::vector<T> out(n_);
        if (prob_) check(psf_filter_backward(prob_->ctx(), dfdrho.data(), out.data()), false);
        else check(psf_list_filter(n_, ptr_.data(), idx_.data(), w_.data(), dfdrho.data(), out.data()), false);
        return out;
    }

private:
    int n_;
    Problem *prob_ = nullptr;
    std::vector<int32_t> ptr_, idx_;
    std::vector<T> w_;
};

// ------------------------------------------------------------------ HeavisideFilter (HeavisideFilter.h:16-98)
// On the structured grid's filter of radius R; beta starts at 1 (HeavisideFilter.h:48).
template <class T>
class HeavisideFilter {
public:
    HeavisideFilter(Problem &p, double R) : n_((int)p.ne()), prob_(&p) { check(psf_filter_setup(p.ctx(), R), false); }
    void UpdateBeta(T beta) { beta_ = beta; }
    std::vector<T> GetFilteredVariables(std::vector<T> s) {
        std::vector<T> out(n_);
        check(psf_heaviside_forward(prob_->ctx(), beta_, s.data(), out.data()), false);
        return out;
    }
    std::vector<T> GetFilteredSensitivitis(std::vector<T> s, std::vector<T> dfdrho) {
        std::vector<T> out(n_);
        check(psf_heaviside_backward(prob_->ctx(), beta_, s.data(), dfdrho.data(), out.data()), false);
        return out;
    }

private:
    int n_;
    Problem *prob_;
    T beta_ = 1.0;
};

// ------------------------------------------------------------------ SensitivityFilter (SensitivityFilter.h:16-99)
// Sigmund's scheme (SensitivityFilter) and Borrvall's (SensitivityFilter2) on the
// structured grid's filter of radius R.
template <class T>
class SensitivityFilter {
public:
    SensitivityFilter(Problem &p, double R, int mode = 0) : n_((int)p.ne()), mode_(mode), prob_(&p) {
        check(psf_filter_setup(p.ctx(), R), false);
    }
    std::vector<T> GetFilteredSensitivitis(std::vector<T> s, std::vector<T> dfds) {
        std::vector<T> out(n_);
        check(psf_sensitivity_filter(prob_->ctx(), mode_, s.data(), dfds.data(), out.data()), false);
        return out;
    }

private:
    int n_, mode_;
    Problem *prob_;
};

template <class T>
class SensitivityFilter2 : public SensitivityFilter<T> {
public:
    SensitivityFilter2(Problem &p, double R) : SensitivityFilter<T>(p, R, 1) {}
};

// ------------------------------------------------------------------ OC (OC.h:16-107)
// The samples' constraint callback (sample_optimize_density_oc.cpp:198-207):
// filtered volume fraction g(x) = sum_i scale1*rho_i(x)/(vf*n) - scale1.
struct VolumeConstraint {
    double vf;
    double scale1;
};

template <class T>
class OC {
public:
    OC(Problem &p, int n, T iota, T lambdamin, T lambdamax, T lambdaeps, T movelimit, const std::vector<T> &xmin,
       const std::vector<T> &xmax)
        : p_(p), n_(n), iota_(iota), lmin_(lambdamin), lmax_(lambdamax), leps_(lambdaeps), move_(movelimit) {
        (void)xmin; (void)xmax;   // stored but unused by the reference's update (OC.h:86-91)
    }
    bool IsConvergence(T f) { return std::fabs(f - prev_) / (f + prev_) < 1.0e-5; }
    // UpdateVariables (OC.h:76-107) with the filtered-volume constraint on the
    // device; the filter is the Problem's (DensityFilter(Problem&, R)).
    void UpdateVariables(std::vector<T> &xk, T f, std::vector<T> dfdx, T g, std::vector<T> dgdx,
                         const VolumeConstraint &c) {
        (void)g;
        double lambda;
        check(psf_oc_update(p_.ctx(), xk.data(), dfdx.data(), dgdx.data(), iota_, lmin_, lmax_, leps_, move_, c.vf,
                            c.scale1, &lambda), false);
        prev_ = f;
    }

private:
    Problem &p_;
    int n_;
    T iota_, lmin_, lmax_, leps_, move_, prev_ = T();
};

// ------------------------------------------------------------------ MMA (MMA.h:18-509)
// One constraint with uniform bounds (the SIMP samples) runs on the Problem's device state
// (psf_mma_init / psf_mma_update); any other m <= 4 or per-variable bounds run on a device MMA
// object of their own (psf_mma_create / psf_mma_update_host).
template <class T>
class MMA {
public:
    // the reference's signature (MMA.h:20-22): a device MMA object of its own
    MMA(int n, int m, T a0, std::vector<T> a, std::vector<T> c, std::vector<T> d, const std::vector<T> &xmin,
        const std::vector<T> &xmax)
        : MMA(nullptr, n, m, a0, a, c, d, xmin, xmax) {}
    // on a Problem: m = 1 with uniform bounds runs on the Problem's device state
    MMA(Problem &p, int n, int m, T a0, std::vector<T> a, std::vector<T> c, std::vector<T> d,
        const std::vector<T> &xmin, const std::vector<T> &xmax)
        : MMA(&p, n, m, a0, a, c, d, xmin, xmax) {}
    MMA(Problem *p, int n, int m, T a0, std::vector<T> a, std::vector<T> c, std::vector<T> d,
        const std::vector<T> &xmin, const std::vector<T> &xmax)
        : p_(p), n_(n), m_(m), a0_(a0), av_(a), cv_(c), dv_(d), xminv_(xmin), xmaxv_(xmax) {
        if (m < 1 || m > 4) throw std::runtime_error("pansfem2_gb300: the device MMA solves 1 <= m <= 4 constraints");
        if ((int)a.size() < m || (int)c.size() < m || (int)d.size() < m || (int)xmin.size() < n || (int)xmax.size() < n)
            throw std::runtime_error("pansfem2_gb300: MMA needs m entries of a, c, d and n of xmin, xmax");
        bool uniform = true;
        for (int j = 1; j < n; j++) uniform = uniform && xmin[j] == xmin[0] && xmax[j] == xmax[0];
        general_ = !(p && m == 1 && uniform);
        if (general_) {
            std::vector<double> a64(a.begin(), a.end()), c64(c.begin(), c.end()), d64(d.begin(), d.end()),
                lo(xmin.begin(), xmin.begin() + n), hi(xmax.begin(), xmax.begin() + n);
            check(psf_mma_create(n, m, a0, a64.data(), c64.data(), d64.data(), lo.data(), hi.data(), &obj_), false);
        }
        init();
    }
    ~MMA() {
        if (obj_) psf_mma_destroy(obj_);
    }
    MMA(const MMA &) = delete;
    MMA &operator=(const MMA &) = delete;
    void SetParameters(T raa0, T albefa, T move, T asyinit, T asydecr, T asyincr, T epsvalue) {
        raa0_ = raa0; albefa_ = albefa; move_ = move; asyinit_ = asyinit; asydecr_ = asydecr; asyincr_ = asyincr;
        eps_ = epsvalue;
        init();
    }
    bool IsConvergence(T f) { return std::fabs(f - prev_) / (f + prev_) < eps_; }
    void UpdateVariables(std::vector<T> &xk, T f, std::vector<T> dfdx, std::vector<T> g,
                         std::vector<std::vector<T> > dgdx) {
        int newton = 0;
        if (general_) {
            std::vector<double> x(xk.begin(), xk.begin() + n_), df(dfdx.begin(), dfdx.begin() + n_),
                gv(g.begin(), g.begin() + m_), dg((size_t)m_ * n_);
            for (int i = 0; i < m_; i++)
                for (int j = 0; j < n_; j++) dg[(size_t)i * n_ + j] = dgdx.at(i).at(j);
            check(psf_mma_update_host(obj_, x.data(), f, df.data(), gv.data(), dg.data(), &newton));
            for (int j = 0; j < n_; j++) xk[j] = x[j];
        } else {
            check(psf_mma_update(p_->ctx(), xk.data(), f, dfdx.data(), g.at(0), dgdx.at(0).data(), &newton));
        }
        prev_ = f;
    }

private:
    void init() {
        if (general_)
            check(psf_mma_set_parameters(obj_, raa0_, albefa_, move_, asyinit_, asydecr_, asyincr_, eps_), false);
        else
            check(psf_mma_init(p_->ctx(), a0_, av_.at(0), cv_.at(0), dv_.at(0), xminv_.at(0), xmaxv_.at(0), raa0_,
                               albefa_, move_, asyinit_, asydecr_, asyincr_, eps_), false);
    }
    Problem *p_;
    int n_, m_;
    T a0_;
    std::vector<T> av_, cv_, dv_, xminv_, xmaxv_;
    bool general_ = false;
    psf_mma *obj_ = nullptr;
    T raa0_ = 1.0e-5, albefa_ = 0.1, move_ = 0.5, asyinit_ = 0.5, asydecr_ = 0.7, asyincr_ = 1.2, eps_ = 1.0e-5;
    T prev_ = T();
};

// ------------------------------------------------------------------ CONLIN (CONLIN.h:17-455), m = 1
template <class T>
class CONLIN {
public:
    CONLIN(Problem &p, int n, int m, T a0, std::vector<T> a, std::vector<T> c, std::vector<T> d,
           const std::vector<T> &xmin, const std::vector<T> &xmax)
        : p_(p), n_(n), a0_(a0), a_(a.at(0)), c_(c.at(0)), d_(d.at(0)), xmin_(xmin.at(0)), xmax_(xmax.at(0)) {
        if (m != 1) throw std::runtime_error("pansfem2_gb300: the device CONLIN solves m = 1 (one constraint)");
        for (int j = 1; j < n && j < (int)xmin.size() && j < (int)xmax.size(); j++)
            if (xmin[j] != xmin[0] || xmax[j] != xmax[0])
                throw std::runtime_error("pansfem2_gb300: the device CONLIN takes uniform bounds (xmin, xmax the same "
                                         "for every variable)");
        init();
    }
    void SetParameters(T move, T epsvalue) {
        move_ = move;
        eps_ = epsvalue;
        init();
    }
    bool IsConvergence(T f) { return std::fabs(f - prev_) / (f + prev_) < eps_; }
    void UpdateVariables(std::vector<T> &xk, T f, std::vector<T> dfdx, std::vector<T> g,
                         std::vector<std::vector<T> > dgdx) {
        int newton = 0;
        check(psf_conlin_update(p_.ctx(), xk.data(), f, dfdx.data(), g.at(0), dgdx.at(0).data(), &newton));
        prev_ = f;
    }

private:
    void init() { check(psf_conlin_init(p_.ctx(), a0_, a_, c_, d_, xmin_, xmax_, move_, eps_), false); }
    Problem &p_;
    int n_;
    T a0_, a_, c_, d_, xmin_, xmax_;
    T move_ = 0.5, eps_ = 1.0e-5;
    T prev_ = T();
};

// ------------------------------------------------------------------ the whole iteration on the device
// One call per iteration of the samples' loop body (filter, volume, solve,
// compliance, sensitivities, filtered sensitivities, OC/MMA/CONLIN update).
class SimpLoop {
public:
    SimpLoop(Problem &p, const psf_simp_params &prm, const std::vector<double> *s0 = nullptr) : p_(p) {
        check(psf_simp_begin(p.ctx(), &prm, s0 ? s0->data() : nullptr), false);
    }
    psf_iter_info Step() {
        psf_iter_info info;
        check(psf_simp_step(p_.ctx(), &info));
        return info;
    }
    std::vector<double> Densities() {
        std::vector<double> rho(p_.ne());
        check(psf_simp_fields(p_.ctx(), nullptr, rho.data(), nullptr, nullptr, nullptr), false);
        return rho;
    }
    std::vector<double> Design() {
        std::vector<double> s(p_.ne());
        check(psf_simp_fields(p_.ctx(), s.data(), nullptr, nullptr, nullptr, nullptr), false);
        return s;
    }

private:
    Problem &p_;
};

// ------------------------------------------------------------------ CSV files (ImportFromCSV.h:22-253)
// One header line, then whitespace-separated records, each split on ','; the first field is
// an id.  Nodes and elements are numbered by their position in the file; in the condition
// files the value fields are the dofs 0, 1, ... and "free" skips one.  Numbers go through
// std::stod / std::stoi, which throw on a bad field, as in the reference.
namespace detail {
// entry d and length of a node row: std::vector<T> (operator[], size) or the reference's
// Vector<T> (operator(), SIZE)
template <class V>
auto entry(V &v, int d, int) -> decltype(v[d]) { return v[d]; }
template <class V>
auto entry(V &v, int d, long) -> decltype(v(d)) { return v(d); }
template <class V>
auto length(const V &v, int) -> decltype((int)v.size()) { return (int)v.size(); }
template <class V>
auto length(const V &v, long) -> decltype((int)v.SIZE()) { return (int)v.SIZE(); }

template <class Record>
bool csv_records(const std::string &fname, const char *what, Record record) {
    std::ifstream in(fname);
    if (!in) {
        std::cout << what << " file " << fname << " open error!" << std::endl;
        return false;
    }
    std::string line;
    std::getline(in, line);   // the header
    std::string token;
    while (in >> token) {
        std::istringstream fields(token);
        std::string id;
        std::getline(fields, id, ',');
        if (!id.empty()) record(id, fields);
    }
    return true;
}
inline bool csv_conditions(std::vector<std::pair<std::pair<int, int>, double> > &out, const std::string &fname) {
    return csv_records(fname, "Dirichlet Condition", [&](const std::string &id, std::istringstream &fields) {
        const int node = std::stoi(id);
        std::string v;
        for (int dof = 0; std::getline(fields, v, ','); dof++)
            if (v != "free") out.push_back({{node, dof}, std::stod(v)});
    });
}
}  // namespace detail

// ImportNodesFromCSV (ImportFromCSV.h:22-58): coordinates in file order
template <class Node>
bool ImportNodesFromCSV(std::vector<Node> &nodes, std::string fname) {
    return detail::csv_records(fname, "Node", [&](const std::string &, std::istringstream &fields) {
        std::vector<double> x;
        std::string v;
        while (std::getline(fields, v, ',')) x.push_back(std::stod(v));
        nodes.push_back(Node(x));
    });
}
// ImportElementsFromCSV (ImportFromCSV.h:63-98)
inline bool ImportElementsFromCSV(std::vector<std::vector<int> > &elements, std::string fname) {
    return detail::csv_records(fname, "Element", [&](const std::string &, std::istringstream &fields) {
        std::vector<int> el;
        std::string v;
        while (std::getline(fields, v, ',')) el.push_back(std::stoi(v));
        elements.push_back(el);
    });
}
// ImportDirichletFromCSV (ImportFromCSV.h:103-137): ((node, dof), value) in file order
template <class T>
bool ImportDirichletFromCSV(std::vector<std::pair<std::pair<int, int>, T> > &ufixed, std::string fname) {
    return detail::csv_conditions(ufixed, fname);
}
// ImportNeumannFromCSV (ImportFromCSV.h:142-176); its open error names the Dirichlet file, as
// the reference's does
template <class T>
bool ImportNeumannFromCSV(std::vector<std::pair<std::pair<int, int>, T> > &qfixed, std::string fname) {
    return detail::csv_conditions(qfixed, fname);
}
// ImportInitialFromCSV (ImportFromCSV.h:181-216): u[node][dof] for the fields that are not
// "free"; a missing field repeats the one before it, as a failed std::getline leaves it
template <class Node>
bool ImportInitialFromCSV(std::vector<Node> &u, std::string fname) {
    return detail::csv_records(fname, "Initial Condition", [&](const std::string &id, std::istringstream &fields) {
        const int node = std::stoi(id);
        std::string v = id;
        for (int dof = 0; dof < detail::length(u[node], 0); dof++) {
            std::getline(fields, v, ',');
            if (v != "free") detail::entry(u[node], dof, 0) = std::stod(v);
        }
    });
}
// ImportPeriodicFromCSV (ImportFromCSV.h:221-253): (master, slave) pairs
inline bool ImportPeriodicFromCSV(std::vector<std::pair<int, int> > &pairs, std::string fname) {
    return detail::csv_records(fname, "Periodic Boundary Condition", [&](const std::string &id, std::istringstream &fields) {
        std::string v = id;
        std::getline(fields, v, ',');
        pairs.push_back({std::stoi(id), std::stoi(v)});
    });
}

// ------------------------------------------------------------------ explicit meshes
// The general path of sample_planestrain.cpp / sample/solid/sample_linear.cpp on the device:
// SetDirichlet + Renumbering, the element loop of stiffness routines and Assembling calls,
// point loads, body forces and edge tractions, CSR(LILCSR&), ScalingCG / CG, Disassembling
// and the reaction loop.  kind is a psf_element_kind (T3 / Q4 plane strain, Q4 heat, H8).
class FemMesh {
public:
    template <class Node>
    FemMesh(int kind, const std::vector<Node> &x, const std::vector<std::vector<int> > &elements) {
        const int dim = kind == PSF_H8_SOLID ? 3 : 2;
        std::vector<double> xs;
        std::vector<int32_t> conn;
        for (auto &xi : x)
            for (int d = 0; d < dim; d++) xs.push_back(detail::entry(const_cast<Node &>(xi), d, 0));
        const int nen = elements.empty() ? 0 : (int)elements[0].size();
        for (auto &el : elements) {
            if ((int)el.size() != nen) throw std::runtime_error("pansfem2_gb300: elements of different sizes");
            conn.insert(conn.end(), el.begin(), el.end());
        }
        nnodes_ = (long long)x.size();
        ne_ = (long long)elements.size();
        ndof_ = kind == PSF_Q4_HEAT ? 1 : dim;
        check(psf_fem_create(kind, nnodes_, xs.data(), ne_, nen, conn.data(), &fem_), false);
    }
    ~FemMesh() { psf_fem_destroy(fem_); }
    FemMesh(const FemMesh &) = delete;
    FemMesh &operator=(const FemMesh &) = delete;
    long long nnodes() const { return nnodes_; }
    int ndof() const { return ndof_; }

    // SetDirichlet + Renumbering (BoundaryCondition.h:19-25, Assembling.h:175-186); returns KDEGREE
    int SetDirichlet(const std::vector<std::pair<std::pair<int, int>, double> > &ufixed) {
        std::vector<int32_t> n, d;
        std::vector<double> v;
        for (auto &u : ufixed) { n.push_back(u.first.first); d.push_back(u.first.second); v.push_back(u.second); }
        int nf = 0;
        check(psf_fem_set_dirichlet(fem_, (int)n.size(), n.data(), d.data(), v.data(), &nf), false);
        return nf;
    }
    // Assembling(F, qfixed, nodetoglobal) (Assembling.h:151-158)
    void SetLoads(const std::vector<std::pair<std::pair<int, int>, double> > &qfixed) {
        std::vector<int32_t> n, d;
        std::vector<double> v;
        for (auto &q : qfixed) { n.push_back(q.first.first); d.push_back(q.first.second); v.push_back(q.second); }
        check(psf_fem_set_loads(fem_, (int)n.size(), n.data(), d.data(), v.data()), false);
    }
    // PlaneStrainBodyForce (PlaneStrain.h:503-534) with a uniform f in the element loop
    void SetBodyForce(double fx, double fy) { check(psf_fem_set_body_force(fem_, fx, fy), false); }
    // PlaneStrainSurfaceForce<ShapeFunction2Line, Gauss1Line> (PlaneStrain.h:421-452) per edge
    void SetEdgeLoads(const std::vector<std::vector<int> > &edges, double tx, double ty) {
        std::vector<int32_t> e;
        for (auto &ed : edges) {
            if (ed.size() != 2) throw std::runtime_error("pansfem2_gb300: an edge has 2 nodes");
            e.insert(e.end(), ed.begin(), ed.end());
        }
        check(psf_fem_set_edge_loads(fem_, (int)edges.size(), e.data(), tx, ty), false);
    }
    // the element loop with modulus E[e] (conductivity for heat), Poisson ratio V and
    // thickness t, then CSR(LILCSR&); returns the number of stored entries
    long long Assemble(const std::vector<double> &E, double V, double t) {
        if ((long long)E.size() != ne_) throw std::runtime_error("pansfem2_gb300: one modulus per element");
        long long nnz = 0;
        check(psf_fem_assemble(fem_, E.data(), V, t, &nnz), false);
        return nnz;
    }
    // ScalingCG (PSF_SOLVE_CSR_JACOBI_F64) or CG (PSF_SOLVE_CSR_CG_F64) + Disassembling: the
    // nodal solution, nnodes x ndof, prescribed values included; the last iterate when the
    // solver reaches itrmax
    std::vector<double> Solve(int solver, int itrmax, double eps, psf_solve_info *info = nullptr) {
        std::vector<double> u(nnodes_ * ndof_);
        psf_solve_info tmp;
        check(psf_fem_solve(fem_, solver, itrmax, eps, u.data(), info ? info : &tmp));
        return u;
    }
    // the reaction loop (sample_planestrain.cpp:66-77): r = sum_e Ke_e u_e over all dofs
    std::vector<double> Reaction(const std::vector<double> &u) {
        std::vector<double> r(nnodes_ * ndof_);
        check(psf_fem_reaction(fem_, u.data(), r.data()), false);
        return r;
    }

private:
    psf_fem *fem_ = nullptr;
    long long nnodes_ = 0, ne_ = 0;
    int ndof_ = 0;
};

}  // namespace PANSFEM2_GB300
