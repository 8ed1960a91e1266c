// C++ front-end over the C ABI (include/cfdg.h) with the reference solver's class
// surface, so a driver written against AmberMond/mycode's Mesh and Solver
// (include/Mesh.hpp, include/Solver.hpp) switches by changing two type names.
//
//   reference                                  here
//   Mesh mesh; mesh.load(path);                cfdg::GpuMesh mesh; mesh.load(path);
//   Solver solver(mesh);                       cfdg::GpuSolver solver(mesh);
//   solver.setNumericalMethod(f, s);           solver.setNumericalMethod(f, s);
//   solver.setFlowConditions(M, P, T);         (same)
//   solver.setFreestreamStatic(M, P, T);       (same)
//   solver.setKinematicViscosity(Re, L);       (same)
//   solver.initialize();                       (same)
//   solver.computeResiduals(U, R, upd);        (same; any 6-double State type)
//   solver.solveImplicit(tol, maxSteps);       (same; returns the per-step record)
//   solver.getSolution();                      (same; vector<StateT>)
//   solver.calculateDrag(), calculateEntropyError(), extractSkinFriction(file)   (same)
//
// Failures throw cfdg::Error (the reference has no error reporting).  Header-only; link
// with libcfdgpu.so.
#pragma once

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cfdg.h"

namespace cfdg {

class Error : public std::runtime_error {
public:
    Error(cfdg_status st, const std::string& what) : std::runtime_error(what), status(st) {}
    cfdg_status status;
};

inline void check(cfdg_status st) {
    if (st != CFDG_OK) throw Error(st, cfdg_last_error());
}

// FluxScheme / SpatialScheme values of include/Types.hpp:38-49
enum class Flux { LLF = CFDG_FLUX_LLF, ROE = CFDG_FLUX_ROE, HLLC = CFDG_FLUX_HLLC, AUSM = CFDG_FLUX_AUSM };
enum class Spatial {
    FIRST_ORDER = CFDG_FIRST_ORDER,
    SECOND_ORDER_CENTRAL = CFDG_SECOND_ORDER_CENTRAL,
    SECOND_ORDER_LIMITED = CFDG_SECOND_ORDER_LIMITED
};

class GpuMesh {
public:
    GpuMesh() = default;
    GpuMesh(const GpuMesh&) = delete;
    GpuMesh& operator=(const GpuMesh&) = delete;
    ~GpuMesh() { cfdg_mesh_destroy(m_); }

    // Mesh::load (src/Mesh.cpp:10-26); CRLF and LF files both load
    void load(const std::string& filename, int renumber = CFDG_RENUMBER_HILBERT) {
        cfdg_mesh* m = nullptr;
        check(cfdg_mesh_load_gmsh(filename.c_str(), renumber, &m));
        cfdg_mesh_destroy(m_);
        m_ = m;
    }
    // from arrays (0-based node ids, -1 pads triangles; boundary edges a, b, tag)
    void create(const std::vector<double>& xy, const std::vector<int>& cells4, const std::vector<int>& bedges3,
                int renumber = CFDG_RENUMBER_HILBERT) {
        cfdg_mesh* m = nullptr;
        check(cfdg_mesh_create((int)(xy.size() / 2), xy.data(), (int)(cells4.size() / 4), cells4.data(),
                               (int)(bedges3.size() / 3), bedges3.empty() ? nullptr : bedges3.data(), renumber, &m));
        cfdg_mesh_destroy(m_);
        m_ = m;
    }
    int getNumCells() const { int n = 0; check(cfdg_mesh_sizes(m_, &n, nullptr, nullptr)); return n; }
    int getNumFaces() const { int n = 0; check(cfdg_mesh_sizes(m_, nullptr, &n, nullptr)); return n; }
    const cfdg_mesh* handle() const { return m_; }

private:
    cfdg_mesh* m_ = nullptr;
};

class GpuSolver {
public:
    explicit GpuSolver(const GpuMesh& mesh) : GpuSolver(mesh, defaults()) {}
    GpuSolver(const GpuMesh& mesh, const cfdg_config& cfg) : n_(mesh.getNumCells()), gamma_(cfg.gamma) {
        check(cfdg_solver_create(mesh.handle(), &cfg, &s_));
    }
    GpuSolver(const GpuSolver&) = delete;
    GpuSolver& operator=(const GpuSolver&) = delete;
    ~GpuSolver() { cfdg_solver_destroy(s_); }

    static cfdg_config defaults() {
        cfdg_config c;
        cfdg_config_default(&c);
        return c;
    }

    void setNumericalMethod(Flux f, Spatial s) { check(cfdg_set_numerical_method(s_, (int)f, (int)s)); }
    void setFlowConditions(double M, double P, double T) { check(cfdg_set_flow_conditions(s_, M, P, T)); }
    void setFreestreamStatic(double M, double P, double T) { check(cfdg_set_freestream_static(s_, M, P, T)); }
    void setKinematicViscosity(double Re, double L) { check(cfdg_set_kinematic_viscosity(s_, Re, L)); }
    void initialize() { check(cfdg_initialize(s_)); }

    // Solver::computeResiduals (src/Solver.cpp:529-801) on any 6-double State type
    template <class StateT>
    void computeResiduals(const std::vector<StateT>& U, std::vector<StateT>& R, bool update_limiters = true) {
        static_assert(sizeof(StateT) == 6 * sizeof(double), "State must be 6 doubles");
        R.resize(U.size());
        check(cfdg_residual(s_, reinterpret_cast<const double*>(U.data()), reinterpret_cast<double*>(R.data()),
                            update_limiters ? 1 : 0));
    }

    // Solver::solveImplicit (src/Solver.cpp:1696-1799); returns the per-step record
    std::vector<cfdg_step> solveImplicit(double tolerance = 1e-6, int maxNewtonstep = 50) {
        std::vector<cfdg_step> trace((size_t)(maxNewtonstep > 0 ? maxNewtonstep : 1));
        int n = 0;
        cfdg_status st = cfdg_solve_implicit(s_, tolerance, maxNewtonstep, trace.data(), &n);
        trace.resize((size_t)n);
        if (st != CFDG_OK && st != CFDG_ERR_NOT_CONVERGED) check(st);
        return trace;
    }

    // Solver::getSolution (include/Solver.hpp:58)
    template <class StateT>
    std::vector<StateT> getSolution() const {
        static_assert(sizeof(StateT) == 6 * sizeof(double), "State must be 6 doubles");
        std::vector<StateT> U((size_t)n_);
        check(cfdg_get_state(s_, reinterpret_cast<double*>(U.data())));
        return U;
    }

    // Solver::timeStepExplicit (src/Solver.cpp:1219-1243); returns norm_L2 of the residual
    double timeStepExplicit(double dt) {
        double r = 0;
        check(cfdg_time_step_explicit(s_, dt, &r));
        return r;
    }

    // Solver::solveUnsteady (src/Solver.cpp:1801-1864); per physical step the Newton steps
    std::vector<int> solveUnsteady(double dt_phy, int maxTimeSteps) {
        std::vector<int> it((size_t)(maxTimeSteps > 0 ? maxTimeSteps : 1));
        check(cfdg_solve_unsteady(s_, dt_phy, maxTimeSteps, it.data(), nullptr));
        it.resize((size_t)(maxTimeSteps > 0 ? maxTimeSteps : 0));
        return it;
    }

    // Solver::calculateDrag (src/Solver.cpp:1307-1325): prints " Drag :<value>" like the
    // reference and returns the value
    double calculateDrag() {
        double d = 0;
        check(cfdg_drag(s_, &d));
        std::cout << " Drag :" << d << std::endl;
        return d;
    }

    // Solver::calculateEntropyError (src/Solver.cpp:1620-1646): prints as the reference
    double calculateEntropyError() {
        double e = 0;
        check(cfdg_entropy_error(s_, &e));
        std::cout << " GRS " << std::endl;
        std::cout << " Cells: " << n_ << std::endl;
        std::cout << " L2 Entropy Error: " << e << std::endl;
        return e;
    }

    // Solver::extractSkinFriction (src/Solver.cpp:1899-1979): x, Cf and the Blasius Cf of
    // the no-slip (tag 4) faces, sorted by x, into a CSV with the reference's columns
    void extractSkinFriction(const std::string& filename) {
        int n = 0;
        check(cfdg_wall_coefficients(s_, 4, nullptr, nullptr, nullptr, &n));
        std::vector<double> x((size_t)n), cp((size_t)n), cf((size_t)n);
        if (n) check(cfdg_wall_coefficients(s_, 4, x.data(), cp.data(), cf.data(), &n));
        double p[6];
        check(cfdg_get_params(s_, p));  // M_inf, P0, T0, Pexit, nu, R_gas
        const double g = gamma_;
        double Ts = p[2] / (1.0 + 0.5 * (g - 1.0) * p[0] * p[0]);
        double u_inf = p[0] * std::sqrt(g * p[5] * Ts);
        std::vector<size_t> order((size_t)n);
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return x[a] < x[b]; });
        std::ofstream out(filename);
        out << "x,Cf,Cf_theory\n";
        for (size_t k : order) {
            double re_x = u_inf * x[k] / p[4];
            out << x[k] << "," << cf[k] << "," << (re_x > 0 ? 0.664 / std::sqrt(re_x) : 0.0) << "\n";
        }
        std::cout << "Skin friction coefficient distribution exported to " << filename << std::endl;
    }

    // computeWallDistances (src/Solver.cpp:1981-2015), per cell in the caller's numbering
    std::vector<double> wallDistances() {
        std::vector<double> d((size_t)n_);
        check(cfdg_wall_distance(s_, d.data()));
        return d;
    }

    // the adjoint: (dR/dU)^T lambda at the current state (no reference counterpart)
    template <class StateT>
    std::vector<StateT> vjp(const std::vector<StateT>& lambda) {
        static_assert(sizeof(StateT) == 6 * sizeof(double), "State must be 6 doubles");
        std::vector<StateT> g(lambda.size());
        check(cfdg_vjp(s_, nullptr, reinterpret_cast<const double*>(lambda.data()), reinterpret_cast<double*>(g.data())));
        return g;
    }

    cfdg_solver* handle() { return s_; }

private:
    int n_ = 0;
    double gamma_ = 1.4;
    cfdg_solver* s_ = nullptr;
};

}  // namespace cfdg
