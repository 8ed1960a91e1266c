// Test infrastructure only: a C-callable harness around the REFERENCE solver
// (AmberMond/mycode src/Solver.cpp + src/Mesh.cpp), compiled from the reference's
// own sources by oracle/build_ref.py into oracle/_ref/libref_<bcset>.so.
// It is the checker that pins the CPU restatement in oracle/cfd_oracle.c; nothing
// in the product links or calls it.
//
// The build includes the (possibly variant-selected) Solver.cpp and Mesh.cpp into
// this one translation unit with private members opened, so the harness can drive
// Mesh::buildConnectivity / computeGeometry (src/Mesh.cpp:102-201) from arrays and
// call the private residual-path members (include/Solver.hpp:116-166) directly.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#define private public
#include REF_SOLVER_CPP
#include REF_MESH_CPP
#undef private

namespace {
struct Handle {
    Mesh mesh;
    Solver* solver = nullptr;
};

void to_states(const double* in, std::vector<State>& out, int n) {
    out.resize(n);
    for (int i = 0; i < n; ++i) {
        const double* s = in + 6 * i;
        out[i] = State(s[0], s[1], s[2], s[3], s[4], s[5]);
    }
}

void from_states(const std::vector<State>& in, double* out) {
    for (size_t i = 0; i < in.size(); ++i) {
        double* s = out + 6 * i;
        s[0] = in[i].rho; s[1] = in[i].rhou; s[2] = in[i].rhov;
        s[3] = in[i].rhoE; s[4] = in[i].rhok; s[5] = in[i].rhow;
    }
}
}  // namespace

extern "C" {

// cells: n_cells x 4 node ids (0-based, -1 pads triangles); bedges: n_bedges x 3 (a, b, tag)
void* ref_create(int n_nodes, const double* xy, int n_cells, const int* cells,
                 int n_bedges, const int* bedges) {
    Handle* h = new Handle();
    Mesh& m = h->mesh;
    m.nodes.resize(n_nodes + 1);
    for (int i = 0; i < n_nodes; ++i) { m.nodes[i + 1].x = xy[2 * i]; m.nodes[i + 1].y = xy[2 * i + 1]; }
    for (int e = 0; e < n_bedges; ++e) {
        int a = bedges[3 * e] + 1, b = bedges[3 * e + 1] + 1;
        m.boundaryEdges[{std::min(a, b), std::max(a, b)}] = bedges[3 * e + 2];
    }
    for (int c = 0; c < n_cells; ++c) {
        Cell cell;
        cell.id = (int)m.cells.size();
        int nv = cells[4 * c + 3] >= 0 ? 4 : 3;
        for (int k = 0; k < nv; ++k) cell.nodes.push_back(cells[4 * c + k] + 1);
        m.cells.push_back(cell);
    }
    m.buildConnectivity();
    m.computeGeometry();
    h->solver = new Solver(m);
    return h;
}

void ref_destroy(void* p) {
    Handle* h = (Handle*)p;
    delete h->solver;
    delete h;
}

void ref_sizes(void* p, int* n_cells, int* n_faces) {
    Handle* h = (Handle*)p;
    *n_cells = (int)h->mesh.cells.size();
    *n_faces = (int)h->mesh.faces.size();
}

// per face: node1, node2 (0-based), owner, neighbor, tag; nx, ny, area, xmid, ymid
void ref_faces(void* p, int* ints5, double* dbl5) {
    Handle* h = (Handle*)p;
    for (size_t f = 0; f < h->mesh.faces.size(); ++f) {
        const Face& F = h->mesh.faces[f];
        ints5[5 * f] = F.node1 - 1; ints5[5 * f + 1] = F.node2 - 1;
        ints5[5 * f + 2] = F.owner; ints5[5 * f + 3] = F.neighbor; ints5[5 * f + 4] = F.bcTag;
        dbl5[5 * f] = F.nx; dbl5[5 * f + 1] = F.ny; dbl5[5 * f + 2] = F.area;
        dbl5[5 * f + 3] = F.x_mid; dbl5[5 * f + 4] = F.y_mid;
    }
}

void ref_cells(void* p, double* vol_xc_yc) {
    Handle* h = (Handle*)p;
    for (size_t c = 0; c < h->mesh.cells.size(); ++c) {
        vol_xc_yc[3 * c] = h->mesh.cells[c].volume;
        vol_xc_yc[3 * c + 1] = h->mesh.cells[c].x_c;
        vol_xc_yc[3 * c + 2] = h->mesh.cells[c].y_c;
    }
}

void ref_set_method(void* p, int flux, int spatial) {
    ((Handle*)p)->solver->setNumericalMethod((FluxScheme)flux, (SpatialScheme)spatial);
}

void ref_set_flow_conditions(void* p, double M, double P, double T) {
    std::streambuf* old = std::cout.rdbuf(nullptr);
    ((Handle*)p)->solver->setFlowConditions(M, P, T);
    std::cout.rdbuf(old);
    std::cout.clear();
}

void ref_set_freestream_static(void* p, double M, double P, double T) {
    ((Handle*)p)->solver->setFreestreamStatic(M, P, T);
}

void ref_set_kinematic_viscosity(void* p, double Re, double L) {
    std::streambuf* old = std::cout.rdbuf(nullptr);
    ((Handle*)p)->solver->setKinematicViscosity(Re, L);
    std::cout.rdbuf(old);
    std::cout.clear();
}

void ref_get_params(void* p, double* out6) {
    Solver* s = ((Handle*)p)->solver;
    out6[0] = s->M_inf; out6[1] = s->P_total_inlet; out6[2] = s->T_total_inlet;
    out6[3] = s->P_static_exit; out6[4] = s->nu; out6[5] = s->R_gas;
}

void ref_initialize(void* p) {
    std::streambuf* old = std::cout.rdbuf(nullptr);
    ((Handle*)p)->solver->initialize();
    std::cout.rdbuf(old);
    std::cout.clear();
}

void ref_set_state(void* p, const double* U) {
    Solver* s = ((Handle*)p)->solver;
    to_states(U, s->U_current, (int)s->mesh.cells.size());
}

void ref_get_state(void* p, double* U) { from_states(((Handle*)p)->solver->U_current, U); }

void ref_residual(void* p, const double* U, double* R, int update_limiters) {
    Solver* s = ((Handle*)p)->solver;
    int n = (int)s->mesh.cells.size();
    std::vector<State> Uin, Rout(n);
    to_states(U, Uin, n);
    s->computeResiduals(Uin, Rout, update_limiters != 0);
    from_states(Rout, R);
}

// the 10 used gradient components per cell, in CellGradient member order
// (drhodx, drhody, dudx, dudy, dvdx, dvdy, dpdx, dpdy, dTdx, dTdy)
void ref_gradients(void* p, const double* U, double* G) {
    Solver* s = ((Handle*)p)->solver;
    int n = (int)s->mesh.cells.size();
    std::vector<State> Uin;
    to_states(U, Uin, n);
    s->computeGradients(Uin);
    for (int i = 0; i < n; ++i) {
        const CellGradient& g = s->cellGradients[i];
        double v[10] = {g.drhodx, g.drhody, g.dudx, g.dudy, g.dvdx, g.dvdy, g.dpdx, g.dpdy, g.dTdx, g.dTdy};
        std::memcpy(G + 10 * i, v, sizeof v);
    }
}

// computeGradients followed by computeLimiters on U
void ref_limiters(void* p, const double* U, double* phi) {
    Solver* s = ((Handle*)p)->solver;
    int n = (int)s->mesh.cells.size();
    std::vector<State> Uin;
    to_states(U, Uin, n);
    s->computeGradients(Uin);
    s->computeLimiters(Uin);
    for (int i = 0; i < n; ++i) phi[i] = s->limiters[i];
}

void ref_get_limiters(void* p, double* phi) {
    Solver* s = ((Handle*)p)->solver;
    for (size_t i = 0; i < s->limiters.size(); ++i) phi[i] = s->limiters[i];
}

void ref_set_limiters(void* p, const double* phi) {
    Solver* s = ((Handle*)p)->solver;
    s->limiters.assign(phi, phi + s->mesh.cells.size());
}

// computeLocalTimeStep on the current state; dt is kept inside the solver for Jv/precond
void ref_local_timestep(void* p, double cfl, double* dt) {
    Solver* s = ((Handle*)p)->solver;
    s->computeLocalTimeStep(cfl);
    for (size_t i = 0; i < s->dt_local.size(); ++i) dt[i] = s->dt_local[i];
}

void ref_preconditioner(void* p, double* D) {
    Solver* s = ((Handle*)p)->solver;
    std::vector<double> d;
    s->computeDiagonalPreconditioner(d);
    for (size_t i = 0; i < d.size(); ++i) D[i] = d[i];
}

void ref_apply_jacobian(void* p, const double* Ub, const double* Rb, const double* v, double* Jv) {
    Solver* s = ((Handle*)p)->solver;
    int n = (int)s->mesh.cells.size();
    std::vector<State> U, R, V, J(n);
    to_states(Ub, U, n); to_states(Rb, R, n); to_states(v, V, n);
    s->applyJacobian(U, R, V, J);
    from_states(J, Jv);
}

int ref_gmres(void* p, const double* Ub, const double* Rb, const double* rhs, double* x) {
    Solver* s = ((Handle*)p)->solver;
    int n = (int)s->mesh.cells.size();
    std::vector<State> U, R, B, X(n);
    to_states(Ub, U, n); to_states(Rb, R, n); to_states(rhs, B, n);
    int it = s->solveGMRES(U, R, B, X);
    from_states(X, x);
    return it;
}

double ref_norm_vm(void* p, const double* R) {
    Solver* s = ((Handle*)p)->solver;
    std::vector<State> V;
    to_states(R, V, (int)s->mesh.cells.size());
    return s->norm_L2_VolumeWeighted(V);
}

// Runs solveImplicit with stdout captured at 17 significant digits and parses the
// per-step log lines (src/Solver.cpp:1725-1726, :1746) into resVM, |R|, CFL, GMRES iters.
int ref_solve_implicit(void* p, double tol, int max_steps, double* res_vm, double* res_abs,
                       double* cfl, int* gmres_iters) {
    Solver* s = ((Handle*)p)->solver;
    std::ostringstream cap;
    std::streambuf* old = std::cout.rdbuf(cap.rdbuf());
    std::streamsize prec = std::cout.precision(17);
    s->solveImplicit(tol, max_steps);
    std::cout.precision(prec);
    std::cout.rdbuf(old);
    std::istringstream in(cap.str());
    std::string line;
    int n = -1;
    while (std::getline(in, line)) {
        int step;
        double a, b, c;
        if (std::sscanf(line.c_str(), "Newton Step %d | Abs Residual Norm: %lf | VM ||R||: %lf | CFL: %lf",
                        &step, &a, &b, &c) == 4) {
            n = step;
            if (step < max_steps) { res_abs[step] = a; res_vm[step] = b; cfl[step] = c; gmres_iters[step] = 0; }
        } else if (n >= 0 && std::sscanf(line.c_str(), "  GMRES Iters: %d", &step) == 1) {
            gmres_iters[n] = step;
        }
    }
    return n + 1;
}

}  // extern "C"

namespace {
// runs f with std::cout captured at 17 significant digits; returns what it printed
template <class Fn>
std::string captured(Fn f) {
    std::ostringstream cap;
    std::streambuf* old = std::cout.rdbuf(cap.rdbuf());
    std::streamsize prec = std::cout.precision(17);
    f();
    std::cout.precision(prec);
    std::cout.rdbuf(old);
    return cap.str();
}
}  // namespace

extern "C" {

// timeStepExplicit (src/Solver.cpp:1219-1243) on the current state (its output captured)
void ref_time_step_explicit(void* p, double dt) {
    Solver* s = ((Handle*)p)->solver;
    captured([&] { s->timeStepExplicit(dt); });
}

// solveUnsteady (src/Solver.cpp:1801-1864) from the current state (its output captured)
void ref_solve_unsteady(void* p, double dt_phy, int n_steps) {
    Solver* s = ((Handle*)p)->solver;
    captured([&] { s->solveUnsteady(dt_phy, n_steps); });
}

// computeWallDistances (src/Solver.cpp:1981-2015)
void ref_wall_distance(void* p, double* d) {
    Solver* s = ((Handle*)p)->solver;
    captured([&] { s->computeWallDistances(); });
    for (size_t i = 0; i < s->wallDistances.size(); ++i) d[i] = s->wallDistances[i];
}

// calculateDrag (src/Solver.cpp:1307-1325) on the current state, parsed from its output
double ref_drag(void* p) {
    Solver* s = ((Handle*)p)->solver;
    std::string out = captured([&] { s->calculateDrag(); });
    double d = 0.0;
    std::sscanf(out.c_str(), " Drag :%lf", &d);
    return d;
}

// calculateEntropyError (src/Solver.cpp:1620-1646), parsed from its output
double ref_entropy_error(void* p) {
    Solver* s = ((Handle*)p)->solver;
    std::string out = captured([&] { s->calculateEntropyError(); });
    size_t k = out.find("L2 Entropy Error:");
    double e = -1.0;
    if (k != std::string::npos) std::sscanf(out.c_str() + k, "L2 Entropy Error: %lf", &e);
    return e;
}

// extractSkinFriction (src/Solver.cpp:1899-1979) into the CSV at path (sorted by x, six
// significant digits); returns the number of rows read back into x, cf (at most cap)
int ref_skin_friction(void* p, const char* path, double* x, double* cf, int cap) {
    Solver* s = ((Handle*)p)->solver;
    captured([&] { s->extractSkinFriction(path); });
    std::ifstream in(path);
    std::string line;
    std::getline(in, line);
    int n = 0;
    while (std::getline(in, line) && n < cap) {
        double a, b, c;
        if (std::sscanf(line.c_str(), "%lf,%lf,%lf", &a, &b, &c) == 3) {
            x[n] = a;
            cf[n] = b;
            ++n;
        }
    }
    return n;
}

}  // extern "C"
