// The reference's default case (AmberMond/mycode src/main.cpp:53-100: bump channel,
// M = 0.5, P = 101325 Pa, T = 300 K, LLF, first order, JFNK to 1e-5) written against
// cfdg::GpuMesh / cfdg::GpuSolver instead of Mesh / Solver.  Prints the residual
// history in the reference's results/residual_history.csv format, then the entropy
// error and the drag as the reference prints them.
//
//   g++ -O2 -std=c++17 -I include bump_main.cpp -L mycode_gb300/_lib -lcfdgpu -o bump_main
//   ./bump_main mesh_file [max_steps]
#include <cstdio>
#include <cstdlib>

#include "cfdg_solver.hpp"

struct State {  // include/Types.hpp:55-82 layout
    double rho, rhou, rhov, rhoE, rhok, rhow;
};

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s mesh_file [max_steps]\n", argv[0]);
        return 2;
    }
    int max_steps = argc > 2 ? std::atoi(argv[2]) : 2500;
    try {
        cfdg::GpuMesh mesh;
        mesh.load(argv[1]);
        cfdg::GpuSolver solver(mesh);
        solver.setFlowConditions(0.5, 101325.0, 300.0);
        solver.initialize();
        solver.setNumericalMethod(cfdg::Flux::LLF, cfdg::Spatial::FIRST_ORDER);
        auto trace = solver.solveImplicit(1e-5, max_steps);
        std::printf("Step, Residual_VM\n");
        for (size_t k = 0; k < trace.size(); ++k) std::printf("%zu, %g\n", k, trace[k].res_vm);
        std::vector<State> U = solver.getSolution<State>();
        std::vector<State> R;
        solver.computeResiduals(U, R, false);
        std::fprintf(stderr, "cells %d steps %zu final %g\n", mesh.getNumCells(), trace.size(),
                     trace.empty() ? 0.0 : trace.back().res_vm);
        std::fflush(stdout);
        // the reference's post-processing (src/main.cpp:91-95)
        std::cout << " Grs " << std::endl;
        solver.calculateEntropyError();
        std::cout << " Drag " << std::endl;
        solver.calculateDrag();
    } catch (const cfdg::Error& e) {
        std::fprintf(stderr, "cfdg error %d: %s\n", (int)e.status, e.what());
        return 1;
    }
    return 0;
}
