/* cfdg — GB300 (sm_103a) residual-and-Newton path for a 2D unstructured
 * cell-centred finite-volume compressible-flow solver.
 *
 * C ABI of libcfdgpu.so.  Plain pointers and sizes only.  It replaces the C++ class
 * surface of the reference solver (AmberMond/mycode): Mesh (include/Mesh.hpp),
 * Solver (include/Solver.hpp) and the flux library (include/Flux.hpp).  Each entry
 * point names the reference interface it stands in for.
 *
 * Conventions
 *  - Every call returns a cfdg_status (0 = ok).  cfdg_last_error() gives the
 *    message of the calling thread's last failure.
 *  - States, residuals and vectors cross the ABI in the reference's layout and
 *    numbering: AoS, 6 doubles per cell {rho, rhou, rhov, rhoE, rhok, rhow}
 *    (struct State, include/Types.hpp:55-82), cells in the order they were given.
 *    The library renumbers the mesh internally and permutes on entry and exit.
 *  - A cfdg_mesh must outlive the solvers made from it (the reference's Solver
 *    holds a const Mesh&, include/Solver.hpp:117).
 *  - One CUDA stream per solver.  A solver is not thread-safe; distinct solvers are
 *    independent.
 *  - There is no CPU fallback: every compute entry point runs on the GPU and
 *    returns CFDG_ERR_CUDA when no usable device exists.
 */
#ifndef CFDG_H
#define CFDG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cfdg_status {
    CFDG_OK = 0,
    CFDG_ERR_ARG = 1,           /* bad argument or size */
    CFDG_ERR_CUDA = 2,          /* CUDA runtime failure or no device */
    CFDG_ERR_NAN = 3,           /* non-finite or non-positive density/pressure found */
    CFDG_ERR_NOT_CONVERGED = 4, /* solve stopped at max_steps above tolerance */
    CFDG_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
    CFDG_ERR_MESH = 6,          /* mesh file or connectivity error */
    CFDG_ERR_UNSUPPORTED = 7    /* option combination not available */
    /* A GMRES breakdown (h_{j+1,j} <= 1e-12, src/Solver.cpp:1553) is not an error: as in the
     * reference the basis vector is left unscaled and the solve goes on; a non-finite
     * solution then surfaces as CFDG_ERR_NAN at the Newton update. */
} cfdg_status;

/* FluxScheme (include/Types.hpp:38-43); AUSM evaluates LLF as in include/Flux.hpp:225 */
enum { CFDG_FLUX_LLF = 0, CFDG_FLUX_ROE = 1, CFDG_FLUX_HLLC = 2, CFDG_FLUX_AUSM = 3 };
/* SpatialScheme (include/Types.hpp:45-49) */
enum { CFDG_FIRST_ORDER = 0, CFDG_SECOND_ORDER_CENTRAL = 1, CFDG_SECOND_ORDER_LIMITED = 2 };
/* boundary-condition sets: the reference's getBoundaryGhostState variants
 * bump (src/Solver.cpp:806-863), supersonic (:973-1011), flat plate / SWBLI (:1088-1139) */
enum { CFDG_BC_BUMP = 0, CFDG_BC_SUPERSONIC = 1, CFDG_BC_PLATE = 2 };
/* initialize variants: bump (src/Solver.cpp:46-65), free stream (:905-920) */
enum { CFDG_INIT_BUMP = 0, CFDG_INIT_FREESTREAM = 1 };
/* arithmetic of the Newton-Krylov loop */
enum { CFDG_FP64 = 0, CFDG_MIXED = 1 };
/* Jacobian-vector product: one-sided finite difference (src/Solver.cpp:1331-1386) or
 * exact forward linearisation (no reference counterpart) */
enum { CFDG_JV_FD = 0, CFDG_JV_EXACT = 1 };
enum { CFDG_RENUMBER_NONE = 0, CFDG_RENUMBER_HILBERT = 1, CFDG_RENUMBER_RCM = 2 };
enum { CFDG_TURB_NONE = 0, CFDG_TURB_SST = 1 };

typedef struct cfdg_config {
    int flux;              /* CFDG_FLUX_*; reference default HLLC (include/Solver.hpp:33) */
    int spatial;           /* CFDG_*_ORDER; reference default SECOND_ORDER_LIMITED (:34) */
    int bcset;             /* CFDG_BC_* */
    int init;              /* CFDG_INIT_* */
    int viscous;           /* 1: subtract the viscous flux (src/Solver.cpp:787 instead of :792) */
    int turbulence;        /* CFDG_TURB_*; SST adds rhok, rhow (no reference counterpart) */
    int precision;         /* CFDG_FP64 or CFDG_MIXED (FP32 Krylov, Jv and preconditioner) */
    int jv;                /* CFDG_JV_FD or CFDG_JV_EXACT */
    int gmres_m;           /* Krylov dimension; reference 40 (src/Solver.cpp:1479) */
    double gmres_tol;      /* relative tolerance; reference 1e-2 (src/Solver.cpp:1587) */
    double gamma;          /* 1.4 (include/Flux.hpp:9, include/Solver.hpp:91) */
    double R_gas;          /* 287 (include/Solver.hpp:92) */
    double Pr;             /* 0.72 (src/Solver.cpp:541) */
    double nu;             /* 0.01 until setKinematicViscosity (include/Solver.hpp:42) */
    double cfl0;           /* 0.1 (src/Solver.cpp:1701) */
    double cfl_max;        /* 1e4 (src/Solver.cpp:1790) */
    int limiter_freeze_step;   /* 150 (src/Solver.cpp:1714) */
    double limiter_freeze_cfl; /* 10 (src/Solver.cpp:1714) */
    /* SST free stream (no reference counterpart) */
    double turb_intensity; /* Tu, e.g. 0.001 */
    double mut_ratio;      /* mu_t / mu in the free stream, e.g. 0.01 */
    double shock_deflection_deg; /* tag-6 post-shock inflow; 0 = unused */
    int renumber;          /* CFDG_RENUMBER_* */
    int device;            /* CUDA device ordinal */
    /* Krylov driver: CFDG_KRYLOV_HOST runs the reference's modified Gram-Schmidt loop with
     * the Hessenberg on the host (one sync per iteration); CFDG_KRYLOV_GRAPH runs the whole
     * solve as one CUDA graph (WHILE node, device Givens, CGS2 orthogonalisation, in its
     * delayed one-reduction form with the exact J v);
     * CFDG_KRYLOV_AUTO picks GRAPH for mixed precision or exact J v, else HOST. */
    int krylov;
    /* graph driver with exact J v: 1 runs each Arnoldi iteration as one persistent kernel
     * with grid barriers between its phases (two-reduction CGS2), 0 (default) as four
     * kernels; measured on the 28,800-cell plate: FP32 basis 63-72 us per iteration
     * persistent vs 54-64 us with the six-kernel body of the time (the four-kernel body
     * since: about 30 us), FP64 exact 186-200 vs 186-211 us */
    int persistent;
    /* graph driver with exact J v: 1 (default) launches the Arnoldi body's kernels after
     * the first with programmatic dependent launch, so each starts while its predecessor's
     * tail (grid reduction, Givens step) runs; 0 launches them plainly */
    int pdl;
    /* persistent Arnoldi kernel: polls of a grid barrier before the wait gives up and the
     * solve reports CFDG_ERR_TIMEOUT (0 = the default, 2^24 polls, seconds in all) */
    int barrier_poll_limit;
    /* graph driver: cfdg_solve_implicit runs its Newton steps in chains of this many, one
     * host synchronisation per chain (the CFL control on the device between the steps;
     * the same trace for any value); 1 = one synchronisation per step.  Default 8. */
    int newton_chain;
    /* Start-up aids for stiff cases, no reference counterpart, off (0) by default so the
     * reference's algorithm is untouched.  Graph driver only.
     * startup_first_order: the first this many Newton steps of a solve use the first-order
     *   scheme, then the configured one.
     * update_limit: each cell's Newton update is scaled so that its density and (to first
     *   order) pressure change by at most this fraction, and with SST rho k and rho w fall
     *   by at most this fraction (e.g. 0.2). */
    int startup_first_order;
    double update_limit;
    /* exact J v Arnoldi body: from this many cells the gather of J v and the iteration's
     * dots run as two kernels (the fused kernel's dependent face gathers hold back its
     * streaming dots on large meshes); the same results bit for bit either way.
     * 0 = the default, 150,000 cells; a negative value never splits. */
    int gather_split_cells;
} cfdg_config;

/* CFDG_KRYLOV_STREAM launches the graph driver's kernels one iteration at a time from a
 * host loop (same arithmetic, one sync per iteration; with timing on every kernel of the
 * exact J v body is timed: stat classes 12-15) */
enum { CFDG_KRYLOV_AUTO = -1, CFDG_KRYLOV_HOST = 0, CFDG_KRYLOV_GRAPH = 1, CFDG_KRYLOV_STREAM = 2 };

/* per-step record of a Newton solve (the reference prints these, src/Solver.cpp:1725-1727, :1746) */
typedef struct cfdg_step {
    double res_vm;         /* volume-weighted L2 of all components (norm_L2_VolumeWeighted) */
    double res_abs;        /* plain L2 (norm_L2) */
    double res_rho;        /* volume-weighted L2 of the density component */
    double cfl;
    int gmres_iters;
    int limiter_updated;
    double seconds;        /* wall time of the step */
    double device_ms;      /* CUDA-event time of the step on the solver's stream (timing on) */
    double krylov_ms;      /* CUDA-event time of the step's Krylov solve (timing on) */
} cfdg_step;

typedef struct cfdg_mesh cfdg_mesh;
typedef struct cfdg_solver cfdg_solver;

const char* cfdg_version(void);
const char* cfdg_last_error(void);
/* number of visible CUDA devices (0 when none) */
cfdg_status cfdg_device_count(int* n);
void cfdg_config_default(cfdg_config* cfg);

/* ---- mesh: Mesh::load / buildConnectivity / computeGeometry (src/Mesh.cpp:10-201) */

/* From arrays: xy[2*n_nodes]; cells[4*n_cells] 0-based node ids, -1 in the fourth
 * slot for a triangle; bedges[3*n_bedges] = (node a, node b, physical tag). */
cfdg_status cfdg_mesh_create(int n_nodes, const double* xy, int n_cells, const int* cells,
                             int n_bedges, const int* bedges, int renumber, cfdg_mesh** out);
/* The same mesh (bit for bit: faces, owners, geometry, renumbering, the device layout) built
 * by kernels on `device` instead of the host (Mesh::buildConnectivity and
 * Mesh::computeGeometry, src/Mesh.cpp:102-201, with the Hilbert renumbering); reverse
 * Cuthill-McKee runs on the host from the GPU's connectivity.  For large meshes: the host
 * build of a 4M-cell mesh takes seconds. */
cfdg_status cfdg_mesh_create_gpu(int n_nodes, const double* xy, int n_cells, const int* cells,
                                 int n_bedges, const int* bedges, int renumber, int device, cfdg_mesh** out);
/* Mesh::load (src/Mesh.cpp:10-26) on a Gmsh 2.2 ASCII file; LF and CRLF both accepted */
cfdg_status cfdg_mesh_load_gmsh(const char* path, int renumber, cfdg_mesh** out);
/* Mesh::getNumCells / getNumFaces (include/Mesh.hpp:25-27) */
cfdg_status cfdg_mesh_sizes(const cfdg_mesh* m, int* n_cells, int* n_faces, int* n_boundary_faces);
/* public Mesh::faces in reference order: ints5 = node1, node2, owner, neighbor, bcTag
 * (0-based nodes); dbl5 = nx, ny, area, x_mid, y_mid (struct Face, include/Types.hpp:16-27) */
cfdg_status cfdg_mesh_faces(const cfdg_mesh* m, int* ints5, double* dbl5);
/* public Mesh::cells: volume, x_c, y_c per cell (struct Cell, include/Types.hpp:30-35) */
cfdg_status cfdg_mesh_cells(const cfdg_mesh* m, double* vol_xc_yc);
/* internal numbering: cell_perm[new] = reference cell, face_perm[new] = reference face */
cfdg_status cfdg_mesh_permutation(const cfdg_mesh* m, int* cell_perm, int* face_perm);
void cfdg_mesh_destroy(cfdg_mesh* m);

/* ---- solver: Solver(const Mesh&) (src/Solver.cpp:7-10) */
cfdg_status cfdg_solver_create(const cfdg_mesh* m, const cfdg_config* cfg, cfdg_solver** out);
void cfdg_solver_destroy(cfdg_solver* s);
/* Solver::setNumericalMethod (include/Solver.hpp:33-36) */
cfdg_status cfdg_set_numerical_method(cfdg_solver* s, int flux, int spatial);
/* Solver::setFlowConditions (src/Solver.cpp:12-32) */
cfdg_status cfdg_set_flow_conditions(cfdg_solver* s, double mach, double p_ref, double t_ref);
/* Solver::setFreestreamStatic (src/Solver.cpp:2017-2025) */
cfdg_status cfdg_set_freestream_static(cfdg_solver* s, double mach, double p_static, double t_static);
/* Solver::setKinematicViscosity (src/Solver.cpp:34-43) */
cfdg_status cfdg_set_kinematic_viscosity(cfdg_solver* s, double reynolds, double l_ref);
/* Solver::initialize (src/Solver.cpp:46-65 / :905-920, chosen by cfg.init) */
cfdg_status cfdg_initialize(cfdg_solver* s);
/* M_inf, P_total_inlet, T_total_inlet, P_static_exit, nu, R_gas (include/Solver.hpp:37-39, :93-95) */
cfdg_status cfdg_get_params(const cfdg_solver* s, double* out6);

/* Solver::getSolution (include/Solver.hpp:58) and its setter */
cfdg_status cfdg_set_state(cfdg_solver* s, const double* U);
cfdg_status cfdg_get_state(cfdg_solver* s, double* U);

/* Solver::timeStepExplicit (src/Solver.cpp:1219-1243): one forward-Euler step of dt with
 * the reference's positivity clamps; res_l2 (may be NULL) gets norm_L2 of the residual
 * the step used (the reference prints it every 100 steps). */
cfdg_status cfdg_time_step_explicit(cfdg_solver* s, double dt, double* res_l2);
/* Solver::solveUnsteady (src/Solver.cpp:1801-1864): n_steps physical steps of dt_phy by
 * dual time stepping (BDF1; per step at most 15 Newton steps to a volume-weighted residual
 * of 1e-6, GMRES with the time term vol / dt_phy, updates relaxed by 0.7).  Per step
 * (arrays may be NULL): the Newton steps taken and the last residual. */
cfdg_status cfdg_solve_unsteady(cfdg_solver* s, double dt_phy, int n_steps, int* newton_steps, double* res_vm);

/* The mixed-precision kernels on their own (solvers created with precision = mixed):
 * the FP32 residual of U (AoS, NULL = current state; the limiter recomputed in FP32 for
 * the limited scheme) and the FP32 exact J v (dual numbers; limiter frozen at the current
 * FP64 limiter, plus v vol / dt with the current dt).  Outputs widened to FP64 AoS. */
cfdg_status cfdg_residual32(cfdg_solver* s, const double* U, double* R);
cfdg_status cfdg_jv32(cfdg_solver* s, const double* Ubase, const double* v, double* Jv);

/* Solver::computeResiduals (src/Solver.cpp:529-801).  U = NULL uses the current state.
 * update_limiters = 0 keeps the last limiter values (the frozen limiter of JFNK). */
cfdg_status cfdg_residual(cfdg_solver* s, const double* U, double* R, int update_limiters);
/* Solver::computeGradients (src/Solver.cpp:81-149): 10 per cell in CellGradient order
 * drho/dx, drho/dy, du/dx, du/dy, dv/dx, dv/dy, dp/dx, dp/dy, dT/dx, dT/dy */
cfdg_status cfdg_gradients(cfdg_solver* s, const double* U, double* grad10);
/* Solver::computeLimiters (src/Solver.cpp:152-253) after computeGradients on U */
cfdg_status cfdg_limiters(cfdg_solver* s, const double* U, double* phi);
cfdg_status cfdg_get_limiters(cfdg_solver* s, double* phi);
cfdg_status cfdg_set_limiters(cfdg_solver* s, const double* phi);
/* Solver::computeLocalTimeStep (src/Solver.cpp:1388-1422) on the current state;
 * keeps dt for cfdg_jv / cfdg_preconditioner / cfdg_gmres */
cfdg_status cfdg_local_timestep(cfdg_solver* s, double cfl, double* dt);
cfdg_status cfdg_set_timestep(cfdg_solver* s, const double* dt);
/* Solver::computeDiagonalPreconditioner (src/Solver.cpp:1424-1465) on the current state */
cfdg_status cfdg_preconditioner(cfdg_solver* s, double* D);
/* Solver::applyJacobian (src/Solver.cpp:1331-1386): Jv = dR/dU v + (vol/dt) v with the
 * limiter frozen.  mode CFDG_JV_FD reproduces the reference's one-sided difference
 * about (U_base, R_base); CFDG_JV_EXACT is the exact linearisation (R_base unused). */
cfdg_status cfdg_jv(cfdg_solver* s, const double* U_base, const double* R_base, const double* v,
                    double* Jv, int mode);
/* Solver::solveGMRES (src/Solver.cpp:1472-1618): one right-preconditioned MGS-GMRES
 * cycle from x0 = 0 for (vol/dt + dR/dU) x = rhs at U_base. */
cfdg_status cfdg_gmres(cfdg_solver* s, const double* U_base, const double* R_base, const double* rhs,
                       double* x, int* iters);
/* Solver::norm_L2_VolumeWeighted (src/Solver.cpp:1280-1303) */
cfdg_status cfdg_norm_vm(cfdg_solver* s, const double* R, double* out);
/* Solver::solveImplicit (src/Solver.cpp:1696-1799) on the device-resident state.
 * trace (may be NULL) receives up to max_steps records; *n_steps the count.
 * Returns CFDG_ERR_NOT_CONVERGED when max_steps ran out above tol. */
cfdg_status cfdg_solve_implicit(cfdg_solver* s, double tol, int max_steps, cfdg_step* trace, int* n_steps);
/* one pseudo-transient Newton step of solveImplicit; *converged set when the
 * step's residual was already below tol (no update made) */
cfdg_status cfdg_newton_step(cfdg_solver* s, double tol, cfdg_step* info, int* converged);
/* k steps of solveImplicit from the driver's current CFL and step counter.  With the graph
 * driver they are enqueued back to back with one host synchronisation per 64 steps: the
 * reference's CFL control (src/Solver.cpp:1747-1750, :1780-1796) and limiter-freeze
 * decision (:1714) run on the device between the steps, with the same arithmetic and the
 * same trace as k single steps.  Stops at convergence (*converged set: that step's
 * residual was below tol, or with tol_rho > 0 its volume-weighted density residual at or
 * below tol_rho after step 5; with the graph driver that step made no update) or an
 * error.  trace (may be NULL) gets the records of the steps taken, *n_done their count. */
cfdg_status cfdg_newton_steps(cfdg_solver* s, double tol, double tol_rho, int k, cfdg_step* trace, int* n_done,
                              int* converged);
/* switch the Krylov driver (CFDG_KRYLOV_HOST or CFDG_KRYLOV_GRAPH) between solves */
cfdg_status cfdg_set_krylov(cfdg_solver* s, int mode);
/* Newton driver state (CFL, step counter) */
cfdg_status cfdg_reset_newton(cfdg_solver* s);
/* The pseudo-transient driver's two loop variables, the CFL number and the step counter
 * of solveImplicit (src/Solver.cpp:1701, :1705), read and restored: a caller that saves
 * the state (cfdg_get_state) and these two can replay the same Newton steps later. */
cfdg_status cfdg_get_newton_state(cfdg_solver* s, double* cfl, int* step);
cfdg_status cfdg_set_newton_state(cfdg_solver* s, double cfl, int step);
/* The CFL cap of the pseudo-transient control (cfdg_config.cfl_max; the reference's
 * hard-coded 1e4, src/Solver.cpp:1790), changed between Newton steps: a continuation
 * schedule can hold the CFL number low through a stiff start-up transient and lift the
 * cap once the flow has settled.  Takes effect from the next step or chain; a current CFL
 * above the new cap is lowered to it. */
cfdg_status cfdg_set_cfl_max(cfdg_solver* s, double cfl_max);

/* Adjoint: gU = (dR/dU)^T lambda for the full residual at U, gradients and limiter
 * recomputed and differentiated along the branches the forward pass took (no
 * reference counterpart).  U = NULL uses the current state. */
cfdg_status cfdg_vjp(cfdg_solver* s, const double* U, const double* lambda, double* gU);

/* Wall quantities (src/Solver.cpp:1307-1325 calculateDrag, :1899-1979
 * extractSkinFriction): per boundary face of the given tag in reference face order,
 * x_mid, Cp (p - p_inf)/q_inf and Cf (one-sided wall shear / q_inf).  *n gets the count;
 * buffers may be NULL to query it. */
cfdg_status cfdg_wall_coefficients(cfdg_solver* s, int tag, double* x_mid, double* cp, double* cf, int* n);
/* computeWallDistances (src/Solver.cpp:1981-2015): per cell (reference numbering), the
 * distance from its centroid to the nearest no-slip (tag 4) face midpoint, 1e10 without
 * such faces.  Computed on the GPU; with SST the same array feeds the model. */
cfdg_status cfdg_wall_distance(cfdg_solver* s, double* d);
/* Wall objectives J(U) of the owner states of boundary faces, summed in reference face
 * order (no reference counterpart except the pressure drag): the adjoint's objectives.
 *   CFDG_OBJ_PRESSURE_DRAG        sum over tag-3 faces of -p A n_x (calculateDrag)
 *   CFDG_OBJ_SKIN_FRICTION_DRAG   sum over tag-4 faces of tau_w A t_x, tau_w = rho nu u_t / dn
 *                                 and t the wall tangent with t_x >= 0 (extractSkinFriction)
 *   CFDG_OBJ_WALL_PRESSURE        sum over tag-4 faces with x0 <= x_mid <= x1 of p A
 * J gets the value; dJdU (AoS, 6 per cell, reference numbering; may be NULL) dJ/dU. */
enum { CFDG_OBJ_PRESSURE_DRAG = 0, CFDG_OBJ_SKIN_FRICTION_DRAG = 1, CFDG_OBJ_WALL_PRESSURE = 2 };
cfdg_status cfdg_objective(cfdg_solver* s, int kind, double x0, double x1, double* J, double* dJdU);
/* calculateDrag (src/Solver.cpp:1307-1325): sum of -p A n_x over tag-3 faces */
cfdg_status cfdg_drag(cfdg_solver* s, double* drag);
/* calculateEntropyError (src/Solver.cpp:1620-1646) */
cfdg_status cfdg_entropy_error(cfdg_solver* s, double* err);

/* ---- device-resident entry points (no host copies): the benchmark's kernel path */
/* R(U_current) into the solver's device residual */
cfdg_status cfdg_residual_device(cfdg_solver* s, int update_limiters);
cfdg_status cfdg_synchronize(cfdg_solver* s);
/* timing: 0 off; 1 CUDA events around every kernel of every residual and exact-J v
 * evaluation and around each Newton step (cfdg_step.device_ms, krylov_ms); 2 around each
 * Newton step only (no events between its kernels) */
cfdg_status cfdg_set_timing(cfdg_solver* s, int on);
/* per-kernel times of the last timed residual evaluation */
cfdg_status cfdg_kernel_times(cfdg_solver* s, double* ms_prim, double* ms_grad, double* ms_flux, double* ms_gather);
/* accumulated per-kernel time and launch count since the last reset (18 classes): 0-3 the
 * residual's prim, grad, flux, gather kernels, 4-7 the same kernels of the exact J v,
 * 8-11 the VJP's forward recomputation, face adjoint and its two cell gathers, 12-15 the
 * stream-driven exact J v Krylov body: second pass of the pending vector + first pass of
 * the last product + z + primitives (+ Givens), gradients (+ SST), fluxes, gather + the
 * iteration's dots; 16-17 are reserved (the FD body's update and final update, not
 * timed) */
cfdg_status cfdg_kernel_stats(cfdg_solver* s, double* ms18, long long* n18, int reset);
/* VJP at the device-resident state with the device residual as lambda (timing path) */
cfdg_status cfdg_vjp_device(cfdg_solver* s);
/* writes `bytes` of device memory on the solver's stream (evicts L2 between timed steps) */
cfdg_status cfdg_flush_l2(cfdg_solver* s, size_t bytes);
/* The volume-weighted residual norm of cfdg_norm_vm for callers that cannot allocate
 * device memory: applications whose GPU memory belongs to their own pool (a library's
 * cudaMalloc would fail or fragment it) and callers on latency-bound paths that cannot
 * afford cudaMalloc's device synchronisation.  No counterpart in the reference.
 * R: device SoA residual, nv planes of n_cells doubles; vol: device cell volumes;
 * out: one device double, receives sqrt(sum_i (sum_c (R_c,i/vol_i)^2) vol_i / sum_i vol_i).
 * stream: a cudaStream_t (NULL = default stream); the call only enqueues work.
 * Allocates nothing: its reduction scratch is a static device array sized for at most
 * 8,388,608 cells (larger n_cells is rejected with CFDG_ERR_ARG).  Every call made outside
 * a stream capture looks that array's address up (cudaGetSymbolAddress) with the device
 * current; a call inside a capture uses the address of the device's last uncaptured call,
 * so make one call before any stream capture (and again after a cudaDeviceReset).  All
 * calls share the array: calls that overlap on the GPU race and must be serialised by
 * the caller. */
cfdg_status cfdg_norm_vm_noalloc(const double* R, const double* vol, long n_cells, int nv, double* out,
                                 void* stream);
/* Throughput of the FP64 pipe of `device`: a stream of independent FP64 fused
 * multiply-adds over every SM, timed with CUDA events (no reference counterpart; the
 * denominator of the FP64 residual's roofline).  *fma_per_s gets thread-level FMAs per
 * second (one FP64 pipe instruction each). */
cfdg_status cfdg_fp64_pipe_rate(int device, double* fma_per_s);
/* kernel launches issued by this solver since creation (all of them are this library's) */
cfdg_status cfdg_launch_count(cfdg_solver* s, long long* n);
/* the Krylov driver in effect: [0] CFDG_KRYLOV_* mode, [1] kernels per Arnoldi iteration
 * of the last built graph body (0 before the first), [2] 1 when the body's kernels use
 * programmatic dependent launch, [3] 1 for the persistent Arnoldi kernel */
cfdg_status cfdg_krylov_info(cfdg_solver* s, int* out4);

#ifdef __cplusplus
}
#endif
#endif /* CFDG_H */
