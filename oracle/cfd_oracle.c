/* CPU oracle for the residual-and-Newton path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solver's algorithm (AmberMond/mycode,
 * src/Solver.cpp, src/Mesh.cpp, include/Flux.hpp), written to reproduce the
 * reference's floating-point operation order so it can be pinned bit-for-bit
 * against the reference itself (oracle/_ref, built by oracle/build_ref.py).
 * Only tests/, the smoke check and the benchmark's CPU-baseline leg load it, and
 * only as the checker; the CUDA library never links or calls it.
 *
 * Build with -ffp-contract=off so that no a*b+c is fused (x86-64 g++ -O2 does not
 * fuse; an aarch64 build would unless told not to).
 *
 * Layout: states are AoS, 6 doubles per cell {rho, rhou, rhov, rhoE, rhok, rhow},
 * cells and faces in the reference's own numbering.
 *
 * Parts with no reference counterpart (SST sources) are marked "parity unpinned".
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NV 6

typedef struct { double r, ru, rv, rE, rk, rw; } st_t;

static inline st_t st(double r, double ru, double rv, double rE, double rk, double rw) {
    st_t s = {r, ru, rv, rE, rk, rw};
    return s;
}
/* State::operator+, -, *scalar (include/Types.hpp:71-81) */
static inline st_t st_add(st_t a, st_t b) { return st(a.r + b.r, a.ru + b.ru, a.rv + b.rv, a.rE + b.rE, a.rk + b.rk, a.rw + b.rw); }
static inline st_t st_sub(st_t a, st_t b) { return st(a.r - b.r, a.ru - b.ru, a.rv - b.rv, a.rE - b.rE, a.rk - b.rk, a.rw - b.rw); }
static inline st_t st_mul(st_t a, double s) { return st(a.r * s, a.ru * s, a.rv * s, a.rE * s, a.rk * s, a.rw * s); }
static inline st_t st_load(const double* p) { return st(p[0], p[1], p[2], p[3], p[4], p[5]); }
static inline void st_store(double* p, st_t s) { p[0] = s.r; p[1] = s.ru; p[2] = s.rv; p[3] = s.rE; p[4] = s.rk; p[5] = s.rw; }
/* std::max / std::min as libstdc++ defines them: max(a,b) = a<b ? b : a; min(a,b) = b<a ? b : a */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

enum { FLUX_LLF = 0, FLUX_ROE = 1, FLUX_HLLC = 2, FLUX_AUSM = 3 };
enum { SP_FIRST = 0, SP_CENTRAL = 1, SP_LIMITED = 2 };
enum { BC_BUMP = 0, BC_SUPERSONIC = 1, BC_PLATE = 2 };
enum { INIT_BUMP = 0, INIT_FREESTREAM = 1 };

/* ------------------------------------------------------------------ mesh */

typedef struct {
    int n_nodes, n_cells, n_faces;
    const double* xy;
    int* cell_nodes; /* n_cells x 4, -1 pads */
    /* faces, in creation order (src/Mesh.cpp:107-141) */
    int *node1, *node2, *owner, *neighbor, *tag;
    double *nx, *ny, *area, *xm, *ym;
    double *vol, *xc, *yc;
} om_mesh;

typedef struct { int64_t key; int val; } hslot;

static uint64_t hmix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

typedef struct { hslot* s; int64_t mask; } htab;

static void ht_init(htab* h, int64_t n) {
    int64_t cap = 16;
    while (cap < 2 * n + 16) cap <<= 1;
    h->s = (hslot*)malloc(sizeof(hslot) * cap);
    for (int64_t i = 0; i < cap; ++i) h->s[i].key = -1;
    h->mask = cap - 1;
}
static hslot* ht_find(htab* h, int64_t key) {
    int64_t i = (int64_t)(hmix((uint64_t)key) & (uint64_t)h->mask);
    while (h->s[i].key != -1 && h->s[i].key != key) i = (i + 1) & h->mask;
    return &h->s[i];
}
static inline int64_t edge_key(int a, int b) {
    int lo = a < b ? a : b, hi = a < b ? b : a;
    return ((int64_t)lo << 32) | (int64_t)(uint32_t)hi;
}

/* Mesh::buildConnectivity (src/Mesh.cpp:102-143) + Mesh::computeGeometry (:148-201).
 * cells: n_cells x 4 node ids (0-based, -1 pads triangles); bedges: n x 3 (a, b, tag),
 * later duplicates overwrite earlier ones as in the std::map of src/Mesh.cpp:72. */
om_mesh* om_mesh_build(int n_nodes, const double* xy, int n_cells, const int* cells,
                       int n_bedges, const int* bedges) {
    om_mesh* m = (om_mesh*)calloc(1, sizeof(om_mesh));
    m->n_nodes = n_nodes;
    m->n_cells = n_cells;
    m->xy = xy;
    m->cell_nodes = (int*)malloc(sizeof(int) * 4 * (size_t)n_cells);
    memcpy(m->cell_nodes, cells, sizeof(int) * 4 * (size_t)n_cells);
    htab bt, et;
    ht_init(&bt, n_bedges);
    for (int e = 0; e < n_bedges; ++e) {
        hslot* s = ht_find(&bt, edge_key(bedges[3 * e], bedges[3 * e + 1]));
        s->key = edge_key(bedges[3 * e], bedges[3 * e + 1]);
        s->val = bedges[3 * e + 2];
    }
    int cap = 4 * n_cells + 4;
    m->node1 = (int*)malloc(sizeof(int) * cap);
    m->node2 = (int*)malloc(sizeof(int) * cap);
    m->owner = (int*)malloc(sizeof(int) * cap);
    m->neighbor = (int*)malloc(sizeof(int) * cap);
    m->tag = (int*)malloc(sizeof(int) * cap);
    ht_init(&et, cap);
    int nf = 0;
    for (int i = 0; i < n_cells; ++i) {
        const int* c = cells + 4 * i;
        int n = c[3] >= 0 ? 4 : 3;
        for (int j = 0; j < n; ++j) {
            int a = c[j], b = c[(j + 1) % n];
            int64_t k = edge_key(a, b);
            hslot* s = ht_find(&et, k);
            if (s->key == k) {
                m->neighbor[s->val] = i;
            } else {
                s->key = k;
                s->val = nf;
                m->node1[nf] = a < b ? a : b;
                m->node2[nf] = a < b ? b : a;
                m->owner[nf] = i;
                m->neighbor[nf] = -1;
                hslot* bs = ht_find(&bt, k);
                m->tag[nf] = (bs->key == k) ? bs->val : 0;
                ++nf;
            }
        }
    }
    free(bt.s);
    free(et.s);
    m->n_faces = nf;
    m->nx = (double*)malloc(sizeof(double) * nf);
    m->ny = (double*)malloc(sizeof(double) * nf);
    m->area = (double*)malloc(sizeof(double) * nf);
    m->xm = (double*)malloc(sizeof(double) * nf);
    m->ym = (double*)malloc(sizeof(double) * nf);
    m->vol = (double*)malloc(sizeof(double) * n_cells);
    m->xc = (double*)malloc(sizeof(double) * n_cells);
    m->yc = (double*)malloc(sizeof(double) * n_cells);
#define X(k) xy[2 * (k)]
#define Y(k) xy[2 * (k) + 1]
    for (int i = 0; i < n_cells; ++i) {
        const int* c = cells + 4 * i;
        if (c[3] < 0) {
            double x1 = X(c[0]), y1 = Y(c[0]), x2 = X(c[1]), y2 = Y(c[1]), x3 = X(c[2]), y3 = Y(c[2]);
            m->vol[i] = 0.5 * fabs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1));
            m->xc[i] = (x1 + x2 + x3) / 3.0;
            m->yc[i] = (y1 + y2 + y3) / 3.0;
        } else {
            double sx = 0, sy = 0, a = 0.0;
            for (int k = 0; k < 4; ++k) { sx += X(c[k]); sy += Y(c[k]); }
            m->xc[i] = sx / 4.0;
            m->yc[i] = sy / 4.0;
            for (int k = 0; k < 4; ++k) {
                int n1 = c[k], n2 = c[(k + 1) % 4];
                a += (X(n1) * Y(n2) - X(n2) * Y(n1));
            }
            m->vol[i] = 0.5 * fabs(a);
        }
    }
    for (int f = 0; f < nf; ++f) {
        double dx = X(m->node2[f]) - X(m->node1[f]);
        double dy = Y(m->node2[f]) - Y(m->node1[f]);
        double A = sqrt(dx * dx + dy * dy);
        m->area[f] = A;
        m->xm[f] = 0.5 * (X(m->node1[f]) + X(m->node2[f]));
        m->ym[f] = 0.5 * (Y(m->node1[f]) + Y(m->node2[f]));
        double nx = dy / A, ny = -dx / A;
        double vx = m->xm[f] - m->xc[m->owner[f]];
        double vy = m->ym[f] - m->yc[m->owner[f]];
        if (vx * nx + vy * ny < 0) { nx = -nx; ny = -ny; }
        m->nx[f] = nx;
        m->ny[f] = ny;
    }
#undef X
#undef Y
    return m;
}

void om_mesh_free(om_mesh* m) {
    if (!m) return;
    free(m->cell_nodes); free(m->node1); free(m->node2); free(m->owner); free(m->neighbor); free(m->tag);
    free(m->nx); free(m->ny); free(m->area); free(m->xm); free(m->ym);
    free(m->vol); free(m->xc); free(m->yc);
    free(m);
}

int om_mesh_n_cells(const om_mesh* m) { return m->n_cells; }
int om_mesh_n_faces(const om_mesh* m) { return m->n_faces; }

void om_mesh_faces(const om_mesh* m, int* ints5, double* dbl5) {
    for (int f = 0; f < m->n_faces; ++f) {
        ints5[5 * f] = m->node1[f]; ints5[5 * f + 1] = m->node2[f];
        ints5[5 * f + 2] = m->owner[f]; ints5[5 * f + 3] = m->neighbor[f]; ints5[5 * f + 4] = m->tag[f];
        dbl5[5 * f] = m->nx[f]; dbl5[5 * f + 1] = m->ny[f]; dbl5[5 * f + 2] = m->area[f];
        dbl5[5 * f + 3] = m->xm[f]; dbl5[5 * f + 4] = m->ym[f];
    }
}

void om_mesh_cells(const om_mesh* m, double* vol_xc_yc) {
    for (int c = 0; c < m->n_cells; ++c) {
        vol_xc_yc[3 * c] = m->vol[c]; vol_xc_yc[3 * c + 1] = m->xc[c]; vol_xc_yc[3 * c + 2] = m->yc[c];
    }
}

/* ------------------------------------------------------------------ flux library */

static const double G = 1.4; /* include/Flux.hpp:9 */

/* getPressure, getSoundSpeed, computeNormalFlux (include/Flux.hpp:12-34) */
static inline double pressure(st_t U) {
    double V2 = (U.ru * U.ru + U.rv * U.rv) / (U.r * U.r);
    return (G - 1.0) * (U.rE - 0.5 * U.r * V2);
}
static inline st_t normal_flux(st_t U, double nx, double ny) {
    double p = pressure(U);
    double u = U.ru / U.r, v = U.rv / U.r;
    double un = u * nx + v * ny;
    return st(U.r * un, U.ru * un + p * nx, U.rv * un + p * ny, (U.rE + p) * un, 0, 0);
}

/* computeFluxHLLC (include/Flux.hpp:36-76) */
static st_t flux_hllc(st_t L, st_t R, double nx, double ny) {
    double pL = pressure(L), pR = pressure(R);
    double uL = L.ru / L.r, uR = R.ru / R.r;
    double vL = L.rv / L.r, vR = R.rv / R.r;
    double unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
    double cL = sqrt(G * pL / L.r), cR = sqrt(G * pR / R.r);
    double hL = (L.rE + pL) / L.r, hR = (R.rE + pR) / R.r;
    double sL = sqrt(L.r), sR = sqrt(R.r);
    double ut = (sL * uL + sR * uR) / (sL + sR);
    double vt = (sL * vL + sR * vR) / (sL + sR);
    double ht = (sL * hL + sR * hR) / (sL + sR);
    double unt = ut * nx + vt * ny;
    double ct = sqrt((G - 1.0) * (ht - 0.5 * (ut * ut + vt * vt)));
    double SL = smin(unL - cL, unt - ct);
    double SR = smax(unR + cR, unt + ct);
    double Ss = (pR - pL + L.r * unL * (SL - unL) - R.r * unR * (SR - unR)) /
                (L.r * (SL - unL) - R.r * (SR - unR));
    if (SL >= 0.0) return normal_flux(L, nx, ny);
    if (SR <= 0.0) return normal_flux(R, nx, ny);
    if (Ss >= 0.0) {
        double coef = L.r * (SL - unL) / (SL - Ss);
        st_t Us = st(coef, coef * (uL + (Ss - unL) * nx), coef * (vL + (Ss - unL) * ny),
                     coef * (L.rE / L.r + (Ss - unL) * (Ss + pL / (L.r * (SL - unL)))), 0, 0);
        return st_add(normal_flux(L, nx, ny), st_mul(st_sub(Us, L), SL));
    } else {
        double coef = R.r * (SR - unR) / (SR - Ss);
        st_t Us = st(coef, coef * (uR + (Ss - unR) * nx), coef * (vR + (Ss - unR) * ny),
                     coef * (R.rE / R.r + (Ss - unR) * (Ss + pR / (R.r * (SR - unR)))), 0, 0);
        return st_add(normal_flux(R, nx, ny), st_mul(st_sub(Us, R), SR));
    }
}

/* computeFluxLLF (include/Flux.hpp:81-108) */
static st_t flux_llf(st_t L, st_t R, double nx, double ny) {
    st_t FL = normal_flux(L, nx, ny), FR = normal_flux(R, nx, ny);
    double pL = pressure(L);
    double uL = L.ru / L.r, vL = L.rv / L.r;
    double unL = uL * nx + vL * ny;
    double cL = sqrt(G * pL / L.r);
    double pR = pressure(R);
    double uR = R.ru / R.r, vR = R.rv / R.r;
    double unR = uR * nx + vR * ny;
    double cR = sqrt(G * pR / R.r);
    double a = smax(fabs(unL) + cL, fabs(unR) + cR);
    st_t D = st_mul(st_sub(R, L), 0.5 * a);
    st_t A = st_mul(st_add(FL, FR), 0.5);
    return st_sub(A, D);
}

/* computeFluxROE with Harten's entropy fix (include/Flux.hpp:112-213) */
static st_t flux_roe(st_t L, st_t R, double nx, double ny) {
    double pL = pressure(L);
    double uL = L.ru / L.r, vL = L.rv / L.r;
    double hL = (L.rE + pL) / L.r;
    double pR = pressure(R);
    double uR = R.ru / R.r, vR = R.rv / R.r;
    double hR = (R.rE + pR) / R.r;
    double sL = sqrt(L.r), sR = sqrt(R.r);
    double inv = 1.0 / (sL + sR);
    double ut = (sL * uL + sR * uR) * inv;
    double vt = (sL * vL + sR * vR) * inv;
    double ht = (sL * hL + sR * hR) * inv;
    double V2 = ut * ut + vt * vt;
    double c2 = (G - 1.0) * (ht - 0.5 * V2);
    double ct = sqrt(smax(c2, 1e-8));
    double unt = ut * nx + vt * ny;
    double utt = -ut * ny + vt * nx;
    double lam[4] = {unt - ct, unt, unt, unt + ct};
    double eps = 0.1 * ct;
    for (int i = 0; i < 4; ++i) {
        if (fabs(lam[i]) < eps) lam[i] = 0.5 * (lam[i] * lam[i] / eps + eps);
        lam[i] = fabs(lam[i]);
    }
    double dr = R.r - L.r, du = uR - uL, dv = vR - vL, dp = pR - pL;
    double dun = du * nx + dv * ny;
    double dut = -du * ny + dv * nx;
    double rt = sL * sR;
    double al0 = 0.5 / c2 * (dp - rt * ct * dun);
    double al1 = dr - dp / c2;
    double al2 = rt * dut;
    double al3 = 0.5 / c2 * (dp + rt * ct * dun);
    double w1 = lam[0] * al0, w2 = lam[1] * al1, w3 = lam[2] * al2, w4 = lam[3] * al3;
    st_t D;
    D.r = w1 * 1.0 + w2 * 1.0 + w3 * 0.0 + w4 * 1.0;
    D.ru = w1 * (ut - ct * nx) + w2 * ut + w3 * (-ny) + w4 * (ut + ct * nx);
    D.rv = w1 * (vt - ct * ny) + w2 * vt + w3 * nx + w4 * (vt + ct * ny);
    D.rE = w1 * (ht - unt * ct) + w2 * (0.5 * V2) + w3 * utt + w4 * (ht + unt * ct);
    D.rk = fabs(unt) * (R.rk / R.r - L.rk / L.r) * rt;
    D.rw = fabs(unt) * (R.rw / R.r - L.rw / L.r) * rt;
    st_t FL = normal_flux(L, nx, ny), FR = normal_flux(R, nx, ny);
    return st_sub(st_mul(st_add(FL, FR), 0.5), st_mul(D, 0.5));
}

/* computeInviscidFlux (include/Flux.hpp:216-227); AUSM falls to LLF */
static st_t inviscid_flux(st_t L, st_t R, double nx, double ny, int scheme) {
    switch (scheme) {
        case FLUX_ROE: return flux_roe(L, R, nx, ny);
        case FLUX_HLLC: return flux_hllc(L, R, nx, ny);
        default: return flux_llf(L, R, nx, ny);
    }
}

/* The inviscid face flux and the normal flux alone, for the known-answer tests of the
 * flux library (consistency F(U, U) = F.n(U), rotational invariance); states AoS, 6 doubles */
void om_inviscid_flux(const double* UL, const double* UR, double nx, double ny, int scheme, double* F) {
    st_t L = st(UL[0], UL[1], UL[2], UL[3], UL[4], UL[5]), R = st(UR[0], UR[1], UR[2], UR[3], UR[4], UR[5]);
    st_t o = inviscid_flux(L, R, nx, ny, scheme);
    F[0] = o.r; F[1] = o.ru; F[2] = o.rv; F[3] = o.rE; F[4] = o.rk; F[5] = o.rw;
}

void om_normal_flux(const double* U, double nx, double ny, double* F) {
    st_t o = normal_flux(st(U[0], U[1], U[2], U[3], U[4], U[5]), nx, ny);
    F[0] = o.r; F[1] = o.ru; F[2] = o.rv; F[3] = o.rE; F[4] = o.rk; F[5] = o.rw;
}

/* ------------------------------------------------------------------ solver */

typedef struct {
    const om_mesh* m;
    int flux, spatial, bcset, viscous, init_mode;
    double gamma, R_gas, Pr, nu;
    double M_inf, P0, T0, Pexit;
    double* grad; /* 10 per cell: rho, u, v, p, T gradients, (x, y) pairs */
    double* phi;  /* limiter per cell */
    double* dt;   /* local time step */
    double* U;    /* current state, 6 per cell */
    double* pc;   /* scratch */
    double* pmax;
    double* pmin;
    int gmres_m;
    double gmres_tol;
    double cfl0;
    int freeze_step;    /* the limiter freezes when step > freeze_step or CFL > freeze_cfl */
    double freeze_cfl;
    double stop_rho;    /* solveImplicit also stops when the density residual is below this */
} om_solver;

enum { GR_RHO = 0, GR_U = 2, GR_V = 4, GR_P = 6, GR_T = 8 };

om_solver* om_solver_create(const om_mesh* m) {
    om_solver* s = (om_solver*)calloc(1, sizeof(om_solver));
    s->m = m;
    s->flux = FLUX_HLLC;      /* include/Solver.hpp:33-34 defaults */
    s->spatial = SP_LIMITED;
    s->bcset = BC_BUMP;
    s->init_mode = INIT_BUMP;
    s->gamma = 1.4;           /* include/Solver.hpp:91-92 */
    s->R_gas = 287.0;
    s->Pr = 0.72;             /* src/Solver.cpp:541 */
    s->nu = 0.01;             /* include/Solver.hpp:42 */
    s->gmres_m = 40;          /* src/Solver.cpp:1479 */
    s->gmres_tol = 1e-2;      /* src/Solver.cpp:1587 */
    s->cfl0 = 0.1;            /* src/Solver.cpp:1700 */
    s->freeze_step = 150;     /* src/Solver.cpp:1714 */
    s->freeze_cfl = 10.0;
    s->stop_rho = 0.0;
    int n = m->n_cells;
    s->grad = (double*)calloc((size_t)10 * n, sizeof(double));
    s->phi = (double*)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) s->phi[i] = 1.0;
    s->dt = (double*)calloc(n, sizeof(double));
    s->U = (double*)calloc((size_t)NV * n, sizeof(double));
    s->pc = (double*)malloc(sizeof(double) * n);
    s->pmax = (double*)malloc(sizeof(double) * n);
    s->pmin = (double*)malloc(sizeof(double) * n);
    return s;
}

void om_solver_free(om_solver* s) {
    if (!s) return;
    free(s->grad); free(s->phi); free(s->dt); free(s->U); free(s->pc); free(s->pmax); free(s->pmin);
    free(s);
}

void om_set_method(om_solver* s, int flux, int spatial) { s->flux = flux; s->spatial = spatial; }
void om_set_case(om_solver* s, int bcset, int viscous, int init_mode) {
    s->bcset = bcset; s->viscous = viscous; s->init_mode = init_mode;
}
void om_set_gmres(om_solver* s, int m, double tol) { s->gmres_m = m; s->gmres_tol = tol; }
void om_set_nu(om_solver* s, double nu) { s->nu = nu; }
/* the first pseudo-time CFL of solveImplicit (the reference hard-codes 0.1) */
void om_set_cfl0(om_solver* s, double cfl0) { s->cfl0 = cfl0; }
/* the limiter-freeze rule of solveImplicit (the reference hard-codes step > 150 ||
 * CFL > 10, src/Solver.cpp:1714); freeze_step = -1 keeps the current limiter throughout */
void om_set_freeze(om_solver* s, int freeze_step, double freeze_cfl) {
    s->freeze_step = freeze_step;
    s->freeze_cfl = freeze_cfl;
}
/* an extra stop of solveImplicit: the volume-weighted density residual below stop_rho
 * (0 = off; the reference stops on the all-component norm only) */
void om_set_stop_rho(om_solver* s, double stop_rho) { s->stop_rho = stop_rho; }

/* setFlowConditions (src/Solver.cpp:12-32) */
void om_set_flow_conditions(om_solver* s, double M, double P, double T) {
    s->M_inf = M;
    double fT = 1.0 + 0.5 * (s->gamma - 1.0) * M * M;
    double fP = pow(fT, s->gamma / (s->gamma - 1.0));
    s->T0 = T * fT;
    s->P0 = P * fP;
    s->Pexit = P;
}
/* setFreestreamStatic (src/Solver.cpp:2017-2025): same arithmetic */
void om_set_freestream_static(om_solver* s, double M, double P, double T) { om_set_flow_conditions(s, M, P, T); }

/* setKinematicViscosity (src/Solver.cpp:34-43) */
void om_set_kinematic_viscosity(om_solver* s, double Re, double L) {
    double fT = 1.0 + 0.5 * (s->gamma - 1.0) * s->M_inf * s->M_inf;
    double Ts = s->T0 / fT;
    double c = sqrt(s->gamma * s->R_gas * Ts);
    double u = s->M_inf * c;
    s->nu = (u * L) / Re;
}

void om_get_params(const om_solver* s, double* out6) {
    out6[0] = s->M_inf; out6[1] = s->P0; out6[2] = s->T0; out6[3] = s->Pexit; out6[4] = s->nu; out6[5] = s->R_gas;
}

/* primitiveToConservative (src/Solver.cpp:498-501) */
static inline st_t p2c(const om_solver* s, double r, double u, double v, double p, double k, double w) {
    double rE = p / (s->gamma - 1.0) + 0.5 * r * (u * u + v * v);
    return st(r, r * u, r * v, rE, r * k, r * w);
}

/* free-stream state used by the frozen inflow / far-field tags (src/Solver.cpp:979-985, :1094-1100)
 * and by the free-stream initialiser (:905-920) */
static st_t freestream(const om_solver* s) {
    double g = s->gamma, M = s->M_inf;
    double fT = 1.0 + 0.5 * (g - 1.0) * M * M;
    double Ts = s->T0 / fT;
    double rho = s->Pexit / (s->R_gas * Ts);
    double c = sqrt(g * s->R_gas * Ts);
    double u = M * c;
    return p2c(s, rho, u, 0.0, s->Pexit, 0.0, 0.0);
}

static st_t slip_ghost(st_t U, double nx, double ny) {
    double u = U.ru / U.r, v = U.rv / U.r;
    double vn = u * nx + v * ny;
    double ug = u - 2.0 * vn * nx, vg = v - 2.0 * vn * ny;
    st_t g = U;
    g.r = U.r; g.ru = U.r * ug; g.rv = U.r * vg; g.rE = U.rE;
    return g;
}

/* getBoundaryGhostState: the bump set (src/Solver.cpp:806-863), the supersonic set
 * (:973-1011) and the laminar-plate / SWBLI set (:1088-1139) */
static st_t ghost(const om_solver* s, st_t U, int f) {
    const om_mesh* m = s->m;
    int tag = m->tag[f];
    double nx = m->nx[f], ny = m->ny[f];
    double g = s->gamma;
    if (s->bcset == BC_BUMP) {
        if (tag == 1) {
            double pin = pressure(U);
            double pu = smin(pin, s->P0 - 1e-4);
            double Tg = s->T0 * pow(pu / s->P0, (g - 1.0) / g);
            double rg = pu / (s->R_gas * Tg);
            double Cp = g * s->R_gas / (g - 1.0);
            double V2 = 2.0 * Cp * (s->T0 - Tg);
            double V = (V2 > 0) ? sqrt(V2) : 0.0;
            return p2c(s, rg, V, 0.0, pu, 0.0, 0.0);
        } else if (tag == 2) {
            double r = U.r, u = U.ru / U.r, v = U.rv / U.r;
            return p2c(s, r, u, v, s->Pexit, 0.0, 0.0);
        } else if (tag == 3) {
            return slip_ghost(U, nx, ny);
        }
        return U;
    } else if (s->bcset == BC_SUPERSONIC) {
        if (tag == 1) return freestream(s);
        if (tag == 2) return U;
        if (tag == 3) return slip_ghost(U, nx, ny);
        return U;
    } else {
        if (tag == 1 || tag == 5) return freestream(s);
        if (tag == 2) return U;
        if (tag == 3) return slip_ghost(U, nx, ny);
        if (tag == 4) {
            double ug = -(U.ru / U.r), vg = -(U.rv / U.r);
            double ek = 0.5 * (U.ru * U.ru + U.rv * U.rv) / U.r;
            double pin = (g - 1.0) * (U.rE - ek);
            double Tin = pin / (U.r * s->R_gas);
            double Tg = Tin;
            double rg = pin / (s->R_gas * Tg);
            return p2c(s, rg, ug, vg, pin, 0.0, 0.0);
        }
        return U;
    }
}

/* initialize: the bump variant (src/Solver.cpp:46-65) or free stream (:905-920) */
void om_initialize(om_solver* s) {
    st_t init;
    if (s->init_mode == INIT_BUMP) {
        double g = s->gamma, p = s->Pexit;
        double fT = pow(s->P0 / p, (g - 1.0) / g);
        double T = s->T0 / fT;
        double rho = p / (s->R_gas * T);
        double V = sqrt(2.0 * (g * s->R_gas / (g - 1.0)) * (s->T0 - T));
        init = p2c(s, rho, V, 0.0, p, 0.0, 0.0);
    } else {
        init = freestream(s);
    }
    for (int i = 0; i < s->m->n_cells; ++i) st_store(s->U + NV * i, init);
}

void om_set_state(om_solver* s, const double* U) { memcpy(s->U, U, sizeof(double) * NV * s->m->n_cells); }
void om_get_state(const om_solver* s, double* U) { memcpy(U, s->U, sizeof(double) * NV * s->m->n_cells); }

/* computeGradients (src/Solver.cpp:81-149) */
void om_gradients(om_solver* s, const double* Uin) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double R = s->R_gas;
    memset(s->grad, 0, sizeof(double) * 10 * (size_t)n);
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        st_t L = st_load(Uin + NV * o);
        st_t Rs = nb >= 0 ? st_load(Uin + NV * nb) : ghost(s, L, f);
        double uL = L.ru / L.r, vL = L.rv / L.r, pL = pressure(L), TL = pL / (L.r * R);
        double uR = Rs.ru / Rs.r, vR = Rs.rv / Rs.r, pR = pressure(Rs), TR = pR / (Rs.r * R);
        double ph[5];
        ph[0] = 0.5 * (L.r + Rs.r);
        ph[1] = 0.5 * (uL + uR);
        ph[2] = 0.5 * (vL + vR);
        ph[3] = 0.5 * (pL + pR);
        ph[4] = 0.5 * (TL + TR);
        double nx = m->nx[f], ny = m->ny[f], A = m->area[f];
        double* go = s->grad + 10 * o;
        for (int q = 0; q < 5; ++q) {
            go[2 * q] += ph[q] * nx * A;
            go[2 * q + 1] += ph[q] * ny * A;
        }
        if (nb >= 0) {
            double* gn = s->grad + 10 * nb;
            for (int q = 0; q < 5; ++q) {
                gn[2 * q] -= ph[q] * nx * A;
                gn[2 * q + 1] -= ph[q] * ny * A;
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        double v = m->vol[i];
        for (int q = 0; q < 10; ++q) s->grad[10 * i + q] /= v;
    }
}

/* computeLimiters: Barth-Jespersen on pressure reconstructed through T
 * (src/Solver.cpp:152-253) */
void om_limiters(om_solver* s, const double* Uin) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double R = s->R_gas;
    for (int i = 0; i < n; ++i) {
        s->phi[i] = 1.0;
        s->pc[i] = pressure(st_load(Uin + NV * i));
        s->pmax[i] = s->pc[i];
        s->pmin[i] = s->pc[i];
    }
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        double pg = 0.0;
        if (nb >= 0) pg = s->pc[nb];
        else pg = pressure(ghost(s, st_load(Uin + NV * o), f));
        s->pmax[o] = smax(s->pmax[o], pg);
        s->pmin[o] = smin(s->pmin[o], pg);
        if (nb >= 0) {
            s->pmax[nb] = smax(s->pmax[nb], s->pc[o]);
            s->pmin[nb] = smin(s->pmin[nb], s->pc[o]);
        }
    }
    const double eps = 1e-12;
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        for (int side = 0; side < 2; ++side) {
            int c = side == 0 ? o : nb;
            if (c < 0) break;
            double dx = m->xm[f] - m->xc[c], dy = m->ym[f] - m->yc[c];
            const double* g = s->grad + 10 * c;
            double rho = Uin[NV * c];
            double Tc = s->pc[c] / (rho * R);
            double Tf = Tc + 1.0 * (g[GR_T] * dx + g[GR_T + 1] * dy);
            double Pf = rho * R * Tf;
            double d2 = Pf - s->pc[c];
            double a = 1.0;
            if (d2 > 0.0) {
                a = (s->pmax[c] - s->pc[c]) / (d2 + eps);
                a = smin(1.0, a);
            } else if (d2 < 0.0) {
                a = (s->pmin[c] - s->pc[c]) / (d2 - eps);
                a = smin(1.0, a);
            }
            s->phi[c] = smin(s->phi[c], a);
        }
    }
}

void om_get_gradients(const om_solver* s, double* G10) { memcpy(G10, s->grad, sizeof(double) * 10 * s->m->n_cells); }
void om_get_limiters(const om_solver* s, double* phi) { memcpy(phi, s->phi, sizeof(double) * s->m->n_cells); }
void om_set_limiters(om_solver* s, const double* phi) { memcpy(s->phi, phi, sizeof(double) * s->m->n_cells); }

/* computeResiduals (src/Solver.cpp:529-801); the viscous flux is subtracted when
 * s->viscous is set (the reference's commented line :787 instead of :792) */
void om_residual(om_solver* s, const double* Uin, double* Rout, int update_limiters) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double g = s->gamma, R = s->R_gas;
    memset(Rout, 0, sizeof(double) * NV * (size_t)n);
    om_gradients(s, Uin);
    if (s->spatial == SP_LIMITED && update_limiters) om_limiters(s, Uin);
    double Cp = g * R / (g - 1.0);
    double Pr = s->Pr;
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        double nx = m->nx[f], ny = m->ny[f];
        st_t L = st_load(Uin + NV * o);
        st_t Rs = nb >= 0 ? st_load(Uin + NV * nb) : ghost(s, L, f);
        st_t Lr, Rr;
        if (s->spatial == SP_FIRST || nb < 0) {
            Lr = L;
            Rr = Rs;
        } else {
            double dxL = m->xm[f] - m->xc[o], dyL = m->ym[f] - m->yc[o];
            double dxR = m->xm[f] - m->xc[nb], dyR = m->ym[f] - m->yc[nb];
            const double* gL = s->grad + 10 * o;
            const double* gR = s->grad + 10 * nb;
            double phL = s->spatial == SP_LIMITED ? s->phi[o] : 0.5;
            double phR = s->spatial == SP_LIMITED ? s->phi[nb] : 0.5;
            double uL = L.ru / L.r, vL = L.rv / L.r;
            double pL = pressure(L);
            double rLf = L.r + phL * (gL[GR_RHO] * dxL + gL[GR_RHO + 1] * dyL);
            double pLf = pL + phL * (gL[GR_P] * dxL + gL[GR_P + 1] * dyL);
            double uLf = uL + phL * (gL[GR_U] * dxL + gL[GR_U + 1] * dyL);
            double vLf = vL + phL * (gL[GR_V] * dxL + gL[GR_V + 1] * dyL);
            if (rLf < 1e-4) rLf = L.r;
            if (pLf < 1e-4) pLf = pL;
            Lr = p2c(s, rLf, uLf, vLf, pLf, 0.0, 0.0);
            double uR = Rs.ru / Rs.r, vR = Rs.rv / Rs.r;
            double pR = pressure(Rs);
            double rRf = Rs.r + phR * (gR[GR_RHO] * dxR + gR[GR_RHO + 1] * dyR);
            double pRf = pR + phR * (gR[GR_P] * dxR + gR[GR_P + 1] * dyR);
            double uRf = uR + phR * (gR[GR_U] * dxR + gR[GR_U + 1] * dyR);
            double vRf = vR + phR * (gR[GR_V] * dxR + gR[GR_V + 1] * dyR);
            if (rRf < 1e-4) rRf = Rs.r;
            if (pRf < 1e-4) pRf = pR;
            Rr = p2c(s, rRf, uRf, vRf, pRf, 0.0, 0.0);
        }
        st_t FE;
        if (nb < 0 && (m->tag[f] == 3 || m->tag[f] == 4)) {
            double pw = pressure(Lr);
            FE = st(0.0, pw * nx, pw * ny, 0.0, 0.0, 0.0);
        } else {
            FE = inviscid_flux(Lr, Rr, nx, ny, s->flux);
        }
        st_t TF = FE;
        if (s->viscous) {
            double rf = 0.5 * (L.r + Rs.r);
            double uf = 0.5 * (L.ru / L.r + Rs.ru / Rs.r);
            double vf = 0.5 * (L.rv / L.r + Rs.rv / Rs.r);
            const double* gL = s->grad + 10 * o;
            const double* gR = nb >= 0 ? s->grad + 10 * nb : gL;
            double dudx, dudy, dvdx, dvdy, dTdx, dTdy;
            if (nb < 0 && m->tag[f] == 4) {
                double dx = m->xm[f] - m->xc[o], dy = m->ym[f] - m->yc[o];
                double d2 = dx * dx + dy * dy;
                double uc = L.ru / L.r, vc = L.rv / L.r;
                dudx = -uc * dx / d2;
                dudy = -uc * dy / d2;
                dvdx = -vc * dx / d2;
                dvdy = -vc * dy / d2;
                dTdx = 0.0;
                dTdy = 0.0;
            } else {
                dudx = 0.5 * (gL[GR_U] + gR[GR_U]);
                dudy = 0.5 * (gL[GR_U + 1] + gR[GR_U + 1]);
                dvdx = 0.5 * (gL[GR_V] + gR[GR_V]);
                dvdy = 0.5 * (gL[GR_V + 1] + gR[GR_V + 1]);
                dTdx = 0.5 * (gL[GR_T] + gR[GR_T]);
                dTdy = 0.5 * (gL[GR_T + 1] + gR[GR_T + 1]);
                /* boundary faces use the owner's centroid for the missing neighbour,
                 * so dist2 = 0 and no correction (defined in place of the reference's
                 * out-of-range read at src/Solver.cpp:729-730) */
                int c2 = nb >= 0 ? nb : o;
                double dxLR = m->xc[c2] - m->xc[o], dyLR = m->yc[c2] - m->yc[o];
                double d2 = dxLR * dxLR + dyLR * dyLR;
                if (d2 > 1e-14) {
                    double du = (Rs.ru / Rs.r) - (L.ru / L.r);
                    double dv = (Rs.rv / Rs.r) - (L.rv / L.r);
                    double a0 = dudx, b0 = dudy, c0 = dvdx, e0 = dvdy;
                    dudx = a0 - (a0 * dxLR + b0 * dyLR - du) * dxLR / d2;
                    dudy = b0 - (a0 * dxLR + b0 * dyLR - du) * dyLR / d2;
                    dvdx = c0 - (c0 * dxLR + e0 * dyLR - dv) * dxLR / d2;
                    dvdy = e0 - (c0 * dxLR + e0 * dyLR - dv) * dyLR / d2;
                }
            }
            double mu = rf * s->nu;
            double k = mu * Cp / Pr;
            double div = dudx + dvdy;
            double txx = mu * (2.0 * dudx - (2.0 / 3.0) * div);
            double tyy = mu * (2.0 * dvdy - (2.0 / 3.0) * div);
            double txy = mu * (dudy + dvdx);
            double qx = -k * dTdx, qy = -k * dTdy;
            st_t FV;
            FV.r = 0.0;
            FV.ru = txx * nx + txy * ny;
            FV.rv = txy * nx + tyy * ny;
            double wx = uf * txx + vf * txy - qx;
            double wy = uf * txy + vf * tyy - qy;
            FV.rE = wx * nx + wy * ny;
            FV.rk = 0.0;
            FV.rw = 0.0;
            TF = st_sub(FE, FV);
        }
        double A = m->area[f];
        st_store(Rout + NV * o, st_add(st_load(Rout + NV * o), st_mul(TF, A)));
        if (nb >= 0) st_store(Rout + NV * nb, st_sub(st_load(Rout + NV * nb), st_mul(TF, A)));
    }
}

/* norm_L2, dot_product, norm_L2_VolumeWeighted (src/Solver.cpp:1250-1303) */
double om_norm(int n, const double* v) {
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* s = v + NV * i;
        sum += s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    }
    return sqrt(sum);
}
double om_dot(int n, const double* a, const double* b) {
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {
        const double* x = a + NV * i;
        const double* y = b + NV * i;
        sum += x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[4] * y[4] + x[5] * y[5];
    }
    return sum;
}
/* the density component of norm_L2_VolumeWeighted: sqrt(sum (R_rho / V)^2 V / sum V) */
double om_norm_vm_rho(const om_solver* s, const double* R) {
    double sq = 0.0, tv = 0.0;
    for (int i = 0; i < s->m->n_cells; ++i) {
        double v = s->m->vol[i];
        double a = R[NV * i] / v;
        sq += a * a * v;
        tv += v;
    }
    if (tv == 0) return 0.0;
    return sqrt(sq / tv);
}

double om_norm_vm(const om_solver* s, const double* R) {
    double sq = 0.0, tv = 0.0;
    for (int i = 0; i < s->m->n_cells; ++i) {
        double v = s->m->vol[i];
        const double* r = R + NV * i;
        double a = r[0] / v, b = r[1] / v, c = r[2] / v, d = r[3] / v, e = r[4] / v, f = r[5] / v;
        double l = a * a + b * b + c * c + d * d + e * e + f * f;
        sq += l * v;
        tv += v;
    }
    if (tv == 0) return 0.0;
    return sqrt(sq / tv);
}

/* computeLocalTimeStep (src/Solver.cpp:1388-1422), on the current state */
void om_local_timestep(om_solver* s, double CFL) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double g = s->gamma;
    double* lam = s->pc;
    for (int i = 0; i < n; ++i) lam[i] = 1e-12;
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        st_t L = st_load(s->U + NV * o);
        double pL = pressure(L);
        double cL = sqrt(g * pL / L.r);
        double unL = (L.ru * m->nx[f] + L.rv * m->ny[f]) / L.r;
        lam[o] += (fabs(unL) + cL) * m->area[f];
        if (nb >= 0) {
            st_t Rr = st_load(s->U + NV * nb);
            double pR = pressure(Rr);
            double cR = sqrt(g * pR / Rr.r);
            double unR = (Rr.ru * (-m->nx[f]) + Rr.rv * (-m->ny[f])) / Rr.r;
            lam[nb] += (fabs(unR) + cR) * m->area[f];
        }
    }
    for (int i = 0; i < n; ++i) s->dt[i] = CFL * m->vol[i] / lam[i];
}
void om_get_dt(const om_solver* s, double* dt) { memcpy(dt, s->dt, sizeof(double) * s->m->n_cells); }
void om_set_dt(om_solver* s, const double* dt) { memcpy(s->dt, dt, sizeof(double) * s->m->n_cells); }

/* computeDiagonalPreconditioner (src/Solver.cpp:1424-1465), on the current state */
void om_preconditioner(om_solver* s, double* D) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double g = s->gamma;
    for (int i = 0; i < n; ++i) D[i] = 0.0;
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        st_t L = st_load(s->U + NV * o);
        st_t Rr = nb >= 0 ? st_load(s->U + NV * nb) : ghost(s, L, f);
        double cL = sqrt(g * pressure(L) / L.r);
        double cR = sqrt(g * (pressure(Rr) > 0 ? pressure(Rr) : 1e-3) / (Rr.r > 0 ? Rr.r : 1e-3));
        double cf = 0.5 * (cL + cR);
        double uf = 0.5 * (L.ru / L.r + Rr.ru / Rr.r);
        double vf = 0.5 * (L.rv / L.r + Rr.rv / Rr.r);
        double vn = fabs(uf * m->nx[f] + vf * m->ny[f]);
        double li = vn + cf;
        double dx = sqrt(m->vol[o]);
        double mu = 0.5 * (L.r + Rr.r) * s->nu;
        double lv = 2.0 * mu / (0.5 * (L.r + Rr.r) * dx + 1e-12);
        double lt = (li + lv) * m->area[f];
        D[o] += lt * 0.5;
        if (nb >= 0) D[nb] += lt * 0.5;
    }
    for (int i = 0; i < n; ++i) {
        double v = m->vol[i];
        D[i] = (v / (s->dt[i] + 1e-30)) + D[i];
        if (D[i] < 1e-12) D[i] = 1e-12;
    }
}

/* applyJacobian: one-sided finite difference with the limiter frozen
 * (src/Solver.cpp:1331-1386) */
void om_apply_jacobian(om_solver* s, const double* Ub, const double* Rb, const double* v, double* Jv) {
    int n = s->m->n_cells;
    double un = om_norm(n, Ub), vn = om_norm(n, v);
    double eps = 1e-7 * (1.0 + un) / (vn + 1e-30);
    double* Up = (double*)malloc(sizeof(double) * NV * (size_t)n);
    double* Rp = (double*)malloc(sizeof(double) * NV * (size_t)n);
    for (int i = 0; i < n; ++i)
        st_store(Up + NV * i, st_add(st_load(Ub + NV * i), st_mul(st_load(v + NV * i), eps)));
    om_residual(s, Up, Rp, 0);
    for (int i = 0; i < n; ++i) {
        st_t t1 = st_mul(st_sub(st_load(Rp + NV * i), st_load(Rb + NV * i)), 1.0 / eps);
        double tc = s->m->vol[i] / (s->dt[i] + 1e-30);
        st_t t2 = st_mul(st_load(v + NV * i), tc);
        st_store(Jv + NV * i, st_add(t1, t2));
    }
    free(Up);
    free(Rp);
}

/* solveGMRES: one right-preconditioned MGS-GMRES cycle from x0 = 0
 * (src/Solver.cpp:1472-1618).  Returns the iteration count k+1. */
int om_gmres(om_solver* s, const double* Ub, const double* Rb, const double* rhs, double* x) {
    int n = s->m->n_cells, m = s->gmres_m;
    size_t len = (size_t)NV * n;
    double* D = (double*)malloc(sizeof(double) * n);
    om_preconditioner(s, D);
    double* V = (double*)calloc((size_t)(m + 1) * len, sizeof(double));
    double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
    double* sn = (double*)calloc(m, sizeof(double));
    double* cs = (double*)calloc(m, sizeof(double));
    double* gv = (double*)calloc(m + 1, sizeof(double));
    double* z = (double*)malloc(sizeof(double) * len);
#define HH(i, j) H[(size_t)(i) * m + (j)]
    for (size_t q = 0; q < len; ++q) x[q] = 0.0;
    double beta = om_norm(n, rhs);
    int k = 0;
    if (beta < 1e-12) { k = -1; goto done; }
    {
        double ib = 1.0 / beta;
        for (int i = 0; i < n; ++i) st_store(V + NV * i, st_mul(st_load(rhs + NV * i), ib));
    }
    gv[0] = beta;
    for (int j = 0; j < m; ++j) {
        k = j;
        double* Vj = V + (size_t)j * len;
        double* Vj1 = V + (size_t)(j + 1) * len;
        for (int i = 0; i < n; ++i) st_store(z + NV * i, st_mul(st_load(Vj + NV * i), 1.0 / D[i]));
        om_apply_jacobian(s, Ub, Rb, z, Vj1);
        for (int i = 0; i <= j; ++i) {
            double* Vi = V + (size_t)i * len;
            HH(i, j) = om_dot(n, Vj1, Vi);
            for (int c = 0; c < n; ++c)
                st_store(Vj1 + NV * c, st_sub(st_load(Vj1 + NV * c), st_mul(st_load(Vi + NV * c), HH(i, j))));
        }
        HH(j + 1, j) = om_norm(n, Vj1);
        if (HH(j + 1, j) > 1e-12) {
            double ih = 1.0 / HH(j + 1, j);
            for (int c = 0; c < n; ++c) st_store(Vj1 + NV * c, st_mul(st_load(Vj1 + NV * c), ih));
        }
        for (int i = 0; i < j; ++i) {
            double t = cs[i] * HH(i, j) + sn[i] * HH(i + 1, j);
            HH(i + 1, j) = -sn[i] * HH(i, j) + cs[i] * HH(i + 1, j);
            HH(i, j) = t;
        }
        double a = HH(j, j), b = HH(j + 1, j);
        if (fabs(b) < 1e-14) { cs[j] = 1.0; sn[j] = 0.0; }
        else {
            double t = sqrt(a * a + b * b);
            cs[j] = a / t;
            sn[j] = b / t;
        }
        HH(j, j) = cs[j] * a + sn[j] * b;
        HH(j + 1, j) = 0.0;
        gv[j + 1] = -sn[j] * gv[j];
        gv[j] = cs[j] * gv[j];
        if (fabs(gv[j + 1]) < s->gmres_tol * beta) break;
    }
    {
        double* y = (double*)malloc(sizeof(double) * (k + 1));
        for (int i = k; i >= 0; --i) {
            y[i] = gv[i];
            for (int l = i + 1; l <= k; ++l) y[i] -= HH(i, l) * y[l];
            y[i] /= HH(i, i);
        }
        for (size_t q = 0; q < len; ++q) x[q] = 0.0;
        for (int i = 0; i <= k; ++i) {
            const double* Vi = V + (size_t)i * len;
            for (int c = 0; c < n; ++c)
                st_store(x + NV * c, st_add(st_load(x + NV * c), st_mul(st_mul(st_load(Vi + NV * c), y[i]), 1.0 / D[c])));
        }
        free(y);
    }
done:
#undef HH
    free(D); free(V); free(H); free(sn); free(cs); free(gv); free(z);
    return k + 1;
}

/* timeStepExplicit (src/Solver.cpp:1219-1243): residual with the limiter updated,
 * U -= R (dt / vol), rho >= 1e-3, rhoE - kinetic energy >= 1e-3.  Returns norm_L2 of the
 * residual used. */
double om_time_step_explicit(om_solver* s, double dt) {
    int n = s->m->n_cells;
    double* R = (double*)malloc(sizeof(double) * NV * (size_t)n);
    om_residual(s, s->U, R, 1);
    double rn = om_norm(n, R);
    for (int i = 0; i < n; ++i) {
        double vol = s->m->vol[i];
        st_t u = st_sub(st_load(s->U + NV * i), st_mul(st_load(R + NV * i), dt / vol));
        if (u.r < 1e-3) u.r = 1e-3;
        double ke = 0.5 * (u.ru * u.ru + u.rv * u.rv) / u.r;
        double ie = u.rE - ke;
        if (ie < 1e-3) u.rE = ke + 1e-3;
        st_store(s->U + NV * i, u);
    }
    free(R);
    return rn;
}

/* solveUnsteady (src/Solver.cpp:1801-1864): dual time stepping, BDF1, at most 15 Newton
 * steps per physical step to 1e-6 (after the first), GMRES with dt_local = dt_phy,
 * updates relaxed by 0.7.  Writes per physical step the Newton steps taken and the last
 * residual. */
void om_solve_unsteady(om_solver* s, double dt_phy, int n_steps, int* newton, double* res_out) {
    int n = s->m->n_cells;
    size_t len = (size_t)NV * n;
    double* Uold = (double*)malloc(sizeof(double) * len);
    double* R = (double*)malloc(sizeof(double) * len);
    double* rhs = (double*)malloc(sizeof(double) * len);
    double* dU = (double*)malloc(sizeof(double) * len);
    for (int i = 0; i < n; ++i) s->dt[i] = dt_phy;
    for (int t = 1; t <= n_steps; ++t) {
        memcpy(Uold, s->U, sizeof(double) * len);
        int taken = 0;
        double resVM = 0.0;
        for (int step = 0; step < 15; ++step) {
            om_residual(s, s->U, R, 1);
            double norm_sq = 0.0, total_vol = 0.0;
            for (int i = 0; i < n; ++i) {
                double vol = s->m->vol[i];
                st_t dUdt = st_mul(st_sub(st_load(s->U + NV * i), st_load(Uold + NV * i)), vol / dt_phy);
                st_t F = st_add(dUdt, st_load(R + NV * i));
                st_store(rhs + NV * i, st_mul(F, -1.0));
                double a = F.r / vol, b = F.ru / vol, c = F.rv / vol, e = F.rE / vol;
                norm_sq += (a * a + b * b + c * c + e * e) * vol;
                total_vol += vol;
            }
            resVM = sqrt(norm_sq / total_vol);
            taken = step;
            if (resVM < 1e-6 && step > 0) break;
            om_gmres(s, s->U, R, rhs, dU);
            for (int i = 0; i < n; ++i)
                st_store(s->U + NV * i, st_add(st_load(s->U + NV * i), st_mul(st_load(dU + NV * i), 0.7)));
            taken = step + 1;
        }
        if (newton) newton[t - 1] = taken;
        if (res_out) res_out[t - 1] = resVM;
    }
    free(Uold); free(R); free(rhs); free(dU);
}

/* solveImplicit: pseudo-transient Newton with the reference CFL schedule, limiter
 * freeze, relaxation and positivity clamps (src/Solver.cpp:1696-1799).  Writes, per
 * step, the volume-weighted and plain residual norms, the CFL and the GMRES count;
 * returns the number of steps logged. */
int om_solve_implicit(om_solver* s, double tol, int max_steps, double* res_vm, double* res_abs,
                      double* cfl_out, int* iters_out, double* res_rho) {
    int n = s->m->n_cells;
    size_t len = (size_t)NV * n;
    double g = s->gamma;
    double CFL = s->cfl0;
    double* R = (double*)malloc(sizeof(double) * len);
    double* rhs = (double*)malloc(sizeof(double) * len);
    double* dU = (double*)malloc(sizeof(double) * len);
    int logged = 0;
    for (int step = 0; step < max_steps; ++step) {
        om_local_timestep(s, CFL);
        int upd = 1;
        if (step > s->freeze_step || CFL > s->freeze_cfl) upd = 0;
        om_residual(s, s->U, R, upd);
        double rvm = om_norm_vm(s, R);
        double rn = om_norm(n, R);
        double rrho = om_norm_vm_rho(s, R);
        res_vm[step] = rvm; res_abs[step] = rn; cfl_out[step] = CFL; iters_out[step] = 0;
        if (res_rho) res_rho[step] = rrho;
        logged = step + 1;
        if (rvm < tol) break;
        if (s->stop_rho > 0.0 && rrho <= s->stop_rho && step > 5) break;
        for (int i = 0; i < n; ++i) st_store(rhs + NV * i, st_mul(st_load(R + NV * i), -1.0));
        int it = om_gmres(s, s->U, R, rhs, dU);
        iters_out[step] = it;
        if (it >= 29) {
            CFL *= 0.5;
            if (CFL < 0.05) CFL = 0.05;
        }
        double relax = 1.0;
        if (rvm > 1e6) relax = 0.5;
        else if (rvm > 2e3 && rvm < 1e2) relax = 0.9;
        for (int i = 0; i < n; ++i) {
            st_t Un = st_add(st_load(s->U + NV * i), st_mul(st_load(dU + NV * i), relax));
            double ke = 0.5 * (Un.ru * Un.ru + Un.rv * Un.rv) / (Un.r + 1e-12);
            double pn = (g - 1.0) * (Un.rE - ke);
            if (Un.r < 1e-5) Un.r = 1e-5;
            if (pn < 1e-5) {
                pn = 1e-5;
                Un.rE = pn / (g - 1.0) + ke;
            }
            st_store(s->U + NV * i, Un);
        }
        if (step > 5) {
            if (rvm > 1e6) CFL *= 1.2;
            else CFL *= 1.5;
            if (it >= 25) CFL *= 0.5;
            if (CFL > 10000) CFL = 10000;
            if (CFL < 0.1) CFL = 0.1;
        }
    }
    free(R); free(rhs); free(dU);
    return logged;
}

/* extractSkinFriction (src/Solver.cpp:1899-1979) before its sort by x: per boundary face
 * of the tag, in face order, x_mid, Cp = (p - p_exit) / q_inf and Cf = rho nu u_t / dn / q_inf
 * from the owner cell.  Returns the face count; the arrays may be NULL. */
int om_wall_coefficients(const om_solver* s, int tag, double* x, double* cp, double* cf) {
    const om_mesh* m = s->m;
    double g = s->gamma;
    double factor_T = 1.0 + 0.5 * (g - 1.0) * s->M_inf * s->M_inf;
    double T_static = s->T0 / factor_T;
    double c_inf = sqrt(g * s->R_gas * T_static);
    double u_inf = s->M_inf * c_inf;
    double rho_inf = s->Pexit / (s->R_gas * T_static);
    double q_inf = 0.5 * rho_inf * u_inf * u_inf;
    int n = 0;
    for (int f = 0; f < m->n_faces; ++f) {
        if (m->neighbor[f] >= 0 || m->tag[f] != tag) continue;
        if (x) {
            int o = m->owner[f];
            st_t U = st_load(s->U + NV * o);
            double uc = U.ru / U.r, vc = U.rv / U.r;
            double tx = -m->ny[f], ty = m->nx[f];
            if (tx < 0) { tx = -tx; ty = -ty; }
            double ut = uc * tx + vc * ty;
            double dx = m->xm[f] - m->xc[o], dy = m->ym[f] - m->yc[o];
            double dn = fabs(dx * m->nx[f] + dy * m->ny[f]);
            if (dn < 1e-12) dn = 1e-12;
            double dudn = ut / dn;
            double mu = U.r * s->nu;
            double tau = mu * dudn;
            x[n] = m->xm[f];
            cf[n] = tau / q_inf;
            cp[n] = (pressure(U) - s->Pexit) / q_inf;
        }
        ++n;
    }
    return n;
}

/* Wall objectives over the owner states, summed in face order, and dJ/dU (AoS, may be
 * NULL): 0 pressure drag -p A n_x over tag 3 (calculateDrag), 1 skin-friction drag
 * tau_w A t_x over tag 4 (tau_w as extractSkinFriction), 2 p A over tag-4 faces with
 * x0 <= x_mid <= x1.  No reference counterpart beyond the pressure drag. */
double om_objective(const om_solver* s, int kind, double x0, double x1, double* grad) {
    const om_mesh* m = s->m;
    int tag = kind == 0 ? 3 : 4;
    double J = 0.0, gm = s->gamma - 1.0;
    if (grad) memset(grad, 0, sizeof(double) * NV * (size_t)m->n_cells);
    for (int f = 0; f < m->n_faces; ++f) {
        if (m->neighbor[f] >= 0 || m->tag[f] != tag) continue;
        double w = 1.0;
        if (kind == 2) w = (m->xm[f] >= x0 && m->xm[f] <= x1) ? 1.0 : 0.0;
        int o = m->owner[f];
        st_t U = st_load(s->U + NV * o);
        double nx = m->nx[f], ny = m->ny[f], A = m->area[f];
        double t, gb[4];
        if (kind == 1) {
            double tx = -ny, ty = nx;
            if (tx < 0) { tx = -tx; ty = -ty; }
            double dx = m->xm[f] - m->xc[o], dy = m->ym[f] - m->yc[o];
            double dn = fabs(dx * nx + dy * ny);
            if (dn < 1e-12) dn = 1e-12;
            double ut = (U.ru / U.r) * tx + (U.rv / U.r) * ty;
            double tau = (U.r * s->nu) * (ut / dn);
            t = tau * A * tx;
            double c = s->nu / dn * A * tx;
            gb[0] = 0.0; gb[1] = c * tx; gb[2] = c * ty; gb[3] = 0.0;
        } else {
            double p = pressure(U), sc = kind == 0 ? -A * nx : A;
            double u = U.ru / U.r, v = U.rv / U.r;
            t = kind == 0 ? -p * A * nx : p * A;
            gb[0] = sc * gm * 0.5 * (u * u + v * v);
            gb[1] = -sc * gm * u;
            gb[2] = -sc * gm * v;
            gb[3] = sc * gm;
        }
        J += w * t;
        if (grad && w != 0.0)
            for (int c = 0; c < 4; ++c) grad[NV * o + c] += w * gb[c];
    }
    return J;
}

/* computeWallDistances (src/Solver.cpp:1981-2015): nearest tag-4 face midpoint, 1e10 without
 * walls.  The no-slip faces are listed once, in face order, so the scan per cell visits the
 * same faces in the same order as the reference's loop over all faces (same minimum) at
 * O(cells x wall faces) instead of O(cells x faces). */
static void wall_distances(const om_mesh* m, double* d) {
    int nw = 0;
    for (int f = 0; f < m->n_faces; ++f)
        if (m->neighbor[f] < 0 && m->tag[f] == 4) ++nw;
    int* wf = (int*)malloc(sizeof(int) * (nw > 0 ? nw : 1));
    nw = 0;
    for (int f = 0; f < m->n_faces; ++f)
        if (m->neighbor[f] < 0 && m->tag[f] == 4) wf[nw++] = f;
    for (int i = 0; i < m->n_cells; ++i) {
        double best = 1e20;
        for (int k = 0; k < nw; ++k) {
            const int f = wf[k];
            double dx = m->xc[i] - m->xm[f], dy = m->yc[i] - m->ym[f];
            double d2 = dx * dx + dy * dy;
            if (d2 < best) best = d2;
        }
        d[i] = nw > 0 ? sqrt(best) : 1e10;
    }
    free(wf);
}

void om_wall_distance(const om_solver* s, double* d) { wall_distances(s->m, d); }

/* calculateDrag: pressure force on tag-3 faces (src/Solver.cpp:1307-1325) */
double om_drag(const om_solver* s) {
    const om_mesh* m = s->m;
    double d = 0.0;
    for (int f = 0; f < m->n_faces; ++f)
        if (m->tag[f] == 3) {
            double p = pressure(st_load(s->U + NV * m->owner[f]));
            d += -p * m->area[f] * m->nx[f];
        }
    return d;
}

/* calculateEntropyError (src/Solver.cpp:1620-1646) */
double om_entropy_error(const om_solver* s) {
    double g = s->gamma, M = s->M_inf;
    double Tinf = s->T0 / (1.0 + 0.5 * (g - 1.0) * M * M);
    double Pinf = s->P0 / pow(1.0 + 0.5 * (g - 1.0) * M * M, g / (g - 1.0));
    double rinf = Pinf / (s->R_gas * Tinf);
    double Sref = Pinf / pow(rinf, g);
    double se = 0.0, tv = 0.0;
    for (int i = 0; i < s->m->n_cells; ++i) {
        st_t U = st_load(s->U + NV * i);
        double p = pressure(U), r = U.r;
        if (p <= 0 || r <= 0) continue;
        double Sl = p / pow(r, g);
        double e = (Sl - Sref) / Sref;
        se += (e * e) * s->m->vol[i];
        tv += s->m->vol[i];
    }
    return sqrt(se / tv);
}

/* ------------------------------------------------------------------ SST (parity unpinned)
 * Menter SST, 2003 variant, as restated from the published model (Menter, Kuntz & Langtry
 * 2003; the "SST-2003" form of the NASA Turbulence Modeling Resource).  The reference has
 * only scaffolding for it (include/Types.hpp:63-68, src/Solver.cpp:1981-2015), so these
 * functions follow the model, not reference code:
 *   mu_t = rho a1 k / max(a1 w, S F2);  P = min(mu_t S^2, 10 beta* rho k w)
 *   S_k = P - beta* rho w k
 *   S_w = gamma rho / mu_t P - beta rho w^2 + 2 (1 - F1) rho sigma_w2 grad k . grad w / w
 * k and w are advected first-order upwind with the Riemann mass flux and diffused with
 * (mu + sigma mu_t); mu_t enters the mean-flow stresses and, over Pr_t = 0.9, the heat flux.
 * Boundary values: free stream at inflow / far field, extrapolation at the pressure outlet
 * and the slip wall, k = 0 and w = 60 nu / (0.075 d^2) at a no-slip wall face. */

static const double SST_BS = 0.09, SST_A1 = 0.31;
static const double SST_SK1 = 0.85, SST_SW1 = 0.5, SST_B1 = 0.075, SST_G1 = 5.0 / 9.0;
static const double SST_SK2 = 1.0, SST_SW2 = 0.856, SST_B2 = 0.0828, SST_G2 = 0.44;

typedef struct {
    const om_mesh* mesh; /* the mesh and settings the arrays below were built for */
    double Tu, ratio, nu;
    double k_inf, w_inf, w_min;
    double* dwall; /* per cell */
    double* g14;   /* gradients of rho, u, v, p, T, k, w */
    double* mut;
    double* F1;
    double* Sk;
    double* Sw;
} om_sst;

static om_sst g_sst;

/* the model's per-mesh arrays; the wall distance is computeWallDistances
 * (src/Solver.cpp:1981-2015) through wall_distances */
static void sst_setup(om_solver* s, double Tu, double ratio) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    free(g_sst.dwall); free(g_sst.g14); free(g_sst.mut); free(g_sst.F1); free(g_sst.Sk); free(g_sst.Sw);
    g_sst.mesh = m;
    g_sst.Tu = Tu;
    g_sst.ratio = ratio;
    g_sst.nu = s->nu;
    g_sst.dwall = (double*)malloc(sizeof(double) * n);
    g_sst.g14 = (double*)calloc((size_t)14 * n, sizeof(double));
    g_sst.mut = (double*)malloc(sizeof(double) * n);
    g_sst.F1 = (double*)malloc(sizeof(double) * n);
    g_sst.Sk = (double*)malloc(sizeof(double) * n);
    g_sst.Sw = (double*)malloc(sizeof(double) * n);
    wall_distances(m, g_sst.dwall);
    double g = s->gamma, M = s->M_inf;
    double fT = 1.0 + 0.5 * (g - 1.0) * M * M;
    double Ts = s->T0 / fT;
    double U = M * sqrt(g * s->R_gas * Ts);
    g_sst.k_inf = 1.5 * (Tu * U) * (Tu * U);
    g_sst.w_inf = g_sst.k_inf / (ratio * s->nu);
    g_sst.w_min = g_sst.w_inf * 1e-6;
}

static st_t ghost_sst(const om_solver* s, st_t U, int f) {
    const om_mesh* m = s->m;
    st_t gs = ghost(s, U, f);
    int tag = m->tag[f];
    int kind = -1; /* 0 free stream, 1 extrapolate, 2 no-slip wall, -1 keep */
    if (s->bcset == BC_BUMP) kind = tag == 1 ? 0 : tag == 2 ? 1 : -1;
    else if (s->bcset == BC_SUPERSONIC) kind = (tag == 1 || tag == 6) ? 0 : -1;
    else kind = (tag == 1 || tag == 5 || tag == 6) ? 0 : tag == 4 ? 2 : -1;
    if (kind == 0) {
        gs.rk = gs.r * g_sst.k_inf;
        gs.rw = gs.r * g_sst.w_inf;
    } else if (kind == 1) {
        gs.rk = gs.r * (U.rk / U.r);
        gs.rw = gs.r * (U.rw / U.r);
    } else if (kind == 2) {
        int o = m->owner[f];
        double dn = fabs((m->xm[f] - m->xc[o]) * m->nx[f] + (m->ym[f] - m->yc[o]) * m->ny[f]);
        if (dn < 1e-30) dn = 1e-30;
        double ww = 60.0 * s->nu / (0.075 * dn * dn);
        gs.rk = -gs.r * (U.rk / U.r);
        gs.rw = gs.r * (2.0 * ww - U.rw / U.r);
    }
    return gs;
}

/* face averages of rho, u, v, p, T, k, w summed Green-Gauss style */
static void sst_gradients(om_solver* s, const double* Uin) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double* G = g_sst.g14;
    memset(G, 0, sizeof(double) * 14 * (size_t)n);
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        st_t L = st_load(Uin + NV * o);
        st_t Rs = nb >= 0 ? st_load(Uin + NV * nb) : ghost_sst(s, L, f);
        double wl[7] = {L.r, L.ru / L.r, L.rv / L.r, pressure(L), 0, L.rk / L.r, L.rw / L.r};
        double wr[7] = {Rs.r, Rs.ru / Rs.r, Rs.rv / Rs.r, pressure(Rs), 0, Rs.rk / Rs.r, Rs.rw / Rs.r};
        wl[4] = wl[3] / (L.r * s->R_gas);
        wr[4] = wr[3] / (Rs.r * s->R_gas);
        double nx = m->nx[f], ny = m->ny[f], A = m->area[f];
        for (int q = 0; q < 7; ++q) {
            double ph = 0.5 * (wl[q] + wr[q]);
            G[14 * o + 2 * q] += ph * nx * A;
            G[14 * o + 2 * q + 1] += ph * ny * A;
            if (nb >= 0) {
                G[14 * nb + 2 * q] -= ph * nx * A;
                G[14 * nb + 2 * q + 1] -= ph * ny * A;
            }
        }
    }
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < 14; ++q) G[14 * i + q] /= m->vol[i];
}

static void sst_cells(om_solver* s, const double* Uin) {
    int n = s->m->n_cells;
    for (int i = 0; i < n; ++i) {
        const double* g = g_sst.g14 + 14 * i;
        double r = Uin[NV * i];
        double k = Uin[NV * i + 4] / r, w = Uin[NV * i + 5] / r;
        double kp = k > 0 ? k : 0.0;
        double wp = w > g_sst.w_min ? w : g_sst.w_min;
        double ux = g[2], uy = g[3], vx = g[4], vy = g[5];
        double kx = g[10], ky = g[11], wx = g[12], wy = g[13];
        double Sxy = 0.5 * (uy + vx);
        double S2 = 2.0 * (ux * ux + vy * vy + 2.0 * Sxy * Sxy);
        double Smag = sqrt(S2 + 1e-30);
        double d = g_sst.dwall[i] > 1e-30 ? g_sst.dwall[i] : 1e-30;
        double gkgw = kx * wx + ky * wy;
        double CD = 2.0 * r * SST_SW2 * gkgw / wp;
        if (CD < 1e-10) CD = 1e-10;
        double sk = sqrt(kp + 1e-30);
        double t1 = sk / (SST_BS * wp * d);
        double t2 = 500.0 * s->nu / (d * d * wp);
        double t3 = 4.0 * r * SST_SW2 * kp / (CD * d * d);
        double arg1 = t1 > t2 ? t1 : t2;
        if (t3 < arg1) arg1 = t3;
        double F1 = tanh(arg1 * arg1 * arg1 * arg1);
        double arg2 = 2.0 * t1 > t2 ? 2.0 * t1 : t2;
        double F2 = tanh(arg2 * arg2);
        double den = SST_A1 * wp > Smag * F2 ? SST_A1 * wp : Smag * F2;
        double mut = r * SST_A1 * kp / den;
        double beta = F1 * SST_B1 + (1.0 - F1) * SST_B2;
        double gam = F1 * SST_G1 + (1.0 - F1) * SST_G2;
        double P = mut * S2;
        double Pl = 10.0 * SST_BS * r * kp * wp;
        if (Pl < P) P = Pl;
        g_sst.mut[i] = mut;
        g_sst.F1[i] = F1;
        g_sst.Sk[i] = P - SST_BS * r * wp * kp;
        g_sst.Sw[i] = gam * r / (mut + 1e-30) * P - beta * r * wp * wp + 2.0 * (1.0 - F1) * r * SST_SW2 * gkgw / wp;
    }
}

/* The residual with the SST model (nv = 6).  The mean-flow face flux is the reference's
 * (reconstruction, Riemann or wall flux, viscous flux) with mu_t added to the viscosity. */
void om_residual_sst(om_solver* s, const double* Uin, double* Rout, double Tu, double ratio) {
    const om_mesh* m = s->m;
    int n = m->n_cells;
    double g = s->gamma, R = s->R_gas;
    if (!g_sst.dwall || g_sst.mesh != s->m || g_sst.Tu != Tu || g_sst.ratio != ratio || g_sst.nu != s->nu)
        sst_setup(s, Tu, ratio);
    memset(Rout, 0, sizeof(double) * NV * (size_t)n);
    if (s->spatial == SP_LIMITED) {
        om_gradients(s, Uin);
        om_limiters(s, Uin);
    }
    sst_gradients(s, Uin);
    sst_cells(s, Uin);
    double Cp = g * R / (g - 1.0);
    const double* G = g_sst.g14;
    for (int f = 0; f < m->n_faces; ++f) {
        int o = m->owner[f], nb = m->neighbor[f];
        double nx = m->nx[f], ny = m->ny[f], A = m->area[f];
        int tag = m->tag[f];
        int wall = nb < 0 && tag == 4;
        st_t L = st_load(Uin + NV * o);
        st_t Rs = nb >= 0 ? st_load(Uin + NV * nb) : ghost_sst(s, L, f);
        st_t Lr = L, Rr = Rs;
        if (s->spatial != SP_FIRST && nb >= 0) {
            double dxL = m->xm[f] - m->xc[o], dyL = m->ym[f] - m->yc[o];
            double dxR = m->xm[f] - m->xc[nb], dyR = m->ym[f] - m->yc[nb];
            const double* gL = G + 14 * o;
            const double* gR = G + 14 * nb;
            double phL = s->spatial == SP_LIMITED ? s->phi[o] : 0.5;
            double phR = s->spatial == SP_LIMITED ? s->phi[nb] : 0.5;
            double pL = pressure(L), pR = pressure(Rs);
            double rLf = L.r + phL * (gL[0] * dxL + gL[1] * dyL), pLf = pL + phL * (gL[6] * dxL + gL[7] * dyL);
            double uLf = L.ru / L.r + phL * (gL[2] * dxL + gL[3] * dyL), vLf = L.rv / L.r + phL * (gL[4] * dxL + gL[5] * dyL);
            if (rLf < 1e-4) rLf = L.r;
            if (pLf < 1e-4) pLf = pL;
            Lr = p2c(s, rLf, uLf, vLf, pLf, 0.0, 0.0);
            double rRf = Rs.r + phR * (gR[0] * dxR + gR[1] * dyR), pRf = pR + phR * (gR[6] * dxR + gR[7] * dyR);
            double uRf = Rs.ru / Rs.r + phR * (gR[2] * dxR + gR[3] * dyR), vRf = Rs.rv / Rs.r + phR * (gR[4] * dxR + gR[5] * dyR);
            if (rRf < 1e-4) rRf = Rs.r;
            if (pRf < 1e-4) pRf = pR;
            Rr = p2c(s, rRf, uRf, vRf, pRf, 0.0, 0.0);
        }
        st_t FE;
        if (nb < 0 && (tag == 3 || tag == 4)) {
            double pw = pressure(Lr);
            FE = st(0.0, pw * nx, pw * ny, 0.0, 0.0, 0.0);
        } else {
            FE = inviscid_flux(Lr, Rr, nx, ny, s->flux);
        }
        /* mean-flow viscous flux with mu + mu_t */
        double mutL = g_sst.mut[o], mutR = nb >= 0 ? g_sst.mut[nb] : mutL;
        double mutf = wall ? 0.0 : 0.5 * (mutL + mutR);
        double F1f = 0.5 * (g_sst.F1[o] + (nb >= 0 ? g_sst.F1[nb] : g_sst.F1[o]));
        const double* gL = G + 14 * o;
        const double* gR = nb >= 0 ? G + 14 * nb : gL;
        double rf = 0.5 * (L.r + Rs.r);
        double uL = L.ru / L.r, vL = L.rv / L.r, uR = Rs.ru / Rs.r, vR = Rs.rv / Rs.r;
        double uf = 0.5 * (uL + uR), vf = 0.5 * (vL + vR);
        double dudx, dudy, dvdx, dvdy, dTdx, dTdy;
        double dxo = m->xm[f] - m->xc[o], dyo = m->ym[f] - m->yc[o];
        double dxlr = nb >= 0 ? m->xc[nb] - m->xc[o] : 0.0, dylr = nb >= 0 ? m->yc[nb] - m->yc[o] : 0.0;
        double d2lr = dxlr * dxlr + dylr * dylr;
        if (wall) {
            double d2 = dxo * dxo + dyo * dyo;
            dudx = -uL * dxo / d2; dudy = -uL * dyo / d2; dvdx = -vL * dxo / d2; dvdy = -vL * dyo / d2;
            dTdx = 0.0; dTdy = 0.0;
        } else {
            dudx = 0.5 * (gL[2] + gR[2]); dudy = 0.5 * (gL[3] + gR[3]);
            dvdx = 0.5 * (gL[4] + gR[4]); dvdy = 0.5 * (gL[5] + gR[5]);
            dTdx = 0.5 * (gL[8] + gR[8]); dTdy = 0.5 * (gL[9] + gR[9]);
            if (d2lr > 1e-14) {
                double cu = (dudx * dxlr + dudy * dylr - (uR - uL)) / d2lr;
                double cv = (dvdx * dxlr + dvdy * dylr - (vR - vL)) / d2lr;
                dudx -= cu * dxlr; dudy -= cu * dylr; dvdx -= cv * dxlr; dvdy -= cv * dylr;
            }
        }
        double mu = rf * s->nu + mutf;
        double kc = rf * s->nu * Cp / s->Pr + mutf * Cp / 0.9;
        double div = dudx + dvdy;
        double txx = mu * (2.0 * dudx - (2.0 / 3.0) * div);
        double tyy = mu * (2.0 * dvdy - (2.0 / 3.0) * div);
        double txy = mu * (dudy + dvdx);
        double wx = uf * txx + vf * txy + kc * dTdx, wy = uf * txy + vf * tyy + kc * dTdy;
        double TF[6];
        TF[0] = FE.r;
        TF[1] = FE.ru - (txx * nx + txy * ny);
        TF[2] = FE.rv - (txy * nx + tyy * ny);
        TF[3] = FE.rE - (wx * nx + wy * ny);
        /* k and w: upwind advection with the mass flux, diffusion with mu + sigma mu_t */
        double mdot = TF[0];
        double kL = L.rk / L.r, wL = L.rw / L.r, kR = Rs.rk / Rs.r, wR = Rs.rw / Rs.r;
        double Fk = (mdot > 0 ? mdot * kL : mdot * kR);
        double Fw = (mdot > 0 ? mdot * wL : mdot * wR);
        double sk = F1f * SST_SK1 + (1.0 - F1f) * SST_SK2, sw = F1f * SST_SW1 + (1.0 - F1f) * SST_SW2;
        double dkn, dwn;
        if (wall) {
            double d2 = dxo * dxo + dyo * dyo, dn = dxo * nx + dyo * ny;
            dkn = (0.0 - kL) * dn / d2;
            dwn = (0.5 * (wL + wR) - wL) * dn / d2;
        } else {
            double kx = 0.5 * (gL[10] + gR[10]), ky = 0.5 * (gL[11] + gR[11]);
            double wxg = 0.5 * (gL[12] + gR[12]), wyg = 0.5 * (gL[13] + gR[13]);
            if (d2lr > 1e-14) {
                double ck = (kx * dxlr + ky * dylr - (kR - kL)) / d2lr;
                double cw = (wxg * dxlr + wyg * dylr - (wR - wL)) / d2lr;
                kx -= ck * dxlr; ky -= ck * dylr; wxg -= cw * dxlr; wyg -= cw * dylr;
            }
            dkn = kx * nx + ky * ny;
            dwn = wxg * nx + wyg * ny;
        }
        double mul = rf * s->nu;
        TF[4] = Fk - (mul + sk * mutf) * dkn;
        TF[5] = Fw - (mul + sw * mutf) * dwn;
        for (int c = 0; c < 6; ++c) {
            Rout[NV * o + c] += TF[c] * A;
            if (nb >= 0) Rout[NV * nb + c] -= TF[c] * A;
        }
    }
    for (int i = 0; i < n; ++i) {
        Rout[NV * i + 4] -= g_sst.Sk[i] * m->vol[i];
        Rout[NV * i + 5] -= g_sst.Sw[i] * m->vol[i];
    }
}

void om_sst_reset(void) {
    free(g_sst.dwall); free(g_sst.g14); free(g_sst.mut); free(g_sst.F1); free(g_sst.Sk); free(g_sst.Sw);
    memset(&g_sst, 0, sizeof g_sst);
}

void om_sst_freestream(om_solver* s, double Tu, double ratio, double* kw) {
    sst_setup(s, Tu, ratio);
    kw[0] = g_sst.k_inf;
    kw[1] = g_sst.w_inf;
}
