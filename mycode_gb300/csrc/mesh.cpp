// Mesh ingest for the GPU solver.
//
// Connectivity and geometry restate Mesh::buildConnectivity and Mesh::computeGeometry
// (AmberMond/mycode src/Mesh.cpp:102-201) with the same face creation order, owner
// choice, node ordering and floating-point expressions (this file is compiled without
// FMA contraction), so face/cell indexing is bit-exact with the reference.  The cells
// are then renumbered along a Hilbert curve (or by reverse Cuthill-McKee), faces are
// sorted by their new owner with boundary faces last, and each cell's face list keeps
// the REFERENCE face order so the per-cell sums add in the reference's order.
#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <numeric>
#include <queue>
#include <sstream>
#include <unordered_map>

namespace cfdg {

namespace {

inline uint64_t edge_key(int a, int b) {
    uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    return ((uint64_t)lo << 32) | hi;
}

// Hilbert index of (x, y) on an n x n grid, n = 2^order (quadrant walk with rotation)
uint64_t hilbert_index(uint32_t x, uint32_t y, int order) {
    const uint32_t n = 1u << order;
    uint64_t d = 0;
    for (uint32_t s = n >> 1; s > 0; s >>= 1) {
        uint32_t rx = (x & s) ? 1u : 0u;
        uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = n - 1 - x;
                y = n - 1 - y;
            }
            std::swap(x, y);
        }
    }
    return d;
}

void order_hilbert(const HostMesh& m, std::vector<int>& perm) {
    double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
    for (int i = 0; i < m.n_cells; ++i) {
        x0 = std::min(x0, m.c_xc[i]); x1 = std::max(x1, m.c_xc[i]);
        y0 = std::min(y0, m.c_yc[i]); y1 = std::max(y1, m.c_yc[i]);
    }
    const int order = 16;
    const double span = std::max(x1 - x0, y1 - y0) + 1e-300;
    const double scale = ((1u << order) - 1) / span;
    std::vector<std::pair<uint64_t, int>> key(m.n_cells);
    for (int i = 0; i < m.n_cells; ++i) {
        uint32_t hx = (uint32_t)((m.c_xc[i] - x0) * scale);
        uint32_t hy = (uint32_t)((m.c_yc[i] - y0) * scale);
        key[i] = {hilbert_index(hx, hy, order), i};
    }
    std::sort(key.begin(), key.end());
    perm.resize(m.n_cells);
    for (int i = 0; i < m.n_cells; ++i) perm[i] = key[i].second;
}

void order_rcm(const HostMesh& m, std::vector<int>& perm) {
    int n = m.n_cells;
    std::vector<int> deg(n, 0), start(n + 1, 0);
    for (int f = 0; f < m.n_faces; ++f)
        if (m.f_n[f] >= 0) { ++deg[m.f_o[f]]; ++deg[m.f_n[f]]; }
    for (int i = 0; i < n; ++i) start[i + 1] = start[i] + deg[i];
    std::vector<int> adj(start[n]), fill(start.begin(), start.end() - 1);
    for (int f = 0; f < m.n_faces; ++f)
        if (m.f_n[f] >= 0) { adj[fill[m.f_o[f]]++] = m.f_n[f]; adj[fill[m.f_n[f]]++] = m.f_o[f]; }
    std::vector<char> seen(n, 0);
    std::vector<int> order;
    order.reserve(n);
    std::vector<int> by_deg(n);
    std::iota(by_deg.begin(), by_deg.end(), 0);
    std::stable_sort(by_deg.begin(), by_deg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
    for (int seed : by_deg) {
        if (seen[seed]) continue;
        std::queue<int> q;
        q.push(seed);
        seen[seed] = 1;
        while (!q.empty()) {
            int c = q.front();
            q.pop();
            order.push_back(c);
            std::vector<int> nb;
            for (int k = start[c]; k < start[c + 1]; ++k)
                if (!seen[adj[k]]) { seen[adj[k]] = 1; nb.push_back(adj[k]); }
            std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
            for (int x : nb) q.push(x);
        }
    }
    perm.assign(order.rbegin(), order.rend());
}

}  // namespace

void order_rcm_host(const HostMesh& m, std::vector<int>& perm) { order_rcm(m, perm); }

std::string build_mesh(HostMesh& m, int n_nodes, const double* xy, int n_cells, const int* cells,
                       int n_bedges, const int* bedges, int renumber) {
    if (n_nodes <= 0 || n_cells <= 0) return "mesh has no nodes or no cells";
    m = HostMesh();
    m.n_nodes = n_nodes;
    m.n_cells = n_cells;
    m.xy.assign(xy, xy + 2 * (size_t)n_nodes);
    m.cell_nodes.assign(cells, cells + 4 * (size_t)n_cells);
    for (int i = 0; i < n_cells; ++i) {
        int nv = cells[4 * i + 3] >= 0 ? 4 : 3;
        for (int k = 0; k < nv; ++k) {
            int v = cells[4 * i + k];
            if (v < 0 || v >= n_nodes) {
                char b[128];
                std::snprintf(b, sizeof b, "cell %d refers to node %d outside [0, %d)", i, v, n_nodes);
                return b;
            }
        }
    }
    std::unordered_map<uint64_t, int> btag;
    btag.reserve(2 * (size_t)n_bedges + 16);
    for (int e = 0; e < n_bedges; ++e) btag[edge_key(bedges[3 * e], bedges[3 * e + 1])] = bedges[3 * e + 2];

    // Mesh::buildConnectivity (src/Mesh.cpp:102-143): faces in order of first appearance
    std::unordered_map<uint64_t, int> e2f;
    e2f.reserve(4 * (size_t)n_cells);
    for (int i = 0; i < n_cells; ++i) {
        const int* c = cells + 4 * i;
        int n = c[3] >= 0 ? 4 : 3;
        for (int j = 0; j < n; ++j) {
            int a = c[j], b = c[(j + 1) % n];
            uint64_t k = edge_key(a, b);
            auto it = e2f.find(k);
            if (it != e2f.end()) {
                if (m.f_n[it->second] >= 0) {
                    char buf[160];
                    std::snprintf(buf, sizeof buf, "edge (%d,%d) is shared by more than two cells", a, b);
                    return buf;
                }
                m.f_n[it->second] = i;
            } else {
                e2f.emplace(k, (int)m.f_o.size());
                m.f_n1.push_back(std::min(a, b));
                m.f_n2.push_back(std::max(a, b));
                m.f_o.push_back(i);
                m.f_n.push_back(-1);
                auto bt = btag.find(k);
                m.f_tag.push_back(bt != btag.end() ? bt->second : 0);
            }
        }
    }
    m.n_faces = (int)m.f_o.size();

    // Mesh::computeGeometry (src/Mesh.cpp:148-201)
    m.c_vol.resize(n_cells);
    m.c_xc.resize(n_cells);
    m.c_yc.resize(n_cells);
    auto X = [&](int k) { return xy[2 * k]; };
    auto Y = [&](int k) { return xy[2 * k + 1]; };
    for (int i = 0; i < n_cells; ++i) {
        const int* c = cells + 4 * i;
        if (c[3] < 0) {
            double x1 = X(c[0]), y1 = Y(c[0]), x2 = X(c[1]), y2 = Y(c[1]), x3 = X(c[2]), y3 = Y(c[2]);
            m.c_vol[i] = 0.5 * std::fabs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1));
            m.c_xc[i] = (x1 + x2 + x3) / 3.0;
            m.c_yc[i] = (y1 + y2 + y3) / 3.0;
        } else {
            double sx = 0, sy = 0, a = 0.0;
            for (int k = 0; k < 4; ++k) { sx += X(c[k]); sy += Y(c[k]); }
            m.c_xc[i] = sx / 4.0;
            m.c_yc[i] = sy / 4.0;
            for (int k = 0; k < 4; ++k) {
                int n1 = c[k], n2 = c[(k + 1) % 4];
                a += (X(n1) * Y(n2) - X(n2) * Y(n1));
            }
            m.c_vol[i] = 0.5 * std::fabs(a);
        }
        if (!(m.c_vol[i] > 0.0)) {
            char b[96];
            std::snprintf(b, sizeof b, "cell %d has zero or invalid area", i);
            return b;
        }
    }
    int nf = m.n_faces;
    m.f_nx.resize(nf); m.f_ny.resize(nf); m.f_area.resize(nf); m.f_xm.resize(nf); m.f_ym.resize(nf);
    for (int f = 0; f < nf; ++f) {
        double dx = X(m.f_n2[f]) - X(m.f_n1[f]);
        double dy = Y(m.f_n2[f]) - Y(m.f_n1[f]);
        double A = std::sqrt(dx * dx + dy * dy);
        m.f_area[f] = A;
        m.f_xm[f] = 0.5 * (X(m.f_n1[f]) + X(m.f_n2[f]));
        m.f_ym[f] = 0.5 * (Y(m.f_n1[f]) + Y(m.f_n2[f]));
        double nx = dy / A, ny = -dx / A;
        double vx = m.f_xm[f] - m.c_xc[m.f_o[f]];
        double vy = m.f_ym[f] - m.c_yc[m.f_o[f]];
        if (vx * nx + vy * ny < 0) { nx = -nx; ny = -ny; }
        m.f_nx[f] = nx;
        m.f_ny[f] = ny;
    }

    // ---- renumbering
    if (renumber == RENUMBER_HILBERT) order_hilbert(m, m.cell_perm);
    else if (renumber == RENUMBER_RCM) order_rcm(m, m.cell_perm);
    else { m.cell_perm.resize(n_cells); std::iota(m.cell_perm.begin(), m.cell_perm.end(), 0); }
    m.cell_inv.assign(n_cells, 0);
    for (int i = 0; i < n_cells; ++i) m.cell_inv[m.cell_perm[i]] = i;

    std::vector<std::pair<std::pair<int, int>, int>> fk(nf);
    int nb = 0;
    for (int f = 0; f < nf; ++f) {
        int o = m.cell_inv[m.f_o[f]];
        bool bnd = m.f_n[f] < 0;
        nb += bnd;
        int other = bnd ? 0 : m.cell_inv[m.f_n[f]];
        // interior faces first, each group ordered by the lower new cell index
        int k0 = (bnd ? (1 << 30) : 0) + (bnd ? o : std::min(o, other));
        fk[f] = {{k0, bnd ? f : std::max(o, other)}, f};
    }
    std::sort(fk.begin(), fk.end());
    m.n_interior = nf - nb;
    m.face_perm.resize(nf);
    m.face_inv.resize(nf);
    for (int s = 0; s < nf; ++s) { m.face_perm[s] = fk[s].second; m.face_inv[fk[s].second] = s; }

    m.fo.resize(nf); m.fn.resize(nf); m.ftag.resize(nf);
    m.nx.resize(nf); m.ny.resize(nf); m.area.resize(nf);
    m.dxo.resize(nf); m.dyo.resize(nf); m.dxn.resize(nf); m.dyn.resize(nf); m.dxlr.resize(nf); m.dylr.resize(nf);
    for (int s = 0; s < nf; ++s) {
        int f = m.face_perm[s];
        int o = m.f_o[f], n = m.f_n[f];
        m.fo[s] = m.cell_inv[o];
        m.fn[s] = n >= 0 ? m.cell_inv[n] : -1;
        m.ftag[s] = m.f_tag[f];
        m.nx[s] = m.f_nx[f];
        m.ny[s] = m.f_ny[f];
        m.area[s] = m.f_area[f];
        // same expressions as the reference's dx_L, dx_R and dx_LR (src/Solver.cpp:564-567, :729-730)
        m.dxo[s] = m.f_xm[f] - m.c_xc[o];
        m.dyo[s] = m.f_ym[f] - m.c_yc[o];
        m.dxn[s] = n >= 0 ? m.f_xm[f] - m.c_xc[n] : 0.0;
        m.dyn[s] = n >= 0 ? m.f_ym[f] - m.c_yc[n] : 0.0;
        int n2 = n >= 0 ? n : o;
        m.dxlr[s] = m.c_xc[n2] - m.c_xc[o];
        m.dylr[s] = m.c_yc[n2] - m.c_yc[o];
        if (n < 0 && m.f_tag[f] == 4) m.wall_faces.push_back(s);
    }
    m.vol.resize(n_cells); m.xc.resize(n_cells); m.yc.resize(n_cells);
    for (int i = 0; i < n_cells; ++i) {
        m.vol[i] = m.c_vol[m.cell_perm[i]];
        m.xc[i] = m.c_xc[m.cell_perm[i]];
        m.yc[i] = m.c_yc[m.cell_perm[i]];
    }
    // per-cell face lists in reference face order
    std::vector<int> cnt(n_cells, 0);
    std::vector<int> tmp(4 * (size_t)n_cells, -1);
    for (int f = 0; f < nf; ++f) {
        int s = m.face_inv[f];
        int o = m.cell_inv[m.f_o[f]];
        if (cnt[o] >= 4) return "a cell has more than four faces";
        tmp[4 * (size_t)o + cnt[o]++] = (s << 1);
        if (m.f_n[f] >= 0) {
            int n = m.cell_inv[m.f_n[f]];
            if (cnt[n] >= 4) return "a cell has more than four faces";
            tmp[4 * (size_t)n + cnt[n]++] = (s << 1) | 1;
        }
    }
    m.cf.assign(4 * (size_t)n_cells, -1);
    for (int i = 0; i < n_cells; ++i)
        for (int k = 0; k < 4; ++k) m.cf[(size_t)k * n_cells + i] = tmp[4 * (size_t)i + k];
    return "";
}

std::string read_gmsh(const std::string& path, std::vector<double>& xy, std::vector<int>& cells,
                      std::vector<int>& bedges) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return "cannot open mesh file " + path;
    std::string line;
    auto strip = [](std::string& s) {
        while (!s.empty() && (s.back() == '\r' || s.back() == '\n' || s.back() == ' ')) s.pop_back();
    };
    std::unordered_map<long, int> remap;
    bool have_nodes = false, have_elems = false;
    while (std::getline(in, line)) {
        strip(line);
        if (line == "$Nodes") {
            std::getline(in, line);
            strip(line);
            long n = std::atol(line.c_str());
            if (n <= 0) return "bad $Nodes count";
            xy.resize(2 * n);
            for (long i = 0; i < n; ++i) {
                if (!std::getline(in, line)) return "truncated $Nodes";
                std::istringstream ss(line);
                long id;
                double x, y, z;
                if (!(ss >> id >> x >> y >> z)) return "bad node line";
                remap[id] = (int)i;
                xy[2 * i] = x;
                xy[2 * i + 1] = y;
            }
            have_nodes = true;
        } else if (line == "$Elements") {
            if (!have_nodes) return "$Elements before $Nodes";
            std::getline(in, line);
            strip(line);
            long n = std::atol(line.c_str());
            for (long e = 0; e < n; ++e) {
                if (!std::getline(in, line)) return "truncated $Elements";
                std::istringstream ss(line);
                long id, type, ntag, tag = 0, t;
                if (!(ss >> id >> type >> ntag)) return "bad element line";
                for (long j = 0; j < ntag; ++j) {
                    ss >> t;
                    if (j == 0) tag = t;
                }
                int nn = type == 1 ? 2 : type == 2 ? 3 : type == 3 ? 4 : 0;
                int v[4] = {-1, -1, -1, -1};
                for (int k = 0; k < nn; ++k) {
                    long q;
                    if (!(ss >> q)) return "bad element node list";
                    auto it = remap.find(q);
                    if (it == remap.end()) return "element refers to an unknown node";
                    v[k] = it->second;
                }
                if (type == 1) { bedges.push_back(v[0]); bedges.push_back(v[1]); bedges.push_back((int)tag); }
                else if (type == 2 || type == 3) for (int k = 0; k < 4; ++k) cells.push_back(v[k]);
            }
            have_elems = true;
        }
    }
    if (!have_nodes || !have_elems) return "no $Nodes/$Elements section in " + path;
    return "";
}

}  // namespace cfdg
