// Host-side mesh ingest: connectivity, geometry, renumbering and the device layout.
#pragma once
#include <string>
#include <vector>

namespace cfdg {

enum Renumber { RENUMBER_NONE = 0, RENUMBER_HILBERT = 1, RENUMBER_RCM = 2 };

struct HostMesh {
    int n_nodes = 0, n_cells = 0, n_faces = 0, n_interior = 0;
    // ---- reference numbering (Mesh::buildConnectivity / computeGeometry order)
    std::vector<double> xy;          // 2 per node
    std::vector<int> cell_nodes;     // 4 per cell, -1 pads triangles
    std::vector<int> f_n1, f_n2, f_o, f_n, f_tag;
    std::vector<double> f_nx, f_ny, f_area, f_xm, f_ym;
    std::vector<double> c_vol, c_xc, c_yc;
    // ---- renumbering
    std::vector<int> cell_perm;      // new -> reference cell
    std::vector<int> cell_inv;       // reference cell -> new
    std::vector<int> face_perm;      // new slot -> reference face
    std::vector<int> face_inv;       // reference face -> new slot
    // ---- device layout (new numbering; faces [0, n_interior) interior)
    std::vector<int> cf;             // [4][n_cells]: (slot << 1) | side, -1 pads
    std::vector<int> fo, fn, ftag;
    std::vector<double> nx, ny, area, dxo, dyo, dxn, dyn, dxlr, dylr, vol, xc, yc;
    std::vector<int> wall_faces;     // new slots of no-slip (tag 4) boundary faces
};

// Builds the mesh from nodes, cells (4 ids per cell, -1 pads triangles, 0-based) and
// tagged boundary edges (a, b, tag).  Returns an empty string on success, else why not.
std::string build_mesh(HostMesh& m, int n_nodes, const double* xy, int n_cells, const int* cells,
                       int n_bedges, const int* bedges, int renumber);

// The same mesh built by kernels on `device` (mesh_gpu.cu): connectivity, geometry, the
// Hilbert renumbering and the device layout; the same HostMesh bit for bit.  *seconds (may
// be null) gets the device time of the build.
std::string build_mesh_gpu(HostMesh& m, int n_nodes, const double* xy, int n_cells, const int* cells,
                           int n_bedges, const int* bedges, int renumber, int device, double* seconds);

// Gmsh 2.2 ASCII reader (LF or CRLF line ends).
std::string read_gmsh(const std::string& path, std::vector<double>& xy, std::vector<int>& cells,
                      std::vector<int>& bedges);

}  // namespace cfdg
