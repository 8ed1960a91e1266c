"""Synthetic 2D meshes for the solver's workloads (seeded, reproducible).

Each generator returns a :class:`MeshSpec`: node coordinates, cells as node
lists (triangles padded with -1 in the fourth slot) and tagged boundary edges,
i.e. exactly what a Gmsh 2.2 ASCII file gives the reference's ``Mesh::load``
(src/Mesh.cpp:30-97): element type 1 = boundary edge with its first physical
tag, type 2 = triangle, type 3 = quad.  Node numbering is 0-based here; the
Gmsh writer adds one.

Physical tags follow the reference meshes: 1 inlet, 2 outlet, 3 slip wall /
symmetry, 4 no-slip wall, 5 far field (mesh/new_laminar_flat_plate's
$PhysicalNames), plus 6 = fixed post-shock inflow state for the
shock/boundary-layer interaction workload.

Recipes (cells, faces):
  wedge         120x80 quads split into 2 triangles, ramp 15 deg from x=0.5,
                1.5 x 1.0 domain, interior jitter +-10 % of the local spacing.
  laminar_plate 240x120 quads, x in [-0.2, 1], y in [0, 0.5], geometric
                wall-normal stretching ratio 1.08.
  turb_plate    480x240 quads, x in [-0.4, 2], y in [0, 1], first spacing for
                y+ < 1 at Re 5e6/m, growth ratio 1.12 capped to fill the height.
  swbli         800x640 stretched quads, the outer half of the rows split into
                triangles, jitter 5 % of the smaller local spacing in both
                directions (isotropic: a per-direction jitter of the streamwise
                spacing would tilt the y+ < 1 wall cells, aspect ratio ~10^3, to
                slivers).
  bump          3x1 channel with a Gaussian bump (height 0.05, width 0.2),
                n_y = round(sqrt(N/6)), n_x = 3 n_y, every quad split in two.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

TAG_INLET, TAG_OUTLET, TAG_SLIP, TAG_NOSLIP, TAG_FARFIELD, TAG_SHOCK_INFLOW = 1, 2, 3, 4, 5, 6


@dataclasses.dataclass
class MeshSpec:
    name: str
    nodes: np.ndarray   # float64 [n_nodes, 2]
    cells: np.ndarray   # int32 [n_cells, 4], node ids, -1 pads triangles
    bedges: np.ndarray  # int32 [n_bedges, 3]: node a, node b, physical tag

    @property
    def n_cells(self) -> int:
        return int(self.cells.shape[0])

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    def expected_faces(self) -> int:
        """Edge count by Euler's relation for a simply connected 2D mesh."""
        nv = np.where(self.cells[:, 3] >= 0, 4, 3)
        return int((nv.sum() + self.bedges.shape[0]) // 2)


def _geometric(n: int, total: float, ratio: float) -> np.ndarray:
    """n spacings growing by ``ratio`` that add up to ``total``; returns n+1 coordinates."""
    if abs(ratio - 1.0) < 1e-14:
        h = np.full(n, total / n)
    else:
        h0 = total * (ratio - 1.0) / (ratio ** n - 1.0)
        h = h0 * ratio ** np.arange(n)
    y = np.concatenate([[0.0], np.cumsum(h)])
    y[-1] = total
    return y


def _capped_geometric(n: int, total: float, first: float, ratio: float) -> np.ndarray:
    """Spacings start at ``first`` and grow by ``ratio`` until they reach the uniform
    spacing that fills the rest of ``total`` with the remaining cells."""
    for n_grow in range(1, n):
        h = first * ratio ** np.arange(n_grow)
        rest = total - h.sum()
        if rest <= 0:
            break
        h_uni = rest / (n - n_grow)
        if h_uni <= h[-1] * ratio:
            sp = np.concatenate([h, np.full(n - n_grow, h_uni)])
            y = np.concatenate([[0.0], np.cumsum(sp)])
            y[-1] = total
            return y
    return _geometric(n, total, ratio)


def _structured(name: str, X: np.ndarray, Y: np.ndarray, split_row, tag_of_edge,
                jitter: float = 0.0, seed: int = 0, isotropic: bool = False) -> MeshSpec:
    """Mesh of the (ny+1) x (nx+1) node grid X, Y.

    Cells are emitted row by row (j outer, i inner).  A quad (a,b,c,d) =
    ((i,j),(i+1,j),(i+1,j+1),(i,j+1)) is either kept or split along a-c into
    (a,b,c) and (a,c,d) when ``split_row(j)`` is true.  Interior nodes move by a
    seeded uniform +-``jitter`` fraction of the smaller adjacent spacing in each
    direction (``isotropic``: of the smaller of the two directions' spacings, in both).
    """
    ny, nx = X.shape[0] - 1, X.shape[1] - 1
    X = X.astype(np.float64).copy()
    Y = Y.astype(np.float64).copy()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        dxl = np.minimum(X[1:-1, 2:] - X[1:-1, 1:-1], X[1:-1, 1:-1] - X[1:-1, :-2])
        dyl = np.minimum(Y[2:, 1:-1] - Y[1:-1, 1:-1], Y[1:-1, 1:-1] - Y[:-2, 1:-1])
        ux = rng.uniform(-1.0, 1.0, size=dxl.shape)
        uy = rng.uniform(-1.0, 1.0, size=dyl.shape)
        if isotropic:
            dxl = dyl = np.minimum(dxl, dyl)
        X[1:-1, 1:-1] += jitter * dxl * ux
        Y[1:-1, 1:-1] += jitter * dyl * uy
    nodes = np.stack([X.ravel(), Y.ravel()], axis=1)

    def nid(i, j):
        return j * (nx + 1) + i

    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    a = nid(ii, jj)
    b = nid(ii + 1, jj)
    c = nid(ii + 1, jj + 1)
    d = nid(ii, jj + 1)
    split = np.array([bool(split_row(j)) for j in range(ny)])
    cells = []
    for j in range(ny):
        if split[j]:
            t1 = np.stack([a[j], b[j], c[j], np.full(nx, -1)], axis=1)
            t2 = np.stack([a[j], c[j], d[j], np.full(nx, -1)], axis=1)
            rows = np.empty((2 * nx, 4), dtype=np.int64)
            rows[0::2] = t1
            rows[1::2] = t2
        else:
            rows = np.stack([a[j], b[j], c[j], d[j]], axis=1)
        cells.append(rows)
    cells = np.concatenate(cells).astype(np.int32)

    bed = []
    for i in range(nx):  # bottom
        n1, n2 = nid(i, 0), nid(i + 1, 0)
        bed.append((n1, n2, tag_of_edge("bottom", 0.5 * (X[0, i] + X[0, i + 1]))))
    for j in range(ny):  # right
        n1, n2 = nid(nx, j), nid(nx, j + 1)
        bed.append((n1, n2, tag_of_edge("right", 0.5 * (Y[j, nx] + Y[j + 1, nx]))))
    for i in range(nx):  # top
        n1, n2 = nid(i, ny), nid(i + 1, ny)
        bed.append((n1, n2, tag_of_edge("top", 0.5 * (X[ny, i] + X[ny, i + 1]))))
    for j in range(ny):  # left
        n1, n2 = nid(0, j), nid(0, j + 1)
        bed.append((n1, n2, tag_of_edge("left", 0.5 * (Y[j, 0] + Y[j + 1, 0]))))
    return MeshSpec(name, nodes, cells, np.asarray(bed, dtype=np.int32))


def _wall_following(xs: np.ndarray, eta: np.ndarray, bottom, top: float):
    X = np.broadcast_to(xs[None, :], (eta.size, xs.size)).copy()
    yb = bottom(xs)[None, :]
    Y = yb + (top - yb) * eta[:, None]
    return X, Y


def wedge(nx: int = 120, ny: int = 80, jitter: float = 0.10, seed: int = 0) -> MeshSpec:
    """15 degree compression ramp from x=0.5 in a 1.5 x 1.0 box, quads split in two.
    Tags as mesh/supersonic_wedge_flow: left and top 1 (frozen free stream), right 2
    (extrapolation), bottom and ramp 3 (slip wall)."""
    t15 = math.tan(math.radians(15.0))
    xs = np.linspace(0.0, 1.5, nx + 1)
    X, Y = _wall_following(xs, np.linspace(0.0, 1.0, ny + 1),
                           lambda x: np.where(x > 0.5, (x - 0.5) * t15, 0.0), 1.0)

    def tag(side, s):
        return {"bottom": TAG_SLIP, "right": TAG_OUTLET}.get(side, TAG_INLET)

    return _structured(f"wedge_{nx}x{ny}", X, Y, lambda j: True, tag, jitter, seed)


def laminar_plate(nx: int = 240, ny: int = 120, ratio: float = 1.08, lead: float = 0.2,
                  length: float = 1.0, height: float = 0.5) -> MeshSpec:
    """Flat plate from x=0 with a symmetry lead-in; tags as mesh/new_laminar_flat_plate:
    1 inlet (left), 2 outlet (right), 3 slip lead-in, 4 no-slip plate, 5 far field (top)."""
    xs = np.linspace(-lead, length, nx + 1)
    X, Y = _wall_following(xs, _geometric(ny, height, ratio), lambda x: 0.0 * x, height)

    def tag(side, s):
        if side == "bottom":
            return TAG_NOSLIP if s > 0.0 else TAG_SLIP
        return {"left": TAG_INLET, "right": TAG_OUTLET, "top": TAG_FARFIELD}[side]

    return _structured(f"laminar_plate_{nx}x{ny}", X, Y, lambda j: False, tag)


def turb_plate(nx: int = 480, ny: int = 240, ratio: float = 1.12, lead: float = 0.4,
               length: float = 2.0, height: float = 1.0, reynolds_per_m: float = 5e6) -> MeshSpec:
    """Turbulent plate: first wall spacing from y+ = 0.5 with a flat-plate skin-friction
    estimate at x = 1, growth ``ratio`` capped so the grid fills ``height``."""
    cf = 0.0576 * reynolds_per_m ** -0.2
    first = 0.5 / (reynolds_per_m * math.sqrt(0.5 * cf))
    xs = np.linspace(-lead, length, nx + 1)
    X, Y = _wall_following(xs, _capped_geometric(ny, height, first, ratio),
                           lambda x: 0.0 * x, height)

    def tag(side, s):
        if side == "bottom":
            return TAG_NOSLIP if s > 0.0 else TAG_SLIP
        return {"left": TAG_INLET, "right": TAG_OUTLET, "top": TAG_FARFIELD}[side]

    return _structured(f"turb_plate_{nx}x{ny}", X, Y, lambda j: False, tag)


def swbli(nx: int = 800, ny: int = 640, length: float = 1.0, height: float = 0.4,
          reynolds_per_m: float = 1e7, jitter: float = 0.05, seed: int = 0) -> MeshSpec:
    """Shock/boundary-layer interaction box: no-slip wall from x=0.1 (slip lead-in),
    free-stream inlet (1), extrapolation outlet (2), the top boundary carries the
    post-shock state of an 8 degree deflection (6).  Rows in the outer half are split.
    Interior nodes move by +-``jitter`` of the smaller local spacing in both directions."""
    cf = 0.0576 * reynolds_per_m ** -0.2
    first = 0.5 / (reynolds_per_m * math.sqrt(0.5 * cf))
    xs = np.linspace(0.0, length, nx + 1)
    X, Y = _wall_following(xs, _capped_geometric(ny, height, first, 1.05),
                           lambda x: 0.0 * x, height)

    def tag(side, s):
        if side == "bottom":
            return TAG_NOSLIP if s > 0.1 * length else TAG_SLIP
        return {"left": TAG_INLET, "right": TAG_OUTLET, "top": TAG_SHOCK_INFLOW}[side]

    return _structured(f"swbli_{nx}x{ny}", X, Y, lambda j: j >= ny // 2, tag, jitter, seed, isotropic=True)


def bump(n_target: int = 64_000, jitter: float = 0.10, seed: int = 0,
         height: float = 0.05, width: float = 0.2) -> MeshSpec:
    """3 x 1 channel, bump y = h exp(-(x/w)^2); tags as mesh/bump_1230.geo:
    1 inlet (left), 2 outlet (right), 3 walls (top and bottom)."""
    ny = int(round(math.sqrt(n_target / 6.0)))
    nx = 3 * ny
    xs = np.linspace(-1.5, 1.5, nx + 1)
    X, Y = _wall_following(xs, np.linspace(0.0, 1.0, ny + 1),
                           lambda x: height * np.exp(-(x / width) ** 2), 1.0)

    def tag(side, s):
        return {"left": TAG_INLET, "right": TAG_OUTLET}.get(side, TAG_SLIP)

    return _structured(f"bump_{2 * nx * ny}", X, Y, lambda j: True, tag, jitter, seed)


def box(nx: int = 3, ny: int = 2, split: bool = False, jitter: float = 0.0, seed: int = 0,
        tags=(TAG_SLIP, TAG_OUTLET, TAG_SLIP, TAG_INLET)) -> MeshSpec:
    """Unit box for small known-answer cases; ``tags`` = (bottom, right, top, left)."""
    X, Y = np.meshgrid(np.linspace(0.0, 1.0, nx + 1), np.linspace(0.0, 1.0, ny + 1))
    names = ("bottom", "right", "top", "left")
    return _structured(f"box_{nx}x{ny}{'t' if split else 'q'}", X, Y, lambda j: split,
                       lambda side, s: tags[names.index(side)], jitter, seed)


def mixed_box(nx: int = 6, ny: int = 4, jitter: float = 0.1, seed: int = 1) -> MeshSpec:
    """Unit box whose upper half is triangles and lower half quads."""
    X, Y = np.meshgrid(np.linspace(0.0, 1.0, nx + 1), np.linspace(0.0, 1.0, ny + 1))
    return _structured(f"mixed_{nx}x{ny}", X, Y, lambda j: j >= ny // 2,
                       lambda side, s: {"left": TAG_INLET, "right": TAG_OUTLET}.get(side, TAG_SLIP),
                       jitter, seed)


WORKLOADS = {
    "wedge": wedge,
    "laminar_plate": laminar_plate,
    "turb_plate": turb_plate,
    "swbli": swbli,
    "bump": bump,
}


def write_gmsh(spec: MeshSpec, path: str, crlf: bool = False) -> None:
    """Gmsh 2.2 ASCII writer (1-based ids; physical tag first, elementary tag second)."""
    nl = "\r\n" if crlf else "\n"
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(spec.n_nodes)]
    out += [f"{i + 1} {x:.17g} {y:.17g} 0" for i, (x, y) in enumerate(spec.nodes)]
    out += ["$EndNodes", "$Elements", str(spec.bedges.shape[0] + spec.n_cells)]
    eid = 1
    for a, b, t in spec.bedges:
        out.append(f"{eid} 1 2 {t} {t} {a + 1} {b + 1}")
        eid += 1
    for c in spec.cells:
        if c[3] < 0:
            out.append(f"{eid} 2 2 100 1 {c[0] + 1} {c[1] + 1} {c[2] + 1}")
        else:
            out.append(f"{eid} 3 2 100 1 {c[0] + 1} {c[1] + 1} {c[2] + 1} {c[3] + 1}")
        eid += 1
    out += ["$EndElements", ""]
    with open(path, "w", newline="") as fh:
        fh.write(nl.join(out))


def read_gmsh(path: str) -> MeshSpec:
    """Minimal Gmsh 2.2 reader (tolerates CRLF) used to feed reference meshes to tests."""
    with open(path, "r", newline="") as fh:
        lines = [l.rstrip("\r\n").rstrip("\r") for l in fh]
    k = lines.index("$Nodes")
    n = int(lines[k + 1])
    ids, xy = [], []
    for l in lines[k + 2:k + 2 + n]:
        p = l.split()
        ids.append(int(p[0]))
        xy.append((float(p[1]), float(p[2])))
    remap = {nid: i for i, nid in enumerate(ids)}
    k = lines.index("$Elements")
    m = int(lines[k + 1])
    cells, bed = [], []
    for l in lines[k + 2:k + 2 + m]:
        p = list(map(int, l.split()))
        typ, ntag = p[1], p[2]
        tag = p[3] if ntag > 0 else 0
        v = [remap[q] for q in p[3 + ntag:]]
        if typ == 1:
            bed.append((v[0], v[1], tag))
        elif typ == 2:
            cells.append((v[0], v[1], v[2], -1))
        elif typ == 3:
            cells.append(tuple(v[:4]))
    return MeshSpec(path, np.asarray(xy, dtype=np.float64), np.asarray(cells, dtype=np.int32),
                    np.asarray(bed, dtype=np.int32).reshape(-1, 3))


def smooth_perturbation(spec_cells_xy: np.ndarray, seed: int, amplitude: float = 0.05) -> np.ndarray:
    """Seeded smooth field in [-amplitude, amplitude] per cell for 4 primitives (rho,u,v,p):
    a sum of three random low-wavenumber sine modes per variable."""
    rng = np.random.default_rng(seed)
    x, y = spec_cells_xy[:, 0], spec_cells_xy[:, 1]
    out = np.zeros((x.size, 4))
    for v in range(4):
        acc = np.zeros_like(x)
        for _ in range(3):
            kx, ky = rng.uniform(0.5, 4.0, size=2)
            ph = rng.uniform(0, 2 * math.pi)
            acc += np.sin(2 * math.pi * (kx * x + ky * y) + ph)
        out[:, v] = amplitude * acc / 3.0
    return out
