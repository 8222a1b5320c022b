"""Synthetic unstructured meshes in the reference's processed-mesh layout.

This plays the role of the reference's mesh preprocessor (pyMeshFV3D) for the
generated benchmark meshes: it produces the arrays that
``read_mesh_file`` (Solver/src/mesh/mesh.c:121-630) would load from the HDF5
file that ``write_mesh`` (tools/pyMeshFV3D/pymeshfv3d/write.py:19-201) writes.

Geometry follows tools/pyMeshFV3D/pymeshfv3d/utilities/geometry.py:
  * cell centre = vertex mean, volume = the tetrahedral decompositions of
    :50-116 (hex 5, prism 3, pyramid 2, tet 1)
  * face centre = vertex mean, area = two-triangle (quad) / triangle (:15-47)
  * normal = normalised cross product of the diagonals (quad) / edges
    (triangle), flipped to point away from cell 0 (:152-183)
  * t1, t2 from the normal (:186-200)
  * interpolation weight lambda = d1 / (d1 + d2), 1 on boundaries (:133-149)
  * cell dx = sum over the cell's faces of |n| * area (process.py:73-77)
Face numbering follows process.py:96-142: faces are numbered in order of first
appearance while walking cells in order and each cell's local faces in the
element table order (utilities/element.py:80-103); a face takes its vertex
order and cell 0 from its first appearance, and each cell's face list is in
ascending face id.

New relative to the reference (which has no periodic faces): periodic faces
are ordinary interior faces between wrapped cells; their second cell's centre
is taken at its periodic image for lambda and ``face_dist_cell_2``.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import numpy as np

# element.py:80-103 local face tables (gmsh vertex ordering)
HEX_FACES = np.array([[0, 1, 2, 3], [4, 5, 6, 7], [0, 4, 7, 3],
                      [0, 4, 5, 1], [1, 5, 6, 2], [3, 7, 6, 2]], dtype=np.int64)
TET_FACES = np.array([[0, 1, 2], [0, 3, 1], [0, 3, 2], [2, 3, 1]], dtype=np.int64)
# element.py:104-122: prism (3 quadrangles, 2 triangles), pyramid (base
# quadrangle, 4 triangles); rows of mixed width as lists.  The reference's
# pyramid table lists (v0, v3, v1) as its fifth face, a triangle inside the
# base, so the side face on the v3-v0 edge is never created and no pyramid
# closes; the side face (v0, v3, v4) is used here.
PRISM_FACES = [[0, 1, 4, 3], [1, 2, 5, 4], [0, 2, 5, 3], [0, 1, 2], [3, 4, 5]]
PYRAMID_FACES = [[0, 1, 2, 3], [0, 1, 4], [1, 2, 4], [2, 3, 4], [0, 3, 4]]
# element kinds: vertices and local faces, in gmsh vertex order
KINDS = {"tet": (4, TET_FACES.tolist()), "pyramid": (5, PYRAMID_FACES),
         "prism": (6, PRISM_FACES), "hex": (8, HEX_FACES.tolist())}

# Kuhn split of a hex (gmsh ordering) into 6 tets along the v0-v6 diagonal;
# translation invariant, hence conforming between neighbours and across
# periodic wraps.
KUHN_TETS = np.array([[0, 1, 2, 6], [0, 1, 5, 6], [0, 3, 2, 6],
                      [0, 3, 7, 6], [0, 4, 5, 6], [0, 4, 7, 6]], dtype=np.int64)

# region / boundary-condition type codes (navier_stokes_module.h:47-59 order)
BC_FLOW, BC_INFLOW, BC_OUTFLOW, BC_WALL_ADIABATIC = 0, 1, 2, 3
BC_WALL_ISOTHERMAL, BC_WALL_SLIP, BC_SYMMETRY, BC_STATE, BC_FUNCTION = 4, 5, 6, 7, 8
BC_PRESSURE_OUTLET = 9  # new: no reference counterpart


@dataclass
class Mesh:
    """Processed mesh arrays in the reference's Mesh_t layout (solver_type.h:22-168)."""
    cell_x: np.ndarray          # (n_cells, 3)
    cell_volume: np.ndarray     # (n_cells,)
    cell_dx: np.ndarray         # (n_cells, 3)
    cell_n_faces: np.ndarray    # (n_cells,) int32
    cell_faces: np.ndarray      # (n_cells, max_cell_faces) int32, -1 padded
    face_cells: np.ndarray      # (n_faces, 2) int32, [:,1] = -1 on boundary faces
    face_boundary: np.ndarray   # (n_faces,) int32, -1 interior else boundary id
    face_area: np.ndarray
    face_lambda: np.ndarray
    face_x: np.ndarray
    face_n: np.ndarray
    face_t1: np.ndarray
    face_t2: np.ndarray
    face_dist_cell_2: np.ndarray  # (n_faces, 3): x_f - x_c1 (periodic image)
    boundary_id: np.ndarray     # (n_boundaries,) region id
    boundary_face: np.ndarray   # (n_boundaries,) face id
    region_names: list = field(default_factory=list)
    region_is_boundary: np.ndarray = None
    name: str = "mesh"

    @property
    def n_cells(self) -> int:
        return int(self.cell_x.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.face_x.shape[0])

    @property
    def n_boundaries(self) -> int:
        return int(self.boundary_id.shape[0])

    @property
    def max_cell_faces(self) -> int:
        return int(self.cell_faces.shape[1])

    @property
    def n_regions(self) -> int:
        return len(self.region_names)

    def arrays(self) -> dict:
        """Contiguous arrays with the dtypes the C interfaces expect."""
        f8 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        i4 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        return dict(
            cell_x=f8(self.cell_x), cell_volume=f8(self.cell_volume), cell_dx=f8(self.cell_dx),
            cell_n_faces=i4(self.cell_n_faces), cell_faces=i4(self.cell_faces),
            face_cells=i4(self.face_cells), face_boundary=i4(self.face_boundary),
            face_area=f8(self.face_area), face_lambda=f8(self.face_lambda),
            face_x=f8(self.face_x), face_n=f8(self.face_n), face_t1=f8(self.face_t1),
            face_t2=f8(self.face_t2), face_dist_cell_2=f8(self.face_dist_cell_2),
            boundary_id=i4(self.boundary_id), boundary_face=i4(self.boundary_face),
            region_is_boundary=i4(self.region_is_boundary))


# ---------------------------------------------------------------------------
# geometry primitives (geometry.py / math.py restated, vectorised)
# ---------------------------------------------------------------------------
def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _len(a):
    return np.sqrt(_dot(a, a))


def _norm(a):
    return a / _len(a)[..., None]


def _mean_vertices(v):
    s = v[..., 0, :]
    for k in range(1, v.shape[-2]):
        s = s + v[..., k, :]
    return s / v.shape[-2]


def _hex_volume(v):
    """geometry.py:74-85 (five tetrahedra of a gmsh-ordered hex)."""
    def tet(a, b, c, d):
        return np.abs(_dot(v[:, a] - v[:, d], _cross(v[:, b] - v[:, d], v[:, c] - v[:, d])))
    vol = tet(5, 1, 6, 4)
    vol = vol + np.abs(_dot(v[:, 1] - v[:, 4], _cross(v[:, 3] - v[:, 4], v[:, 6] - v[:, 4])))
    vol = vol + np.abs(_dot(v[:, 1] - v[:, 4], _cross(v[:, 0] - v[:, 4], v[:, 3] - v[:, 4])))
    vol = vol + np.abs(_dot(v[:, 6] - v[:, 4], _cross(v[:, 3] - v[:, 4], v[:, 7] - v[:, 4])))
    vol = vol + np.abs(_dot(v[:, 3] - v[:, 1], _cross(v[:, 6] - v[:, 1], v[:, 2] - v[:, 1])))
    return vol * (1.0 / 6.0)


def _tet_volume(v):
    """geometry.py:104-109."""
    a = v[:, 1] - v[:, 0]
    b = v[:, 2] - v[:, 0]
    c = v[:, 3] - v[:, 0]
    return np.abs(_dot(a, _cross(b, c))) * (1.0 / 6.0)


def _prism_volume(v):
    """geometry.py:86-95 (three tetrahedra from vertex 0)."""
    a, b, c, d, e = (v[:, k] - v[:, 0] for k in range(1, 6))
    vol = np.abs(_dot(a, _cross(b, e)))
    vol = vol + np.abs(_dot(a, _cross(e, d)))
    vol = vol + np.abs(_dot(d, _cross(e, c)))
    return vol * (1.0 / 6.0)


def _pyramid_volume(v):
    """geometry.py:96-103 (two tetrahedra on the base diagonal)."""
    a, b, c, d = (v[:, k] - v[:, 0] for k in range(1, 5))
    vol = np.abs(_dot(a, _cross(b, d)))
    vol = vol + np.abs(_dot(b, _cross(c, d)))
    return vol * (1.0 / 6.0)


_VOLUME = {"tet": _tet_volume, "pyramid": _pyramid_volume, "prism": _prism_volume, "hex": _hex_volume}


def _face_area_normal(v):
    """geometry.py:29-40 (area) and :165-172 (normal, before orientation)."""
    if v.shape[1] == 4:
        a = v[:, 1] - v[:, 0]
        b = v[:, 2] - v[:, 0]
        c = v[:, 3] - v[:, 0]
        area = (_len(_cross(a, b)) + _len(_cross(b, c))) * 0.5
        n = _norm(_cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 1]))
    else:
        a = v[:, 1] - v[:, 0]
        b = v[:, 2] - v[:, 0]
        area = _len(_cross(a, b)) * 0.5
        n = _norm(_cross(a, b))
    return area, n


def _tangents(n):
    """geometry.py:186-200."""
    n0, n1, n2 = n[:, 0], n[:, 1], n[:, 2]
    z = np.zeros_like(n0)
    pick = np.abs(n0) > np.abs(n1)
    t1 = np.where(pick[:, None], np.stack([-n2, z, n0], axis=1), np.stack([z, -n2, n1], axis=1))
    t1 = _norm(t1)
    t2 = _norm(_cross(t1, n))
    return t1, t2


# ---------------------------------------------------------------------------
# generic builder: cells (node ids + per-vertex periodic shifts) -> Mesh
# ---------------------------------------------------------------------------
def build_mesh(nodes, cell_nodes, cell_shift, cell_type, boundary_region_of_face=None,
               region_names=("flow",), region_is_boundary=(0,), name="mesh", boundary_region_of_nodes=None):
    """Assemble a processed mesh.

    nodes:       (n_nodes, 3) unique node coordinates
    cell_nodes:  (n_cells, nv) node ids in gmsh element order (rows of a
                 mixed mesh padded with -1 to its widest element)
    cell_shift:  (n_cells, nv, 3) translation added to each vertex (periodic
                 unwrapping), zeros for non-periodic meshes
    cell_type:   "hex", "tet", "prism" or "pyramid", or one of those per cell
    boundary_region_of_face: callable(face_x (m,3), face_n (m,3)) -> region ids
                 for the unmatched (boundary) faces
    boundary_region_of_nodes: alternatively callable(face node ids (m, fv),
                 each row sorted; with faces of 3 and 4 nodes, triangles
                 carry a leading -1) -> region ids
    """
    cell_nodes = np.asarray(cell_nodes, dtype=np.int64)
    n_cells = cell_nodes.shape[0]
    kinds = np.full(n_cells, cell_type, dtype=object) if isinstance(cell_type, str) else np.asarray(cell_type, dtype=object)
    if kinds.shape != (n_cells,) or not set(kinds.tolist()) <= set(KINDS):
        raise ValueError(f"cell kinds must be among {sorted(KINDS)}")
    # per kind: vertex means and volumes; local faces in tmp_faces order
    # (cell-major, element-table order), rows padded to 4 nodes
    nfl = np.array([len(KINDS[k][1]) for k in kinds], dtype=np.int64)
    lf_start = np.concatenate([[0], np.cumsum(nfl)[:-1]])
    n_lf = int(nfl.sum())
    cell_x = np.zeros((n_cells, 3))
    cell_volume = np.zeros(n_cells)
    lf_nodes = np.full((n_lf, 4), -1, dtype=np.int64)
    lf_nv = np.zeros(n_lf, dtype=np.int64)
    lf_verts = np.zeros((n_lf, 4, 3))
    lf_shift = np.zeros((n_lf, 4, 3))
    lf_cell = np.repeat(np.arange(n_cells, dtype=np.int64), nfl)
    for kind, (nv, table) in KINDS.items():
        sel = np.nonzero(kinds == kind)[0]
        if sel.shape[0] == 0:
            continue
        cn = cell_nodes[sel, :nv]
        verts = nodes[cn] + cell_shift[sel, :nv]               # unwrapped vertices
        cell_x[sel] = _mean_vertices(verts)
        cell_volume[sel] = _VOLUME[kind](verts)
        for j, face in enumerate(table):
            rows = lf_start[sel] + j
            w = len(face)
            lf_nodes[rows, :w] = cn[:, face]
            lf_nv[rows] = w
            lf_verts[rows, :w] = verts[:, face]
            lf_shift[rows, :w] = cell_shift[sel][:, face]
    fw = 4 if np.any(lf_nv == 4) else 3                         # face width of the mesh
    if np.all(lf_nv == fw):
        lf_nodes, lf_verts, lf_shift = lf_nodes[:, :fw], lf_verts[:, :fw], lf_shift[:, :fw]
    key_nodes = np.sort(lf_nodes, axis=1)                       # triangles: leading -1
    order = np.lexsort(tuple(key_nodes[:, k] for k in range(key_nodes.shape[1] - 1, -1, -1)))
    ks = key_nodes[order]
    same_next = np.zeros(ks.shape[0], dtype=bool)
    same_next[:-1] = np.all(ks[1:] == ks[:-1], axis=1)
    if np.any(same_next[:-1] & same_next[1:]):
        raise ValueError("a face is shared by more than two cells")
    first = np.ones(ks.shape[0], dtype=bool)
    first[1:] = ~same_next[:-1]                                  # start of a key group
    grp_first = order[first]                                     # first appearance index
    has_pair = same_next[first]
    grp_second = np.full(grp_first.shape[0], -1, dtype=np.int64)
    idx_first = np.nonzero(first)[0]
    grp_second[has_pair] = order[idx_first[has_pair] + 1]
    # face numbering = order of first appearance (process.py:106-134)
    fo = np.argsort(grp_first, kind="stable")
    f_first = grp_first[fo]
    f_second = grp_second[fo]
    n_faces = f_first.shape[0]

    c0 = lf_cell[f_first]
    c1 = np.where(f_second >= 0, lf_cell[np.maximum(f_second, 0)], -1)
    fverts = lf_verts[f_first]
    fnv = lf_nv[f_first]
    face_x = np.zeros((n_faces, 3))
    face_area = np.zeros(n_faces)
    n = np.zeros((n_faces, 3))
    for w in (3, 4):
        sel = np.nonzero(fnv == w)[0]
        if sel.shape[0]:
            face_x[sel] = _mean_vertices(fverts[sel, :w])
            face_area[sel], n[sel] = _face_area_normal(fverts[sel, :w])
    d = face_x - cell_x[c0]
    cos_angle = _dot(d, n) / (_len(d) * _len(n))
    angle = np.arccos(np.clip(cos_angle, -1.0, 1.0)) * 180 / np.pi
    flip = (angle > 90.0) & (angle < 270.0)
    n = np.where(flip[:, None], -n, n)
    t1, t2 = _tangents(n)

    # periodic image of cell 1: shift that maps its face vertices onto cell 0's
    interior = c1 >= 0
    shift = np.zeros((n_faces, 3))
    if np.any(interior):
        # exact lattice vector: the same node seen from cell 0 and from cell 1
        fi = np.nonzero(interior)[0]
        node0 = lf_nodes[f_first[fi], 0]
        pos = np.argmax(lf_nodes[f_second[fi]] == node0[:, None], axis=1)
        shift[fi] = lf_shift[f_first[fi], 0] - lf_shift[f_second[fi], pos]
    x_c1 = np.zeros((n_faces, 3))
    x_c1[interior] = cell_x[c1[interior]] + shift[interior]
    d1 = _dot(n, face_x - cell_x[c0]) / face_area
    d2 = _dot(n, x_c1 - face_x) / face_area
    lam = np.ones(n_faces)
    lam[interior] = d1[interior] / (d1[interior] + d2[interior])
    if np.any(lam[interior] <= 0.0) or np.any(lam[interior] >= 1.0):
        raise ValueError("degenerate interpolation weight")
    dist2 = np.zeros((n_faces, 3))
    dist2[interior] = face_x[interior] - x_c1[interior]

    # cell face lists (ascending face id) and dx
    fid = np.arange(n_faces, dtype=np.int64)
    owner = np.concatenate([c0, c1[interior]])
    ofid = np.concatenate([fid, fid[interior]])
    o = np.lexsort((ofid, owner))
    owner, ofid = owner[o], ofid[o]
    counts = np.bincount(owner, minlength=n_cells)
    mcf = int(counts.max())
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    slot = np.arange(owner.shape[0]) - starts[owner]
    cell_faces = np.full((n_cells, mcf), -1, dtype=np.int64)
    cell_faces[owner, slot] = ofid
    cell_dx = np.zeros((n_cells, 3))
    contrib = np.abs(n) * face_area[:, None]
    for s in range(mcf):                          # summed in face-list order
        has = cell_faces[:, s] >= 0
        cell_dx[has] = cell_dx[has] + contrib[cell_faces[has, s]]

    # boundaries: one per boundary face, in face order
    bfaces = np.nonzero(~interior)[0]
    face_boundary = np.full(n_faces, -1, dtype=np.int64)
    face_boundary[bfaces] = np.arange(bfaces.shape[0])
    if bfaces.shape[0] > 0:
        if boundary_region_of_nodes is not None:
            boundary_id = np.asarray(boundary_region_of_nodes(np.sort(lf_nodes[f_first[bfaces]], axis=1)),
                                     dtype=np.int64)
        elif boundary_region_of_face is not None:
            boundary_id = np.asarray(boundary_region_of_face(face_x[bfaces], n[bfaces]), dtype=np.int64)
        else:
            raise ValueError("mesh has boundary faces but no boundary regions")
    else:
        boundary_id = np.zeros(0, dtype=np.int64)

    return Mesh(cell_x=cell_x, cell_volume=cell_volume, cell_dx=cell_dx,
                cell_n_faces=counts.astype(np.int32), cell_faces=cell_faces.astype(np.int32),
                face_cells=np.stack([c0, c1], axis=1).astype(np.int32),
                face_boundary=face_boundary.astype(np.int32), face_area=face_area,
                face_lambda=lam, face_x=face_x, face_n=n, face_t1=t1, face_t2=t2,
                face_dist_cell_2=dist2, boundary_id=boundary_id.astype(np.int32),
                boundary_face=bfaces.astype(np.int32), region_names=list(region_names),
                region_is_boundary=np.asarray(region_is_boundary, dtype=np.int32), name=name)


def _structured(nx, ny, nz, xs, ys, zs, periodic, jitter=0.0, seed=0, lengths=None):
    """Node array + hex connectivity (gmsh order) + per-vertex periodic shifts."""
    px, py, pz = periodic
    mx, my, mz = nx + (0 if px else 1), ny + (0 if py else 1), nz + (0 if pz else 1)
    X, Y, Z = np.meshgrid(xs[:mx], ys[:my], zs[:mz], indexing="ij")
    nodes = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)        # node id = (i*my + j)*mz + k
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hx = np.diff(xs).min(); hy = np.diff(ys).min(); hz = np.diff(zs).min()
        jit = rng.uniform(-jitter, jitter, size=nodes.shape) * np.array([hx, hy, hz])
        ii, jj, kk = np.meshgrid(np.arange(mx), np.arange(my), np.arange(mz), indexing="ij")
        fixed = np.zeros((mx, my, mz, 3), dtype=bool)   # keep non-periodic walls planar
        if not px:
            fixed[[0, -1], :, :, 0] = True
        if not py:
            fixed[:, [0, -1], :, 1] = True
        if not pz:
            fixed[:, :, [0, -1], 2] = True
        jit[fixed.reshape(-1, 3)] = 0.0
        nodes = nodes + jit
    Lx, Ly, Lz = lengths
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # cell id = i + nx*(j + ny*k): x fastest
    i = i.transpose(2, 1, 0).reshape(-1); j = j.transpose(2, 1, 0).reshape(-1)
    k = k.transpose(2, 1, 0).reshape(-1)
    off = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                    [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    vi = i[:, None] + off[None, :, 0]
    vj = j[:, None] + off[None, :, 1]
    vk = k[:, None] + off[None, :, 2]
    shift = np.zeros(vi.shape + (3,))
    if px:
        shift[..., 0] = np.where(vi == nx, Lx, 0.0); vi = vi % nx
    if py:
        shift[..., 1] = np.where(vj == ny, Ly, 0.0); vj = vj % ny
    if pz:
        shift[..., 2] = np.where(vk == nz, Lz, 0.0); vk = vk % nz
    cell_nodes = (vi * my + vj) * mz + vk
    return nodes, cell_nodes, shift


def periodic_hex_box(n, length=1.0, jitter=0.0, seed=20240601, name=None):
    """n^3 hexes on [0, length]^3, periodic on all faces; optional node jitter
    (uniform +-jitter * spacing per axis, numpy PCG64 stream of `seed`)."""
    xs = np.linspace(0.0, length, n + 1)
    nodes, cn, sh = _structured(n, n, n, xs, xs, xs, (True, True, True), jitter, seed,
                                (length, length, length))
    return build_mesh(nodes, cn, sh, "hex", name=name or f"hex{n}")


def periodic_tet_box(n, length=1.0, name=None):
    """n^3 hexes on [0, length]^3, each split into 6 Kuhn tetrahedra, periodic."""
    xs = np.linspace(0.0, length, n + 1)
    nodes, cn, sh = _structured(n, n, n, xs, xs, xs, (True, True, True), 0.0, 0,
                                (length, length, length))
    tn = cn[:, KUHN_TETS].reshape(-1, 4)
    ts = sh[:, KUHN_TETS, :].reshape(-1, 4, 3)
    return build_mesh(nodes, tn, ts, "tet", name=name or f"tet{n}")


def mixed_parts(n, length=1.0, jitter=0.0, seed=20240601, periodic=True):
    """Nodes, cells (rows padded with -1), vertex shifts and kinds of an n^3
    hex box on [0, length]^3 with two other element kinds mixed in: the
    columns (i, j) with (i + 2 j) % 5 == 0 split into two prisms per hex
    along the v0-v2 diagonal (their triangles meet only inside the column,
    across the periodic wrap too), and outside those columns every hex with
    (i + j + k) % 4 == 1 split into six pyramids on its faces around its
    vertex mean (a node of its own).  Every face matches its neighbour's:
    faces of 3 and 4 nodes, cells of 5 and 6 faces."""
    xs = np.linspace(0.0, length, n + 1)
    nodes, cn, sh = _structured(n, n, n, xs, xs, xs, (periodic,) * 3, jitter, seed, (length, length, length))
    c = np.arange(n ** 3)
    i, j, k = c % n, (c // n) % n, c // (n * n)
    prism_col = (i + 2 * j) % 5 == 0
    pyr = ~prism_col & ((i + j + k) % 4 == 1)
    rows, shifts, kinds, extra = [], [], [], []
    n0 = nodes.shape[0]
    for cell in range(n ** 3):
        v, d = cn[cell], sh[cell]
        if prism_col[cell]:
            for sub in ([0, 1, 2, 4, 5, 6], [0, 2, 3, 4, 6, 7]):
                rows.append(list(v[sub]) + [-1, -1])
                shifts.append(np.vstack([d[sub], np.zeros((2, 3))]))
                kinds.append("prism")
        elif pyr[cell]:
            apex = n0 + len(extra)
            extra.append(_mean_vertices((nodes[v] + d)[None])[0])
            for f in HEX_FACES:
                rows.append(list(v[f]) + [apex, -1, -1, -1])
                shifts.append(np.vstack([d[f], np.zeros((4, 3))]))
                kinds.append("pyramid")
        else:
            rows.append(list(v))
            shifts.append(d)
            kinds.append("hex")
    all_nodes = np.vstack([nodes, np.asarray(extra).reshape(-1, 3)])
    return all_nodes, np.asarray(rows, dtype=np.int64), np.asarray(shifts), kinds


def mixed_box(n, length=1.0, jitter=0.0, seed=20240601, periodic=True, name=None):
    """The mixed hexahedron / prism / pyramid box of ``mixed_parts``:
    periodic, or with all outer faces in region 1 ("wall")."""
    nodes, rows, shifts, kinds = mixed_parts(n, length, jitter, seed, periodic)
    if periodic:
        return build_mesh(nodes, rows, shifts, kinds, name=name or f"mixed{n}")
    return build_mesh(nodes, rows, shifts, kinds, boundary_region_of_face=lambda fx, fn: np.ones(fx.shape[0]),
                      region_names=("flow", "wall"), region_is_boundary=(0, 1), name=name or f"mixed{n}w")


def stretched_coords(n, length, ratio):
    """Two-sided geometric stretching: spacing grows by `ratio` from both walls."""
    if n % 2:
        raise ValueError("two-sided stretching needs an even cell count")
    half = n // 2
    h = np.array([ratio ** i for i in range(half)])
    h = h / h.sum() * (0.5 * length)
    hs = np.concatenate([h, h[::-1]])
    y = np.concatenate([[0.0], np.cumsum(hs)])
    y[-1] = length
    return y


def channel(nx=96, ny=48, nz=48, lx=2.0, ly=1.0, lz=1.0, ratio=1.1, name=None, tets=False):
    """Stretched-hex channel: walls at y=0 and y=ly, inflow x=0, pressure outlet
    x=lx, periodic in z.  Regions: 0 flow, 1 inflow, 2 outlet, 3 wall.
    tets=True splits every hex into 6 Kuhn tetrahedra."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = stretched_coords(ny, ly, ratio)
    zs = np.linspace(0.0, lz, nz + 1)
    nodes, cn, sh = _structured(nx, ny, nz, xs, ys, zs, (False, False, True), 0.0, 0,
                                (lx, ly, lz))
    kind = "hex"
    if tets:
        cn = cn[:, KUHN_TETS].reshape(-1, 4)
        sh = sh[:, KUHN_TETS, :].reshape(-1, 4, 3)
        kind = "tet"

    def regions(fx, fn):
        r = np.full(fx.shape[0], 3)                      # walls
        r[np.abs(fx[:, 0]) < 1e-12] = 1                  # inflow
        r[np.abs(fx[:, 0] - lx) < 1e-12] = 2             # outlet
        return r

    return build_mesh(nodes, cn, sh, kind, boundary_region_of_face=regions,
                      region_names=("flow", "inflow", "outlet", "wall"),
                      region_is_boundary=(0, 1, 1, 1),
                      name=name or f"channel{'_tet' if tets else ''}{nx}x{ny}x{nz}")


def mesh_checksum(mesh: Mesh) -> str:
    import hashlib
    h = hashlib.sha256()
    for k, v in sorted(mesh.arrays().items()):
        h.update(k.encode())
        h.update(np.ascontiguousarray(v).tobytes())
    return h.hexdigest()[:16]
