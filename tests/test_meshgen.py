"""Synthetic meshes against the reference preprocessor's geometry definitions
(tools/pyMeshFV3D/pymeshfv3d/utilities/geometry.py, process.py:47-78)."""
import numpy as np
import pytest

from conftest import reference_tree_present
from fv3d_gb300 import meshgen as mg


def test_sizes_match_configs():
    m = mg.periodic_hex_box(4)
    assert (m.n_cells, m.n_faces, m.n_boundaries) == (64, 192, 0)
    m = mg.periodic_tet_box(3)
    assert (m.n_cells, m.n_faces) == (162, 324)
    m = mg.channel(8, 4, 4)
    assert m.n_boundaries == 2 * 4 * 4 + 2 * 8 * 4
    assert m.n_faces == 9 * 4 * 4 + 8 * 5 * 4 + 8 * 4 * 4


@pytest.mark.parametrize("maker,closure", [
    # non-planar quads: the reference's area (two triangles) and normal
    # (diagonal cross product) are not exactly consistent, so cells close
    # only to O(jitter^2)
    (lambda: mg.periodic_hex_box(4, 2 * np.pi, jitter=0.1, seed=7), 2e-2),
    (lambda: mg.periodic_tet_box(3), 1e-12),
    (lambda: mg.channel(6, 4, 4), 1e-12),
])
def test_mesh_invariants(maker, closure):
    m = maker()
    # closed cells: sum_f n A (outward) = 0
    s = np.zeros((m.n_cells, 3))
    for k in range(m.max_cell_faces):
        f = m.cell_faces[:, k]
        ok = f >= 0
        sign = np.where(m.face_cells[f[ok], 0] == np.nonzero(ok)[0], 1.0, -1.0)
        s[ok] += sign[:, None] * m.face_n[f[ok]] * m.face_area[f[ok], None]
    assert np.abs(s).max() < closure * max(1.0, m.face_area.max())
    # face lists ascending, each interior face in two lists
    for i in range(m.n_cells):
        fl = m.cell_faces[i, : m.cell_n_faces[i]]
        assert np.all(np.diff(fl) > 0)
    assert np.all((m.face_lambda > 0) & (m.face_lambda <= 1))
    assert np.all(np.abs(np.linalg.norm(m.face_n, axis=1) - 1) < 1e-14)
    # normal points from cell 0 to cell 1 (periodic image)
    inter = m.face_cells[:, 1] >= 0
    d = -m.face_dist_cell_2[inter] + (m.face_x[inter] - m.cell_x[m.face_cells[inter, 0]])
    assert np.all(np.einsum("ij,ij->i", d, m.face_n[inter]) > 0)


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
def test_geometry_matches_reference_preprocessor():
    import refgeom
    element, geometry = refgeom.load()
    ET = element.ElementType
    m = mg.periodic_hex_box(3, 2 * np.pi, jitter=0.1, seed=3)
    xs = np.linspace(0.0, 2 * np.pi, 4)
    nodes, cn, sh = mg._structured(3, 3, 3, xs, xs, xs, (True, True, True), 0.1, 3,
                                   (2 * np.pi,) * 3)
    # cells
    for c in range(m.n_cells):
        v = nodes[cn[c]] + sh[c]
        cell = element.Cell(ET.HEXAEDER, list(range(8)), 0)
        assert abs(geometry.calc_volume(v, cell) - m.cell_volume[c]) < 1e-13
        assert np.allclose(v.mean(axis=0), m.cell_x[c], rtol=0, atol=1e-14)
    # faces: rebuild each face's vertices from cell 0's frame
    lf = mg.HEX_FACES
    for f in range(m.n_faces):
        c0, c1 = m.face_cells[f]
        v0 = nodes[cn[c0]] + sh[c0]
        # find the local face of c0 whose centre is this face's centre
        cands = [k for k in range(6) if np.allclose(v0[lf[k]].mean(axis=0), m.face_x[f], atol=1e-12)]
        assert len(cands) == 1
        fv = v0[lf[cands[0]]]
        face = element.Face(ET.QUADRANGLE, list(range(4)))
        face.cell_ids = [0, 1]
        x_c1 = m.face_x[f] - m.face_dist_cell_2[f]
        cells = [types_cell(m.cell_x[c0]), types_cell(x_c1)]
        face.x_v = fv.mean(axis=0)
        face.area = geometry.calc_area(fv, face)
        face.n_v = geometry.calc_normal(fv, cells, face)
        face.t1_v = geometry.calc_t1(face)
        face.t2_v = geometry.calc_t2(face)
        face.weight = geometry.calc_weight(cells, face)
        assert abs(face.area - m.face_area[f]) < 1e-13
        assert np.allclose(face.n_v, m.face_n[f], atol=1e-14)
        assert np.allclose(face.t1_v, m.face_t1[f], atol=1e-14)
        assert np.allclose(face.t2_v, m.face_t2[f], atol=1e-14)
        assert abs(face.weight - m.face_lambda[f]) < 1e-13


class types_cell:
    def __init__(self, x):
        self.x_v = np.asarray(x)


def test_mixed_element_geometry():
    """Prism and pyramid geometry (geometry.py:86-103) on the mixed box: with
    planar faces every cell closes (sum of outward n A = 0) and the volumes
    tile the box; the pyramids of a split hex add up to the hex."""
    m = mg.mixed_box(5)
    assert m.n_boundaries == 0 and sorted(set(m.cell_n_faces.tolist())) == [5, 6]
    s = np.zeros((m.n_cells, 3))
    np.add.at(s, m.face_cells[:, 0], m.face_n * m.face_area[:, None])
    np.add.at(s, m.face_cells[:, 1], -(m.face_n * m.face_area[:, None]))
    assert np.abs(s).max() < 1e-15
    assert abs(m.cell_volume.sum() - 1.0) < 1e-14
    assert np.all((m.face_lambda > 0) & (m.face_lambda < 1))
    h = 1.0 / 5
    pyr = m.cell_n_faces == 5
    assert np.allclose(m.cell_volume[pyr].reshape(-1), np.where(np.isclose(m.cell_volume[pyr], h ** 3 / 6),
                                                                 h ** 3 / 6, h ** 3 / 2))
