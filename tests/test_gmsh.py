"""Gmsh reader, ASCII MSH 4.1 (the reference preprocessor's format) and 2.2:
meshes written as Gmsh files in either format and read back give the same
processed mesh (faces, geometry, regions) as the in-memory generators, so
the two formats give identical meshes; the 4.1 files this module writes read
the same through the reference's own reader; unsupported inputs are
rejected."""
import os

import numpy as np
import pytest

from fv3d_gb300 import gmsh, meshgen as mg

VERSIONS = ["4.1", "2.2"]


def channel_parts(nx=6, ny=4, nz=4):
    xs = np.linspace(0, 2, nx + 1)
    ys = mg.stretched_coords(ny, 1.0, 1.1)
    zs = np.linspace(0, 1, nz + 1)
    nodes, cn, sh = mg._structured(nx, ny, nz, xs, ys, zs, (False, False, False), 0.0, 0, (2.0, 1.0, 1.0))

    def region(x):
        return 1 if abs(x[0]) < 1e-12 else (2 if abs(x[0] - 2.0) < 1e-12 else 3)

    ref = mg.build_mesh(nodes, cn, sh, "hex",
                        boundary_region_of_face=lambda fx, fn: np.array([region(x) for x in fx]),
                        region_names=("flow", "inflow", "outlet", "wall"), region_is_boundary=(0, 1, 1, 1))
    count, first = {}, {}
    for c in range(cn.shape[0]):
        for lf in mg.HEX_FACES:
            key = tuple(sorted(cn[c, lf]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, cn[c, lf])
    bnd = [(region(nodes[list(k)].mean(axis=0)), list(first[k])) for k, n in count.items() if n == 1]
    return nodes, cn, bnd, ref


@pytest.mark.parametrize("version", VERSIONS)
def test_round_trip_matches_generator(tmp_path, version):
    nodes, cn, bnd, ref = channel_parts()
    p = os.path.join(tmp_path, f"channel{version}.msh")
    gmsh.write_msh(p, nodes, cn, "hex", bnd, {(2, 1): "inflow", (2, 2): "outlet", (2, 3): "wall", (3, 4): "fluid"},
                   version=version)
    m = gmsh.read_msh(p)
    assert m.region_names == ["flow", "inflow", "outlet", "wall"]
    for f in ("face_cells", "cell_faces", "boundary_id", "boundary_face", "face_boundary"):
        assert np.array_equal(getattr(m, f), getattr(ref, f)), f
    for f in ("cell_x", "cell_volume", "cell_dx", "face_x", "face_n", "face_area", "face_lambda"):
        assert np.allclose(getattr(m, f), getattr(ref, f), rtol=0, atol=1e-14), f


def test_rejects_unsupported(tmp_path):
    for fmt in ("4.1 0 8", "3.0 0 8", "4.1 1 8"):           # no nodes; an unknown version; binary
        with pytest.raises((ValueError, KeyError)):
            gmsh.read_msh(f"$MeshFormat\n{fmt}\n$EndMeshFormat\n")
    nodes, cn, bnd, _ = channel_parts(2, 2, 2)
    p = os.path.join(tmp_path, "nophys.msh")
    gmsh.write_msh(p, nodes, cn, "hex", bnd[1:], {(2, 1): "a", (2, 2): "b", (2, 3): "c"})
    with pytest.raises(ValueError, match="no physical surface"):
        gmsh.read_msh(p)


def unwrap_to_lattice(nodes, cn, sh, dims, periodic):
    """A periodic structured mesh (unique nodes + vertex shifts, as meshgen
    builds it) as Gmsh writes one: every lattice node its own node, the
    periodic surfaces linked slave -> master."""
    nx, ny, nz = dims
    mx, my, mz = (n + (0 if p else 1) for n, p in zip(dims, periodic))
    lengths = [sh[..., a].max() for a in range(3)]
    u = cn
    k, j, i = u % mz, (u // mz) % my, u // (mz * my)
    idx = [i + np.where(sh[..., 0] != 0, nx, 0), j + np.where(sh[..., 1] != 0, ny, 0),
           k + np.where(sh[..., 2] != 0, nz, 0)]
    full = (idx[0] * (ny + 1) + idx[1]) * (nz + 1) + idx[2]
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    base = (np.minimum(I, mx - 1) * my + np.minimum(J, my - 1)) * mz + np.minimum(K, mz - 1)
    wrap = [(I == nx) & periodic[0], (J == ny) & periodic[1], (K == nz) & periodic[2]]
    base = ((np.where(wrap[0], 0, I) * my + np.where(wrap[1], 0, J)) * mz + np.where(wrap[2], 0, K))
    lat = nodes[base] + np.stack([np.where(w, L, 0.0) for w, L in zip(wrap, lengths)], axis=1)
    master_of = ((np.where(wrap[0], 0, I) * (ny + 1) + np.where(wrap[1], 0, J)) * (nz + 1)
                 + np.where(wrap[2], 0, K))
    links = [(int(a), int(b)) for a, b in zip(np.arange(lat.shape[0]), master_of) if a != b]
    return lat, full, links


def by_translation(lat, pairs):
    """Group (slave, master) pairs into links of one translation each."""
    out = {}
    for a, b in pairs:
        out.setdefault(tuple(np.round(lat[a] - lat[b], 9)), []).append((a, b))
    return list(out.values())


@pytest.mark.parametrize("version", VERSIONS)
def test_periodic_channel_matches_generator(tmp_path, version):
    """z-periodic channel: the periodic surfaces' physical group gets no
    region, the z faces join the cells across the period as the generator's
    periodic faces do."""
    nx, ny, nz = 6, 4, 4
    ref = mg.channel(nx, ny, nz)
    xs = np.linspace(0, 2, nx + 1)
    ys = mg.stretched_coords(ny, 1.0, 1.1)
    zs = np.linspace(0, 1, nz + 1)
    nodes, cn, sh = mg._structured(nx, ny, nz, xs, ys, zs, (False, False, True), 0.0, 0, (2.0, 1.0, 1.0))
    lat, full, links = unwrap_to_lattice(nodes, cn, sh, (nx, ny, nz), (False, False, True))
    count = {}
    for c in range(full.shape[0]):
        for lf in mg.HEX_FACES:
            key = tuple(sorted(full[c, lf]))
            count.setdefault(key, [0, full[c, lf]])[0] += 1

    def tag(x):
        if abs(x[0]) < 1e-12:
            return 1
        if abs(x[0] - 2.0) < 1e-12:
            return 2
        return 5 if (abs(x[2]) < 1e-12 or abs(x[2] - 1.0) < 1e-12) else 3

    bnd = [(tag(lat[list(k)].mean(axis=0)), list(v[1])) for k, v in count.items() if v[0] == 1]
    p = os.path.join(tmp_path, "pchannel.msh")
    gmsh.write_msh(p, lat, full, "hex", bnd,
                   {(2, 1): "inflow", (2, 2): "outlet", (2, 3): "wall", (2, 5): "periodic-z", (3, 4): "fluid"},
                   periodic=by_translation(lat, links), version=version)
    m = gmsh.read_msh(p)
    assert m.region_names == ["flow", "inflow", "outlet", "wall"]
    for f in ("face_cells", "cell_faces", "boundary_id", "boundary_face", "face_boundary"):
        assert np.array_equal(getattr(m, f), getattr(ref, f)), f
    for f in ("cell_x", "cell_volume", "cell_dx", "face_x", "face_n", "face_area", "face_lambda",
              "face_dist_cell_2"):
        assert np.allclose(getattr(m, f), getattr(ref, f), rtol=0, atol=1e-14), f


@pytest.mark.parametrize("kind", ["hex", "tet"])
@pytest.mark.parametrize("version", VERSIONS)
def test_fully_periodic_box_matches_generator(tmp_path, kind, version):
    """Jittered periodic hex box / Kuhn tet box (links along all three axes,
    edge and corner nodes reached through chains of links)."""
    n = 4
    xs = np.linspace(0.0, 1.0, n + 1)
    jit = 0.1 if kind == "hex" else 0.0
    nodes, cn, sh = mg._structured(n, n, n, xs, xs, xs, (True, True, True), jit, 20240601, (1.0, 1.0, 1.0))
    lat, full, links = unwrap_to_lattice(nodes, cn, sh, (n, n, n), (True, True, True))
    # chains: link each slave to a node that is itself a slave where possible
    I = np.arange(lat.shape[0])
    k, j, i = I % (n + 1), (I // (n + 1)) % (n + 1), I // ((n + 1) ** 2)
    chained = []
    for a, b in links:
        if i[a] == n and (j[a] == n or k[a] == n):
            b = int(a - n * (n + 1) ** 2)            # only x unwrapped: a slave of the y/z links
        chained.append((a, b))
    if kind == "hex":
        ref = mg.periodic_hex_box(n, jitter=jit)
        cells = full
    else:
        ref = mg.periodic_tet_box(n)
        cells = full[:, mg.KUHN_TETS].reshape(-1, 4)
    p = os.path.join(tmp_path, "box.msh")
    gmsh.write_msh(p, lat, cells, kind, [], {(3, 1): "fluid"}, periodic=by_translation(lat, chained),
                   version=version)
    m = gmsh.read_msh(p)
    assert m.region_names == ["flow"] and m.n_boundaries == 0
    for f in ("face_cells", "cell_faces"):
        assert np.array_equal(getattr(m, f), getattr(ref, f)), f
    for f in ("cell_x", "cell_volume", "cell_dx", "face_x", "face_n", "face_area", "face_lambda",
              "face_dist_cell_2"):
        assert np.allclose(getattr(m, f), getattr(ref, f), rtol=0, atol=1e-13), f


@pytest.mark.parametrize("version", VERSIONS)
def test_rejects_rotational_periodic_links(tmp_path, version):
    nx, ny, nz = 2, 2, 2
    xs = np.linspace(0, 1, 3)
    nodes, cn, sh = mg._structured(nx, ny, nz, xs, xs, xs, (False, False, True), 0.0, 0, (1.0, 1.0, 1.0))
    lat, full, links = unwrap_to_lattice(nodes, cn, sh, (nx, ny, nz), (False, False, True))
    links = [(a, b) for a, b in links]
    a, b = links[0]
    links[0] = (a, b + 1)                              # not the common translation
    p = os.path.join(tmp_path, "rot.msh")
    gmsh.write_msh(p, lat, full, "hex", [], {(3, 1): "fluid"}, periodic=[links], version=version)
    with pytest.raises(ValueError, match="translational"):
        gmsh.read_msh(p)


@pytest.mark.parametrize("jitter", [0.0, 0.1])
@pytest.mark.parametrize("version", VERSIONS)
def test_mixed_elements_round_trip(tmp_path, jitter, version):
    """Hexahedra, prisms and pyramids in one Gmsh file (element types 5, 6,
    7) give the generator's mixed mesh; cells have 5 and 6 faces, faces 3
    and 4 nodes."""
    nodes, rows, shifts, kinds = mg.mixed_parts(4, jitter=jitter, periodic=False)
    ref = mg.mixed_box(4, jitter=jitter, periodic=False)
    count, first = {}, {}
    for c, kind in zip(rows, kinds):
        for face in mg.KINDS[kind][1]:
            key = tuple(sorted(int(v) for v in c[face]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, [int(v) for v in c[face]])
    bnd = [(1, first[k]) for k, n in count.items() if n == 1]
    p = os.path.join(tmp_path, "mixed.msh")
    gmsh.write_msh(p, nodes, rows, kinds, bnd, {(2, 1): "wall", (3, 2): "fluid"}, version=version)
    m = gmsh.read_msh(p)
    assert m.region_names == ["flow", "wall"]
    assert sorted(set(np.bincount(m.cell_n_faces).nonzero()[0])) == [5, 6]
    for f in ("face_cells", "cell_faces", "cell_n_faces", "boundary_id", "boundary_face", "face_boundary"):
        assert np.array_equal(getattr(m, f), getattr(ref, f)), f
    for f in ("cell_x", "cell_volume", "cell_dx", "face_x", "face_n", "face_area", "face_lambda"):
        assert np.allclose(getattr(m, f), getattr(ref, f), rtol=0, atol=1e-14), f


@pytest.mark.parametrize("version", VERSIONS)
def test_rejects_cyclic_periodic_links(tmp_path, version):
    xs = np.linspace(0, 1, 3)
    nodes, cn, sh = mg._structured(2, 2, 2, xs, xs, xs, (False, False, True), 0.0, 0, (1.0, 1.0, 1.0))
    lat, full, links = unwrap_to_lattice(nodes, cn, sh, (2, 2, 2), (False, False, True))
    a, b = links[0]
    p = os.path.join(tmp_path, "cyc.msh")
    gmsh.write_msh(p, lat, full, "hex", [], {(3, 1): "fluid"}, periodic=[[(a, b), (b, a)]], version=version)
    with pytest.raises(ValueError, match="cyclic"):
        gmsh.read_msh(p)


def test_both_formats_give_identical_meshes(tmp_path):
    """The mixed hexahedron / prism / pyramid mesh through MSH 4.1 and 2.2:
    every array of the processed meshes is identical."""
    nodes, rows, shifts, kinds = mg.mixed_parts(3, jitter=0.1, periodic=False)
    count, first = {}, {}
    for c, kind in zip(rows, kinds):
        for face in mg.KINDS[kind][1]:
            key = tuple(sorted(int(v) for v in c[face]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, [int(v) for v in c[face]])
    bnd = [(1 + (k[0] % 2), first[k]) for k, n in count.items() if n == 1]
    out = {}
    for version in VERSIONS:
        p = os.path.join(tmp_path, f"m{version}.msh")
        gmsh.write_msh(p, nodes, rows, kinds, bnd, {(2, 1): "a", (2, 2): "b", (3, 3): "fluid"}, version=version)
        out[version] = gmsh.read_msh(p)
    a, b = out["4.1"], out["2.2"]
    assert a.region_names == b.region_names == ["flow", "a", "b"]
    for k, v in a.arrays().items():
        assert np.array_equal(v, b.arrays()[k]), k


def load_reference_reader():
    """The reference preprocessor's Gmsh reader (reader/gmsh.py), run from its
    source text with stand-ins for the element and mesh records it builds
    (its package imports VTK, absent here); no file of the reference tree is
    written."""
    import sys
    import types
    from conftest import REFERENCE
    src = os.path.join(REFERENCE, "tools", "pyMeshFV3D", "pymeshfv3d", "reader", "gmsh.py")
    if not os.path.exists(src):
        pytest.skip("reference tree absent")

    class ElementType:
        POINT, LINE, TRIANGLE, QUADRANGLE, TETRAEDER, HEXAEDER, PRISM, PYRAMID = range(8)

    class Element:
        def __init__(self, etype, nodes, region):
            self.type, self.nodes, self.region = etype, nodes, region

    class Mesh:
        def __init__(self, name, elements, regions, vertices):
            self.name, self.elements, self.regions, self.vertices = name, elements, regions, vertices

    util = types.ModuleType("pymeshfv3d.utilities")
    util.ElementType, util.Element, util.Mesh = ElementType, Element, Mesh
    saved = {k: sys.modules.get(k) for k in ("pymeshfv3d", "pymeshfv3d.utilities")}
    sys.modules["pymeshfv3d"] = types.ModuleType("pymeshfv3d")
    sys.modules["pymeshfv3d.utilities"] = util
    try:
        ns = {"__name__": "reference_gmsh_reader"}
        exec(compile(open(src).read(), src, "exec"), ns)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return ns["read_handler_gmsh"], ElementType


def test_reference_reader_reads_the_41_files(tmp_path):
    """A channel and the mixed box written as MSH 4.1 here, read by the
    reference preprocessor's own reader: the same vertices, the same volume
    elements (kind and nodes) and boundary elements with the region of their
    physical group (its tag - 1)."""
    read_ref, ET = load_reference_reader()
    kind_of = {"hex": ET.HEXAEDER, "tet": ET.TETRAEDER, "prism": ET.PRISM, "pyramid": ET.PYRAMID}
    nodes, cn, bnd, _ = channel_parts(4, 2, 2)
    mixed_nodes, mixed_rows, _, mixed_kinds = mg.mixed_parts(2, jitter=0.1, periodic=False)
    count, first = {}, {}
    for c, kind in zip(mixed_rows, mixed_kinds):
        for face in mg.KINDS[kind][1]:
            key = tuple(sorted(int(v) for v in c[face]))
            count[key] = count.get(key, 0) + 1
            first.setdefault(key, [int(v) for v in c[face]])
    mixed_bnd = [(1, first[k]) for k, n in count.items() if n == 1]
    cases_ = [(nodes, cn, ["hex"] * len(cn), bnd, {(2, 1): "inflow", (2, 2): "outlet", (2, 3): "wall",
                                                    (3, 4): "fluid"}),
              (mixed_nodes, mixed_rows, mixed_kinds, mixed_bnd, {(2, 1): "wall", (3, 2): "fluid"})]
    for i, (nd, rows, kinds, b, names) in enumerate(cases_):
        p = os.path.join(tmp_path, f"ref{i}.msh")
        gmsh.write_msh(p, nd, rows, kinds, b, names, version="4.1")
        m = read_ref(p)
        assert m.regions == [names[k] for k in sorted(names, key=lambda x: x[1])]
        assert np.array_equal(np.asarray(m.vertices), nd)
        surf = [e for e in m.elements if e.type in (ET.TRIANGLE, ET.QUADRANGLE)]
        vol = [e for e in m.elements if e.type not in (ET.TRIANGLE, ET.QUADRANGLE)]
        assert sorted((e.region, tuple(e.nodes)) for e in surf) == sorted((t - 1, tuple(c)) for t, c in b)
        vol_tag = max(t for d, t in names if d == 3)
        want = sorted((kind_of[k], tuple(int(v) for v in r if v >= 0)) for r, k in zip(rows, kinds))
        assert sorted((e.type, tuple(e.nodes)) for e in vol) == want
        assert {e.region for e in vol} == {vol_tag - 1}
