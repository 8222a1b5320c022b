"""Gmsh MSH 2.2 reader: a channel written as a Gmsh file and read back gives
the same processed mesh (faces, geometry, regions) as the in-memory
generator; unsupported inputs are rejected."""
import os

import numpy as np
import pytest

from fv3d_gb300 import gmsh, meshgen as mg


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


def test_round_trip_matches_generator(tmp_path):
    nodes, cn, bnd, ref = channel_parts()
    p = os.path.join(tmp_path, "channel.msh")
    gmsh.write_msh(p, nodes, cn, "hex", bnd, {(2, 1): "inflow", (2, 2): "outlet", (2, 3): "wall", (3, 4): "fluid"})
    m = gmsh.read_msh(p)
    assert m.region_names == ["flow", "inflow", "outlet", "wall"]
    for f in ("face_cells", "cell_faces", "boundary_id", "boundary_face", "face_boundary"):
        assert np.array_equal(getattr(m, f), getattr(ref, f)), f
    for f in ("cell_x", "cell_volume", "cell_dx", "face_x", "face_n", "face_area", "face_lambda"):
        assert np.allclose(getattr(m, f), getattr(ref, f), rtol=0, atol=1e-14), f


def test_rejects_unsupported(tmp_path):
    with pytest.raises(ValueError):
        gmsh.read_msh("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
    nodes, cn, bnd, _ = channel_parts(2, 2, 2)
    p = os.path.join(tmp_path, "nophys.msh")
    gmsh.write_msh(p, nodes, cn, "hex", bnd[1:], {(2, 1): "a", (2, 2): "b", (2, 3): "c"})
    with pytest.raises(ValueError, match="no physical surface"):
        gmsh.read_msh(p)
