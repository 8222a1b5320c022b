"""fv3d_global_residual_noalloc: the residual reduction with its scratch in
a static device array (no device allocation), called through the C ABI and
compared with fv3d_global_residual on two calls in a row.  Collected last so
that it also runs after every other GPU test in the same process.

Who needs it: a caller that may not allocate device memory while it runs
(a fixed device-memory budget carved out up front, or a section of a host
program where allocation calls are not allowed) still gets the residual
norms; what it gives up is the mesh size, at most FV3D_NOALLOC_MAX_CELLS
cells."""
import ctypes as C

import numpy as np
import pytest

from fv3d_gb300 import api, cases, meshgen as mg

pytestmark = pytest.mark.gpu

_f8p = C.POINTER(C.c_double)
MAX_CELLS = 2097152  # FV3D_NOALLOC_MAX_CELLS of include/fv3d_gpu.h


def noalloc(s, dt):
    out = np.full(5, np.nan)
    st = s.lib.fv3d_global_residual_noalloc(s.h, dt, out.ctypes.data_as(_f8p))
    assert st == 0, s.lib.fv3d_last_error(s.h).decode()
    return out


def device_free_bytes():
    """Free device memory as the CUDA runtime reports it (cudaMemGetInfo)."""
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    else:
        pytest.skip("no CUDA runtime library to query free memory")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_residual_equals_allocating_entry_point(precision):
    c = cases.tgv_tet(6)
    with api.from_case(c, precision) as s:
        results = []
        for call in range(2):
            if call == 1:
                s.step_explicit("rk33", 2, 0.5)   # a different state for the second call
            s.time_derivative(0.0)
            ref = s.global_residual(0.01)
            got = noalloc(s, 0.01)
            assert np.all(np.isfinite(got))
            assert np.array_equal(got, ref), (call, got, ref)
            results.append(got)
        assert not np.array_equal(results[0], results[1])


def test_noalloc_residual_two_contexts_one_after_the_other():
    """Two contexts of different sizes share the one static array in turn."""
    outs = []
    for n in (5, 4):
        c = cases.tgv_tet(n)
        with api.from_case(c, "fp64") as s:
            s.time_derivative(0.0)
            outs.append((s.global_residual(1.0), noalloc(s, 1.0)))
    for ref, got in outs:
        assert np.array_equal(got, ref)


def test_noalloc_calls_leave_free_device_memory_unchanged():
    """After a first call (which looks up the array's address), further calls
    change the device's free memory by nothing: they allocate nothing."""
    c = cases.tgv_tet(8)
    with api.from_case(c, "fp64") as s:
        s.time_derivative(0.0)
        noalloc(s, 1.0)
        before = device_free_bytes()
        for _ in range(5):
            noalloc(s, 1.0)
        assert device_free_bytes() == before


def isolated_cells(n):
    """n unit cells, each closed by one wall face of its own: the cheapest
    valid mesh of a given cell count."""
    i = np.arange(n)
    x = np.stack([i % 1000, (i // 1000) % 1000, i // 1000000], axis=1).astype(np.float64)
    nrm = np.tile([1.0, 0.0, 0.0], (n, 1))
    return mg.Mesh(cell_x=x, cell_volume=np.ones(n), cell_dx=np.ones((n, 3)),
                   cell_n_faces=np.ones(n, np.int32), cell_faces=i.astype(np.int32)[:, None],
                   face_cells=np.stack([i, -np.ones(n, np.int64)], axis=1).astype(np.int32),
                   face_boundary=i.astype(np.int32), face_area=np.ones(n), face_lambda=np.ones(n),
                   face_x=x + nrm * 0.5, face_n=nrm, face_t1=np.tile([0.0, 1.0, 0.0], (n, 1)),
                   face_t2=np.tile([0.0, 0.0, 1.0], (n, 1)), face_dist_cell_2=np.zeros((n, 3)),
                   boundary_id=np.zeros(n, np.int32), boundary_face=i.astype(np.int32),
                   region_names=["wall"], region_is_boundary=np.ones(1, np.int32), name="isolated")


def test_noalloc_refuses_a_mesh_beyond_its_limit():
    """One cell past FV3D_NOALLOC_MAX_CELLS: FV3D_ERR_UNSUPPORTED (2) with a
    message naming the limit; the allocating entry point still works."""
    c = cases.euler16(4)                     # its physics parameters
    m = isolated_cells(MAX_CELLS + 1)
    prim = np.array([[0.0, 0.0, 0.0, 1 / 1.4, 1 / 1.4]])
    with api.Solver(m, c.params, [mg.BC_WALL_ADIABATIC], prim, "fp64", "none") as s:
        out = np.full(5, np.nan)
        st = s.lib.fv3d_global_residual_noalloc(s.h, 1.0, out.ctypes.data_as(_f8p))
        assert st == 2
        assert str(MAX_CELLS) in s.lib.fv3d_last_error(s.h).decode()
        assert np.all(np.isnan(out))
