"""ctypes front end to the CPU oracles (TEST INFRASTRUCTURE ONLY).

``Oracle("restated")`` loads oracle/liboracle.so, this repository's FP64 C
restatement of the reference hot path; ``Oracle("reference")`` loads
oracle/_ref/libfv3d_ref.so, the reference's own C sources built against the
basec stand-in (present only where the reference tree was available at build
time).  Both implement oracle/fv3d_oracle.h and hold one global instance.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {
    "restated": os.path.join(HERE, "liboracle.so"),
    "reference": os.path.join(HERE, "_ref", "libfv3d_ref.so"),
    # the restatement under AddressSanitizer / UndefinedBehaviorSanitizer:
    # load only in a process started with libasan preloaded
    "restated_san": os.path.join(HERE, "_san", "liboracle_san.so"),
}


def reference_tree() -> str:
    """The reference source tree: FV3D_REFERENCE_TREE when set, else the
    default of the build recipe oracle/Makefile.ref (the one file that names
    where the tree lies on the build machine)."""
    env = os.environ.get("FV3D_REFERENCE_TREE")
    if env:
        return env
    p = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "print-ref"],
                       capture_output=True, text=True)
    return p.stdout.strip() if p.returncode == 0 else ""


def reference_tree_present() -> bool:
    return os.path.isdir(os.path.join(reference_tree(), "src", "Solver"))


_f8p = C.POINTER(C.c_double)
_i4p = C.POINTER(C.c_int)


class OrcMesh(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("n_boundaries", C.c_int),
                ("max_cell_faces", C.c_int), ("n_regions", C.c_int),
                ("cell_x", _f8p), ("cell_volume", _f8p), ("cell_dx", _f8p),
                ("cell_n_faces", _i4p), ("cell_faces", _i4p), ("face_cells", _i4p),
                ("face_boundary", _i4p), ("face_area", _f8p), ("face_lambda", _f8p),
                ("face_x", _f8p), ("face_n", _f8p), ("face_t1", _f8p), ("face_t2", _f8p),
                ("face_dist_cell_2", _f8p), ("boundary_id", _i4p), ("boundary_face", _i4p),
                ("region_is_boundary", _i4p)]


class OrcParams(C.Structure):
    _fields_ = [("kappa", C.c_double), ("R_mix", C.c_double), ("mu_mix", C.c_double),
                ("Pr", C.c_double), ("cfl_scale", C.c_double), ("dfl_scale", C.c_double),
                ("flux_scheme", C.c_int), ("reconstruction", C.c_int), ("limiter", C.c_int),
                ("gradient", C.c_int)]


def build(which: str = "restated", quiet: bool = True) -> str:
    """Compile the oracle library (gcc).  "reference" needs the reference tree."""
    mk = "Makefile.ref" if which == "reference" else "Makefile"
    args = ["make", "-s", "-f", os.path.join(HERE, mk)]
    if which == "reference" and os.environ.get("FV3D_REFERENCE_TREE"):
        args.append(f"REF={os.environ['FV3D_REFERENCE_TREE']}")
    elif which == "restated_san":
        args.append("sanitize")
    subprocess.run(args, check=True, capture_output=quiet)
    return LIBS[which]


def available(which: str) -> bool:
    return os.path.exists(LIBS[which])


def _ptr(a, t):
    return a.ctypes.data_as(t)


# the instance whose init() last set up each library's global state
_ACTIVE = {}


class Oracle:
    """One oracle instance.  The libraries keep global state, as the
    reference does, so instances of one library share it: only the instance
    initialised last may be used (any other raises instead of computing on
    the other instance's mesh and settings)."""

    def __init__(self, which: str = "restated"):
        path = LIBS[which]
        if not os.path.exists(path):
            build(which)
        self.which = which
        self._lib = C.CDLL(path)
        L = self._lib
        L.orc_init.argtypes = [C.POINTER(OrcMesh), C.POINTER(OrcParams), _i4p, _f8p]
        L.orc_error.restype = C.c_char_p
        for name in ("orc_set_conserved", "orc_get_total", "orc_get_flux"):
            getattr(L, name).argtypes = [_f8p]
        L.orc_time_derivative.argtypes = [C.c_double, _f8p]
        L.orc_get_gradients.argtypes = [_f8p, _f8p, _f8p]
        L.orc_get_face_states.argtypes = [_f8p, _f8p]
        L.orc_timestep_convective.argtypes = [C.c_double]
        L.orc_timestep_convective.restype = C.c_double
        L.orc_calc_ns_timestep.restype = C.c_double
        L.orc_step_lserkw2.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_step_ssprk3.argtypes = [C.c_double, C.c_double]
        L.orc_global_residual.argtypes = [C.c_double, _f8p]
        L.orc_step_newton.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                      C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                      _i4p, _i4p]
        L.orc_get_jacobian.argtypes = [_f8p]
        self._keep = None

    @property
    def lib(self):
        if _ACTIVE.get(self.which) is not self:
            raise RuntimeError(f"oracle[{self.which}]: another instance of this library was initialised "
                               "since this one (they share its global state), or this one never was")
        return self._lib

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle[{self.which}]: {self.lib.orc_error().decode()}")

    def init(self, mesh, params: dict, region_type, region_prim):
        a = mesh.arrays()
        self._keep = a
        self.nc, self.nf, self.nb = mesh.n_cells, mesh.n_faces, mesh.n_boundaries
        m = OrcMesh(mesh.n_cells, mesh.n_faces, mesh.n_boundaries, mesh.max_cell_faces,
                    mesh.n_regions)
        for k, v in a.items():
            setattr(m, k, _ptr(v, _i4p if v.dtype == np.int32 else _f8p))
        p = OrcParams(params["kappa"], params["R_mix"], params["mu_mix"], params["Pr"],
                      params.get("cfl_scale", 1.0), params.get("dfl_scale", 1.0),
                      params["flux_scheme"], params["reconstruction"], params["limiter"],
                      params.get("gradient", 0))
        rt = np.ascontiguousarray(region_type, dtype=np.int32)
        rp = np.ascontiguousarray(region_prim, dtype=np.float64).reshape(-1)
        self._keep2 = (m, p, rt, rp)
        _ACTIVE[self.which] = self
        self._check(self.lib.orc_init(C.byref(m), C.byref(p), _ptr(rt, _i4p), _ptr(rp, _f8p)))

    def set_conserved(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == (self.nc, 5)
        self._check(self.lib.orc_set_conserved(_ptr(u, _f8p)))

    def total(self):
        out = np.zeros((self.nc + self.nb, 10))
        self._check(self.lib.orc_get_total(_ptr(out, _f8p)))
        return out

    def conserved(self):
        return self.total()[: self.nc, :5].copy()

    def time_derivative(self, t=0.0):
        out = np.zeros((self.nc, 5))
        self._check(self.lib.orc_time_derivative(t, _ptr(out, _f8p)))
        return out

    def gradients(self):
        g = [np.zeros((self.nc + self.nb, 10)) for _ in range(3)]
        self._check(self.lib.orc_get_gradients(*[_ptr(x, _f8p) for x in g]))
        return g

    def face_states(self):
        l, r = np.zeros((self.nf, 10)), np.zeros((self.nf, 10))
        self._check(self.lib.orc_get_face_states(_ptr(l, _f8p), _ptr(r, _f8p)))
        return l, r

    def flux(self):
        out = np.zeros((self.nf, 5))
        self._check(self.lib.orc_get_flux(_ptr(out, _f8p)))
        return out

    def timestep_convective(self, cfl):
        return self.lib.orc_timestep_convective(cfl)

    def calc_ns_timestep(self):
        return self.lib.orc_calc_ns_timestep()

    def step_lserkw2(self, scheme, iter_, t, dt):
        self._check(self.lib.orc_step_lserkw2(scheme, iter_, t, dt))

    def step_ssprk3(self, t, dt):
        self._check(self.lib.orc_step_ssprk3(t, dt))

    def global_residual(self, dt):
        out = np.zeros(5)
        self._check(self.lib.orc_global_residual(dt, _ptr(out, _f8p)))
        return out

    def step_newton(self, iter_, t, dt, scheme=0, solver=1, max_iter_inner=100,
                    tolerance_lsoe=1e-12, max_iter_lsoe=100, krylov_dims=15,
                    krylov_restarts=2, is_transient=True):
        ni, nl = C.c_int(0), C.c_int(0)
        self._check(self.lib.orc_step_newton(scheme, solver, max_iter_inner, tolerance_lsoe,
                                             max_iter_lsoe, krylov_dims, krylov_restarts,
                                             int(is_transient), iter_, t, dt, C.byref(ni),
                                             C.byref(nl)))
        return ni.value, nl.value

    def jacobian(self):
        out = np.zeros((self.nc, 5, 5))
        self._check(self.lib.orc_get_jacobian(_ptr(out, _f8p)))
        return out  # out[i, col, row] (column-major blocks)
