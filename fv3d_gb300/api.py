"""Python host interface over the C ABI of libfv3d_gb300.so (include/fv3d_gpu.h).

Mirrors the reference solver's entry points for the hot path:
``Solver(...)`` ~ init_mesh + navier_stokes_initialize + boundary_initialize
+ init_reconstruction/init_limiter; ``time_derivative`` ~
finite_volume_time_derivative; ``step_explicit`` ~ timestep_lserkw2 driven by
timedisc; ``timestep`` ~ calc_ns_timestep; ``global_residual`` ~
calc_global_residual.  Errors raise ``FV3DError`` carrying the status code
(the reference aborts instead).

There is no CPU fallback: without the compiled CUDA library (or without a GPU)
every call fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfv3d_gb300.so")

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "UNSUPPORTED", 3: "NONFINITE", 4: "NOT_CONVERGED",
          5: "STAGNATED_FALLBACK", 6: "DEVICE", 7: "TIMEOUT", 8: "BOUNDS", 9: "STATE"}
SCHEMES = {"euler": 0, "rk33": 1, "rk45": 2, "ssprk3": 3}
PRECISION = {"fp64": 0, "mixed": 1}
RENUMBER = {"none": 0, "morton": 1, "rcm": 2}


class FV3DError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_f8p = C.POINTER(C.c_double)
_i4p = C.POINTER(C.c_int)


class Config(C.Structure):
    _fields_ = [("kappa", C.c_double), ("R_mix", C.c_double), ("mu_mix", C.c_double),
                ("Pr", C.c_double), ("cfl_scale", C.c_double), ("dfl_scale", C.c_double),
                ("flux_scheme", C.c_int), ("reconstruction", C.c_int), ("limiter", C.c_int),
                ("gradient", C.c_int), ("precision", C.c_int), ("renumber", C.c_int),
                ("device", C.c_int)]


class MeshArrays(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("n_boundaries", C.c_int),
                ("max_cell_faces", C.c_int), ("n_regions", C.c_int),
                ("cell_x", _f8p), ("cell_volume", _f8p), ("cell_dx", _f8p),
                ("cell_n_faces", _i4p), ("cell_faces", _i4p), ("face_cells", _i4p),
                ("face_boundary", _i4p), ("face_area", _f8p), ("face_lambda", _f8p),
                ("face_x", _f8p), ("face_n", _f8p), ("face_t1", _f8p), ("face_t2", _f8p),
                ("face_dist_cell_2", _f8p), ("boundary_id", _i4p), ("boundary_face", _i4p),
                ("region_is_boundary", _i4p)]


class StepStats(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("steps", C.c_int),
                ("elapsed_ms", C.c_double)]


class ImplicitOpts(C.Structure):
    _fields_ = [("cfl_start", C.c_double), ("cfl_max", C.c_double), ("tol_rel", C.c_double),
                ("max_newton", C.c_int), ("krylov_dim", C.c_int), ("eta", C.c_double),
                ("fd_eps", C.c_double), ("jv_precision", C.c_int), ("preconditioner", C.c_int),
                ("pc_refresh", C.c_int), ("max_restarts", C.c_int), ("sync_every", C.c_int),
                ("inner_dim", C.c_int), ("inner_sweeps", C.c_int), ("inner_omega", C.c_double),
                ("fallback", C.c_int)]


class ImplicitStats(C.Structure):
    _fields_ = [("newton_steps", C.c_int), ("gmres_iterations", C.c_int),
                ("jv_evaluations", C.c_int), ("rejected_steps", C.c_int), ("fallbacks", C.c_int),
                ("converged", C.c_int), ("res0", C.c_double), ("res_final", C.c_double),
                ("rel_res", C.c_double), ("wall_ms", C.c_double), ("cfl_final", C.c_double)]


class NewtonOpts(C.Structure):
    _fields_ = [("scheme", C.c_int), ("max_iter_inner", C.c_int), ("is_transient", C.c_int)]


class NewtonStats(C.Structure):
    _fields_ = [("n_inner", C.c_int), ("err0", C.c_double), ("err", C.c_double)]


EXACT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double))
ITERATION_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int)
OUTPUT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double)


class TimedOpts(C.Structure):
    _fields_ = [("implicit", C.c_int), ("scheme", C.c_int), ("max_iter", C.c_int), ("is_transient", C.c_int),
                ("abort_residual", C.c_double), ("t_start", C.c_double), ("t_end", C.c_double),
                ("cfl", C.c_double), ("max_iter_inner", C.c_int), ("on_iteration", ITERATION_FN),
                ("user", C.c_void_p), ("iter_start", C.c_int), ("i_output_data", C.c_int),
                ("on_output", OUTPUT_FN)]


class TimedStats(C.Structure):
    _fields_ = [("iter", C.c_int), ("t", C.c_double), ("dt", C.c_double), ("res", C.c_double * 5),
                ("stop_reason", C.c_int)]


class MlpTrainOpts(C.Structure):
    _fields_ = [("epochs", C.c_int), ("batch", C.c_int), ("lr", C.c_double), ("seed", C.c_ulonglong)]


class MlpTrainStats(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("samples", C.c_int),
                ("steps", C.c_int), ("wall_ms", C.c_double)]


_f4p = C.POINTER(C.c_float)

PRECONDITIONERS = {"block_jacobi": 0, "lumped": 1, "learned": 2, "none": 3, "coupled": 4}

EXPORTS = {
    "fv3d_create": ([C.POINTER(Config), C.POINTER(C.c_void_p)], C.c_int),
    "fv3d_destroy": ([C.c_void_p], C.c_int),
    "fv3d_last_error": ([C.c_void_p], C.c_char_p),
    "fv3d_version": ([], C.c_char_p),
    "fv3d_mesh_from_arrays": ([C.c_void_p, C.POINTER(MeshArrays)], C.c_int),
    "fv3d_mesh_load_h5": ([C.c_void_p, C.c_char_p], C.c_int),
    "fv3d_get_permutation": ([C.c_void_p, _i4p], C.c_int),
    "fv3d_set_region": ([C.c_void_p, C.c_int, C.c_int, _f8p], C.c_int),
    "fv3d_set_state": ([C.c_void_p, _f8p], C.c_int),
    "fv3d_get_state": ([C.c_void_p, _f8p], C.c_int),
    "fv3d_get_conserved": ([C.c_void_p, _f8p], C.c_int),
    "fv3d_get_time_derivative": ([C.c_void_p, _f8p], C.c_int),
    "fv3d_get_bdf_history": ([C.c_void_p, C.c_int, _f8p, C.POINTER(C.c_int)], C.c_int),
    "fv3d_set_bdf_history": ([C.c_void_p, C.c_int, C.c_int, _f8p], C.c_int),
    "fv3d_time_derivative": ([C.c_void_p, C.c_double, _f8p], C.c_int),
    "fv3d_timestep": ([C.c_void_p, C.c_double, _f8p], C.c_int),
    "fv3d_step_explicit_io": ([C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, _f8p, _f8p,
                               C.POINTER(StepStats)], C.c_int),
    "fv3d_step_explicit": ([C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                            C.POINTER(StepStats)], C.c_int),
    "fv3d_global_residual": ([C.c_void_p, C.c_double, _f8p], C.c_int),
    "fv3d_global_residual_noalloc": ([C.c_void_p, C.c_double, _f8p], C.c_int),
    "fv3d_profile_stage": ([C.c_void_p, C.c_int, C.c_double, _f8p], C.c_int),
    "fv3d_profile_step": ([C.c_void_p, C.c_int, C.c_int, C.c_double, _f8p], C.c_int),
    "fv3d_get_stream": ([C.c_void_p, C.POINTER(C.c_void_p)], C.c_int),
    "fv3d_device_state": ([C.c_void_p, C.POINTER(_f8p)], C.c_int),
    "fv3d_selftest_bounded_wait": ([C.c_void_p, C.c_int, C.POINTER(C.c_int), _f8p], C.c_int),
    "fv3d_implicit_default_opts": ([C.POINTER(ImplicitOpts)], C.c_int),
    "fv3d_solve_implicit": ([C.c_void_p, C.POINTER(ImplicitOpts), C.POINTER(ImplicitStats)], C.c_int),
    "fv3d_implicit_history": ([C.c_void_p, _f8p, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "fv3d_get_blocks": ([C.c_void_p, _f8p], C.c_int),
    "fv3d_jacobian_vector": ([C.c_void_p, C.c_int, C.c_double, _f8p, _f8p], C.c_int),
    "fv3d_get_coupled_blocks": ([C.c_void_p, C.c_int, _f8p, _f8p, _i4p, C.POINTER(C.c_int)], C.c_int),
    "fv3d_step_newton": ([C.c_void_p, C.POINTER(NewtonOpts), C.c_int, C.c_double, C.c_double,
                          C.POINTER(NewtonStats)], C.c_int),
    "fv3d_timedisc": ([C.c_void_p, C.POINTER(TimedOpts), C.POINTER(TimedStats)], C.c_int),
    "fv3d_set_exact_function": ([C.c_void_p, EXACT_FN, C.c_void_p, C.c_int, C.c_double], C.c_int),
    "fv3d_mlp_num_params": ([], C.c_int),
    "fv3d_mlp_init": ([C.c_void_p, C.c_ulonglong], C.c_int),
    "fv3d_mlp_get_params": ([C.c_void_p, _f4p], C.c_int),
    "fv3d_mlp_set_params": ([C.c_void_p, _f4p], C.c_int),
    "fv3d_mlp_forward": ([C.c_void_p, _f4p, C.c_int, _f4p], C.c_int),
    "fv3d_mlp_grad": ([C.c_void_p, _f4p, _f4p, C.c_int, _f8p, _f4p], C.c_int),
    "fv3d_mlp_harvest": ([C.c_void_p, C.c_int, C.c_int], C.c_int),
    "fv3d_mlp_dataset": ([C.c_void_p, C.POINTER(C.c_int)], C.c_int),
    "fv3d_mlp_train": ([C.c_void_p, C.POINTER(MlpTrainOpts), C.POINTER(MlpTrainStats)], C.c_int),
    "fv3d_mlp_adam_step": ([C.c_void_p, _f4p, C.c_double], C.c_int),
    "fv3d_mlp_set_kernel": ([C.c_void_p, C.c_int], C.c_int),
    "fv3d_profile_mlp": ([C.c_void_p, C.c_int, _f8p], C.c_int),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Load (once) the compiled CUDA library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FV3DError(6, f"CUDA library {path} not built (run __graft_entry__.build())")
    lib = C.CDLL(path)
    for name, (args, res) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _p(a, t):
    return a.ctypes.data_as(t)


class Solver:
    """One GPU solver context for a mesh (FV3D's global solver state, per handle)."""

    def __init__(self, mesh, params: dict, region_type, region_prim, precision: str = "fp64",
                 renumber: str = "morton", device: int = 0):
        self.lib = load_library()
        self.h = C.c_void_p()
        cfg = Config(params["kappa"], params["R_mix"], params["mu_mix"], params["Pr"],
                     params.get("cfl_scale", 1.0), params.get("dfl_scale", 1.0),
                     params["flux_scheme"], params["reconstruction"], params["limiter"],
                     params.get("gradient", 0), PRECISION[precision], RENUMBER[renumber], device)
        st = self.lib.fv3d_create(C.byref(cfg), C.byref(self.h))
        if st != 0:
            raise FV3DError(st, "fv3d_create failed (no CUDA device or bad configuration)")
        self.nc = mesh.n_cells
        self.precision = precision
        a = mesh.arrays()
        m = MeshArrays(mesh.n_cells, mesh.n_faces, mesh.n_boundaries, mesh.max_cell_faces,
                       mesh.n_regions)
        for k, v in a.items():
            setattr(m, k, _p(v, _i4p if v.dtype == np.int32 else _f8p))
        self._check(self.lib.fv3d_mesh_from_arrays(self.h, C.byref(m)))
        for r, (t, prim) in enumerate(zip(region_type, np.asarray(region_prim, dtype=np.float64))):
            pr = np.ascontiguousarray(prim, dtype=np.float64)
            self._check(self.lib.fv3d_set_region(self.h, r, int(t), _p(pr, _f8p)))

    def _check(self, st):
        if st != 0:
            raise FV3DError(st, self.lib.fv3d_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.fv3d_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state ----
    def set_state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        if u.shape != (self.nc, 5):
            raise ValueError(f"state must have shape ({self.nc}, 5)")
        self._check(self.lib.fv3d_set_state(self.h, _p(u, _f8p)))

    def get_state(self):
        out = np.empty((self.nc, 10))
        self._check(self.lib.fv3d_get_state(self.h, _p(out, _f8p)))
        return out

    def get_conserved(self, out=None):
        """Conserved state (n_cells, 5); `out` (C-contiguous float64, e.g. a
        pinned host buffer) is filled in place when given."""
        if out is None:
            out = np.empty((self.nc, 5))
        if out.shape != (self.nc, 5) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (n_cells, 5)")
        self._check(self.lib.fv3d_get_conserved(self.h, _p(out, _f8p)))
        return out

    def get_time_derivative(self):
        """phi_dt (n_cells, 5) of the last residual evaluation."""
        out = np.empty((self.nc, 5))
        self._check(self.lib.fv3d_get_time_derivative(self.h, _p(out, _f8p)))
        return out

    def bdf_history(self):
        """The implicit step's phi_old stages, a list of (n_cells, 5) arrays
        (empty before the first implicit step)."""
        n = C.c_int()
        self._check(self.lib.fv3d_get_bdf_history(self.h, 0, None, C.byref(n)))
        out = []
        for k in range(n.value):
            a = np.empty((self.nc, 5))
            self._check(self.lib.fv3d_get_bdf_history(self.h, k, _p(a, _f8p), None))
            out.append(a)
        return out

    def set_bdf_history(self, scheme, stages):
        """Restart history: `stages` the phi_old arrays of `scheme` (euler: 1,
        bdf2: 2), after set_state with the restart state."""
        a = np.ascontiguousarray(np.stack([np.asarray(x, dtype=np.float64) for x in stages]))
        if a.shape[1:] != (self.nc, 5):
            raise ValueError(f"history stages must have shape ({self.nc}, 5)")
        self._check(self.lib.fv3d_set_bdf_history(self.h, {"euler": 0, "bdf2": 1}[scheme], a.shape[0],
                                                  _p(a, _f8p)))

    def permutation(self):
        out = np.empty(self.nc, dtype=np.int32)
        self._check(self.lib.fv3d_get_permutation(self.h, _p(out, _i4p)))
        return out

    # ---- hot path ----
    def time_derivative(self, t: float = 0.0):
        out = np.empty((self.nc, 5))
        self._check(self.lib.fv3d_time_derivative(self.h, t, _p(out, _f8p)))
        return out

    def timestep(self, cfl: float) -> float:
        dt = C.c_double()
        self._check(self.lib.fv3d_timestep(self.h, cfl, C.byref(dt)))
        return dt.value

    def step_explicit(self, scheme: str, n_steps: int, cfl: float = 0.0, dt_fixed: float = 0.0):
        st = StepStats()
        self._check(self.lib.fv3d_step_explicit(self.h, SCHEMES[scheme], n_steps, cfl, dt_fixed,
                                                C.byref(st)))
        return {"t": st.t, "dt": st.dt, "steps": st.steps, "elapsed_ms": st.elapsed_ms}

    def step_explicit_io(self, scheme: str, n_steps: int, cfl: float = 0.0, u_in=None, u_out=None,
                         dt_fixed: float = 0.0):
        """Host state in, n_steps explicit steps, host state out, in one call
        with one synchronisation (u_in / u_out: C-contiguous float64 arrays
        of shape (n_cells, 5), page-locked for direct access; may be the same
        array; None keeps the state on the device)."""
        for u in (u_in, u_out):
            if u is not None and (u.shape != (self.nc, 5) or u.dtype != np.float64 or not u.flags.c_contiguous):
                raise ValueError("host states must be C-contiguous float64 arrays of shape (n_cells, 5)")
        st = StepStats()
        self._check(self.lib.fv3d_step_explicit_io(
            self.h, SCHEMES[scheme], n_steps, cfl, dt_fixed, None if u_in is None else _p(u_in, _f8p),
            None if u_out is None else _p(u_out, _f8p), C.byref(st)))
        return {"t": st.t, "dt": st.dt, "steps": st.steps, "elapsed_ms": st.elapsed_ms}

    def global_residual(self, dt: float):
        out = np.empty(5)
        self._check(self.lib.fv3d_global_residual(self.h, dt, _p(out, _f8p)))
        return out

    def profile_stage(self, n_reps: int = 10, cfl: float = 0.5):
        out = np.empty(3)
        self._check(self.lib.fv3d_profile_stage(self.h, n_reps, cfl, _p(out, _f8p)))
        return out

    def profile_step(self, scheme: str = "rk33", n_steps: int = 10, cfl: float = 0.5):
        """Per-launch kernel times (ms) of real steps: [gradient pass, flux pass
        (both averaged over every stage), last stage's flux pass]."""
        out = np.empty(3)
        self._check(self.lib.fv3d_profile_step(self.h, SCHEMES[scheme], n_steps, cfl, _p(out, _f8p)))
        return out

    # ---- implicit steady solve ----
    def solve_implicit(self, check: bool = True, **kw):
        """Pseudo-transient Newton-Krylov to ||R||/||R_0|| <= tol_rel.  Keyword
        arguments override fv3d_implicit_default_opts (preconditioner may be
        a name).  Returns the statistics as a dict (raises on failure when
        `check`)."""
        o = ImplicitOpts()
        self._check(self.lib.fv3d_implicit_default_opts(C.byref(o)))
        for k, v in kw.items():
            if k in ("preconditioner", "fallback") and isinstance(v, str):
                v = PRECONDITIONERS[v]
            if k == "jv_precision" and isinstance(v, str):
                v = {"fp64": 0, "fp32": 1, "fp32_fp64_arnoldi": 2}[v]
            setattr(o, k, v)
        st = ImplicitStats()
        rc = self.lib.fv3d_solve_implicit(self.h, C.byref(o), C.byref(st))
        out = {f: getattr(st, f) for f, _ in ImplicitStats._fields_}
        out["status"] = rc
        if check and rc != 0:
            self._check(rc)
        return out

    def implicit_history(self):
        n = C.c_int()
        self._check(self.lib.fv3d_implicit_history(self.h, None, 0, C.byref(n)))
        out = np.empty(n.value)
        self._check(self.lib.fv3d_implicit_history(self.h, _p(out, _f8p), n.value, C.byref(n)))
        return out

    def jacobian_vector(self, z, precision: str = "fp64", fd_eps: float = 1e-7):
        """J z of the implicit solve's finite differences at the current
        state ((n_cells, 5) in and out, reference order): FP64 or FP32
        residuals ("fp64" / "fp32")."""
        z = np.ascontiguousarray(z, dtype=np.float64)
        if z.shape != (self.nc, 5):
            raise ValueError(f"z must have shape ({self.nc}, 5)")
        out = np.empty((self.nc, 5))
        self._check(self.lib.fv3d_jacobian_vector(self.h, {"fp64": 0, "fp32": 1}[precision], fd_eps,
                                                  _p(z, _f8p), _p(out, _f8p)))
        return out

    def coupled_blocks(self, which: str = "ausm"):
        """Blocks of the last coupled-preconditioner build: (diag (n_cells, 5,
        5), slots (n_cells, max_slots, 5, 5), neighbour (n_cells, max_slots)),
        row-major blocks, reference order; which "ausm" (P_A) or "rusanov"
        (P_R: inverted diagonal blocks)."""
        w = {"ausm": 0, "rusanov": 1}[which]
        ms = C.c_int()
        self._check(self.lib.fv3d_get_coupled_blocks(self.h, w, None, None, None, C.byref(ms)))
        d = np.empty((self.nc, 5, 5))
        o = np.empty((self.nc, ms.value, 5, 5))
        nb = np.empty((self.nc, ms.value), dtype=np.int32)
        self._check(self.lib.fv3d_get_coupled_blocks(self.h, w, _p(d, _f8p), _p(o, _f8p), _p(nb, _i4p),
                                                     C.byref(ms)))
        return d, o, nb

    def blocks(self):
        out = np.empty((self.nc, 5, 5))
        self._check(self.lib.fv3d_get_blocks(self.h, _p(out, _f8p)))
        return out  # out[i, col, row]

    def step_newton(self, iter_: int, t: float, dt: float, scheme: str = "euler", max_iter_inner: int = 100,
                    is_transient: bool = True, check: bool = True):
        """timestep_newton (implicit.c:224-351): one implicit BE / BDF2 step with
        the lumped Jacobian; returns the stats (n_inner, err0, err)."""
        o = NewtonOpts({"euler": 0, "bdf2": 1}[scheme], max_iter_inner, int(is_transient))
        st = NewtonStats()
        rc = self.lib.fv3d_step_newton(self.h, C.byref(o), iter_, t, dt, C.byref(st))
        if check:
            self._check(rc)
        return {"n_inner": st.n_inner, "err0": st.err0, "err": st.err, "status": rc}

    def set_exact_function(self, fn, id_=0, t=0.0):
        """set_exact_function + set_solution: fn(id, t, x[3]) -> phi (10 values,
        the reference's phi_total row; the conserved entries are used)."""
        def cb(_user, i, tt, x, phi):
            out = fn(i, tt, np.array([x[0], x[1], x[2]]))
            for j in range(min(10, len(out))):
                phi[j] = float(out[j])

        f = EXACT_FN(cb)
        self._check(self.lib.fv3d_set_exact_function(self.h, f, None, id_, t))

    def timedisc(self, scheme="rk33", implicit=False, max_iter=1000, is_transient=True, abort_residual=1e-10,
                 t_start=0.0, t_end=0.2, cfl=0.5, max_iter_inner=100, check=True, iter_start=0,
                 i_output_data=0, on_output=None):
        """timedisc (timedisc.c:134-222): returns the final stats and the
        per-iteration rows (iter, t, dt, res[5], n_inner) print_residual prints.
        on_output(iter, t) is called where the reference calls write_output
        (i_output_data: -1 first and last, 0 never, k > 0 also every k-th);
        iter_start > 0 continues a restart."""
        rows = []

        def on_iter(_user, it, t, dt, res, n_inner):
            rows.append((it, t, dt, [res[j] for j in range(5)], n_inner))

        errors = []

        def on_out(_user, it, t):
            try:
                on_output(it, t)
            except Exception as e:      # no exception may cross the C frames
                errors.append(e)

        cb = ITERATION_FN(on_iter)
        ocb = OUTPUT_FN(on_out) if on_output is not None else OUTPUT_FN()
        sch = {"euler": 0, "bdf2": 1}[scheme] if implicit else SCHEMES[scheme]
        o = TimedOpts(int(implicit), sch, max_iter, int(is_transient), abort_residual, t_start, t_end, cfl,
                      max_iter_inner, cb, None, iter_start, i_output_data, ocb)
        st = TimedStats()
        rc = self.lib.fv3d_timedisc(self.h, C.byref(o), C.byref(st))
        if errors:
            raise errors[0]
        if check:
            self._check(rc)
        return {"iter": st.iter, "t": st.t, "dt": st.dt, "res": list(st.res), "stop_reason": st.stop_reason,
                "status": rc}, rows

    # ---- learned preconditioner ----
    def mlp_init(self, seed: int = 1):
        self._check(self.lib.fv3d_mlp_init(self.h, seed))

    def mlp_params(self):
        out = np.empty(self.lib.fv3d_mlp_num_params(), dtype=np.float32)
        self._check(self.lib.fv3d_mlp_get_params(self.h, _p(out, _f4p)))
        return out

    def mlp_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.fv3d_mlp_set_params(self.h, _p(p, _f4p)))

    def mlp_forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.empty((X.shape[0], 5), dtype=np.float32)
        self._check(self.lib.fv3d_mlp_forward(self.h, _p(X, _f4p), X.shape[0], _p(Y, _f4p)))
        return Y

    def mlp_grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.empty(self.lib.fv3d_mlp_num_params(), dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.fv3d_mlp_grad(self.h, _p(X, _f4p), _p(T, _f4p), X.shape[0],
                                           C.byref(loss), _p(g, _f4p)))
        return loss.value, g

    def mlp_harvest(self, per_step: int, max_samples: int):
        self._check(self.lib.fv3d_mlp_harvest(self.h, per_step, max_samples))

    def mlp_dataset(self) -> int:
        n = C.c_int()
        self._check(self.lib.fv3d_mlp_dataset(self.h, C.byref(n)))
        return n.value

    def mlp_train(self, epochs=5, batch=4096, lr=1e-3, seed=7):
        st = MlpTrainStats()
        self._check(self.lib.fv3d_mlp_train(self.h, C.byref(MlpTrainOpts(epochs, batch, lr, seed)),
                                            C.byref(st)))
        return {f: getattr(st, f) for f, _ in MlpTrainStats._fields_}

    def mlp_set_kernel(self, kind: str):
        """The network's inference kernels: "tcgen05" (default) or "mma_sync"."""
        self._check(self.lib.fv3d_mlp_set_kernel(self.h, {"mma_sync": 0, "tcgen05": 1}[kind]))

    def profile_mlp(self, n_reps: int = 20) -> float:
        """Average ms of one application of the network on the mesh."""
        ms = C.c_double()
        self._check(self.lib.fv3d_profile_mlp(self.h, n_reps, C.byref(ms)))
        return ms.value

    def mlp_adam_step(self, grad, lr=1e-3):
        """One Adam step of the parameters with the given gradient."""
        g = np.ascontiguousarray(grad, dtype=np.float32)
        self._check(self.lib.fv3d_mlp_adam_step(self.h, _p(g, _f4p), lr))

    def selftest_bounded_wait(self, limit_us: int = 2000):
        """(timed_out, elapsed_ms) of a bounded wait on a phase nothing completes."""
        flag, ms = C.c_int(), C.c_double()
        self._check(self.lib.fv3d_selftest_bounded_wait(self.h, limit_us, C.byref(flag), C.byref(ms)))
        return flag.value, ms.value

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.fv3d_get_stream(self.h, C.byref(s)))
        return s.value or 0


def from_case(case, precision="fp64", renumber="morton", device=0) -> Solver:
    s = Solver(case.mesh, case.params, case.region_type, case.region_prim, precision, renumber, device)
    s.set_state(case.u0)
    return s
