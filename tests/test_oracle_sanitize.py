"""The FP64 oracle's C code under AddressSanitizer and
UndefinedBehaviorSanitizer: every path the parity tests use, on small
meshes, in a child process with the sanitizer runtime preloaded (no GPU)."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _runtime(name):
    try:
        p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
    except OSError:
        return None
    return p if os.path.isabs(p) and os.path.exists(p) else None


SCRIPT = textwrap.dedent("""
    import sys
    sys.path.insert(0, ROOT)
    import numpy as np
    from fv3d_gb300 import cases, meshgen as mg
    from oracle import oracle as orc
    o = orc.Oracle("restated_san")
    def run(c, steps=2, newton=False):
        o.init(c.mesh, c.params, c.region_type, c.region_prim)
        o.set_conserved(c.u0)
        o.time_derivative(0.0); o.gradients(); o.face_states(); o.flux(); o.total()
        o.calc_ns_timestep(); o.global_residual(1e-3)
        for k in range(steps):
            o.step_lserkw2(1, k, 0.0, o.timestep_convective(0.5))
        o.step_ssprk3(0.0, o.timestep_convective(0.5))
        if newton:
            for k in range(2):
                o.step_newton(k, 0.0, o.timestep_convective(1.0), scheme=k, solver=1, krylov_dims=15,
                              krylov_restarts=2)
            o.jacobian()
    run(cases.euler16(3))
    run(cases.tgv_tet(3))
    run(cases.tgv_hex(3))                                   # least squares
    run(cases.tgv_mixed(3))                                 # 5- and 6-face cells
    c = cases.channel(4, 4, 3)
    c.params["mu_mix"] = 0.01
    run(c, newton=True)                                     # pressure outlet, walls
    for t in (mg.BC_OUTFLOW, mg.BC_WALL_ISOTHERMAL, mg.BC_WALL_SLIP, mg.BC_SYMMETRY, mg.BC_STATE):
        c.region_type[2] = t
        run(c, steps=1)
    bad = c.mesh.face_boundary.copy()
    bad[np.nonzero(bad >= 0)[0][0]] = 10 ** 6
    c.mesh.face_boundary = bad
    try:
        o.init(c.mesh, c.params, c.region_type, c.region_prim)
        raise SystemExit("corrupt mesh accepted")
    except RuntimeError:
        pass
    print("sanitized oracle ok")
""")


@pytest.mark.skipif(_runtime("libasan.so") is None, reason="no AddressSanitizer runtime for gcc")
def test_oracle_clean_under_asan_and_ubsan():
    from oracle import oracle as orc
    orc.build("restated_san")
    env = dict(os.environ, LD_PRELOAD=_runtime("libasan.so"),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=0:exitcode=23",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    p = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + SCRIPT], env=env, capture_output=True,
                       text=True, timeout=600)
    report = p.stdout[-2000:] + p.stderr[-4000:]
    assert p.returncode == 0, report
    assert "AddressSanitizer" not in p.stderr and "runtime error" not in p.stderr, report
    assert "sanitized oracle ok" in p.stdout
