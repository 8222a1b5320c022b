"""Generates the full-run fixtures fullrun_*.npz: the FP64 CPU solution of
the benchmark configurations at their stated step counts, for the GPU tests
in tests/test_gpu_fullrun.py.

  tgv_tet64   1,572,864 tetrahedra, Green-Gauss + Barth-Jespersen, Rusanov,
              viscous, Taylor-Green vortex at Mach 0.8; 500 RK3-3 steps at
              CFL 0.5.  Run by the reference's own C sources
              (oracle/_ref/libfv3d_ref.so), about 20 minutes on one core.
  tgv_hex64   262,144 jittered hexahedra, least-squares gradients +
              Barth-Jespersen, AUSM, viscous, TGV at Mach 0.1; 200 RK3-3
              steps at CFL 0.5.  Least-squares gradients have no reference
              counterpart, so this one runs on the FP64 restatement
              (oracle/liboracle.so), which is bit-identical to the
              reference build on everything the reference has.
  euler16     4,096 hexahedra, first-order Euler, Rusanov; 100 RK3-3 steps at
              CFL 0.5 on the reference build (the configuration's SSP-RK3 is
              new and is checked live against the restatement).

The time step of every step is the convective one at the CFL (computed by
the CPU code on its own state, as the GPU computes it on the device).  Each
fixture stores the final time, every step's dt, the per-variable L2 norms
and volume-weighted totals of the whole final state, and the final state of
every `stride`-th cell (reference cell order) with their indices.

Run where the reference tree exists (the FP64 restatement alone for
tgv_hex64):  python tests/golden/make_fullrun.py [name ...]
Each case runs in a process of its own (the CPU libraries hold global
state); with no names every case runs, all at once.
"""
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fv3d_gb300 import cases  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# name: (case factory, oracle library, RK3-3 steps, CFL, sampled-cell stride)
RUNS = {
    "tgv_tet64": (lambda: cases.tgv_tet(64), "reference", 500, 0.5, 512),
    "tgv_hex64": (lambda: cases.tgv_hex(64), "restated", 200, 0.5, 128),
    "euler16": (lambda: cases.euler16(16), "reference", 100, 0.5, 1),
}
RK33 = 1  # the reference's explicit scheme code for RK3-3 (explicit.c:19-39)


def run(name):
    make, which, steps, cfl, stride = RUNS[name]
    c = make()
    o = orc.Oracle(which)
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    t, dts = 0.0, []
    t0 = time.time()
    for k in range(steps):
        dt = o.timestep_convective(cfl)
        o.step_lserkw2(RK33, k, t, dt)
        t += dt
        dts.append(dt)
        if k % 50 == 0:
            print(f"{name}: step {k}/{steps} t={t:.6f} ({time.time() - t0:.0f} s)", flush=True)
    u = o.conserved()
    idx = np.arange(0, c.mesh.n_cells, stride, dtype=np.int64)
    np.savez_compressed(
        os.path.join(HERE, f"fullrun_{name}.npz"),
        oracle=np.array(which), steps=np.array(steps), cfl=np.array(cfl), t=np.array(t),
        dt=np.array(dts), l2=np.linalg.norm(u, axis=0),
        totals=(u * c.mesh.cell_volume[:, None]).sum(axis=0),
        cells=idx, u=u[idx], cpu_seconds=np.array(time.time() - t0))
    print(f"{name}: done, t={t:.6f}, {time.time() - t0:.0f} s", flush=True)


def main(names):
    if len(names) == 1:
        run(names[0])
        return
    procs = [subprocess.Popen([sys.executable, os.path.abspath(__file__), n]) for n in names]
    rc = [p.wait() for p in procs]
    if any(rc):
        raise SystemExit(f"failed: {[n for n, r in zip(names, rc) if r]}")


if __name__ == "__main__":
    main(sys.argv[1:] or list(RUNS))
