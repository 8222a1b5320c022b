"""The ctypes binding of the C ABI: an explicit run, then the implicit
steady channel with the learned preconditioner trained on pairs that a
plain Newton-Krylov solve harvests."""
from fv3d_gb300 import api, cases
case = cases.tgv_tet(64)
with api.Solver(case.mesh, case.params, case.region_type, case.region_prim,
                precision="mixed") as s:
    s.set_state(case.u0)
    stats = s.step_explicit("rk33", 500, cfl=0.5)
    phi_total = s.get_state()          # reference phi_total layout (n, 10)

# implicit steady solve; the learned preconditioner trained on pairs that a
# plain Newton-Krylov solve harvests
c = cases.channel()
with api.from_case(c, "fp64") as s:
    s.mlp_init(seed=5)
    s.mlp_harvest(100000, 20000000)    # (features, r) -> dU pairs, 100,000 cells per Newton step
    s.solve_implicit(preconditioner="none", max_restarts=3, max_newton=200, check=False)
    s.mlp_harvest(0, 20000000)
    s.mlp_train(epochs=4, batch=16384, lr=2e-3)
    s.set_state(c.u0)
    stats = s.solve_implicit(preconditioner="learned", check=False)
