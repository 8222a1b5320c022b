"""CPU evidence (oracle/smoother_study.py) for the design of the learned
part: on the channel's Rusanov matrix at CFL 1e4, per-cell maps fitted with
full knowledge of the exact solutions (upper bounds for any per-cell
network) do not improve on damped block-Jacobi sweeps, while one global
damping does improve on plain sweeps."""
from fv3d_gb300 import cases
from oracle import smoother_study as ss


def test_per_cell_maps_do_not_beat_damped_sweeps():
    r = ss.study(cases.channel(24, 16, 8), k=4)
    print(r)
    assert r["damped_0.7"] < 0.8 * r["plain"]                   # measured 0.37 against 0.53
    assert r["per_cell_first_map"] > 0.95 * r["plain"]          # 0.52: no gain
    assert r["per_cell_damping"] > 0.97 * r["damped_0.7"]       # 0.38: no gain over one damping
    assert r["per_cell_update_map"] > 1.5 * r["damped_0.7"]     # fitted to the error, it amplifies
