"""Output and restart files (write_output / read_restart_data datasets in a
NumPy container): names, datasets and the round trip, on the host side
with a stand-in for the solver context."""
import os

import numpy as np

from fv3d_gb300 import output


class FakeSolver:
    def __init__(self, n, stages):
        rng = np.random.default_rng(3)
        self.phi = rng.standard_normal((n, 10))
        self.dt = rng.standard_normal((n, 5))
        self.hist = [rng.standard_normal((n, 5)) for _ in range(stages)]

    def get_state(self):
        return self.phi

    def get_time_derivative(self):
        return self.dt

    def bdf_history(self):
        return self.hist


def test_explicit_output_round_trip(tmp_path):
    s = FakeSolver(7, 0)
    p = output.write_output(s, "tgv", 12, 0.25, str(tmp_path))
    assert os.path.basename(p) == "tgv.000000012.npz"
    r = output.read_restart(p)
    assert r["iter"] == 12 and r["t"] == 0.25 and r["phi_old"] == []
    assert np.array_equal(r["phi_total"], s.phi) and np.array_equal(r["phi_dt"], s.dt)
    with np.load(p) as z:
        assert sorted(z.files) == ["iter", "phi_dt", "phi_total", "t"]


def test_implicit_output_keeps_the_bdf_history(tmp_path):
    s = FakeSolver(5, 2)
    p = output.write_output(s, "channel", 0, 0.0, str(tmp_path))
    with np.load(p) as z:
        assert int(z["n_stages"]) == 2 and "phi_old:0" in z.files and "phi_old:1" in z.files
    r = output.read_restart(p)
    assert len(r["phi_old"]) == 2
    for a, b in zip(r["phi_old"], s.hist):
        assert np.array_equal(a, b)
