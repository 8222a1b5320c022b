"""Learned preconditioner: hand-written forward / backward / Adam kernels
against a CPU FP64 reference (PyTorch autograd on CPU, with the BF16
rounding of weights and inputs the kernels apply), training, and its use
inside FGMRES with the block-Jacobi fallback."""
import numpy as np
import pytest

from fv3d_gb300 import api, cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NP = 11013


def bf16(a):
    t = torch.tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float64)
    return t


def unpack(p):
    p = torch.tensor(p, dtype=torch.float64)
    o = 0
    shapes = [(64, 36), (64,), (64, 64), (64,), (64, 64), (64,), (5, 64), (5,)]
    out = []
    for s in shapes:
        n = int(np.prod(s))
        out.append(p[o:o + n].reshape(s))
        o += n
    return out


def torch_loss(params, X, T):
    W0, b0, W1, b1, W2, b2, W3, b3 = params
    gelu = torch.nn.functional.gelu
    a = gelu(X @ W0.T + b0)
    a = gelu(a @ W1.T + b1)
    a = gelu(a @ W2.T + b2)
    y = a @ W3.T + b3
    return ((y - T) ** 2).sum(dim=1).mean(), y


@pytest.fixture(scope="module")
def solver():
    c = cases.channel(8, 4, 4)
    s = api.from_case(c, "fp64")
    s.mlp_init(3)
    yield s
    s.close()


def test_forward_and_gradient_match_cpu_fp64(solver):
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(NP) * 0.2).astype(np.float32)
    solver.mlp_set_params(p)
    X = rng.standard_normal((256, 36)).astype(np.float32)
    T = rng.standard_normal((256, 5)).astype(np.float32)
    loss, g = solver.mlp_grad(X, T)
    Y = solver.mlp_forward(X)
    # weights and inputs rounded to BF16 as the kernels use them; biases FP32
    ps = [t.clone() for t in unpack(p)]
    for i in (0, 2, 4, 6):
        ps[i] = bf16(ps[i].numpy())
    ps = [t.clone().requires_grad_(True) for t in ps]
    L, y = torch_loss(ps, bf16(X), torch.tensor(T, dtype=torch.float64))
    L.backward()
    gref = torch.cat([t.grad.reshape(-1) for t in ps]).numpy()
    assert np.abs(Y - y.detach().numpy()).max() / np.abs(y.detach().numpy()).max() < 3e-2
    assert abs(loss - L.item()) / L.item() < 2e-2
    rel = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    assert rel < 3e-2, rel


def test_training_reduces_loss_on_harvested_pairs(solver):
    solver.mlp_init(11)
    solver.set_state(cases.channel(8, 4, 4).u0)
    solver.mlp_harvest(128, 200000)     # every cell of the 8x4x4 channel, every Newton step
    st = solver.solve_implicit(preconditioner="block_jacobi", tol_rel=1e-6, max_newton=300, check=False)
    n = solver.mlp_dataset()
    assert n >= 128 * min(st["newton_steps"], 8)
    st = solver.mlp_train(epochs=30, batch=512, lr=2e-3)
    assert st["loss_last"] < 0.7 * st["loss_first"], st


def test_learned_preconditioner_converges_to_the_same_answer():
    c = cases.channel(12, 8, 4)
    o = orc.Oracle("restated")
    with api.from_case(c, "fp64") as s:
        s.mlp_init(5)
        s.mlp_harvest(256, 400000)
        base = s.solve_implicit(preconditioner="block_jacobi", tol_rel=1e-8)
        s.mlp_train(epochs=20, batch=1024, lr=2e-3)
        s.mlp_harvest(0, 400000)
        s.set_state(c.u0)
        st = s.solve_implicit(preconditioner="learned", tol_rel=1e-8)
        u = s.get_conserved()
    assert st["converged"] == 1 and base["converged"] == 1
    o.init(c.mesh, c.params, c.region_type, c.region_prim)
    o.set_conserved(c.u0)
    r0 = np.linalg.norm(o.time_derivative(0.0))
    o.set_conserved(u)
    r1 = np.linalg.norm(o.time_derivative(0.0))
    assert r1 / r0 <= 1e-7


def test_stagnating_network_falls_back_to_block_jacobi():
    """An all-zero network makes every learned solve stagnate; each Newton
    step is redone with block Jacobi and counted."""
    c = cases.channel(8, 4, 4)
    with api.from_case(c, "fp64") as s:
        s.mlp_init(1)
        s.mlp_set_params(np.zeros(NP, dtype=np.float32))
        st = s.solve_implicit(preconditioner="learned", tol_rel=1e-6, max_newton=200)
    assert st["converged"] == 1
    assert st["fallbacks"] == st["newton_steps"]
