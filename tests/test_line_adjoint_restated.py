"""The hand-derived 1-D reverse passes (tests/line_adjoint_restated.py,
restating csrc/mpm_line_adjoint.cu) against torch autograd of the float64
1-D restatement (oracle.mpm_torch.TorchLine), whose forward is first checked
against the NumPy oracle: the derivation the 1-D kernels implement, pinned
without a GPU."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import mpm_oracle as O
from oracle import mpm_torch as T
import line_cases as LC
from line_adjoint_restated import LineRestated


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def case(material, scheme, vu, pvc, steps=50):
    solver, g = LC.bar(O, dtype=np.float64, scheme=scheme, material=material, sim_steps=steps,
                       velocity_update=vu, pvc=pvc)
    n = len(solver.mesh.particles[0])
    E = None
    if material != "newtonian":
        E = 1e6 * np.exp(0.3 * np.random.Generator(np.random.PCG64(3)).normal(size=n))
        solver, g = LC.bar(O, dtype=np.float64, scheme=scheme, material=material, sim_steps=steps,
                           velocity_update=vu, pvc=pvc, E=E)
    return solver, g, E


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("material", ["linear", "simple", "newtonian"])
def test_line_forward_matches_numpy_oracle(material, scheme, reinit):
    solver, g, E = case(material, scheme, False, True)
    sim, st = T.from_line_solver(solver, g)
    Et = None if E is None else torch.tensor(E)
    for i in range(50):
        solver.step(i, g, reinit=reinit)
        st = sim.step(st, i, E=Et, reinit=reinit)
    p = solver.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1)) < 1e-14
    assert rel(st["v"].numpy(), p.velocity.reshape(-1)) < 1e-13
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-13


@pytest.mark.parametrize("pvc", [False, True])
@pytest.mark.parametrize("vu", [False, True])
@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("material", ["linear", "simple", "newtonian"])
def test_line_restated_reverse_matches_autograd(material, scheme, reinit, vu, pvc):
    solver, g, E = case(material, scheme, vu, pvc)
    tl, st0 = T.from_line_solver(solver, g)
    n = len(st0["x"])
    rng = np.random.Generator(np.random.PCG64(5))
    W, U = rng.normal(size=n), rng.normal(size=n)
    r = LineRestated(tl, reinit=reinit)
    st = {k: st0[k].numpy().copy() for k in st0}
    got, end = r.gradient(st, E, 50, W, U)

    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    Et = None if E is None else torch.tensor(E, requires_grad=True)
    end_t = tl.run(dict(st0, x=x0, v=v0), 50, E=Et, reinit=reinit)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-14
    assert rel(end["v"], end_t["v"].detach().numpy()) < 1e-13
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9
    if E is not None:
        assert rel(got["E"], Et.grad.numpy()) < 1e-9
