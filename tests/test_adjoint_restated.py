"""The hand-derived reverse passes (restated in NumPy float64) against torch
autograd of the float64 oracle: the derivation the CUDA adjoint implements."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
from oracle import mpm_torch as T
from adjoint_restated import Restated


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def sheared(p):
    return np.stack([1.5 + 0.4 * p[:, 0] + 0.8 * p[:, 1], 0.6 + 0.5 * p[:, 0] - 0.3 * p[:, 1]],
                    axis=1)


def case(velocity_update, steps=24, scheme="usf", velocity=(1.5, 0.6)):
    # USL at dt 1e-3 blows up within these steps (a free-surface node's mass
    # falls towards zero); 2.5e-4 keeps it stable
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, info = workloads.differentiation(O, n=16, sim_steps=steps, dt=dt,
                                           velocity=velocity, dtype=np.float64, scheme=scheme)
    o.velocity_update = velocity_update
    o.mpm_scheme.velocity_update = velocity_update
    tsim, st0 = T.from_solver(o, g)
    return tsim, st0, info


@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("vu", [False, True])
def test_restated_forward_matches_oracle(vu, scheme):
    tsim, st0, info = case(vu, scheme=scheme)
    E = info["E"]
    r = Restated(tsim)
    st = {k: st0[k].numpy().copy() for k in ("x", "v", "sig", "rho", "nv")}
    for _ in range(24):
        st, _ = r.forward(st, E)
    with torch.no_grad():
        ref = tsim.run(dict(st0), 24, E=torch.tensor(E))
    assert rel(st["x"], ref["x"].numpy()) < 1e-13
    assert rel(st["v"], ref["v"].numpy()) < 1e-12
    assert rel(st["sig"], ref["sig"].numpy()) < 1e-12


@pytest.mark.parametrize("velocity", ["uniform", "sheared"])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("vu", [False, True])
def test_restated_reverse_matches_autograd(vu, scheme, velocity):
    tsim, st0, info = case(vu, scheme=scheme, velocity=(1.5, 0.6) if velocity == "uniform" else sheared)
    n = info["np"]
    rng = np.random.Generator(np.random.PCG64(5))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    E = info["E"]
    r = Restated(tsim)
    st = {k: st0[k].numpy().copy() for k in ("x", "v", "sig", "rho", "nv")}
    got, _ = r.gradient(st, E, 24, W, U)

    Et = torch.tensor(E, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    s = dict(st0, x=x0, v=v0)
    end = tsim.run(s, 24, E=Et)
    L = (end["x"] * torch.tensor(W)).sum() + (end["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9


@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("vu", [False, True])
def test_restated_reverse_matches_autograd_solve_semantics(vu, scheme):
    """``solve`` semantics: the volume is carried from step to step (its update
    V' = V f has an adjoint of its own) and the mass is a constant; the
    restated reverse passes against autograd of the same program."""
    tsim, st0, info = case(vu, scheme=scheme, velocity=sheared)
    n = info["np"]
    rng = np.random.Generator(np.random.PCG64(7))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    E = info["E"]
    r = Restated(tsim, reinit=False)
    st = {k: st0[k].numpy().copy() for k in ("x", "v", "sig", "rho", "nv", "vol", "mass")}
    got, end = r.gradient(st, E, 24, W, U)

    Et = torch.tensor(E, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    s = dict(st0, x=x0, v=v0)
    end_t = tsim.run(s, 24, E=Et, reinit=False)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-13
    assert rel(end["vol"], end_t["vol"].detach().numpy()) < 1e-12
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9
    # the carried volume changes the gradient: solve_jit's differs
    rj = Restated(tsim)
    gj, _ = rj.gradient({k: st0[k].numpy().copy() for k in ("x", "v", "sig", "rho", "nv")}, E, 24, W, U)
    assert rel(gj["E"], got["E"]) > 1e-6


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_restated_reverse_matches_autograd_with_particle_traction(scheme, reinit):
    """A ramped particle traction on the top layer, under both volume
    semantics: the traction's terms of the shape-function and volume
    adjoints against autograd."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, info = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=sheared,
                                           dtype=np.float64, scheme=scheme, traction=(1, -2.0e3))
    tsim, st0 = T.from_solver(o, g)
    n = info["np"]
    rng = np.random.Generator(np.random.PCG64(9))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    E = info["E"]
    r = Restated(tsim, reinit=reinit)
    keys = ("x", "v", "sig", "rho", "nv") + (() if reinit else ("vol", "mass", "psize"))
    got, end = r.gradient({k: st0[k].numpy().copy() for k in keys}, E, 24, W, U)

    Et = torch.tensor(E, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    end_t = tsim.run(dict(st0, x=x0, v=v0), 24, E=Et, reinit=reinit)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-13
    assert rel(end["v"], end_t["v"].detach().numpy()) < 1e-12
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9


@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("vu", [False, True])
def test_restated_reverse_matches_autograd_with_particle_velocity_constraints(vu, scheme):
    """Overlapping particle velocity constraints: the cleared end-of-step
    velocity adjoints against autograd."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, info = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=sheared,
                                           dtype=np.float64, scheme=scheme)
    o.velocity_update = vu
    o.mpm_scheme.velocity_update = vu
    n = info["np"]
    o.mesh.particle_velocity_constraints = [
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 7), dir=0, velocity=1.6),
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(3, n, 5), dir=1, velocity=0.5)]
    tsim, st0 = T.from_solver(o, g)
    rng = np.random.Generator(np.random.PCG64(11))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    E = info["E"]
    r = Restated(tsim)
    got, end = r.gradient({k: st0[k].numpy().copy() for k in ("x", "v", "sig", "rho", "nv")},
                          E, 24, W, U)
    Et = torch.tensor(E, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    end_t = tsim.run(dict(st0, x=x0, v=v0), 24, E=Et)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-13
    assert rel(end["v"], end_t["v"].detach().numpy()) < 1e-12
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_restated_reverse_matches_autograd_elastic_newtonian_mixture(scheme, reinit):
    """Elastic and Newtonian particles in one population: the Newtonian stress
    is total (no adjoint to the start-of-step stress) and reads the
    accumulated centroid volumetric strain, whose adjoint the reverse carries."""
    from mixed_cases import mixed_newtonian
    o, g, E0 = mixed_newtonian(O, scheme, dtype=np.float64)
    tsim, st0 = T.from_solver(o, g)
    n = len(E0)
    rng = np.random.Generator(np.random.PCG64(13))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    r = Restated(tsim, reinit=reinit)
    assert r.newt.any() and not r.newt.all()
    keys = ("x", "v", "sig", "rho", "nv", "vsc") + (() if reinit else ("vol", "mass"))
    got, end = r.gradient({k: st0[k].numpy().copy() for k in keys}, E0, 24, W, U)
    Et = torch.tensor(E0, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    end_t = tsim.run(dict(st0, x=x0, v=v0), 24, E=Et, reinit=reinit)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-13
    assert rel(end["sig"], end_t["sig"].detach().numpy()) < 1e-12
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9
    assert np.all(got["E"][r.newt] == 0.0)


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_restated_reverse_matches_autograd_simple_material_nodal_force(scheme, reinit):
    """SimpleMaterial with a per-particle E under a ramped concentrated nodal
    force (a constant of the state: it changes the trajectory, not the
    reverse passes)."""
    from mixed_cases import simple_with_nodal_force
    o, g, E0 = simple_with_nodal_force(O, scheme, dtype=np.float64)
    tsim, st0 = T.from_solver(o, g)
    n = len(E0)
    rng = np.random.Generator(np.random.PCG64(17))
    W = rng.normal(size=(n, 2))
    U = rng.normal(size=(n, 2))
    r = Restated(tsim, reinit=reinit)
    assert r.simple.all() and r.cnf
    keys = ("x", "v", "sig", "rho", "nv", "vsc") + (() if reinit else ("vol", "mass"))
    got, end = r.gradient({k: st0[k].numpy().copy() for k in keys}, E0, 24, W, U)
    Et = torch.tensor(E0, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    end_t = tsim.run(dict(st0, x=x0, v=v0), 24, E=Et, reinit=reinit)
    assert rel(end["x"], end_t["x"].detach().numpy()) < 1e-13
    L = (end_t["x"] * torch.tensor(W)).sum() + (end_t["v"] * torch.tensor(U)).sum()
    L.backward()
    assert rel(got["E"], Et.grad.numpy()) < 1e-9
    assert rel(got["x"], x0.grad.numpy()) < 1e-9
    assert rel(got["v"], v0.grad.numpy()) < 1e-9
