"""The float64 torch restatement (the gradient oracle) against the NumPy oracle.

Its forward must equal the NumPy oracle run in float64, and its autograd
gradient must agree with central finite differences of that oracle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
from oracle import mpm_torch as T


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle(scheme):
    o, g, _ = workloads.plain_scaleup(O, n=16, scheme=scheme, sim_steps=6, dtype=np.float64)
    sim, st = T.from_solver(o, g)
    for i in range(6):
        o.step(i, g)
        st = sim.step(st, i)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-14
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-14
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-14
    assert rel(st["rho"].numpy(), p.density.reshape(-1)) < 1e-14


def test_forward_matches_with_motion():
    o, g, _ = workloads.plain_small(O, sim_steps=30, dt=2e-3, velocity=(0.6, 0.25), dtype=np.float64)
    sim, st = T.from_solver(o, g)
    for i in range(30):
        o.step(i, g)
        st = sim.step(st, i)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12


def _loss_from(st, target):
    return ((st["x"] - target) ** 2).sum(1).mean()


def test_autograd_matches_finite_differences():
    """dL/dE of L = mean |x_K - x_target|^2 w.r.t. a per-particle E field."""
    n, steps = 12, 30
    o, g, info = workloads.plain_scaleup(O, n=n, sim_steps=steps, dtype=np.float64)
    # a stiff, fast-responding variant: larger dt so the field matters in 30 steps
    o.dt = 2e-4
    o.mpm_scheme.dt = 2e-4
    sim, st0 = T.from_solver(o, g)
    rng = np.random.Generator(np.random.PCG64(3))
    E0 = 1e6 * np.exp(0.5 * rng.normal(size=info["np"]))
    target = st0["x"].detach() + 1e-4
    E = torch.tensor(E0, dtype=torch.float64, requires_grad=True)
    L = _loss_from(sim.run(dict(st0), steps, E=E), target)
    L.backward()
    grad = E.grad.numpy()
    u = rng.normal(size=info["np"])
    h = 1e-3 * np.linalg.norm(E0) / np.linalg.norm(u)

    def loss(Ev):
        with torch.no_grad():
            return float(_loss_from(sim.run(dict(st0), steps, E=torch.tensor(Ev)), target))

    fd = (loss(E0 + h * u) - loss(E0 - h * u)) / (2 * h)
    assert abs(fd - grad @ u) <= 1e-5 * abs(fd) + 1e-30, (fd, grad @ u)


def _sheared(p):
    return np.stack([1.5 + 0.4 * p[:, 0] + 0.8 * p[:, 1], 0.6 + 0.5 * p[:, 0] - 0.3 * p[:, 1]],
                    axis=1)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle_solve_semantics(scheme):
    """``solve`` semantics (volume carried from step to step, mass constant):
    the restatement's ``reinit=False`` step against the oracle's."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, _ = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=_sheared,
                                        dtype=np.float64, scheme=scheme)
    sim, st = T.from_solver(o, g)
    for i in range(24):
        o.step(i, g, reinit=False)
        st = sim.step(st, i, E=torch.tensor(o.mesh.particles[0].youngs_modulus, dtype=torch.float64),
                      reinit=False)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-12
    assert rel(st["rho"].numpy(), p.density.reshape(-1)) < 1e-13
    assert rel(st["vol"].numpy(), p.volume.reshape(-1)) < 1e-13
    assert np.array_equal(st["mass"].numpy(), p.mass.reshape(-1))


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle_with_particle_traction(scheme, reinit):
    """A ramped particle traction on the top layer (t = f(t) tau V / size at
    force time) under both volume semantics."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, _ = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=_sheared,
                                        dtype=np.float64, scheme=scheme, traction=(1, -2.0e3))
    sim, st = T.from_solver(o, g)
    assert sim.tractions
    E = torch.tensor(o.mesh.particles[0].youngs_modulus, dtype=torch.float64)
    for i in range(24):
        o.step(i, g, reinit=reinit)
        st = sim.step(st, i, E=E, reinit=reinit)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-12


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle_with_particle_velocity_constraints(scheme):
    """Particle velocity constraints, overlapping, later entries winning."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, info = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=_sheared,
                                           dtype=np.float64, scheme=scheme)
    n = info["np"]
    o.mesh.particle_velocity_constraints = [
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 7), dir=0, velocity=1.6),
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(3, n, 5), dir=1, velocity=0.5),
        O.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 14), dir=0, velocity=-0.2)]
    sim, st = T.from_solver(o, g)
    assert len(sim.pcons) == 3
    E = torch.tensor(o.mesh.particles[0].youngs_modulus, dtype=torch.float64)
    for i in range(24):
        o.step(i, g)
        st = sim.step(st, i, E=E)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert np.array_equal(st["v"].numpy()[::14, 0], np.full(len(range(0, n, 14)), -0.2))
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12


@pytest.mark.parametrize("reinit", [True, False])
@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle_elastic_newtonian_mixture(scheme, reinit):
    """Elastic and Newtonian particles in one population (the Newtonian stress
    is total, from the rate and the accumulated centroid volumetric strain)."""
    from mixed_cases import mixed_newtonian
    o, g, E0 = mixed_newtonian(O, scheme, dtype=np.float64)
    sim, st = T.from_solver(o, g)
    E = torch.tensor(E0, dtype=torch.float64)
    for i in range(24):
        o.step(i, g, reinit=reinit)
        st = sim.step(st, i, E=E, reinit=reinit)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-12
    assert rel(st["vsc"].numpy(), p.volumetric_strain_centroid.reshape(-1)) < 1e-12


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_forward_matches_numpy_oracle_simple_material_nodal_force(scheme):
    """SimpleMaterial with a per-particle E and a ramped concentrated nodal force."""
    from mixed_cases import simple_with_nodal_force
    o, g, E0 = simple_with_nodal_force(O, scheme, dtype=np.float64)
    sim, st = T.from_solver(o, g)
    E = torch.tensor(E0, dtype=torch.float64)
    for i in range(24):
        o.step(i, g)
        st = sim.step(st, i, E=E)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-13
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-12
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-12


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_float32_forward_tracks_the_float32_oracle(scheme):
    """In float32 the torch restatement runs the oracle's float32 program (the
    one the GPU adjoint is compared with) up to the order of its sums."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    o, g, info = workloads.differentiation(O, n=16, sim_steps=24, dt=dt, velocity=_sheared,
                                           scheme=scheme)
    sim, st = T.from_solver(o, g, dtype=torch.float32)
    E = torch.tensor(info["E"], dtype=torch.float32)
    for i in range(24):
        o.step(i, g)
        st = sim.step(st, i, E=E)
    p = o.mesh.particles[0]
    assert rel(st["x"].numpy(), p.loc.reshape(-1, 2)) < 1e-6
    assert rel(st["v"].numpy(), p.velocity.reshape(-1, 2)) < 1e-5
    assert rel(st["sig"].numpy(), p.stress.reshape(-1, 6)[:, :4]) < 1e-5
