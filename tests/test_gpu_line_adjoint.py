"""The hand-written 1-D adjoint (csrc/mpm_line_adjoint.cu) against central
differences of the float64 oracle.

A loss L = sum(w * x_end) + sum(u * v_end) with seeded weights is
differentiated along seeded directions of the per-particle Young's modulus,
the initial positions and the initial velocities: the GPU's
dL/dE . dE (and likewise for x0, v0) must match (L(+) - L(-)) / 2 eps of two
float64 oracle runs within 1e-3 (relative to |FD|, or to a tenth of the summed
|terms| where a random direction cancels).  Besides the solve_jit cases,
solve semantics (``reinit=False``: constant mass, carried volume) and the
build's Newtonian material are checked the same way.  The last case is the
reference's own optimisation example (examples/optim_1d.py): one SimpleMaterial particle,
USL, 1000 steps, the gradient of |v_end - v_target| in E."""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300.autograd import explicit_run
from oracle import mpm_oracle as O
import line_cases as L

pytestmark = pytest.mark.gpu

TOL = 1e-3


def oracle_end(case, steps, E, x0=None, v0=None):
    case = dict(case)
    reinit = case.pop("reinit", True)
    solver, g = L.bar(O, dtype=np.float64, E=E, sim_steps=steps, **case)
    p = solver.mesh.particles[0]
    if x0 is not None:
        p.loc[:] = np.asarray(x0, np.float64).reshape(-1, 1, 1)
    if v0 is not None:
        p.velocity[:] = np.asarray(v0, np.float64).reshape(-1, 1, 1)
    for i in range(steps):
        solver.step(i, g, reinit=reinit)
    return p.loc.reshape(-1).copy(), p.velocity.reshape(-1).copy()


# vshift=8: every particle crosses into the next element during the 40 steps,
# so the reversed steps follow changing element populations (per-step re-sorts)
CASES = [dict(scheme="usf"), dict(scheme="usl"), dict(scheme="usf", material="simple"),
         dict(scheme="usl", material="simple", nx=12, ppe=1),
         dict(scheme="usf", velocity_update=True),
         dict(scheme="usf", vshift=8.0), dict(scheme="usl", vshift=8.0),
         dict(scheme="usf", pvc=True), dict(scheme="usl", pvc=True, vshift=8.0),
         dict(scheme="usf", reinit=False), dict(scheme="usl", reinit=False, vshift=8.0),
         dict(scheme="usf", material="newtonian"), dict(scheme="usl", material="newtonian", reinit=False)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}={v}" for k, v in c.items()))
def test_line_adjoint_matches_central_differences(built, case):
    case = dict(dict(nx=20, ppe=2), **case)
    reinit = case.get("reinit", True)
    bar_case = {k: v for k, v in case.items() if k != "reinit"}
    steps = 40
    gs0, g = L.bar(O, sim_steps=steps, **bar_case)
    p0 = gs0.mesh.particles[0]
    n = len(p0.loc)
    x0 = p0.loc.reshape(-1).astype(np.float64)
    v0 = p0.velocity.reshape(-1).astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(11))
    E = 1e6 * np.exp(rng.uniform(-0.3, 0.3, n))
    w = rng.standard_normal(n)
    u = rng.standard_normal(n)
    gs, g = L.bar(D, sim_steps=steps, E=E.astype(np.float32), **bar_case)
    sim = gs.simulation(g, reinit=reinit)
    gs._upload(sim)
    sim.initialize()
    sim.record(steps)
    out = sim.adjoint(w.astype(np.float32).reshape(n, 1), u.astype(np.float32).reshape(n, 1))
    sim.close()
    assert out["loc"].shape == (n, 1) and out["velocity"].shape == (n, 1)

    def loss(**kw):
        x, v = oracle_end(case, steps, **kw)
        return float(w @ x + u @ v)

    checks = {
        "E": (out["youngs_modulus"].astype(np.float64), E, 1e-4,
              lambda d, s: loss(E=E * (1 + s * d), x0=x0, v0=v0), True),
        "x0": (out["loc"].reshape(-1).astype(np.float64), x0, 1e-6,
               lambda d, s: loss(E=E, x0=x0 + s * d, v0=v0), False),
        "v0": (out["velocity"].reshape(-1).astype(np.float64), v0, 1e-3,
               lambda d, s: loss(E=E, x0=x0, v0=v0 + s * d), False),
    }
    for name, (grad, base, eps, f, relative) in checks.items():
        d = rng.standard_normal(n)
        # E is perturbed relatively: dE = E * d * eps
        dirn = base * d if relative else d
        fd = (f(d, eps) - f(d, -eps)) / (2 * eps)
        ad = float(grad @ dirn)
        # relative to the size of the summed terms (a random direction may cancel)
        scale = max(abs(fd), 0.1 * float(np.abs(grad * dirn).sum()), 1e-30)
        assert abs(ad - fd) <= TOL * scale, (name, ad, fd)


def test_optim_1d_gradient(built):
    """examples/optim_1d.py: loss |v_end - v_target| with v_target from E = 100,
    gradient in E at E = 105 through explicit_run (torch autograd)."""
    torch = pytest.importorskip("torch")
    steps = 1000
    target_solver, g = L.point(D, E=100.0)
    target = target_solver.solve_jit(g)["velocity"].reshape(-1)

    def oracle_v(E):
        s, g0 = L.point(O, E=np.array([E]), dtype=np.float64)
        for i in range(steps):
            s.step(i, g0, reinit=True)
        return s.mesh.particles[0].velocity.reshape(-1).astype(np.float64)

    mpm, g = L.point(D, E=105.0)
    E = torch.tensor([105.0], dtype=torch.float64, requires_grad=True)
    x, v = explicit_run(mpm, g, E, nsteps=steps)
    loss = torch.linalg.norm(v.reshape(-1).double() - torch.tensor(target, dtype=torch.float64))
    loss.backward()
    h = 1e-3
    fd = (np.linalg.norm(oracle_v(105.0 + h) - target) -
          np.linalg.norm(oracle_v(105.0 - h) - target)) / (2 * h)
    got = float(E.grad[0])
    assert abs(got - fd) <= 1e-2 * abs(fd), (got, fd)
    # the float32 forward under the per-particle E equals the material-E run
    o, g0 = L.point(O, E=np.array([105.0]))
    ref = o.solve_jit(g0)["velocity"].reshape(-1)
    assert np.array_equal(v.detach().numpy().reshape(-1), ref)
