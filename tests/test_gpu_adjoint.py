"""The CUDA adjoint (mpm_record / mpm_adjoint) against the gradient oracle.

The oracle is torch autograd of the restatement in oracle.mpm_torch, whose
float64 gradient is checked against central finite differences on the CPU
(tests/test_oracle_torch.py) and whose reverse passes equal the hand-derived
ones (tests/test_adjoint_restated.py).  The GPU adjoint is the exact adjoint
of the float32 program, so it is compared with float32 autograd (normwise
relative error <= 1e-3); against float64 autograd it must be within 1e-3 or
as close as float32 autograd is (within 3x) -- the float32 program's own
conditioning (the position gradient under velocity_update differs from
float64 by ~3e-3 in float32 autograd too).
The initial velocity field is sheared: under a uniform velocity the strain
rates are zero in exact arithmetic, and whether the reference's flush
(|a| < 1e-12 -> 0, zero derivative) blocks them then depends on round-off
ties (see oracle/mpm_torch.py), which makes the velocity gradient of that
degenerate input differ between any two summation orders.  A central finite
difference of the float64 oracle checks a directional derivative in E.
"""
import numpy as np
import pytest

import diffmpm_gb300 as D
from diffmpm_gb300 import workloads
from oracle import mpm_oracle as O
from mixed_cases import mixed_newtonian

torch = pytest.importorskip("torch")
from oracle import mpm_torch as T  # noqa: E402

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def sheared(p):
    """Initial velocity (1.5 + 0.4 x + 0.8 y, 0.6 + 0.5 x - 0.3 y): particles
    change cell, and every strain rate is far from the flush threshold."""
    return np.stack([1.5 + 0.4 * p[:, 0] + 0.8 * p[:, 1], 0.6 + 0.5 * p[:, 0] - 0.3 * p[:, 1]],
                    axis=1)


CASE = dict(n=16, sim_steps=24, dt=1e-3, velocity=sheared)


def case_args(kw):
    """CASE with overrides; USL steps at dt 2.5e-4 (at 1e-3 a free-surface
    node's mass falls towards zero within the steps and USL blows up)."""
    args = dict(CASE, **kw)
    if args.get("scheme") == "usl" and "dt" not in kw:
        args["dt"] = 2.5e-4
    return args


def gpu_sim(vu=False, block=None, **kw):
    args = case_args(kw)
    gs, g, info = workloads.differentiation(D, **args)
    gs.velocity_update = vu
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    if block:
        sim.set_block_steps(block)
    return gs, sim, g, info


def seeds(n, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.normal(size=(n, 2)).astype(np.float32), rng.normal(size=(n, 2)).astype(np.float32)


def autograd_ref(vu, W, U, dtype=torch.float32, **kw):
    """Gradients of L = <W, x_end> + <U, v_end> by autograd of the oracle in
    ``dtype`` (float32: the same discrete program as the GPU)."""
    args = case_args(kw)
    npd = np.float32 if dtype == torch.float32 else np.float64
    o, g, info = workloads.differentiation(O, dtype=npd, **args)
    o.velocity_update = vu
    o.mpm_scheme.velocity_update = vu
    tsim, st0 = T.from_solver(o, g, dtype=dtype)
    Et = torch.tensor(info["E"], dtype=dtype, requires_grad=True)
    x0 = st0["x"].clone().requires_grad_(True)
    v0 = st0["v"].clone().requires_grad_(True)
    end = tsim.run(dict(st0, x=x0, v=v0), args["sim_steps"], E=Et)
    L = (end["x"] * torch.tensor(W, dtype=dtype)).sum() + (end["v"] * torch.tensor(U, dtype=dtype)).sum()
    L.backward()
    return {"youngs_modulus": Et.grad.numpy(), "loc": x0.grad.numpy(), "velocity": v0.grad.numpy(),
            "x_end": end["x"].detach().numpy()}


@pytest.mark.parametrize("scheme", ["usf", "usl"])
@pytest.mark.parametrize("vu", [False, True])
def test_adjoint_matches_autograd(built, vu, scheme):
    gs, sim, g, info = gpu_sim(vu, scheme=scheme)
    W, U = seeds(info["np"])
    sim.record(CASE["sim_steps"], 10)
    x_end = sim.read("loc")
    got = sim.adjoint(W, U)
    ref = autograd_ref(vu, W, U, scheme=scheme)
    ref64 = autograd_ref(vu, W, U, dtype=torch.float64, scheme=scheme)
    fwd = rel(x_end, ref64["x_end"])
    assert fwd < 1e-5
    for k in ("youngs_modulus", "loc", "velocity"):
        e, e64 = rel(got[k], ref[k]), rel(got[k], ref64[k])
        # as close to float64 as float32 autograd itself is (within 3x)
        assert e < GRAD_TOL and e64 <= max(GRAD_TOL, 3.0 * rel(ref[k], ref64[k])), (k, e, e64)


def test_adjoint_checkpoint_interval_and_repeat(built):
    """Every re-run segment reproduces the recorded run bit for bit (the
    adjoint checks this itself and raises otherwise); a repeated call (the
    handle is left at the recorded end) gives the same bits; and the gradient
    hardly depends on the checkpoint interval (the interval splits the step
    blocks, which moves the re-sorts and so the order of float32 sums)."""
    outs = []
    for K in (1, 7, CASE["sim_steps"]):
        gs, sim, g, info = gpu_sim()
        W, U = seeds(info["np"])
        sim.record(CASE["sim_steps"], K)
        outs.append(sim.adjoint(W, U))
        again = sim.adjoint(W, U)
        for k in again:
            assert np.array_equal(again[k], outs[-1][k]), (K, k)
    for o in outs[1:]:
        for k in o:
            assert rel(o[k], outs[0][k]) < 1e-5, k


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_across_resorts(built, scheme):
    """Short step blocks re-sort the particles between blocks; the recorded
    re-sorts are replayed and the adjoint arrays permuted across them."""
    steps = CASE["sim_steps"] if scheme == "usf" else 96   # USL: 4x the steps at dt / 4
    gs, sim, g, info = gpu_sim(block=3, scheme=scheme, sim_steps=steps)
    W, U = seeds(info["np"])
    before = sim.counters()["resorts"]
    sim.record(steps, 10)
    assert sim.counters()["resorts"] > before + 1
    a = sim.adjoint(W, U)
    ref = autograd_ref(False, W, U, scheme=scheme, sim_steps=steps)
    for k in a:
        assert rel(a[k], ref[k]) < GRAD_TOL, k


def _direct_adjoint(gs, g, E, W, U, steps, ckpt=8):
    """record + adjoint through the Simulation API (no autograd)."""
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.write("youngs_modulus", np.asarray(E, np.float32))
    sim.initialize()
    sim.record(steps, ckpt)
    return sim.adjoint(W, U)


def test_autograd_function(built):
    from diffmpm_gb300.autograd import explicit_run
    gs, g, info = workloads.differentiation(D, **CASE)
    n = info["np"]
    W, U = seeds(n, 9)
    dev = torch.device("cuda:0")
    E = torch.tensor(info["E"], dtype=torch.float32, device=dev, requires_grad=True)
    v0 = torch.tensor(gs.mesh.particles[0].velocity.reshape(n, 2), device=dev, requires_grad=True)
    x, v = explicit_run(gs, g, E, velocity=v0, checkpoint_steps=8)
    L = (x * torch.tensor(W, device=dev)).sum() + (v * torch.tensor(U, device=dev)).sum()
    L.backward()
    direct = _direct_adjoint(gs, g, info["E"], W, U, CASE["sim_steps"])
    assert np.array_equal(E.grad.cpu().numpy(), direct["youngs_modulus"])
    assert np.array_equal(v0.grad.cpu().numpy(), direct["velocity"])


def test_autograd_function_is_reentrant(built):
    """Two forwards with different E before either backward, then the two
    backwards in reverse order, then a forward-only evaluation between a
    forward and its backward: every gradient equals the one of the same run
    differentiated alone (each forward records into its own simulation)."""
    from diffmpm_gb300.autograd import explicit_run
    gs, g, info = workloads.differentiation(D, **CASE)
    n = info["np"]
    W, U = seeds(n, 9)
    dev = torch.device("cuda:0")
    Es = [info["E"], info["E"] * (1.0 + 0.3 * np.sin(np.arange(n)))]
    want = [_direct_adjoint(gs, g, Ek, W, U, CASE["sim_steps"]) for Ek in Es]
    tW, tU = torch.tensor(W, device=dev), torch.tensor(U, device=dev)
    leaves = [torch.tensor(Ek, dtype=torch.float32, device=dev, requires_grad=True) for Ek in Es]
    losses = []
    for E in leaves:
        x, v = explicit_run(gs, g, E, checkpoint_steps=8)
        losses.append((x * tW).sum() + (v * tU).sum())
    for k in (1, 0):
        losses[k].backward()
        assert np.array_equal(leaves[k].grad.cpu().numpy(), want[k]["youngs_modulus"]), k
    E = torch.tensor(Es[0], dtype=torch.float32, device=dev, requires_grad=True)
    x, v = explicit_run(gs, g, E, checkpoint_steps=8)
    L = (x * tW).sum() + (v * tU).sum()
    with torch.no_grad():
        explicit_run(gs, g, torch.tensor(Es[1], dtype=torch.float32, device=dev), checkpoint_steps=8)
    L.backward()
    assert np.array_equal(E.grad.cpu().numpy(), want[0]["youngs_modulus"])


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_directional_derivative_vs_finite_differences(built, scheme):
    """<dL/dE, u> from the GPU against a central difference of the float64
    oracle, L = mean |x_end - x_target|^2 (the differentiation workload's loss)
    on a 32 x 32 mesh for 40 steps."""
    kw = dict(n=32, sim_steps=40, dt=2e-4, velocity=(0.5, 0.0), scheme=scheme)
    gs, sim, g, info = gpu_sim(**kw)
    n = info["np"]
    rng = np.random.Generator(np.random.PCG64(21))
    o, g64, info64 = workloads.differentiation(O, dtype=np.float64, **dict(CASE, **kw))
    tsim, st0 = T.from_solver(o, g64)
    target = st0["x"].numpy() + rng.normal(scale=1e-3, size=(n, 2))
    sim.record(kw["sim_steps"], 16)
    x_end = sim.read("loc").astype(np.float64)
    dl_dx = (2.0 / n) * (x_end - target)
    grad = sim.adjoint(dl_dx.astype(np.float32), want=("youngs_modulus",))["youngs_modulus"]
    E0 = info64["E"]
    u = rng.normal(size=n) * E0
    h = 1e-4

    def loss(Ev):
        with torch.no_grad():
            end = tsim.run(dict(st0), kw["sim_steps"], E=torch.tensor(Ev))
        return float(((end["x"].numpy() - target) ** 2).sum(1).mean())

    fd = (loss(E0 + h * u) - loss(E0 - h * u)) / (2 * h)
    gd = float(np.dot(grad.astype(np.float64), u))
    assert abs(gd - fd) <= GRAD_TOL * abs(fd), (gd, fd)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_with_particle_tractions(built, scheme):
    """A ramped traction on the top particle layer (both directions in turn):
    directional derivatives in E, x_0 and v_0 against central differences of
    the float64 NumPy oracle (the restated reverse passes with tractions are
    pinned against autograd on the CPU, tests/test_adjoint_restated.py)."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    for d, val in ((1, -2.0e3), (0, 1.5e3)):
        kw = dict(n=16, sim_steps=24, dt=dt, velocity=sheared, scheme=scheme, traction=(d, val))
        gs, sim, g, info = gpu_sim(**kw)
        n = info["np"]
        W, U = seeds(n, 17)
        sim.record(kw["sim_steps"], 10)
        got = sim.adjoint(W, U)
        rng = np.random.Generator(np.random.PCG64(23))
        E0 = info["E"]

        def loss(E=None, dx=None, dv=None):
            o, og, _ = workloads.differentiation(O, dtype=np.float64, E=E0 if E is None else E,
                                                 **dict(CASE, **kw))
            p = o.mesh.particles[0]
            if dx is not None:
                p.loc[:] = p.loc + dx.reshape(-1, 1, 2)
            if dv is not None:
                p.velocity[:] = p.velocity + dv.reshape(-1, 1, 2)
            for i in range(kw["sim_steps"]):
                o.step(i, og, reinit=True)
            return float((p.loc.reshape(-1, 2) * W).sum() + (p.velocity.reshape(-1, 2) * U).sum())

        for name, h, perturb, grad in (
                ("youngs_modulus", 1e-4, lambda u, s_: dict(E=E0 * (1 + s_ * u)), lambda u: (got["youngs_modulus"] * E0 * u).sum()),
                ("loc", 1e-6, lambda u, s_: dict(dx=s_ * u), lambda u: (got["loc"].reshape(-1) * u).sum()),
                ("velocity", 1e-4, lambda u, s_: dict(dv=s_ * u), lambda u: (got["velocity"].reshape(-1) * u).sum())):
            u = rng.normal(size=n if name == "youngs_modulus" else 2 * n)
            fd = (loss(**perturb(u, h)) - loss(**perturb(u, -h))) / (2 * h)
            gd = float(grad(u))
            # float32 adjoint against the float64 program's derivative
            tol = 2e-3 if name == "youngs_modulus" else 5e-3
            assert abs(gd - fd) <= tol * max(abs(fd), 1e-12), (d, name, gd, fd)
        sim.close()


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_with_particle_velocity_constraints(built, scheme):
    """Particle velocity constraints (one in x on every 7th particle, one in y
    on every 5th from the 4th): directional derivatives in E, x_0 and v_0
    against central differences of the float64 oracle, which applies the
    constraints after each particle velocity update like the GPU.  The
    constrained particles are dragged through the block, so the run is close
    to a change of cell assignment: the position differences use h = 1e-7
    (at 1e-6 some directions already cross one)."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    kw = dict(n=16, sim_steps=24, dt=dt, velocity=sheared, scheme=scheme)

    def build(api, **extra):
        s, g, info = workloads.differentiation(api, **dict(kw, **extra))
        n = info["np"]
        s.mesh.particle_velocity_constraints = [
            api.ParticleVelocityConstraint(pset=0, pids=np.arange(0, n, 7), dir=0, velocity=1.6),
            api.ParticleVelocityConstraint(pset=0, pids=np.arange(3, n, 5), dir=1, velocity=0.5)]
        return s, g, info

    gs, g, info = build(D)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    n = info["np"]
    W, U = seeds(n, 19)
    sim.record(kw["sim_steps"], 10)
    got = sim.adjoint(W, U)
    sim.close()
    E0 = info["E"]
    rng = np.random.Generator(np.random.PCG64(29))

    def loss(E=None, dx=None, dv=None):
        o, og, _ = build(O, dtype=np.float64, E=E0 if E is None else E)
        p = o.mesh.particles[0]
        if dx is not None:
            p.loc[:] = p.loc + dx.reshape(-1, 1, 2)
        if dv is not None:
            p.velocity[:] = p.velocity + dv.reshape(-1, 1, 2)
        for i in range(kw["sim_steps"]):
            o.step(i, og, reinit=True)
        return float((p.loc.reshape(-1, 2) * W).sum() + (p.velocity.reshape(-1, 2) * U).sum())

    for name, h, perturb, grad in (
            ("youngs_modulus", 1e-4, lambda u, s_: dict(E=E0 * (1 + s_ * u)), lambda u: (got["youngs_modulus"] * E0 * u).sum()),
            ("loc", 1e-7, lambda u, s_: dict(dx=s_ * u), lambda u: (got["loc"].reshape(-1) * u).sum()),
            ("velocity", 1e-6, lambda u, s_: dict(dv=s_ * u), lambda u: (got["velocity"].reshape(-1) * u).sum())):
        u = rng.normal(size=n if name == "youngs_modulus" else 2 * n)
        fd = (loss(**perturb(u, h)) - loss(**perturb(u, -h))) / (2 * h)
        gd = float(grad(u))
        tol = 2e-3 if name == "youngs_modulus" else 5e-3
        assert abs(gd - fd) <= tol * max(abs(fd), 1e-12), (name, gd, fd)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_solve_semantics(built, scheme):
    """solve semantics (no per-step volume set-up: constant mass, the volume
    carried from step to step): directional derivatives in E, x_0 and v_0
    against central differences of the float64 oracle stepped the same way."""
    dt = 1e-3 if scheme == "usf" else 2.5e-4
    kw = dict(n=16, sim_steps=24, dt=dt, velocity=sheared, scheme=scheme)
    gs, g, info = workloads.differentiation(D, **kw)
    sim = gs.simulation(g, reinit=False)
    gs._upload(sim)
    sim.initialize()
    n = info["np"]
    W, U = seeds(n, 31)
    sim.record(kw["sim_steps"], 10)
    got = sim.adjoint(W, U)
    sim.close()
    E0 = info["E"]
    rng = np.random.Generator(np.random.PCG64(37))

    def loss(E=None, dx=None, dv=None):
        o, og, _ = workloads.differentiation(O, dtype=np.float64, E=E0 if E is None else E, **kw)
        p = o.mesh.particles[0]
        if dx is not None:
            p.loc[:] = p.loc + dx.reshape(-1, 1, 2)
        if dv is not None:
            p.velocity[:] = p.velocity + dv.reshape(-1, 1, 2)
        for i in range(kw["sim_steps"]):
            o.step(i, og, reinit=False)
        return float((p.loc.reshape(-1, 2) * W).sum() + (p.velocity.reshape(-1, 2) * U).sum())

    for name, h, perturb, grad in (
            ("youngs_modulus", 1e-4, lambda u, s_: dict(E=E0 * (1 + s_ * u)), lambda u: (got["youngs_modulus"] * E0 * u).sum()),
            ("loc", 1e-7, lambda u, s_: dict(dx=s_ * u), lambda u: (got["loc"].reshape(-1) * u).sum()),
            ("velocity", 1e-6, lambda u, s_: dict(dv=s_ * u), lambda u: (got["velocity"].reshape(-1) * u).sum())):
        u = rng.normal(size=n if name == "youngs_modulus" else 2 * n)
        fd = (loss(**perturb(u, h)) - loss(**perturb(u, -h))) / (2 * h)
        gd = float(grad(u))
        tol = 2e-3 if name == "youngs_modulus" else 5e-3
        assert abs(gd - fd) <= tol * max(abs(fd), 1e-12), (name, gd, fd)


def test_adjoint_needs_a_current_recording(built):
    """(Every 2-D configuration is differentiable; the 1-D refusals are in
    test_gpu_line.py.)  The adjoint needs a recording that is still current."""
    gs, sim, g, info = gpu_sim()
    with pytest.raises(D.MpmError) as e:
        sim.adjoint(np.zeros((info["np"], 2), np.float32))
    assert e.value.code == 6
    sim.record(4, 2)
    sim.step(1)
    with pytest.raises(D.MpmError) as e:
        sim.adjoint(np.zeros((info["np"], 2), np.float32))
    assert e.value.code == 6


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_adjoint_newtonian_mixed(built, scheme):
    """Elastic and Newtonian particles in one population (the Newtonian stress
    is total: it reads the accumulated centroid volumetric strain, which the
    adjoint then carries): directional derivatives in E, x_0 and v_0 against
    central differences of the float64 oracle."""
    gs, g, E0 = mixed_newtonian(D, scheme)
    sim = gs.simulation(g, reinit=True)
    gs._upload(sim)
    sim.initialize()
    n = len(E0)
    W, U = seeds(n, 43)
    sim.record(24, 10)
    got = sim.adjoint(W, U)
    sim.close()
    rng = np.random.Generator(np.random.PCG64(47))

    def loss(E=None, dx=None, dv=None):
        o, og, _ = mixed_newtonian(O, scheme, dtype=np.float64, E=E0 if E is None else E)
        p = o.mesh.particles[0]
        if dx is not None:
            p.loc[:] = p.loc + dx.reshape(-1, 1, 2)
        if dv is not None:
            p.velocity[:] = p.velocity + dv.reshape(-1, 1, 2)
        for i in range(24):
            o.step(i, og, reinit=True)
        return float((p.loc.reshape(-1, 2) * W).sum() + (p.velocity.reshape(-1, 2) * U).sum())

    for name, h, perturb, grad in (
            ("youngs_modulus", 1e-4, lambda u, s_: dict(E=E0 * (1 + s_ * u)), lambda u: (got["youngs_modulus"] * E0 * u).sum()),
            ("loc", 1e-7, lambda u, s_: dict(dx=s_ * u), lambda u: (got["loc"].reshape(-1) * u).sum()),
            ("velocity", 1e-6, lambda u, s_: dict(dv=s_ * u), lambda u: (got["velocity"].reshape(-1) * u).sum())):
        u = rng.normal(size=n if name == "youngs_modulus" else 2 * n)
        fd = (loss(**perturb(u, h)) - loss(**perturb(u, -h))) / (2 * h)
        gd = float(grad(u))
        tol = 2e-3 if name == "youngs_modulus" else 5e-3
        assert abs(gd - fd) <= tol * max(abs(fd), 1e-12), (name, gd, fd)


@pytest.mark.parametrize("scheme", ["usf", "usl"])
def test_empty_tile_split_gives_the_same_bits(built, scheme):
    """A 64^2 mesh whose particles fill [0.1, 0.9] x [0, 0.6] has tiles that
    neither store nor can receive a particle in a step block.  Launched apart
    (their node update only) or through the step kernels with the other
    tiles, forward state and every gradient are bit for bit the same, with
    re-sorts between blocks (time steps within the explicit stability limit
    of the 64^2 cells)."""
    steps, dt, block = (60, 2.5e-4, 6) if scheme == "usf" else (160, 3e-5, 16)
    out = []
    for min_empty in (0, 2 ** 31 - 1):
        gs, sim, g, info = gpu_sim(block=block, scheme=scheme, n=64, sim_steps=steps, dt=dt)
        sim.set_empty_split(min_empty)
        W, U = seeds(info["np"])
        before = sim.counters()["resorts"]
        sim.record(steps, 20)
        assert sim.counters()["resorts"] > before
        state = {k: sim.read(k).copy() for k in ("loc", "velocity", "stress", "strain", "density")}
        out.append((state, sim.adjoint(W, U)))
        sim.close()
    (s0, a0), (s1, a1) = out
    for k in s0:
        assert np.array_equal(s0[k], s1[k]), k
    for k in a0:
        assert np.array_equal(a0[k], a1[k]), k
