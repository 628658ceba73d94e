"""Edge cases of the step on the GPU: no particles, one particle, particles
exactly on cell edges, on the mesh's right edge, and several particle sets of
different sizes (advanced as one population)."""
import numpy as np
import pytest

import diffmpm_gb300 as D
from oracle import mpm_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def block(api, pts, sets=None, steps=10, dt=1e-4, **kw):
    """A 10 x 10 mesh on [0, 1]^2 with the bottom fixed and particles at
    ``pts``; ``sets`` splits them into several particle sets (sizes)."""
    n, h = 10, 0.1
    mat = api.LinearElastic({"density": 1000, "youngs_modulus": 1e4, "poisson_ratio": 0.3})
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    bottom = (jj.reshape(-1) * (n + 1) + ii.reshape(-1))[jj.reshape(-1) == 0]
    cons = [(bottom, api.Constraint(0, 0.0)), (bottom, api.Constraint(1, 0.0))]
    el = api.Quadrilateral4Node((n, n), n * n, (h, h), cons, **kw)
    sizes = sets or [len(pts)]
    psets, o = [], 0
    for k in sizes:
        p = np.asarray(pts[o:o + k], np.float64).reshape(-1, 1, 2)
        psets.append(api.Particles(p, mat, np.zeros(k, dtype=np.int32), **kw))
        psets[-1].velocity[:] = np.array([0.05, -0.02]).reshape(1, 1, 2)
        o += k
    mesh = api.Mesh2D({"particles": psets, "elements": el, "particle_surface_traction": []})
    return api.MPMExplicit(mesh, dt, scheme="usf", sim_steps=steps), np.array([0.0, -9.81])


def test_no_particles(built):
    sim = D.Simulation((4, 4), (0.25, 0.25), 1e-3,
                       materials=[D.LinearElastic({"density": 1.0, "youngs_modulus": 1.0,
                                                   "poisson_ratio": 0.0})])
    sim.set_particles(np.zeros((0, 2), np.float32))
    sim.initialize()
    sim.step(7)
    assert sim.step_index == 7
    assert sim.read("loc").shape == (0, 2) and sim.read("stress").shape == (0, 6)
    sim.close()


def test_one_particle(built):
    pts = np.array([[0.43, 0.57]])
    gs, g = block(D, pts, steps=20)
    os_, _ = block(O, pts, steps=20)
    a, b = gs.solve_jit(g), os_.solve_jit(g)
    for k in ("loc", "velocity", "stress"):
        assert rel(a[k], b[k]) <= 1e-5, k


def test_particles_on_cell_edges(built):
    """Particles exactly on interior node lines x = float(i) * h belong to the
    cell above/right of the line (element.py:820-840), as in the oracle."""
    h = np.float32(0.1)
    xs = np.array([np.float32(3) * h, np.float32(5) * h, 0.45, 0.62], np.float64)
    ys = np.array([0.35, np.float32(4) * h, np.float32(6) * h, 0.55], np.float64)
    pts = np.stack([xs, ys], axis=1)
    gs, g = block(D, pts, steps=15)
    os_, _ = block(O, pts, steps=15)
    assert np.array_equal(gs.mesh.particles[0].element_ids, os_.mesh.particles[0].element_ids)
    a, b = gs.solve_jit(g), os_.solve_jit(g)
    for k in ("loc", "velocity", "stress"):
        assert rel(a[k], b[k]) <= 1e-5, k


def test_particle_on_the_right_edge_is_outside(built):
    """x = float(10) * h is the mesh's right edge: the reference gives it an
    element id past the mesh; this build reports it."""
    pts = np.array([[0.5, 0.5], [float(np.float32(10) * np.float32(0.1)), 0.5]])
    with pytest.raises(D.OutOfMeshError):
        block(D, pts, steps=2)


def test_ragged_particle_sets_are_one_population(built):
    """Three sets of 7, 1 and 24 particles step exactly like the same 32
    particles in one set (this build's semantics for several sets), which
    match the oracle run on the single set."""
    rng = np.random.Generator(np.random.PCG64(8))
    pts = rng.uniform(0.25, 0.75, size=(32, 2))
    many, g = block(D, pts, sets=[7, 1, 24], steps=25)
    one, _ = block(D, pts, steps=25)
    ref, _ = block(O, pts, steps=25)
    got = []
    for solver in (many, one):
        sim = solver.simulation(g, reinit=True)
        solver._upload(sim)
        sim.initialize()
        sim.step(25)
        got.append({k: sim.read(k) for k in ("loc", "velocity", "stress")})
    c = ref.solve_jit(g)
    for k in got[0]:
        assert np.array_equal(got[0][k], got[1][k]), k
        ref = np.asarray(c[k]).reshape(got[1][k].shape)
        if k == "stress":   # a loose, slowly moving cloud: stresses at round-off (1 mPa floor)
            assert np.linalg.norm(got[1][k] - ref) <= 1e-3 * np.sqrt(ref.size), k
        else:
            assert rel(got[1][k], ref) <= 1e-5, k
