"""Explicit MPM driver with the reference's surface (diffmpm/solver.py:19-222).

``MPMExplicit(mesh, dt, scheme, velocity_update, sim_steps, out_steps, out_dir,
writer_func)`` with ``solve_jit(gravity)`` and ``solve(gravity)``.  Every step
runs in the CUDA library (engine.Simulation); the Python objects hold the
initial state, as the reference's pytrees do.

* ``solve_jit`` is pure like the reference's: it starts from the objects'
  state, advances ``sim_steps`` steps with the per-step volume/mass set-up of
  the reference's ``lax.fori_loop`` (solver.py:100-111, 213), calls
  ``writer_func((arrays, i), None, out_dir=..., max_steps=...)`` after step i
  when ``i % out_steps == 0`` (solver.py:203-210) and returns the final
  ``{"loc", "velocity", "stress", "strain"}`` (solver.py:214-222).
* ``solve`` runs without the per-step set-up, records every step
  (solver.py:116-157) and leaves the final state in the objects.
"""
from __future__ import annotations

from collections import defaultdict

import numpy as np

from .engine import Simulation
from .writers import AsyncOutput
from .functions import Linear

_schemes = ("usf", "usl")


class SimulationLease:
    """Holds one pooled simulation (``MPMExplicit.lease_simulation``) and puts
    it back into its pool when released or garbage-collected."""

    def __init__(self, sim, pool):
        self.sim, self._pool = sim, pool

    def release(self):
        if self.sim is not None:
            self._pool.append(self.sim)
            self.sim = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class MPMExplicit:
    __particle_props = ("loc", "velocity", "stress", "strain")

    def __init__(self, mesh, dt, scheme="usf", velocity_update=False, sim_steps=1, out_steps=1,
                 out_dir="results/", writer_func=None):
        if scheme not in _schemes:
            raise ValueError(f"Please select scheme from {_schemes}. Found {scheme}")
        self.mesh = mesh
        self.dt = dt
        self.scheme = scheme
        self.velocity_update = velocity_update
        self.sim_steps = sim_steps
        self.out_steps = out_steps
        self.out_dir = out_dir
        self.writer_func = writer_func
        self._sims = {}
        self._idle = {}      # leased simulations returned to the pool, per key
        # the constructor's volume set-up (solver.py:81-85), run on the GPU
        sim = self.simulation(np.zeros(2), reinit=True)
        self._upload(sim)
        sim.initialize()
        self._pull_setup(sim)

    # ------------------------------------------------------------------
    def _population(self):
        sets = self.mesh.particles
        mats, mat_index = [], {}
        for p in sets:
            for m in p.materials:
                if id(m) not in mat_index:
                    mat_index[id(m)] = len(mats)
                    mats.append(m)
        offsets = np.cumsum([0] + [len(p) for p in sets])
        return sets, mats, mat_index, offsets

    def _functions(self):
        fns = []
        for f in list(self.mesh.elements.concentrated_nodal_forces) + list(self.mesh.particle_tractions):
            if isinstance(f.function, Linear) and all(f.function is not g for g in fns):
                fns.append(f.function)
        return fns

    def simulation(self, gravity, reinit=True) -> Simulation:
        """The GPU simulation for this configuration (cached per mode, scheme,
        velocity update and dt), with ``gravity`` set."""
        g = np.broadcast_to(np.asarray(gravity, dtype=np.float64).reshape(-1), (2,))
        key = (bool(reinit), self.scheme, bool(self.velocity_update), float(self.dt))
        if key not in self._sims:
            self._sims[key] = self._new_simulation(reinit, g)
        return self._with_gravity(self._sims[key], g)

    def _new_simulation(self, reinit, g) -> Simulation:
        el = self.mesh.elements
        _, mats, _, _ = self._population()
        sim = Simulation(
            el.nelements, el.el_len, self.dt, scheme=self.scheme,
            velocity_update=self.velocity_update, reinit_each_step=reinit, gravity=g,
            constraints=el.constraints, functions=self._functions(),
            nodal_forces=el.concentrated_nodal_forces, materials=mats,
            ndim=getattr(el, "ndim", 2))
        sim.gravity = tuple(g)
        return sim

    @staticmethod
    def _with_gravity(sim, g):
        if sim.gravity != tuple(g):
            sim.set_gravity(g)
            sim.gravity = tuple(g)
        return sim

    def lease_simulation(self, gravity, reinit=True) -> "SimulationLease":
        """A simulation of this configuration that no other lease holds: an
        idle one from this solver's pool, or a new one.  It goes back to the
        pool when the lease is released or garbage-collected, so that every
        recorded run (``record``) stays intact until its holder lets go --
        the autograd function takes one lease per forward."""
        g = np.broadcast_to(np.asarray(gravity, dtype=np.float64).reshape(-1), (2,))
        key = (bool(reinit), self.scheme, bool(self.velocity_update), float(self.dt))
        pool = self._idle.setdefault(key, [])
        sim = pool.pop() if pool else self._new_simulation(reinit, g)
        return SimulationLease(self._with_gravity(sim, g), pool)

    def _upload(self, sim: Simulation):
        sets, mats, mat_index, offsets = self._population()
        ndim = sim.ndim
        loc = np.concatenate([p.loc.reshape(len(p), ndim) for p in sets])
        mids = np.concatenate([np.asarray([mat_index[id(p.materials[k])] for k in p.material_ids],
                                          dtype=np.int32).reshape(-1) for p in sets])
        sim.set_particles(loc, mids)
        sim.write("velocity", np.concatenate([p.velocity.reshape(len(p), ndim) for p in sets]))
        sim.write("stress", np.concatenate([p.stress.reshape(len(p), 6) for p in sets]))
        sim.write("strain", np.concatenate([p.strain.reshape(len(p), 6) for p in sets]))
        sim.write("density", np.concatenate([p.density.reshape(-1) for p in sets]))
        sim.write("volumetric_strain_centroid",
                  np.concatenate([p.volumetric_strain_centroid.reshape(-1) for p in sets]))
        if any(p.youngs_modulus is not None for p in sets):
            E = []
            for p in sets:
                if p.youngs_modulus is not None:
                    E.append(p.youngs_modulus)
                else:
                    E.append(np.full(len(p), -1.0, dtype=np.float32))
            sim.write("youngs_modulus", np.concatenate(E))
        sim.write_nodal("velocity", self.mesh.elements.nodes.velocity.reshape(-1, ndim))
        pids, dirs, vals, fns = [], [], [], []
        for pt in self.mesh.particle_tractions:
            psets = pt.pset if isinstance(pt.pset, (list, tuple, np.ndarray)) else [pt.pset]
            ids = np.asarray(pt.pids, dtype=np.int64).reshape(-1)
            for s in psets:
                pids.extend((offsets[int(s)] + ids).tolist())
                dirs.extend([int(pt.dir)] * ids.size)
                vals.extend([float(pt.traction)] * ids.size)
                fns.extend([pt.function] * ids.size)
        if pids:
            sim.set_tractions(pids, dirs, vals, fns)
        pids, dirs, vals = [], [], []
        for pc in getattr(self.mesh, "particle_velocity_constraints", []):
            psets = pc.pset if isinstance(pc.pset, (list, tuple, np.ndarray)) else [pc.pset]
            ids = np.asarray(pc.pids, dtype=np.int64).reshape(-1)
            for s in psets:
                pids.extend((offsets[int(s)] + ids).tolist())
                dirs.extend([int(pc.dir)] * ids.size)
                vals.extend([float(pc.velocity)] * ids.size)
        if pids:
            sim.set_particle_velocity_constraints(pids, dirs, vals)

    def _pull_setup(self, sim: Simulation):
        sets, _, _, offsets = self._population()
        e = sim.read("element_ids")
        vol = sim.read("volume")
        mass = sim.read("mass")
        ndim = sim.ndim
        for k, p in enumerate(sets):
            sl = slice(offsets[k], offsets[k + 1])
            p.element_ids = e[sl].copy()
            p.volume = vol[sl].reshape(-1, 1, 1).copy()
            p.mass = mass[sl].reshape(-1, 1, 1).copy()
            size = np.sqrt(p.volume) if ndim == 2 else p.volume
            p.size = np.broadcast_to(size, p.loc.shape).astype(np.float32).copy()
        self.mesh.elements.volume[:] = self._element_volume()

    def _element_volume(self):
        """Element volume by the reference's formula (element.py:903-909), the
        value the library uses; in 1-D the element length x_{e+1} - x_e."""
        el = self.mesh.elements
        if getattr(el, "ndim", 2) == 1:
            x = el.nodes.loc.reshape(-1)
            return (x[1:] - x[:-1]).reshape(-1, 1, 1)
        a = c = np.float32(el.el_len[1])
        b = d = np.float32(el.el_len[0])
        p = q = np.sqrt(a * a + b * b)
        t = a * a + c * c - b * b - d * d
        return np.float32(0.25) * np.sqrt(np.float32(4) * p * p * q * q - t * t)

    def _arrays(self, sim: Simulation, squeeze_each=True, read=None):
        """The reference's output dict: per field, the sets' arrays stacked
        (solver.py:190-197, 214-222); ``read`` supplies the fields already
        read (original order), else they are read from ``sim``."""
        sets, _, _, offsets = self._population()
        out = {}
        for name in self.__particle_props:
            a = sim.read(name) if read is None else read[name]
            per = []
            for k, p in enumerate(sets):
                v = a[offsets[k]:offsets[k + 1]]
                shape = (len(p), 1, sim.ndim) if name in ("loc", "velocity") else (len(p), 6, 1)
                v = v.reshape(shape)
                per.append(v.squeeze() if squeeze_each else v)
            out[name] = np.array(per)
        return out

    # ------------------------------------------------------------------
    def solve_jit(self, gravity) -> dict:
        sim = self.simulation(gravity, reinit=True)
        self._upload(sim)
        sim.initialize()
        done = 0
        if self.writer_func is not None:
            # the output of step i is copied to pinned host memory behind the
            # next steps and written by a host thread (writers.AsyncOutput)
            out = AsyncOutput(sim, self.__particle_props,
                              lambda read: self._arrays(sim, read=read), self.writer_func,
                              out_dir=self.out_dir, max_steps=self.sim_steps)
            try:
                for i in range(0, self.sim_steps, self.out_steps):
                    sim.step(i + 1 - done)
                    done = i + 1
                    out.submit(i)
                sim.step(self.sim_steps - done)
            finally:
                out.close()
        else:
            sim.step(self.sim_steps)
        return {k: v.squeeze() for k, v in self._arrays(sim, squeeze_each=False).items()}

    def solve(self, gravity) -> dict:
        sim = self.simulation(gravity, reinit=False)
        self._upload(sim)
        sim.initialize()
        sets, _, _, offsets = self._population()
        result = defaultdict(list)
        for _ in range(self.sim_steps):
            sim.step(1)
            loc, vel = sim.read("loc"), sim.read("velocity")
            stress, strain = sim.read("stress"), sim.read("strain")
            for k, p in enumerate(sets):
                sl = slice(offsets[k], offsets[k + 1])
                result["position"].append(loc[sl].reshape(-1, 1, sim.ndim))
                result["velocity"].append(vel[sl].reshape(-1, 1, sim.ndim))
                result["stress"].append(stress[sl, :2])
                result["strain"].append(strain[sl, :2])
        for k, p in enumerate(sets):
            sl = slice(offsets[k], offsets[k + 1])
            p.loc = sim.read("loc")[sl].reshape(p.loc.shape)
            p.velocity = sim.read("velocity")[sl].reshape(p.velocity.shape)
            p.stress = sim.read("stress")[sl].reshape(p.stress.shape)
            p.strain = sim.read("strain")[sl].reshape(p.strain.shape)
            p.density = sim.read("density")[sl].reshape(p.density.shape)
        return {k: np.asarray(v) for k, v in result.items()}
