"""Differentiable restatement of the explicit MPM step -- TEST INFRASTRUCTURE.

A PyTorch (CPU, float64 or float32) restatement of the same step as ``oracle.mpm_oracle``
(and of the reference's diffmpm step it restates), written so that autograd
gives the exact discrete gradient of a loss with respect to the per-particle
Young's modulus and the initial particle state.  It is the gradient oracle of
the hand-written CUDA adjoint; ``tests/test_oracle_torch.py`` checks that its
forward agrees with the NumPy oracle run in float64, and the adjoint tests also
check it against central finite differences of that oracle.

Scope: Quadrilateral4Node mesh, USF or USL, the per-step volume set-up of
``solve_jit`` (diffmpm/solver.py:81-85, 100-111) or the carried volume and
constant mass of ``solve`` (``reinit=False``; diffmpm/solver.py:116-157,
particle.py:324-327), LinearElastic (per-particle E or the material's) and
SimpleMaterial and the build's Newtonian material (total stress from the
rate and the accumulated centroid volumetric strain), gravity, velocity
constraints, concentrated nodal forces,
particle tractions (t = f(t) tau V / size at force time, mesh.py:60-77,
particle.py:329-343) and the build's particle velocity constraints (set after
the particle velocity update, in list order).  Particle cell ids and counts are piecewise constant in
the positions and carry no gradient; so are the flush-to-zero masks.

The float32 form is the gradient oracle of the float32 GPU adjoint: the
reference's flush |a| < 1e-12 -> 0 has zero derivative, and a quantity that is
zero in exact arithmetic (the strain rate of a uniform velocity field) lands
below the threshold in float64 round-off (~1e-16) but above it in float32
(~1e-6), so float32 and float64 programs can differ in which paths carry
gradient.  Against float32 autograd the masks agree.
"""
from __future__ import annotations

import numpy as np
import torch

from .mpm_oracle import le_coefficients

FLUSH = 1e-12


def _flush(a):
    return torch.where(a.abs() < FLUSH, torch.zeros_like(a), a)


class TorchMPM:
    """One simulation: mesh, materials, boundary conditions; ``run`` advances a
    state dict of tensors ``x (N,2), v (N,2), sig (N,4: xx yy zz xy),
    eps (N,3: xx yy xy), rho (N,), vsc (N,)``, the persistent nodal velocity
    ``nv`` and, for solve semantics, ``vol (N,)``, ``mass (N,)`` and
    ``psize (N,)`` (the particle size of the set-up, which tractions divide by)."""

    def __init__(self, nx, ny, hx, hy, dt, gravity, constraints, materials, mat_ids,
                 scheme="usf", velocity_update=False, nodal_forces=(), tractions=(),
                 particle_constraints=(), dtype=torch.float64):
        self.nx, self.ny = nx, ny
        f = self.dtype = dtype
        self.hx, self.hy = float(hx), float(hy)
        # node coordinates as the reference forms them: float(i) * h in the
        # working precision (diffmpm/element.py:669-679)
        self.node_x = torch.arange(nx + 1, dtype=f) * torch.tensor(self.hx, dtype=f)
        self.node_y = torch.arange(ny + 1, dtype=f) * torch.tensor(self.hy, dtype=f)
        self.dt = float(dt)
        self.g = torch.tensor(np.broadcast_to(np.asarray(gravity, float).reshape(-1), (2,)), dtype=f)
        nn = (nx + 1) * (ny + 1)
        self.nn = nn
        # constraint masks/values in application order: last one wins per (node, dir)
        self.cmask = torch.zeros(nn, 2, dtype=torch.bool)
        self.cval = torch.zeros(nn, 2, dtype=f)
        for ids, d, vel in constraints:
            ids = torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1))
            self.cmask[ids, d] = True
            self.cval[ids, d] = float(vel)
        self.cnf = [(torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1)), d, float(F), fn)
                    for ids, d, F, fn in nodal_forces]
        # particle tractions (pids, dir, tau, function or None for Unit)
        self.tractions = [(torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1)), int(d),
                           float(tau), fn) for ids, d, tau, fn in tractions]
        # particle velocity constraints (pids, dir, velocity), later entries win
        self.pcons = [(torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1)), int(d),
                       float(vel)) for ids, d, vel in particle_constraints]
        a, b, c = self.hy, self.hx, self.hy
        p = np.sqrt(a * a + b * b)
        t = a * a + c * c - b * b - b * b
        self.vol_el = 0.25 * np.sqrt(4 * p * p * p * p - t * t)
        self.scheme = scheme
        self.velocity_update = velocity_update
        self.mat_ids = torch.as_tensor(np.asarray(mat_ids, dtype=np.int64))
        self.materials = materials

    # ------------------------------------------------------------------
    def _locate(self, x):
        with torch.no_grad():
            i = torch.searchsorted(self.node_x, x[:, 0].contiguous(), right=True) - 1
            j = torch.searchsorted(self.node_y, x[:, 1].contiguous(), right=True) - 1
        if ((i < 0) | (i >= self.nx) | (j < 0) | (j >= self.ny)).any():
            raise ValueError("particle outside the mesh")
        return i, j

    def _geometry(self, x):
        i, j = self._locate(x)
        e = j * self.nx + i
        x0, x1 = self.node_x[i], self.node_x[i + 1]
        y0, y1 = self.node_y[j], self.node_y[j + 1]
        rx, ry = 2.0 / (x1 - x0), 2.0 / (y1 - y0)
        xi = (x[:, 0] - (x0 + x1) / 2) * rx
        eta = (x[:, 1] - (y0 + y1) / 2) * ry
        ll = j * (self.nx + 1) + i
        ids = torch.stack([ll, ll + 1, ll + self.nx + 2, ll + self.nx + 1], dim=1)
        a, b, c, d = 1 - xi, 1 + xi, 1 - eta, 1 + eta
        N = torch.stack([0.25 * a * c, 0.25 * b * c, 0.25 * b * d, 0.25 * a * d], dim=1)
        Gx = torch.stack([-0.25 * c, 0.25 * c, 0.25 * d, -0.25 * d], dim=1) * rx[:, None]
        Gy = torch.stack([-0.25 * a, -0.25 * b, 0.25 * b, 0.25 * a], dim=1) * ry[:, None]
        Gcx = torch.stack([-0.25 * rx, 0.25 * rx, 0.25 * rx, -0.25 * rx], dim=1)
        Gcy = torch.stack([-0.25 * ry, -0.25 * ry, 0.25 * ry, 0.25 * ry], dim=1)
        return e, ids, N, Gx, Gy, Gcx, Gcy

    def _scatter(self, ids, vals):
        out = torch.zeros((self.nn,) + vals.shape[2:], dtype=vals.dtype)
        return out.index_add(0, ids.reshape(-1), vals.reshape((-1,) + vals.shape[2:]))

    def _constrain(self, v, a=None):
        v = torch.where(self.cmask, self.cval, v)
        if a is not None:
            a = torch.where(self.cmask, torch.zeros_like(a), a)
        return v, a

    def _stress(self, s, E, sr, dvol, vsc_new):
        """Stress update of particle.py:315-322 for the particle's material."""
        dt = self.dt
        d0, d1, d3 = sr[:, 0] * dt, sr[:, 1] * dt, sr[:, 2] * dt
        out = s.clone()
        for k, mat in enumerate(self.materials):
            sel = self.mat_ids == k
            if not bool(sel.any()):
                continue
            kind = type(mat).__name__
            if kind == "LinearElastic":
                c1, c2, c3 = le_coefficients(float(mat.properties["poisson_ratio"]))
                Ek = E[sel] if E is not None else torch.full((int(sel.sum()),),
                                                             float(mat.properties["youngs_modulus"]),
                                                             dtype=self.dtype)
                a1, a2, G = Ek * c1, Ek * c2, Ek * c3
                ds = torch.stack([a1 * d0[sel] + a2 * d1[sel], a2 * d0[sel] + a1 * d1[sel],
                                  a2 * d0[sel] + a2 * d1[sel], G * d3[sel]], dim=1)
            elif kind == "SimpleMaterial":
                # a per-particle E replaces the material's (as in the oracle)
                Es = E[sel] if E is not None else torch.full((int(sel.sum()),), float(mat.properties["E"]),
                                                             dtype=self.dtype)
                ds = torch.stack([d0[sel] * Es, d1[sel] * Es, torch.zeros_like(d0[sel]),
                                  d3[sel] * Es], dim=1)
            elif kind == "Newtonian":
                # the build's total stress: K vsc' I + 2 mu dev(rate), rate_zz = 0,
                # s_xy = mu rate_xy (oracle.mpm_oracle.Newtonian)
                K = float(mat.properties["bulk_modulus"])
                mu = float(mat.properties["dynamic_viscosity"])
                kv = K * vsc_new[sel]
                t3 = (sr[sel, 0] + sr[sel, 1]) / 3.0
                tot = torch.stack([kv + 2.0 * mu * (sr[sel, 0] - t3), kv + 2.0 * mu * (sr[sel, 1] - t3),
                                   kv - 2.0 * mu * t3, mu * sr[sel, 2]], dim=1)
                out = out.index_put((sel.nonzero()[:, 0],), tot)
                continue
            else:
                raise NotImplementedError(kind)
            out = out.index_put((sel.nonzero()[:, 0],), s[sel] + ds)
        return out

    def _strain(self, st, Gx, Gy, ids, vn, Gcx, Gcy):
        vx, vy = vn[ids, 0], vn[ids, 1]
        r0 = _flush((Gx * vx).sum(1))
        r1 = _flush((Gy * vy).sum(1))
        r3 = _flush((Gx * vy).sum(1) + (Gy * vx).sum(1))
        c0 = _flush((Gcx * vx).sum(1))
        c1 = _flush((Gcy * vy).sum(1))
        dvol = self.dt * (c0 + c1)
        return torch.stack([r0, r1, r3], dim=1), dvol

    def step(self, st, i, E=None, reinit=True):
        """One step, returns the new state dict: solve_jit's (R0 + scheme:
        volume V_el / count and mass V rho set up again) or, with ``reinit``
        False, solve's (the state's carried ``vol`` and constant ``mass``;
        the volume update V' = V (1 + dvol) is carried to the next step)."""
        x, v, s, eps, rho, vsc, nvo = (st[k] for k in ("x", "v", "sig", "eps", "rho", "vsc", "nv"))
        e, ids, N, Gx, Gy, Gcx, Gcy = self._geometry(x)
        if reinit:
            with torch.no_grad():
                cnt = torch.bincount(e, minlength=self.nx * self.ny).to(self.dtype)
            V0 = self.vol_el / cnt[e]
            m = V0 * rho
        else:
            V0, m = st["vol"], st["mass"]
        M = self._scatter(ids, m[:, None] * N)
        P = _flush(self._scatter(ids, (N[:, :, None] * (m[:, None] * v)[:, None, :])))
        safeM = torch.where(M == 0, torch.ones_like(M), M)
        vn = torch.where((M == 0)[:, None], nvo, P / safeM[:, None])
        vn, _ = self._constrain(_flush(vn))
        out = dict(st)
        V = V0
        if self.scheme == "usf":
            sr, dvol = self._strain(st, Gx, Gy, ids, vn, Gcx, Gcy)
            vsc = vsc + dvol
            s = self._stress(s, E, sr, dvol, vsc)
            eps = eps + sr * self.dt
            V = V0 * (1 + dvol)
            rho = rho / (1 + dvol)
        Vend = V
        fx = Gx * s[:, 0:1] + Gy * s[:, 3:4]
        fy = Gy * s[:, 1:2] + Gx * s[:, 3:4]
        fint = self._scatter(ids, torch.stack([-V[:, None] * fx, -V[:, None] * fy], dim=2))
        fext = self._scatter(ids, N[:, :, None] * (m[:, None] * self.g[None, :])[:, None, :])
        t = float(np.float64(i) * self.dt)
        if self.tractions:
            size0 = torch.sqrt(V0) if reinit else st["psize"]
            n = x.shape[0]
            cols = [torch.zeros(n, dtype=self.dtype), torch.zeros(n, dtype=self.dtype)]
            for pids, d, tau, fn in self.tractions:
                fval = 1.0 if fn is None else float(np.interp(t, fn.xvalues, fn.fxvalues))
                cols[d] = cols[d].index_add(0, pids, (fval * tau) * V[pids] / size0[pids])
            trac = torch.stack(cols, dim=1)
            fext = fext + self._scatter(ids, N[:, :, None] * trac[:, None, :])
        for nid, d, F, fn in self.cnf:
            fval = 1.0 if fn is None else float(np.interp(t, fn.xvalues, fn.fxvalues))
            col = torch.zeros(self.nn, 2, dtype=self.dtype)
            col[:, d] = torch.zeros(self.nn, dtype=self.dtype).index_add(
                0, nid, torch.full((nid.numel(),), fval * F, dtype=self.dtype))
            fext = fext + col
        tot = fint + fext
        a = torch.where((M == 0)[:, None], torch.zeros_like(tot), tot / safeM[:, None])
        vb = vn + a * self.dt
        vb, a = self._constrain(vb, a)
        vb, a = _flush(vb), _flush(a)
        vhat = (N[:, :, None] * vb[ids]).sum(1)
        ahat = (N[:, :, None] * a[ids]).sum(1)
        vp = vhat if self.velocity_update else v + ahat * self.dt
        if self.pcons:
            pmask = torch.zeros_like(vp, dtype=torch.bool)
            pval = torch.zeros_like(vp)
            for pids, d, vel in self.pcons:
                pmask[pids, d] = True
                pval[pids, d] = vel
            vp = torch.where(pmask, pval, vp)
        xp = x + vhat * self.dt
        if self.scheme == "usl":
            sr, dvol = self._strain(st, Gx, Gy, ids, vb, Gcx, Gcy)
            vsc = vsc + dvol
            s = self._stress(s, E, sr, dvol, vsc)
            eps = eps + sr * self.dt
            Vend = V0 * (1 + dvol)
            rho = rho / (1 + dvol)
        out.update(x=xp, v=vp, sig=s, eps=eps, rho=rho, vsc=vsc, nv=vb)
        if not reinit:
            out.update(vol=Vend, mass=m)
        return out

    def run(self, st, nsteps, E=None, start=0, reinit=True):
        for i in range(start, start + nsteps):
            st = self.step(st, i, E, reinit)
        return st


def from_solver(solver, gravity, dtype=torch.float64):
    """TorchMPM and initial state dict from an ``oracle.mpm_oracle``
    MPMExplicit built for one particle set (float64, or float32 with
    ``dtype=torch.float32`` for the float32 discrete program)."""
    el = solver.mesh.elements
    ps = solver.mesh.particles[0]
    nx, ny = el.nelements
    cons = [(ids, c.dir, c.velocity) for ids, c in el.constraints]
    nfs = [(f.node_ids, f.dir, f.force, None if type(f.function).__name__ == "Unit" else f.function)
           for f in el.concentrated_nodal_forces]
    trs = [(t.pids, t.dir, t.traction, None if type(t.function).__name__ == "Unit" else t.function)
           for t in solver.mesh.particle_tractions]
    pcs = [(c.pids, c.dir, c.velocity) for c in solver.mesh.particle_velocity_constraints]
    sim = TorchMPM(nx, ny, float(el.el_len[0]), float(el.el_len[1]), solver.dt, gravity, cons,
                   ps.materials, ps.material_ids, scheme=solver.scheme,
                   velocity_update=solver.velocity_update, nodal_forces=nfs, tractions=trs,
                   particle_constraints=pcs, dtype=dtype)
    f = dtype
    n = len(ps)
    s = ps.stress.reshape(n, 6)
    e = ps.strain.reshape(n, 6)
    st = {
        "x": torch.tensor(ps.loc.reshape(n, 2), dtype=f),
        "v": torch.tensor(ps.velocity.reshape(n, 2), dtype=f),
        "sig": torch.tensor(np.stack([s[:, 0], s[:, 1], s[:, 2], s[:, 3]], 1), dtype=f),
        "eps": torch.tensor(np.stack([e[:, 0], e[:, 1], e[:, 3]], 1), dtype=f),
        "rho": torch.tensor(ps.density.reshape(n), dtype=f),
        "vsc": torch.tensor(ps.volumetric_strain_centroid.reshape(n), dtype=f),
        "nv": torch.tensor(el.nodes.velocity.reshape(-1, 2), dtype=f),
        # the set-up of the constructor (solver.py:81-85), which solve carries
        "vol": torch.tensor(ps.volume.reshape(n), dtype=f),
        "mass": torch.tensor(ps.mass.reshape(n), dtype=f),
        "psize": torch.tensor(ps.size.reshape(n, -1)[:, 0], dtype=f),
    }
    return sim, st


class TorchLine:
    """The 1-D step (Linear1D elements on [0, nx h], one particle set) in the
    same terms as ``TorchMPM``, for autograd of the 1-D runs: the oracle's
    Linear1D semantics (element volume = its length, strain rate
    ``[dN/dx . v, 0, 0, 0, 0, 0]``, centroid rate equal to it), USF or USL,
    solve_jit or solve semantics, LinearElastic and SimpleMaterial (material or
    per-particle E) and the build's Newtonian, gravity, node constraints,
    concentrated nodal forces and particle velocity constraints.  State:
    ``x, v (N,), sig (N,4), rho, vsc (N,), nv (nn,)`` and, for solve semantics,
    ``vol, mass (N,)``."""

    def __init__(self, nx, h, dt, gravity, constraints, materials, mat_ids, scheme="usf",
                 velocity_update=False, nodal_forces=(), particle_constraints=(), dtype=torch.float64):
        self.nx, self.dtype = nx, dtype
        self.node_x = torch.arange(nx + 1, dtype=dtype) * torch.tensor(float(h), dtype=dtype)
        self.dt = float(dt)
        self.g = float(np.asarray(gravity, float).reshape(-1)[0])
        self.nn = nx + 1
        self.cmask = torch.zeros(self.nn, dtype=torch.bool)
        self.cval = torch.zeros(self.nn, dtype=dtype)
        for ids, d, vel in constraints:
            ids = torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1))
            self.cmask[ids] = True
            self.cval[ids] = float(vel)
        self.cnf = [(torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1)), float(F), fn)
                    for ids, d, F, fn in nodal_forces]
        self.pcons = [(torch.as_tensor(np.asarray(ids, dtype=np.int64).reshape(-1)), float(vel))
                      for ids, d, vel in particle_constraints]
        self.scheme, self.velocity_update = scheme, velocity_update
        self.mat_ids = torch.as_tensor(np.asarray(mat_ids, dtype=np.int64))
        self.materials = materials

    def _geometry(self, x):
        with torch.no_grad():
            e = torch.searchsorted(self.node_x, x.contiguous(), right=True) - 1
        if ((e < 0) | (e >= self.nx)).any():
            raise ValueError("particle outside the mesh")
        x0, x1 = self.node_x[e], self.node_x[e + 1]
        r = 2.0 / (x1 - x0)
        xi = (x - (x0 + x1) / 2) * r
        N = torch.stack([0.5 * (1 - xi), 0.5 * (1 + xi)], dim=1)
        dN = torch.stack([-0.5 * r, 0.5 * r], dim=1)
        return e, torch.stack([e, e + 1], dim=1), N, dN, x1 - x0

    def _scatter(self, ids, vals):
        return torch.zeros(self.nn, dtype=vals.dtype).index_add(0, ids.reshape(-1), vals.reshape(-1))

    def _stress(self, s, E, r, vsc_new):
        dt = self.dt
        d0 = r * dt
        out = s.clone()
        for k, mat in enumerate(self.materials):
            sel = self.mat_ids == k
            if not bool(sel.any()):
                continue
            kind = type(mat).__name__
            if kind == "LinearElastic":
                c1, c2, _ = le_coefficients(float(mat.properties["poisson_ratio"]))
                Ek = E[sel] if E is not None else torch.full((int(sel.sum()),),
                                                             float(mat.properties["youngs_modulus"]),
                                                             dtype=self.dtype)
                a1, a2 = Ek * c1, Ek * c2
                new = s[sel] + torch.stack([a1 * d0[sel], a2 * d0[sel], a2 * d0[sel],
                                            torch.zeros_like(d0[sel])], dim=1)
            elif kind == "SimpleMaterial":
                Es = E[sel] if E is not None else torch.full((int(sel.sum()),), float(mat.properties["E"]),
                                                             dtype=self.dtype)
                z = torch.zeros_like(d0[sel])
                new = s[sel] + torch.stack([Es * d0[sel], z, z, z], dim=1)
            elif kind == "Newtonian":
                K = float(mat.properties["bulk_modulus"])
                mu = float(mat.properties["dynamic_viscosity"])
                kv, t3 = K * vsc_new[sel], r[sel] / 3.0
                new = torch.stack([kv + 2.0 * mu * (r[sel] - t3), kv - 2.0 * mu * t3,
                                   kv - 2.0 * mu * t3, torch.zeros_like(kv)], dim=1)
            else:
                raise NotImplementedError(kind)
            out = out.index_put((sel.nonzero()[:, 0],), new)
        return out

    def step(self, st, i, E=None, reinit=True):
        x, v, s, rho, vsc, nvo = (st[k] for k in ("x", "v", "sig", "rho", "vsc", "nv"))
        e, ids, N, dN, length = self._geometry(x)
        if reinit:
            with torch.no_grad():
                cnt = torch.bincount(e, minlength=self.nx).to(self.dtype)
            V0 = length / cnt[e]
            m = V0 * rho
        else:
            V0, m = st["vol"], st["mass"]
        M = self._scatter(ids, m[:, None] * N)
        P = _flush(self._scatter(ids, N * (m * v)[:, None]))
        safeM = torch.where(M == 0, torch.ones_like(M), M)
        vA = _flush(torch.where(M == 0, nvo, P / safeM))
        vA = torch.where(self.cmask, self.cval, vA)

        def rate(nvel):
            return _flush((dN * nvel[ids]).sum(1))

        V = V0
        Vend = V0
        if self.scheme == "usf":
            r = rate(vA)
            dvol = self.dt * r
            vsc = vsc + dvol
            s = self._stress(s, E, r, vsc)
            V = V0 * (1 + dvol)
            Vend = V
            rho = rho / (1 + dvol)
        fint = self._scatter(ids, (-V * s[:, 0])[:, None] * dN)
        fext = self._scatter(ids, N * (m * self.g)[:, None])
        t = float(np.float64(i) * self.dt)
        for nid, F, fn in self.cnf:
            fval = 1.0 if fn is None else float(np.interp(t, fn.xvalues, fn.fxvalues))
            fext = fext + torch.zeros(self.nn, dtype=self.dtype).index_add(
                0, nid, torch.full((nid.numel(),), fval * F, dtype=self.dtype))
        tot = fint + fext
        a = torch.where(M == 0, torch.zeros_like(tot), tot / safeM)
        vb = vA + a * self.dt
        vb = _flush(torch.where(self.cmask, self.cval, vb))
        a = _flush(torch.where(self.cmask, torch.zeros_like(a), a))
        vhat = (N * vb[ids]).sum(1)
        ahat = (N * a[ids]).sum(1)
        vp = vhat if self.velocity_update else v + ahat * self.dt
        for pids, vel in self.pcons:
            vp = vp.index_put((pids,), torch.full((pids.numel(),), vel, dtype=self.dtype))
        xp = x + vhat * self.dt
        if self.scheme == "usl":
            r = rate(vb)
            dvol = self.dt * r
            vsc = vsc + dvol
            s = self._stress(s, E, r, vsc)
            Vend = V0 * (1 + dvol)
            rho = rho / (1 + dvol)
        out = dict(st, x=xp, v=vp, sig=s, rho=rho, vsc=vsc, nv=vb)
        if not reinit:
            out.update(vol=Vend, mass=m)
        return out

    def run(self, st, nsteps, E=None, start=0, reinit=True):
        for i in range(start, start + nsteps):
            st = self.step(st, i, E, reinit)
        return st


def from_line_solver(solver, gravity, dtype=torch.float64):
    """TorchLine and initial state from an ``oracle.mpm_oracle`` MPMExplicit
    on a Linear1D mesh with one particle set."""
    el = solver.mesh.elements
    ps = solver.mesh.particles[0]
    cons = [(ids, c.dir, c.velocity) for ids, c in el.constraints]
    nfs = [(f.node_ids, f.dir, f.force, None if type(f.function).__name__ == "Unit" else f.function)
           for f in el.concentrated_nodal_forces]
    pcs = [(c.pids, c.dir, c.velocity) for c in solver.mesh.particle_velocity_constraints]
    sim = TorchLine(el.nx, float(el.el_len), solver.dt, gravity, cons, ps.materials, ps.material_ids,
                    scheme=solver.scheme, velocity_update=solver.velocity_update, nodal_forces=nfs,
                    particle_constraints=pcs, dtype=dtype)
    n = len(ps)
    s = ps.stress.reshape(n, 6)
    f = dtype
    st = {
        "x": torch.tensor(ps.loc.reshape(n), dtype=f),
        "v": torch.tensor(ps.velocity.reshape(n), dtype=f),
        "sig": torch.tensor(np.stack([s[:, 0], s[:, 1], s[:, 2], s[:, 3]], 1), dtype=f),
        "rho": torch.tensor(ps.density.reshape(n), dtype=f),
        "vsc": torch.tensor(ps.volumetric_strain_centroid.reshape(n), dtype=f),
        "nv": torch.tensor(el.nodes.velocity.reshape(-1), dtype=f),
        "vol": torch.tensor(ps.volume.reshape(n), dtype=f),
        "mass": torch.tensor(ps.mass.reshape(n), dtype=f),
    }
    return sim, st
