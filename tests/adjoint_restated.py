"""NumPy float64 restatement of the hand-written adjoint -- TEST INFRASTRUCTURE.

The four reverse passes of diffmpm_gb300/csrc/mpm_adjoint_kernels.cu written
out with NumPy scatters, over a float64 forward that keeps the same tape (the
particle state at each step start, nodal mass, vA, vB, aB).  The CPU tests
check that this restatement equals torch autograd of ``oracle.mpm_torch``, so
the derivation the CUDA kernels implement is pinned without a GPU; the GPU
tests then compare the kernels with autograd directly.

Scope as the CUDA adjoint: USF or USL; the per-step volume set-up of
solve_jit or the carried volume and constant mass of solve (``reinit``
False: V' = V f carries its own adjoint, and the mass none); LinearElastic
or SimpleMaterial with a per-particle E and the build's Newtonian; gravity,
velocity constraints, concentrated nodal forces; particle tractions
(t = f(t) tau V / size: the shape-function adjoint gains F-bar . t and, where
the volume at force time varies, the volume adjoint N F-bar . t / V); and
particle velocity constraints (a held component of the end-of-step velocity
is a constant: its adjoint is cleared before the reverse passes).  USL
reverses in six passes (the order of the CUDA launches): U, the stress
update after G2P (strain-rate adjoints from the updated nodal velocities
vB); G, their transposed gather to the nodes; then passes 1-4 as for USF,
with the forces of pass 2 on the start-of-step stress and volume and no
strain-rate gather in pass 3.
"""
from __future__ import annotations

import numpy as np

from oracle.mpm_oracle import le_coefficients

FLUSH = 1e-12


def flush(a):
    return np.where(np.abs(a) < FLUSH, 0.0, a)


class Restated:
    def __init__(self, tsim, reinit=True):
        """``tsim``: an ``oracle.mpm_torch.TorchMPM`` (mesh, constraints,
        material); ``reinit``: solve_jit semantics (else solve's)."""
        self.reinit = reinit
        self.nx, self.ny = tsim.nx, tsim.ny
        self.node_x = tsim.node_x.numpy()
        self.node_y = tsim.node_y.numpy()
        self.dt = tsim.dt
        self.g = tsim.g.numpy()
        self.cmask = tsim.cmask.numpy()
        self.cval = tsim.cval.numpy()
        self.vol_el = float(tsim.vol_el)
        self.nn = tsim.nn
        self.vu = bool(tsim.velocity_update)
        assert tsim.scheme in ("usf", "usl")
        self.usl = tsim.scheme == "usl"
        # per-particle material parameters: LinearElastic coefficients of E, or
        # the Newtonian bulk modulus and viscosity (a total-stress material)
        mid = tsim.mat_ids.numpy()
        n = len(mid)
        self.c1, self.c2, self.c3 = np.zeros(n), np.zeros(n), np.zeros(n)
        self.newt, self.K, self.mu = np.zeros(n, bool), np.zeros(n), np.zeros(n)
        self.simple, self.Es = np.zeros(n, bool), np.zeros(n)
        for k, mat in enumerate(tsim.materials):
            sel = mid == k
            kind = type(mat).__name__
            if kind == "LinearElastic":
                c = le_coefficients(float(mat.properties["poisson_ratio"]))
                self.c1[sel], self.c2[sel], self.c3[sel] = c
            elif kind == "SimpleMaterial":   # sigma += E deps (E per particle if given)
                self.simple[sel] = True
                self.Es[sel] = float(mat.properties["E"])
            elif kind == "Newtonian":
                self.newt[sel] = True
                self.K[sel] = float(mat.properties["bulk_modulus"])
                self.mu[sel] = float(mat.properties["dynamic_viscosity"])
            else:
                raise NotImplementedError(kind)
        self.tractions = [(pids.numpy(), d, tau, fn) for pids, d, tau, fn in tsim.tractions]
        self.cnf = [(ids.numpy(), d, F, fn) for ids, d, F, fn in tsim.cnf]
        self.pcons = [(pids.numpy(), d, vel) for pids, d, vel in tsim.pcons]

    def geometry(self, x):
        i = np.searchsorted(self.node_x, x[:, 0], side="right") - 1
        j = np.searchsorted(self.node_y, x[:, 1], side="right") - 1
        x0, x1 = self.node_x[i], self.node_x[i + 1]
        y0, y1 = self.node_y[j], self.node_y[j + 1]
        rx, ry = 2.0 / (x1 - x0), 2.0 / (y1 - y0)
        xi = (x[:, 0] - (x0 + x1) / 2) * rx
        eta = (x[:, 1] - (y0 + y1) / 2) * ry
        ll = j * (self.nx + 1) + i
        ids = np.stack([ll, ll + 1, ll + self.nx + 2, ll + self.nx + 1], 1)
        a, b, c, d = 1 - xi, 1 + xi, 1 - eta, 1 + eta
        N = np.stack([0.25 * a * c, 0.25 * b * c, 0.25 * b * d, 0.25 * a * d], 1)
        Gx = np.stack([-0.25 * c, 0.25 * c, 0.25 * d, -0.25 * d], 1) * rx[:, None]
        Gy = np.stack([-0.25 * a, -0.25 * b, 0.25 * b, 0.25 * a], 1) * ry[:, None]
        Gcx = np.stack([-0.25 * rx, 0.25 * rx, 0.25 * rx, -0.25 * rx], 1)
        Gcy = np.stack([-0.25 * ry, -0.25 * ry, 0.25 * ry, 0.25 * ry], 1)
        e = j * self.nx + i
        return dict(e=e, ids=ids, N=N, Gx=Gx, Gy=Gy, Gcx=Gcx, Gcy=Gcy, rx=rx, ry=ry)

    def rates(self, G, nv):
        """Strain rates (xx, yy, xy) and centroid rates of nodal velocities nv."""
        ids = G["ids"]
        vx, vy = nv[ids, 0], nv[ids, 1]
        r0 = flush((G["Gx"] * vx).sum(1))
        r1 = flush((G["Gy"] * vy).sum(1))
        r3 = flush((G["Gx"] * vy).sum(1) + (G["Gy"] * vx).sum(1))
        c0 = flush((G["Gcx"] * vx).sum(1))
        c1 = flush((G["Gcy"] * vy).sum(1))
        return r0, r1, r3, c0, c1

    def stress(self, s, E, r0, r1, r3, vsc2):
        """Elastic increment, or the Newtonian total stress from the rates and
        the updated centroid volumetric strain vsc2."""
        dt = self.dt
        d0, d1, d3 = r0 * dt, r1 * dt, r3 * dt
        a1, a2, Gm = E * self.c1, E * self.c2, E * self.c3
        out = s + np.stack([a1 * d0 + a2 * d1, a2 * d0 + a1 * d1, a2 * d0 + a2 * d1, Gm * d3], 1)
        if self.simple.any():
            Es = E if E is not None else self.Es
            si = s + np.stack([Es * d0, Es * d1, 0 * d0, Es * d3], 1)
            out = np.where(self.simple[:, None], si, out)
        if self.newt.any():
            kv, t3, mu = self.K * vsc2, (r0 + r1) / 3.0, self.mu
            tot = np.stack([kv + 2 * mu * (r0 - t3), kv + 2 * mu * (r1 - t3), kv - 2 * mu * t3,
                            mu * r3], 1)
            out = np.where(self.newt[:, None], tot, out)
        return out

    def stress_reverse(self, sb, E, r0, r1, r3):
        """Rate adjoints (masked where a rate was flushed), dL/dE, the adjoint
        of the updated centroid volumetric strain and the particles whose
        stress is total (their start-of-step stress passes no adjoint)."""
        r0b, r1b, r3b, Eb = self.stress_reverse_elastic(sb, E, r0, r1, r3)
        if self.simple.any():
            Es = E if E is not None else self.Es
            dt, sm = self.dt, self.simple
            r0b = np.where(sm, np.where(r0 != 0, Es * sb[:, 0] * dt, 0.0), r0b)
            r1b = np.where(sm, np.where(r1 != 0, Es * sb[:, 1] * dt, 0.0), r1b)
            r3b = np.where(sm, np.where(r3 != 0, Es * sb[:, 3] * dt, 0.0), r3b)
            Eb = np.where(sm, r0 * dt * sb[:, 0] + r1 * dt * sb[:, 1] + r3 * dt * sb[:, 3], Eb)
        vscb = np.zeros_like(r0)
        if self.newt.any():
            tr = sb[:, 0] + sb[:, 1] + sb[:, 2]
            t3b = -2 * self.mu * tr
            nw = self.newt
            r0b = np.where(nw, np.where(r0 != 0, 2 * self.mu * sb[:, 0] + t3b / 3, 0.0), r0b)
            r1b = np.where(nw, np.where(r1 != 0, 2 * self.mu * sb[:, 1] + t3b / 3, 0.0), r1b)
            r3b = np.where(nw, np.where(r3 != 0, self.mu * sb[:, 3], 0.0), r3b)
            Eb = np.where(nw, 0.0, Eb)
            vscb = np.where(nw, self.K * tr, 0.0)
        return r0b, r1b, r3b, Eb, vscb, self.newt

    def stress_reverse_elastic(self, sb, E, r0, r1, r3):
        """D^T sb dt (masked where a rate was flushed) and dL/dE."""
        dt = self.dt
        d0, d1, d3 = r0 * dt, r1 * dt, r3 * dt
        a1, a2, Gm = E * self.c1, E * self.c2, E * self.c3
        d0b = a1 * sb[:, 0] + a2 * sb[:, 1] + a2 * sb[:, 2]
        d1b = a2 * sb[:, 0] + a1 * sb[:, 1] + a2 * sb[:, 2]
        d3b = Gm * sb[:, 3]
        Eb = (self.c1 * (d0 * sb[:, 0] + d1 * sb[:, 1])
              + self.c2 * (d1 * sb[:, 0] + d0 * sb[:, 1] + (d0 + d1) * sb[:, 2])
              + self.c3 * d3 * sb[:, 3])
        r0b = np.where(r0 != 0, d0b * dt, 0.0)
        r1b = np.where(r1 != 0, d1b * dt, 0.0)
        r3b = np.where(r3 != 0, d3b * dt, 0.0)
        return r0b, r1b, r3b, Eb

    def rate_gather(self, G, r0b, r1b, r3b, c0b, c1b):
        """Transposed strain-rate gather: nodal-velocity adjoint."""
        Gx, Gy, Gcx, Gcy = G["Gx"], G["Gy"], G["Gcx"], G["Gcy"]
        return self.scatter(G["ids"], np.stack([Gx * r0b[:, None] + Gy * r3b[:, None] + Gcx * c0b[:, None],
                                                Gy * r1b[:, None] + Gx * r3b[:, None] + Gcy * c1b[:, None]], 2))

    def scatter(self, ids, vals):
        out = np.zeros((self.nn,) + vals.shape[2:])
        np.add.at(out, ids.reshape(-1), vals.reshape((-1,) + vals.shape[2:]))
        return out

    # ------------------------------------------------------------------
    def forward(self, st, E, i=0):
        """One step; returns (new state, tape).  State: x (n,2), v (n,2),
        sig (n,4: xx yy zz xy), rho (n,), nv (nn,2); under solve semantics
        also vol (n,) and mass (n,)."""
        x, v, s, rho, nvo = st["x"], st["v"], st["sig"], st["rho"], st["nv"]
        G = self.geometry(x)
        ids, N, Gx, Gy = G["ids"], G["N"], G["Gx"], G["Gy"]
        if self.reinit:
            cnt = np.bincount(G["e"], minlength=self.nx * self.ny).astype(float)
            V0 = self.vol_el / cnt[G["e"]]
            m = V0 * rho
        else:
            V0, m = st["vol"], st["mass"]
        M = self.scatter(ids, m[:, None] * N)
        P = flush(self.scatter(ids, N[:, :, None] * (m[:, None] * v)[:, None, :]))
        safe = np.where(M == 0, 1.0, M)
        vA = np.where((M == 0)[:, None], nvo, P / safe[:, None])
        vA = np.where(self.cmask, self.cval, flush(vA))
        vsc = st["vsc"] if "vsc" in st else np.zeros_like(rho)
        if self.usl:   # forces on the start-of-step stress and volume
            s2, V, rho2 = s, V0, rho
        else:
            r0, r1, r3, c0, c1 = self.rates(G, vA)
            f = 1 + self.dt * (c0 + c1)
            vsc2 = vsc + self.dt * (c0 + c1)
            s2 = self.stress(s, E, r0, r1, r3, vsc2)
            V = V0 * f
            rho2 = rho / f
        Vend = V
        fx = Gx * s2[:, 0:1] + Gy * s2[:, 3:4]
        fy = Gy * s2[:, 1:2] + Gx * s2[:, 3:4]
        F = self.scatter(ids, np.stack([-V[:, None] * fx, -V[:, None] * fy], 2))
        F = F + self.scatter(ids, N[:, :, None] * (m[:, None] * self.g[None, :])[:, None, :])
        # concentrated nodal forces at step i (constants: no adjoint)
        for nid, d, Fv, fn in self.cnf:
            fval = 1.0 if fn is None else float(np.interp(float(np.float64(i) * self.dt), fn.xvalues,
                                                          fn.fxvalues))
            np.add.at(F[:, d], nid, fval * Fv)
        # particle tractions at step i: tq = sum f(t) tau / size, t = tq V
        tq = np.zeros_like(x)
        if self.tractions:
            size0 = np.sqrt(V0) if self.reinit else st["psize"]
            t = float(np.float64(i) * self.dt)
            for pids, d, tau, fn in self.tractions:
                fval = 1.0 if fn is None else float(np.interp(t, fn.xvalues, fn.fxvalues))
                np.add.at(tq[:, d], pids, (fval * tau) / size0[pids])
            F = F + self.scatter(ids, N[:, :, None] * (tq * V[:, None])[:, None, :])
        a = np.where((M == 0)[:, None], 0.0, F / safe[:, None])
        vB = vA + a * self.dt
        vB = flush(np.where(self.cmask, self.cval, vB))
        aB = flush(np.where(self.cmask, 0.0, a))
        vhat = (N[:, :, None] * vB[ids]).sum(1)
        ahat = (N[:, :, None] * aB[ids]).sum(1)
        v2 = vhat if self.vu else v + ahat * self.dt
        if self.pcons:
            v2 = v2.copy()
            for pids, d, vel in self.pcons:
                v2[pids, d] = vel
        x2 = x + vhat * self.dt
        if self.usl:   # stress update from vB at the start-of-step positions
            r0, r1, r3, c0, c1 = self.rates(G, vB)
            f = 1 + self.dt * (c0 + c1)
            vsc2 = vsc + self.dt * (c0 + c1)
            s2 = self.stress(s, E, r0, r1, r3, vsc2)
            rho2 = rho / f
            Vend = V0 * f
        tape = dict(x=x, v=v, sig=s, rho=rho, M=M, vA=vA, vB=vB, aB=aB, vol=V0, mass=m, tq=tq,
                    vsc=vsc)
        out = dict(x=x2, v=v2, sig=s2, rho=rho2, nv=vB, vsc=vsc2)
        if not self.reinit:
            out.update(vol=Vend, mass=m)
            if "psize" in st:
                out["psize"] = st["psize"]
        return out, tape

    # ------------------------------------------------------------------
    def reverse(self, tape, lam, E):
        """Reverse of one step: ``lam`` (x, v, sig, rho and vsc adjoints of the
        step's end state, and vol under solve semantics) -> adjoints of its
        start state; returns (lam, dL/dE part)."""
        dt = self.dt
        x, v, s, rho = tape["x"], tape["v"], tape["sig"], tape["rho"]
        M, vA, vB, aB = tape["M"], tape["vA"], tape["vB"], tape["aB"]
        G = self.geometry(x)
        ids, N, Gx, Gy = G["ids"], G["N"], G["Gx"], G["Gy"]
        live = (M != 0)[:, None]
        safe = np.where(M == 0, 1.0, M)
        V0, m = tape["vol"], tape["mass"]
        lvol = None if self.reinit else lam["vol"]
        lvsc = lam["vsc"] if "vsc" in lam else np.zeros_like(rho)
        if self.pcons:   # held velocity components are constants after G2P
            lam = dict(lam, v=lam["v"].copy())
            for pids, d, _ in self.pcons:
                lam["v"][pids, d] = 0.0
        sb = lam["sig"].copy()
        vBb = np.zeros((self.nn, 2))
        if self.usl:
            # pass U: the stress update after G2P; the stress adjoint passes
            # through to the start of the step
            r0, r1, r3, c0, c1 = self.rates(G, vB)
            f = 1 + dt * (c0 + c1)
            r0b, r1b, r3b, Eb, vscb, total = self.stress_reverse(sb, E, r0, r1, r3)
            sb[total] = 0.0   # a total stress: the start-of-step stress passes none
            lvsc = lvsc + vscb   # vsc' = vsc + dvol
            fb = -lam["rho"] * (rho / f) / f + lvsc
            if not self.reinit:   # V' = V0 f carries the volume to the next step
                fb = fb + lvol * V0
                lvol = lvol * f
            rhob = lam["rho"] / f
            c0b = np.where(c0 != 0, fb * dt, 0.0)
            c1b = np.where(c1 != 0, fb * dt, 0.0)
            # pass G: its transposed strain-rate gather (vB adjoint)
            vBb = self.rate_gather(G, r0b, r1b, r3b, c0b, c1b)
            s2, V, nvr = s, V0, vB
        # pass 1: transposed G2P, reverse nodal update
        gh = lam["x"] * dt + (lam["v"] if self.vu else 0.0)
        hh = np.zeros_like(gh) if self.vu else lam["v"] * dt
        vBb = vBb + self.scatter(ids, N[:, :, None] * gh[:, None, :])
        aBb = self.scatter(ids, N[:, :, None] * hh[:, None, :])
        wb = np.where(self.cmask | (vB == 0), 0.0, vBb) * live
        ab = (np.where(self.cmask | (aB == 0), 0.0, aBb) + wb * dt) * live
        Fb = ab / safe[:, None]
        Mb = -(ab * aB).sum(1) / safe
        # pass 2: forces (and the USF stress update)
        if not self.usl:
            r0, r1, r3, c0, c1 = self.rates(G, vA)
            f = 1 + dt * (c0 + c1)
            s2 = self.stress(s, E, r0, r1, r3, tape["vsc"] + dt * (c0 + c1))
            V = V0 * f
            nvr = vA
        fbx, fby = Fb[ids, 0], Fb[ids, 1]
        fg = fbx * self.g[0] + fby * self.g[1]
        Nb = (gh[:, None, 0] * vB[ids, 0] + gh[:, None, 1] * vB[ids, 1]
              + hh[:, None, 0] * aB[ids, 0] + hh[:, None, 1] * aB[ids, 1] + m[:, None] * fg)
        mb = (N * fg).sum(1)
        fx = Gx * s2[:, 0:1] + Gy * s2[:, 3:4]
        fy = Gy * s2[:, 1:2] + Gx * s2[:, 3:4]
        Vb = -(fbx * fx + fby * fy).sum(1)
        if self.tractions:   # F-bar . t, t = tq V
            tq = tape["tq"]
            tr = tq * V[:, None]
            Nb = Nb + fbx * tr[:, None, 0] + fby * tr[:, None, 1]
            Vb = Vb + (N * (fbx * tq[:, None, 0] + fby * tq[:, None, 1])).sum(1)
        sb[:, 0] -= V * (fbx * Gx).sum(1)
        sb[:, 1] -= V * (fby * Gy).sum(1)
        sb[:, 3] -= V * (fbx * Gy + fby * Gx).sum(1)
        Gxb = -V[:, None] * (fbx * s2[:, 0:1] + fby * s2[:, 3:4])
        Gyb = -V[:, None] * (fbx * s2[:, 3:4] + fby * s2[:, 1:2])
        if self.usl:
            if self.reinit:
                rhob = rhob + V0 * mb
            else:   # the forces used the start volume
                lvol = lvol + Vb
        else:
            r0b, r1b, r3b, Eb, vscb, total = self.stress_reverse(sb, E, r0, r1, r3)
            sb[total] = 0.0   # a total stress: the start-of-step stress passes none
            lvsc = lvsc + vscb   # vsc' = vsc + dvol
            Vt = Vb if self.reinit else Vb + lvol
            fb = Vt * V0 - lam["rho"] * (rho / f) / f + lvsc
            rhob = lam["rho"] / f + (V0 * mb if self.reinit else 0.0)
            if not self.reinit:
                lvol = Vt * f
            c0b = np.where(c0 != 0, fb * dt, 0.0)
            c1b = np.where(c1 != 0, fb * dt, 0.0)
        vx, vy = nvr[ids, 0], nvr[ids, 1]
        Gxb = Gxb + r0b[:, None] * vx + r3b[:, None] * vy
        Gyb = Gyb + r1b[:, None] * vy + r3b[:, None] * vx
        sgn = np.array([1.0, -1.0, 1.0, -1.0])
        rxy = 0.25 * G["rx"] * G["ry"]
        xb = lam["x"].copy()
        xb[:, 0] += (Nb * Gx).sum(1) + rxy * (Gyb * sgn).sum(1)
        xb[:, 1] += (Nb * Gy).sum(1) + rxy * (Gxb * sgn).sum(1)
        # pass 3: (USF) transposed strain-rate gather, reverse nodal velocity
        vAb = wb if self.usl else wb + self.rate_gather(G, r0b, r1b, r3b, c0b, c1b)
        ub = np.where(self.cmask | (vA == 0), 0.0, vAb) * live
        Qb = ub / safe[:, None]
        Mbt = Mb - (ub * vA).sum(1) / safe
        # pass 4: mass and momentum P2G
        t = Qb[ids, 0] * v[:, None, 0] + Qb[ids, 1] * v[:, None, 1] + Mbt[ids]
        mb2 = (N * t).sum(1)
        vb = (0.0 if self.vu else lam["v"]) + m[:, None] * np.stack(
            [(N * Qb[ids, 0]).sum(1), (N * Qb[ids, 1]).sum(1)], 1)
        if self.reinit:   # m = V0 rho (under solve semantics a constant)
            rhob = rhob + V0 * mb2
        xb[:, 0] += (m[:, None] * t * Gx).sum(1)
        xb[:, 1] += (m[:, None] * t * Gy).sum(1)
        out = dict(x=xb, v=vb, sig=sb, rho=rhob, vsc=lvsc)
        if not self.reinit:
            out["vol"] = lvol
        return out, Eb

    def gradient(self, st0, E, nsteps, dl_dx, dl_dv=None):
        """Forward ``nsteps`` steps keeping every tape, then the reverse sweep;
        returns dict(E, x, v) of gradients at the start."""
        tapes, st = [], dict(st0)
        for i in range(nsteps):
            st, tp = self.forward(st, E, i)
            tapes.append(tp)
        n = st0["x"].shape[0]
        dt = st0["x"].dtype
        lam = dict(x=np.array(dl_dx, dt), v=np.zeros((n, 2), dt) if dl_dv is None else np.array(dl_dv, dt),
                   sig=np.zeros((n, 4), dt), rho=np.zeros(n, dt))
        if not self.reinit:
            lam["vol"] = np.zeros(n, dt)
        gE = np.zeros(n, dt)
        for tp in reversed(tapes):
            lam, Eb = self.reverse(tp, lam, E)
            gE += Eb
        return dict(E=gE, x=lam["x"], v=lam["v"]), st
