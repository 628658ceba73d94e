"""NumPy float64 restatement of the hand-written 1-D adjoint -- TEST INFRASTRUCTURE.

The reverse passes of diffmpm_gb300/csrc/mpm_line_adjoint.cu (Linear1D
elements) written out with NumPy over a float64 forward that keeps the same
tape (each step's start state and its nodal mass, velocity after kinematics,
velocity and acceleration after the update).  The CPU tests check it against
torch autograd of ``oracle.mpm_torch.TorchLine``, so the derivation the 1-D
kernels implement is pinned without a GPU.

Per reversed step, as the kernels run it (particles in original order):
0 (USL) the stress update after G2P; 1 G2P; 2 transposed G2P (+ the USL
strain-rate gather) and the nodal update; 3 the forces (+ the USF stress
update); 4 (USF) the transposed strain-rate gather and the nodal velocity;
5 the mass and momentum sums and, under solve_jit semantics, m = V0 rho.
Scope as the kernels: USF or USL, solve_jit or solve semantics,
LinearElastic and SimpleMaterial (material or per-particle E), the build's
Newtonian, gravity, node constraints, concentrated nodal forces, particle
velocity constraints.
"""
from __future__ import annotations

import numpy as np

from oracle.mpm_oracle import le_coefficients

FLUSH = 1e-12


def flush(a):
    return np.where(np.abs(a) < FLUSH, 0.0, a)


class LineRestated:
    def __init__(self, tl, reinit=True):
        """``tl``: an ``oracle.mpm_torch.TorchLine``; ``reinit``: solve_jit
        semantics (else solve's)."""
        self.reinit = reinit
        self.nx, self.nn = tl.nx, tl.nn
        self.node_x = tl.node_x.numpy()
        self.dt, self.g = tl.dt, tl.g
        self.cmask, self.cval = tl.cmask.numpy(), tl.cval.numpy()
        self.cnf = [(ids.numpy(), F, fn) for ids, F, fn in tl.cnf]
        self.pcons = [(ids.numpy(), vel) for ids, vel in tl.pcons]
        self.usl = tl.scheme == "usl"
        self.vu = bool(tl.velocity_update)
        mid = tl.mat_ids.numpy()
        n = len(mid)
        self.kind = np.zeros(n, int)           # 0 LinearElastic, 1 Simple, 2 Newtonian
        self.c1, self.c2 = np.zeros(n), np.zeros(n)
        self.Emat, self.K, self.mu = np.zeros(n), np.zeros(n), np.zeros(n)
        for k, mat in enumerate(tl.materials):
            sel = mid == k
            name = type(mat).__name__
            if name == "LinearElastic":
                c1, c2, _ = le_coefficients(float(mat.properties["poisson_ratio"]))
                self.c1[sel], self.c2[sel] = c1, c2
                self.Emat[sel] = float(mat.properties["youngs_modulus"])
            elif name == "SimpleMaterial":
                self.kind[sel] = 1
                self.Emat[sel] = float(mat.properties["E"])
            else:
                self.kind[sel] = 2
                self.K[sel] = float(mat.properties["bulk_modulus"])
                self.mu[sel] = float(mat.properties["dynamic_viscosity"])

    def geometry(self, x):
        e = np.searchsorted(self.node_x, x, side="right") - 1
        x0, x1 = self.node_x[e], self.node_x[e + 1]
        r = 2.0 / (x1 - x0)
        xi = (x - (x0 + x1) / 2) * r
        N = np.stack([0.5 * (1 - xi), 0.5 * (1 + xi)], 1)
        dN = np.stack([-0.5 * r, 0.5 * r], 1)
        return e, np.stack([e, e + 1], 1), N, dN, x1 - x0

    def scatter(self, ids, vals):
        out = np.zeros(self.nn)
        np.add.at(out, ids.reshape(-1), vals.reshape(-1))
        return out

    def stress(self, s, E, r, vsc2):
        d0 = r * self.dt
        Ep = self.Emat if E is None else E
        le = s + np.stack([Ep * self.c1 * d0, Ep * self.c2 * d0, Ep * self.c2 * d0, 0 * d0], 1)
        si = s + np.stack([Ep * d0, 0 * d0, 0 * d0, 0 * d0], 1)
        kv, t3 = self.K * vsc2, r / 3.0
        nw = np.stack([kv + 2 * self.mu * (r - t3), kv - 2 * self.mu * t3, kv - 2 * self.mu * t3, 0 * kv], 1)
        k = self.kind[:, None]
        return np.where(k == 0, le, np.where(k == 1, si, nw))

    # ------------------------------------------------------------------
    def forward(self, st, E, i=0):
        x, v, s, rho, vsc, nvo = st["x"], st["v"], st["sig"], st["rho"], st["vsc"], st["nv"]
        e, ids, N, dN, length = self.geometry(x)
        if self.reinit:
            cnt = np.bincount(e, minlength=self.nx).astype(float)
            V0 = length / cnt[e]
            m = V0 * rho
        else:
            V0, m = st["vol"], st["mass"]
        M = self.scatter(ids, m[:, None] * N)
        P = flush(self.scatter(ids, N * (m * v)[:, None]))
        safe = np.where(M == 0, 1.0, M)
        vA = flush(np.where(M == 0, nvo, P / safe))
        vA = np.where(self.cmask, self.cval, vA)
        rate = lambda nv: flush((dN * nv[ids]).sum(1))   # noqa: E731
        s2, V, Vend, rho2, vsc2 = s, V0, V0, rho, vsc
        if not self.usl:
            r = rate(vA)
            vsc2 = vsc + self.dt * r
            s2 = self.stress(s, E, r, vsc2)
            V = Vend = V0 * (1 + self.dt * r)
            rho2 = rho / (1 + self.dt * r)
        F = self.scatter(ids, (-V * s2[:, 0])[:, None] * dN) + self.scatter(ids, N * (m * self.g)[:, None])
        t = float(np.float64(i) * self.dt)
        for nid, Fv, fn in self.cnf:
            fval = 1.0 if fn is None else float(np.interp(t, fn.xvalues, fn.fxvalues))
            np.add.at(F, nid, fval * Fv)
        a = np.where(M == 0, 0.0, F / safe)
        vB = flush(np.where(self.cmask, self.cval, vA + a * self.dt))
        a = flush(np.where(self.cmask, 0.0, a))
        vhat = (N * vB[ids]).sum(1)
        ahat = (N * a[ids]).sum(1)
        v2 = vhat if self.vu else v + ahat * self.dt
        if self.pcons:
            v2 = v2.copy()
            for pids, vel in self.pcons:
                v2[pids] = vel
        x2 = x + vhat * self.dt
        if self.usl:
            r = rate(vB)
            vsc2 = vsc + self.dt * r
            s2 = self.stress(s, E, r, vsc2)
            Vend = V0 * (1 + self.dt * r)
            rho2 = rho / (1 + self.dt * r)
        tape = dict(x=x, v=v, sig=s, rho=rho, vsc=vsc, vol=V0, mass=m, M=M, vA=vA, vB=vB, a=a)
        out = dict(x=x2, v=v2, sig=s2, rho=rho2, vsc=vsc2, nv=vB)
        if not self.reinit:
            out.update(vol=Vend, mass=m)
        return out, tape

    # ------------------------------------------------------------------
    def rev_stress(self, L, tape, E, G, nv, sb, Vb):
        """Reverse of the strain / volume / density / stress update driven by
        the nodal velocities ``nv``: updates the particle adjoints ``L`` (to
        the start of the update) and returns the rate adjoint."""
        dt = self.dt
        e, ids, N, dN = G
        r = flush((dN * nv[ids]).sum(1))
        f = 1 + dt * r
        d0 = r * dt
        Ep = self.Emat if E is None else E
        k = self.kind
        rb_le = dt * (Ep * self.c1 * sb[:, 0] + Ep * self.c2 * sb[:, 1] + Ep * self.c2 * sb[:, 2])
        Eb_le = d0 * (self.c1 * sb[:, 0] + self.c2 * sb[:, 1] + self.c2 * sb[:, 2])
        rb_si, Eb_si = dt * Ep * sb[:, 0], d0 * sb[:, 0]
        tr = sb[:, 0] + sb[:, 1] + sb[:, 2]
        rb_nw = 2 * self.mu * sb[:, 0] - 2 * self.mu * tr / 3.0
        rb = np.where(k == 0, rb_le, np.where(k == 1, rb_si, rb_nw))
        Eb = np.where(k == 0, Eb_le, np.where(k == 1, Eb_si, 0.0))
        vscb = np.where(k == 2, self.K * tr, 0.0)
        total = k == 2
        V0, rho0 = tape["vol"], tape["rho"]
        Vt = Vb if self.reinit else Vb + L["vol"]
        fb = V0 * Vt - L["rho"] * (rho0 / f) / f
        vsc1 = L["vsc"] + vscb
        rb = rb + dt * (fb + vsc1)
        rb = np.where(r == 0, 0.0, rb)
        L["rho"] = L["rho"] / f
        L["vsc"] = vsc1
        if not self.reinit:
            L["vol"] = Vt * f
        L["sig"] = np.where(total[:, None], 0.0, sb)
        L["E"] = L["E"] + Eb
        return rb

    def reverse(self, tape, L, E):
        """Reverse of one step: ``L`` (x, v, sig, rho, vsc, E and, under solve
        semantics, vol adjoints of the step's end state) -> the start's."""
        dt = self.dt
        L = {k: np.array(v, copy=True) for k, v in L.items()}
        x, v, rho = tape["x"], tape["v"], tape["rho"]
        M, vA, vB, a = tape["M"], tape["vA"], tape["vB"], tape["a"]
        e, ids, N, dN, length = self.geometry(x)
        G = (e, ids, N, dN)
        nz = np.zeros(len(x))
        rU = self.rev_stress(L, tape, E, G, vB, L["sig"], nz) if self.usl else nz
        # pass 1: G2P
        lv = L["v"].copy()
        for pids, _ in self.pcons:
            lv[pids] = 0.0
        gh = L["x"] * dt + (lv if self.vu else 0.0)
        hh = 0.0 * gh if self.vu else lv * dt
        X = L["x"] + gh * (dN * vB[ids]).sum(1) + hh * (dN * a[ids]).sum(1)
        Vv = 0.0 * lv if self.vu else lv
        # pass 2: transposed G2P (+ USL rate gather), nodal update
        vbb = self.scatter(ids, N * gh[:, None]) + self.scatter(ids, dN * rU[:, None])
        ab = self.scatter(ids, N * hh[:, None])
        vbb = np.where(self.cmask | (vB == 0), 0.0, vbb)
        ab = np.where(self.cmask | (a == 0), 0.0, ab)
        at = ab + vbb * dt
        ok = (M != 0) & (at != 0)
        safe = np.where(M == 0, 1.0, M)
        Fb = np.where(ok, at / safe, 0.0)
        Mb = np.where(ok, -(at * a) / safe, 0.0)
        # pass 3: forces (+ USF stress update)
        V0 = tape["vol"]
        m = tape["mass"]
        SF = (N * Fb[ids]).sum(1)
        SD = (dN * Fb[ids]).sum(1)
        xb = X + m * self.g * SD
        mb = self.g * SF
        if self.usl:
            sxx, V = tape["sig"][:, 0], V0
            L["sig"] = L["sig"].copy()
            L["sig"][:, 0] += -V * SD
            if not self.reinit:
                L["vol"] = L["vol"] + (-sxx * SD)
            rF = nz
        else:
            r = flush((dN * vA[ids]).sum(1))
            s2 = self.stress(tape["sig"], E, r, tape["vsc"] + dt * r)
            sxx, V = s2[:, 0], V0 * (1 + dt * r)
            sb = L["sig"].copy()
            sb[:, 0] += -V * SD
            rF = self.rev_stress(L, tape, E, G, vA, sb, -sxx * SD)
        # pass 4: (USF) transposed rate gather, reverse nodal velocity
        vab = vbb + self.scatter(ids, dN * rF[:, None])
        ok = ~self.cmask & (M != 0) & (vA != 0)
        Pb = np.where(ok, vab / safe, 0.0)
        Mb = np.where(ok, Mb - (vab * vA) / safe, Mb)
        # pass 5: mass and momentum sums, m = V0 rho
        SM, SP = (N * Mb[ids]).sum(1), (N * Pb[ids]).sum(1)
        DM, DP = (dN * Mb[ids]).sum(1), (dN * Pb[ids]).sum(1)
        mb = mb + SM + v * SP
        L["x"] = xb + m * DM + m * v * DP
        L["v"] = Vv + m * SP
        if self.reinit:
            L["rho"] = L["rho"] + V0 * mb
        return L

    def gradient(self, st0, E, nsteps, dl_dx, dl_dv=None):
        tapes, st = [], dict(st0)
        for i in range(nsteps):
            st, tp = self.forward(st, E, i)
            tapes.append(tp)
        n = len(st0["x"])
        L = dict(x=np.array(dl_dx, float), v=np.zeros(n) if dl_dv is None else np.array(dl_dv, float),
                 sig=np.zeros((n, 4)), rho=np.zeros(n), vsc=np.zeros(n), E=np.zeros(n))
        if not self.reinit:
            L["vol"] = np.zeros(n)
        for tp in reversed(tapes):
            L = self.reverse(tp, L, E)
        return dict(E=L["E"], x=L["x"], v=L["v"]), st
