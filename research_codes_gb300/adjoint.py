"""Gradient of a smooth bound-mass functional after K leapfrog steps with
respect to the initial positions and velocities.

    L = sum_i m_i sigmoid(-e_i / e0),  e_i = |v_i - v_cm|^2 / 2 + pot_i + u_i

with v_cm the density-weighted mean velocity (analysis/common.py:71-90) and e0
a fixed energy scale: the smooth form of the bound mass of
analysis/unbound_mass/unbound_mass.py:10-27 (a particle with e < 0 is bound).

The derivative is hand-written: the engine's sph_system_adjoint_forces gives
the vector-Jacobian product of one force evaluation (density with its three
smoothing-length passes and gradient pass, EOS and Balsara switch, tree
gravity, hydro, alpha source); the leapfrog predictor and corrector
(hdr_hgas.hpp:646-665), linear in the state for a fixed dt, are reversed here.
The forward run keeps the full state every `every` steps; the backward pass
recomputes each segment from its checkpoint, then reverses its steps one by
one, repeating each step's force evaluation (sph_system_predict +
compute_forces) so that the lists, tree and intermediates of that evaluation
are the ones differentiated.

Held fixed, as for any derivative of this code: the time step (the run uses
one constant dt, below the CFL limit), the interaction lists and tree of
every evaluation, and e0.  The derivative needs monopole gravity, alpha_u = 0
and no clamp of h (see sph_system_adjoint_forces).
"""
import numpy as np

STATE = ("pos", "vel", "uene", "alph", "alphu", "acc", "udot", "adot", "adotu", "ksr")
STEP_FIELDS = ("acc", "udot", "adot", "adotu")   # restored with set_field after an upload


def bound_mass(mass, vel, pot, uene, dens, e0):
    """(L, dL/d{vel, uene, pot, dens}) of the smooth bound-mass functional."""
    w = dens.sum()
    vcm = (dens[:, None] * vel).sum(0) / w
    dv = vel - vcm
    e = 0.5 * (dv * dv).sum(1) + pot + uene
    z = -e / e0
    sig = 0.5 * (1.0 + np.tanh(0.5 * z))   # logistic, overflow-free
    L = float((mass * sig).sum())
    eb = -mass * sig * (1.0 - sig) / e0
    vcmb = -(eb[:, None] * dv).sum(0)
    return L, {"vel": eb[:, None] * dv + dens[:, None] / w * vcmb, "uene": eb.copy(), "pot": eb.copy(),
               "dens": dv @ vcmb / w}


def energy_scale(ps, fraction=0.01):
    """fraction x the mean |e_i| of the system's current state (e0 of the loss)."""
    vel, pot, uene, dens = (ps.download(k) for k in ("vel", "pot", "uene", "dens"))
    vcm = (dens[:, None] * vel).sum(0) / dens.sum()
    e = 0.5 * ((vel - vcm) ** 2).sum(1) + pot + uene
    return fraction * float(np.mean(np.abs(e)))


class BoundMassRun:
    """K steps of a ParticleSystem from fixed initial conditions (mass, uene,
    alph, ksr guess, ids) with variable initial positions and velocities.

    forward(x0, v0) -> L; backward() -> (dL/dx0, dL/dv0) of the last forward.
    """

    def __init__(self, ps, ic, steps=20, every=5, dt=None, e0=None):
        self.ps = ps
        self.ic = {k: np.array(v, copy=True) for k, v in ic.items()}
        self.ic.setdefault("alphu", np.zeros(ps.n))
        self.steps = int(steps)
        self.every = max(1, int(every))
        if dt is None:
            # half the first CFL step of the initial state, as the run's constant dt
            self._upload(self.ic["pos"], self.ic["vel"])
            ps.compute_forces()
            ps.step(1)
            dt = 0.5 * ps.clock()[1]
        self.dt = float(dt)
        # a constant dt: update_dt never doubles beyond dt_max and halves only
        # below the CFL limit, which the forward checks
        ps.set_params(dt_max=self.dt)
        if e0 is None:
            self._upload(self.ic["pos"], self.ic["vel"])
            ps.compute_forces()
            e0 = energy_scale(ps)
        self.e0 = float(e0)
        self._ckpt = None

    # -- state
    def _upload(self, x, v):
        s = dict(self.ic)
        s["pos"], s["vel"] = np.asarray(x, np.float64), np.asarray(v, np.float64)
        self.ps.upload(s)
        self.ps.set_clock(time=0.0, dt=self.dt if hasattr(self, "dt") else -1.0)

    def _save(self):
        st = {k: self.ps.download(k) for k in STATE}
        st["time"] = self.ps.clock()[0]
        return st

    def _restore(self, st):
        s = dict(self.ic)
        for k in ("pos", "vel", "uene", "alph", "alphu", "ksr"):
            s[k] = st[k]
        self.ps.upload(s)
        for k in STEP_FIELDS:
            self.ps.set_field(k, st[k])
        self.ps.set_clock(time=st["time"], dt=self.dt)

    def _step(self):
        self.ps.step(1)
        dt = self.ps.clock()[1]
        if dt != self.dt:
            raise RuntimeError(f"the run's time step changed ({dt} != {self.dt}): lower dt")

    # -- forward
    def forward(self, x0, v0):
        ps = self.ps
        self._upload(x0, v0)
        ps.compute_forces()                 # F0: the accelerations of the initial state
        self._ckpt = {0: self._save()}
        for n in range(self.steps):
            self._step()
            if (n + 1) % self.every == 0 and n + 1 < self.steps:
                self._ckpt[n + 1] = self._save()
        self._final = {k: ps.download(k) for k in ("vel", "pot", "uene", "dens")}
        self._final["mass"] = self.ic["mass"]
        L, self._lossb = bound_mass(self._final["mass"], self._final["vel"], self._final["pot"],
                                    self._final["uene"], self._final["dens"], self.e0)
        return L

    # -- backward
    def backward(self):
        if self._ckpt is None:
            raise RuntimeError("backward() needs a forward() first")
        ps, dt, n_all = self.ps, self.dt, self.steps
        z = lambda w: np.zeros((ps.n, 3) if w == 3 else ps.n)  # noqa: E731
        sb = {"pos": z(3), "vel": self._lossb["vel"], "uene": self._lossb["uene"], "alph": z(1), "acc": z(3),
              "udot": z(1), "adot": z(1), "ksr": z(1)}
        extra = {"pot": self._lossb["pot"], "dens": self._lossb["dens"]}   # the last evaluation only
        starts = sorted(self._ckpt)
        for s0 in reversed(starts):
            s1 = min(s0 + self.every, n_all)
            # recompute the segment's starting states
            self._restore(self._ckpt[s0])
            states = [self._ckpt[s0]]
            for _ in range(s0 + 1, s1):
                self._step()
                states.append(self._save())
            for n in reversed(range(s0, s1)):
                self._restore(states[n - s0])
                ps.predict()
                ps.compute_forces()
                # corrector: v = v2 + a dt/2, u = u2 + udot dt/2, alpha = alpha2 + adot dt/2
                seed = {"acc": sb["acc"] + 0.5 * dt * sb["vel"], "udot": sb["udot"] + 0.5 * dt * sb["uene"],
                        "adot": sb["adot"] + 0.5 * dt * sb["alph"], "ksr": sb["ksr"]}
                if n == n_all - 1:
                    seed.update(extra)
                g = ps.adjoint_forces(seed)
                v2b, u2b, a2b = sb["vel"], sb["uene"], sb["alph"]
                xpb = sb["pos"] + g["pos"]
                vpb, upb, apb = g["vel"], g["uene"], g["alph"]
                # predictor: x' = x + v dt + a dt^2/2, v' = v + a dt, v2 = v + a dt/2, likewise u, alpha
                sb = {"pos": xpb, "vel": dt * xpb + vpb + v2b, "acc": 0.5 * dt * dt * xpb + dt * vpb + 0.5 * dt * v2b,
                      "uene": upb + u2b, "udot": dt * upb + 0.5 * dt * u2b, "alph": apb + a2b,
                      "adot": dt * apb + 0.5 * dt * a2b, "ksr": g["ksr"]}
        # F0: the initial accelerations, h and alpha rates as functions of x0, v0
        self._upload(self._ckpt[0]["pos"], self._ckpt[0]["vel"])
        ps.compute_forces()
        g = ps.adjoint_forces({"acc": sb["acc"], "udot": sb["udot"], "adot": sb["adot"], "ksr": sb["ksr"]})
        return sb["pos"] + g["pos"], sb["vel"] + g["vel"]


def autograd_function():
    """torch.autograd.Function: BoundMass.apply(x0, v0, run) -> L (a 0-d tensor)."""
    import torch

    class BoundMass(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, v0, run):
            L = run.forward(x0.detach().cpu().double().numpy(), v0.detach().cpu().double().numpy())
            ctx.run = run
            ctx.dev = (x0.device, x0.dtype)
            return torch.tensor(L, dtype=torch.float64, device=x0.device)

        @staticmethod
        def backward(ctx, gL):
            xb, vb = ctx.run.backward()
            dev, dtp = ctx.dev
            g = gL.detach().to(torch.float64).cpu().item()
            return (torch.as_tensor(g * xb, device=dev, dtype=dtp), torch.as_tensor(g * vb, device=dev, dtype=dtp),
                    None)

    return BoundMass
