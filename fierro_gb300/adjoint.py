"""The discrete adjoint of the SGH cycle loop from Python.

* ``SGHFunction`` -- a ``torch.autograd.Function`` over fierro_adj_forward /
  fierro_adj_backward: inputs per-element initial sie and gamma (a scalar or per
  element), outputs the final element density, pressure and sie.
* ``DensityMismatch`` -- J = sum_e M_e (rho_e - rho_target_e)^2 at the final
  state, its gradient through the adjoint, and central finite differences of
  the same forward along seeded directions (the gradient check), optionally of
  the frozen-branch forward (the forward's switches held at the base run's
  decisions, so the differences do not straddle them).

The parameters enter the way fierro_adj_forward defines them: the initial
state's sie is replaced and pressure / sound speed are recomputed from it with
the ideal-gas EOS, so a perturbed run is "the same deck with another initial
energy field".
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import sgh


class SGHFunction:
    """Namespace for the autograd Function (torch is imported lazily)."""

    _cls = None

    @classmethod
    def get(cls):
        if cls._cls is None:
            import torch

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, sie0, gamma, solver, state0, cycles, ckpt_every):
                    solver.set_state(state0)
                    g = gamma.detach().cpu().double().numpy()
                    solver.adj_forward(sie0.detach().cpu().double().numpy(), g if g.ndim else float(g),
                                       int(cycles), int(ckpt_every))
                    st = solver.get_state()
                    ctx.solver = solver
                    ctx.scalar_gamma = gamma.dim() == 0
                    return (torch.from_numpy(st["elem_den"].copy()), torch.from_numpy(st["elem_pres"].copy()),
                            torch.from_numpy(st["elem_sie"][1].copy()))

                @staticmethod
                def backward(ctx, dden, dpres, dsie):
                    def np_or_none(t):
                        return None if t is None else t.detach().cpu().double().numpy()

                    sb, gb, _ = ctx.solver.adj_backward(den=np_or_none(dden), pres=np_or_none(dpres),
                                                        sie=np_or_none(dsie))
                    gg = (torch.tensor(float(np.sum(gb)), dtype=torch.float64) if ctx.scalar_gamma
                          else torch.from_numpy(gb))
                    return torch.from_numpy(sb), gg, None, None, None, None

            cls._cls = _F
        return cls._cls

    @classmethod
    def apply(cls, sie0, gamma, solver, state0, cycles, ckpt_every=20):
        """(den, pres, sie) of the final state; differentiable in sie0 and gamma."""
        return cls.get().apply(sie0, gamma, solver, state0, cycles, ckpt_every)


def eos_state(state0: dict, sie0: np.ndarray, gamma: np.ndarray) -> dict:
    """A copy of a set-up state with sie replaced and pressure / sound speed
    recomputed by the ideal-gas EOS (eos.cpp:35-43), for the oracle."""
    st = {k: v.copy() for k, v in state0.items()}
    st["elem_sie"][:] = sie0[None, :]
    st["elem_statev"][:, 0] = gamma
    den = st["elem_den"]
    st["elem_pres"] = (gamma - 1.0) * sie0 * den
    c = np.sqrt(gamma * (gamma - 1.0) * sie0)
    csmin = st["elem_statev"][:, 1]
    st["elem_sspd"] = np.where(c < csmin, csmin, c)
    return st


class DensityMismatch:
    """J(sie0, gamma) = sum_e M_e (rho_e(T) - rho_target_e)^2 after `cycles` cycles."""

    def __init__(self, problem, target_den: np.ndarray, cycles: int, ckpt_every: int = 20,
                 solver: Optional[sgh.SGHSolver] = None):
        self.problem = problem
        self.solver = solver or sgh.SGHSolver(problem)
        self.state0 = sgh.setup(problem)
        self.mass = self.state0["elem_mass"].copy()
        self.sie0 = self.state0["elem_sie"][1].copy()
        self.gamma0 = self.state0["elem_statev"][:, 0].copy()
        self.target = np.asarray(target_den, dtype=np.float64)
        self.cycles = int(cycles)
        self.ckpt_every = int(ckpt_every)

    def value(self, den: np.ndarray) -> float:
        return float(np.sum(self.mass * (den - self.target) ** 2))

    def forward(self, sie0=None, gamma=None) -> float:
        """J through the GPU forward (fierro_adj_forward)."""
        s = self.solver
        s.set_state(self.state0)
        s.adj_forward(self.sie0 if sie0 is None else sie0, self.gamma0 if gamma is None else gamma,
                      self.cycles, self.ckpt_every)
        st = s.get_state()
        self.last_den = st["elem_den"]
        return self.value(st["elem_den"])

    def gradient(self, sie0=None, gamma=None):
        """(J, dJ/dsie0 [Ne], dJ/dgamma per element [Ne], dJ/dvel0 [Nn,3])."""
        J = self.forward(sie0, gamma)
        seed = 2.0 * self.mass * (self.last_den - self.target)
        sb, gb, vb = self.solver.adj_backward(den=seed)
        return J, sb, gb, vb

    def gradient_frozen(self, sie0=None, gamma=None):
        """gradient() with the forward's branch decisions recorded, after which
        every forward() of this object runs with them frozen (the frozen-branch
        forward, fierro_adj_branches): central differences of that forward are
        the derivative the adjoint computes, not a secant across a switch."""
        s = self.solver
        s.adj_branches(sgh.ADJ_BRANCHES_RECORD)
        out = self.gradient(sie0, gamma)
        s.adj_branches(sgh.ADJ_BRANCHES_FREEZE)
        return out

    def unfreeze(self):
        """Plain forwards again (frees the branch record)."""
        self.solver.adj_branches(sgh.ADJ_BRANCHES_OFF)

    def directions(self, n: int, seed: int = 2024):
        """Seeded directions: sie0 scaled per element by U(-1,1) (relative to its
        value, so the 1e-10 background and the blast element move alike) and a
        gamma shift U(-1,1) applied to every element."""
        rng = np.random.default_rng(seed)
        out = []
        for _ in range(n):
            out.append((self.sie0 * rng.uniform(-1.0, 1.0, self.sie0.size), float(rng.uniform(-1.0, 1.0))))
        return out

    def fd(self, d_sie: np.ndarray, d_gamma: float, h: float = 1e-6, forward=None) -> float:
        """Central difference of J along (d_sie, d_gamma) with step h."""
        f = forward or self.forward
        jp = f(self.sie0 + h * d_sie, self.gamma0 + h * d_gamma)
        jm = f(self.sie0 - h * d_sie, self.gamma0 - h * d_gamma)
        return (jp - jm) / (2.0 * h)

    def fd5(self, d_sie: np.ndarray, d_gamma: float, h: float = 1e-6, forward=None):
        """Central differences of J along (d_sie, d_gamma) at step h from the
        four values J(x + k h d), k = -2, -1, 1, 2: the three-point difference
        (J(h) - J(-h)) / 2h, whose error is h^2 J3 / 6 (J3 the third derivative
        along the direction), and the five-point one
        (8 (J(h) - J(-h)) - (J(2h) - J(-2h))) / 12h, whose error is O(h^4).
        Returns (three_point, five_point)."""
        f = forward or self.forward
        j = {k: f(self.sie0 + k * h * d_sie, self.gamma0 + k * h * d_gamma) for k in (-2, -1, 1, 2)}
        d1 = j[1] - j[-1]
        d2 = j[2] - j[-2]
        return d1 / (2.0 * h), (8.0 * d1 - d2) / (12.0 * h)

    def fd_consistent(self, d_sie: np.ndarray, d_gamma: float, steps=(1e-5, 1e-6, 1e-7, 1e-8), forward=None):
        """Central differences at several steps; returns (estimate, step, spread,
        table).  J is piecewise smooth (the forward's switches: limiter, Mach
        switch, CFL minimiser, dt clamps), so a step can straddle a kink; the
        estimate is taken at the step whose value agrees best with the next
        smaller step's, judged by the differences alone, and `spread` is that
        disagreement (relative)."""
        vals = [self.fd(d_sie, d_gamma, h=h, forward=forward) for h in steps]
        best = None
        for i in range(len(steps) - 1):
            a, b = vals[i], vals[i + 1]
            spread = abs(a - b) / max(abs(b), 1e-300)
            if best is None or spread < best[2]:
                best = (a, steps[i], spread)
        return best[0], best[1], best[2], list(zip(steps, vals))


def sedov_target(n: int, cycles: int, jitter: float = 0.1, seed: int = 7, energy: float = 0.3, **kw):
    """Target density: the same Sedov deck with origin energy `energy`, run on the GPU."""
    from .problems import sedov
    p = sedov(n, energy=energy, jitter=jitter, seed=seed, cycles=cycles, **kw)
    st = sgh.setup(p)
    with sgh.SGHSolver(p) as s:
        s.set_state(st)
        s.run(cycles)
        return s.get_state()["elem_den"].copy()
