"""Gradients of field-energy diagnostics through the discrete adjoint of the FP64 step.

The reference has no adjoint; this is the differentiable form of its 2D periodic
Weibel run (2d/proj/weibel/app.f90): the plasma of ``load_weibel2d`` (electron
beams +-drift along one axis with thermal spread u_th, cold ions) plus seed
fields made of Fourier modes with amplitudes a_k, advanced nsteps fused steps
(particle__solv, field__fdtd_i, the periodic boundaries, sort__bucket), scored
by the energy_history field sums (2d/proj/weibel/app.f90:502-534).

The gradient comes from the library's hand-written reverse sweep
(``Pic2D.adjoint_record`` / ``adjoint_reverse``: the Boris push and spline
gather/scatter differentiated per particle, the transposed field stencils and
the adjoint CG solve with the same symmetric operator, states kept every K
steps and recomputed in between).  The map from the loader's parameters to the
initial state is linear in each of them, so the parameter gradients are sums
over the per-particle and per-cell adjoints:

  * electrons: u = u_th n + s drift e_axis, with n the seeded normal deviates
    and s = +1 for even row slots k, -1 for odd ones (the loader's alternation,
    recovered from the particle ids -(row * npr + k + 1));
    dL/d drift = sum_e s lam_u[axis],  dL/d u_th = sum_e n . lam_u;
  * seed fields: uf[comp] interior = sum_k a_k m_k(i, j) with periodic ghost
    copies; dL/d a_k = <m_k, lam_uf folded onto the interior>.
"""
import dataclasses
import math
import time

import numpy as np

from .pic2d import Pic2D

PI = 4.0 * math.atan(1.0)


def wrap_ghosts(core):
    """(ncomp, nx, ny) interior values -> (ncomp, nx+4, ny+4) with the periodic ghost copies."""
    return np.asfortranarray(np.pad(core, ((0, 0), (2, 2), (2, 2)), mode="wrap"))


def fold_ghosts(a):
    """Transpose of ``wrap_ghosts``: (ncomp, nx+4, ny+4) -> (ncomp, nx, ny), each ghost entry
    added onto the interior cell it copies."""
    nc, nxg, nyg = a.shape
    nx, ny = nxg - 4, nyg - 4
    out = np.zeros((nc, nx, ny))
    ix = (np.arange(nxg) - 2) % nx
    iy = (np.arange(nyg) - 2) % ny
    np.add.at(out, (slice(None), ix[:, None], iy[None, :]), a)
    return out


class SeedModes:
    """Seed field of one component as a sum of Fourier modes on the cell indices:
    m_k(i, j) = cos(2 pi (mx_k i / nx + my_k j / ny) + phase_k)."""

    def __init__(self, nx, ny, modes, comp=2):
        self.nx, self.ny, self.comp = nx, ny, comp
        self.modes = np.asarray(modes, dtype=float).reshape(-1, 3)
        i = np.arange(nx)[:, None]
        j = np.arange(ny)[None, :]
        self.basis = np.stack([np.cos(2 * PI * (mx * i / nx + my * j / ny) + ph) for mx, my, ph in self.modes])

    @classmethod
    def lowest(cls, nx, ny, count=64, comp=2):
        """The `count` longest-wavelength modes, each as a cos and a sin phase: wave vectors
        (mx, my) with mx > 0 or (mx == 0, my > 0), ordered by |m|^2 then mx, my."""
        ks = sorted(((mx, my) for mx in range(0, 9) for my in range(-8, 9) if mx > 0 or (mx == 0 and my > 0)),
                    key=lambda m: (m[0] ** 2 + m[1] ** 2, m[0], m[1]))
        modes = []
        for mx, my in ks:
            modes.append((mx, my, 0.0))
            modes.append((mx, my, -0.5 * PI))
            if len(modes) >= count:
                break
        return cls(nx, ny, modes[:count], comp)

    @property
    def count(self):
        return len(self.modes)

    def field(self, amps):
        return np.tensordot(np.asarray(amps, dtype=float), self.basis, axes=1)

    def grad(self, g):
        """dL/da_k from dL/d(interior field of this component), shape (nx, ny)"""
        return np.tensordot(self.basis, g, axes=([1, 2], [0, 1]))


def field_energy(uf, which="B"):
    """energy_history field sums over the interior: sum B^2 / 8pi ("B"), sum E^2 / 8pi ("E")
    or both ("EB"); returns (value, d value / d uf)."""
    comps = {"B": (0, 1, 2), "E": (3, 4, 5), "EB": (0, 1, 2, 3, 4, 5)}[which]
    lam = np.zeros_like(uf, order="F")
    val = 0.0
    for k in comps:
        f = uf[k, 2:-2, 2:-2]
        val += float((f * f).sum()) / (8 * PI)
        lam[k, 2:-2, 2:-2] = f / (4 * PI)
    return val, lam


def electron_parameters(u, ids, np2, drift, u_th, axis):
    """Per electron slot of a freshly loaded state: (valid, s, n) with u = u_th n + s drift e_axis.

    u: (3, slots, ny, nsp) momenta, ids: (slots, ny, nsp) id column, np2: (ny, nsp) counts.
    The beam sign s alternates with the slot k of the particle in its row at loading,
    recovered from the id -(row * npr + k + 1); n = 0 where u_th = 0."""
    isp = 1
    npr = max(int(np2[:, isp].max()), 1)
    counts = np2[:, isp]
    valid = np.arange(u.shape[1])[:, None] < counts[None, :]                 # (slots, ny)
    pid = -np.ascontiguousarray(ids[:, :, isp]).view(np.int64)
    k = np.where(valid, (pid - 1) % npr, 0)
    s = np.where(valid, np.where(k % 2 == 0, 1.0, -1.0), 0.0)
    ue = np.where(valid[None], u[:, :, :, isp], 0.0)
    ue[axis] -= drift * s
    n = ue / u_th if u_th != 0 else np.zeros_like(ue)
    return valid, s, n


class FieldEnergyProblem:
    """One differentiable Weibel run: L(drift, u_th, a) = field energy after nsteps steps.

    ``forward`` loads the plasma (device loader, seed of the plasma description),
    adds the seed modes, records the run and returns L; ``backward`` reverses the
    recorded run and returns (dL/d drift, dL/d u_th, dL/d a).  With
    ``adjoint_precision="mixed"`` the reverse push and deposit run in FP32 per particle
    (the trajectory, the field adjoint, the adjoint CG and all sums stay FP64)."""

    def __init__(self, plasma, nsteps, every, modes: SeedModes = None, which="B", cg_rtol=1e-13,
                 cg_ite_max=2000, adjoint_precision="fp64"):
        if plasma.bc != "periodic":
            raise ValueError("the adjoint covers the periodic run")
        self.p = plasma
        self.nsteps, self.every = int(nsteps), int(every)
        self.modes = modes
        self.which = which
        self.cg_rtol, self.cg_ite_max = cg_rtol, cg_ite_max
        self.adjoint_precision = adjoint_precision  # "mixed": FP32 reverse push and deposit sweeps
        self.sim = None
        self._init = None
        self.timings = {}  # seconds of the last value / record / reverse calls (synchronous C calls)

    def close(self):
        for name in ("sim", "_mixed"):
            g = getattr(self, name, None)
            if g is not None:
                g.close()
                setattr(self, name, None)

    def _context(self):
        if self.sim is None:
            self.sim = Pic2D(self.p, precision="fp64")
            self.sim.cg_tolerance(self.cg_rtol, self.cg_ite_max)
            self.sim.adjoint_precision(self.adjoint_precision)
        return self.sim

    def load(self, drift, u_th, amps=None):
        """Put the initial state for these parameters into the context."""
        g = self._context()
        g.p = dataclasses.replace(self.p, drift=float(drift), u_the=float(u_th))
        g.load_weibel()
        if self.modes is not None and amps is not None and self.modes.count:
            uf = g.get_fields()
            core = np.zeros((6, self.p.nx, self.p.ny))
            core[self.modes.comp] = self.modes.field(amps)
            uf += wrap_ghosts(core)
            g.put_fields(uf)
        return g

    def value(self, drift, u_th, amps=None):
        """L without recording (the forward alone, for finite differences and timing)."""
        g = self.load(drift, u_th, amps)
        t0 = time.perf_counter()
        g.step(self.nsteps)
        self.timings["forward"] = time.perf_counter() - t0
        return field_energy(g.get_fields(), self.which)[0]

    def value_mixed(self, drift, u_th, amps=None):
        """L from the mixed-precision path (integer cell + FP32 offset, FP32 push and deposit,
        FP64 fields) on the same plasma: the forward the FP64 adjoint is the reference for."""
        if getattr(self, "_mixed", None) is None:
            self._mixed = Pic2D(self.p, precision="mixed")
            self._mixed.cg_tolerance(self.cg_rtol, self.cg_ite_max)
        g = self._mixed
        g.p = dataclasses.replace(self.p, drift=float(drift), u_the=float(u_th))
        g.load_weibel()
        if self.modes is not None and amps is not None and self.modes.count:
            uf = g.get_fields()
            core = np.zeros((6, self.p.nx, self.p.ny))
            core[self.modes.comp] = self.modes.field(amps)
            g.put_fields(uf + wrap_ghosts(core))
        t0 = time.perf_counter()
        g.step(self.nsteps)
        self.timings["forward_mixed"] = time.perf_counter() - t0
        return field_energy(g.get_fields(), self.which)[0]

    def forward(self, drift, u_th, amps=None):
        g = self.load(drift, u_th, amps)
        st = g.get_state()
        self._init = (float(drift), float(u_th), st.up[2:5].copy(), st.up[5].copy(), st.np2.copy())
        t0 = time.perf_counter()
        g.adjoint_record(self.nsteps, self.every)
        self.timings["record"] = time.perf_counter() - t0
        val, self._lam = field_energy(g.get_fields(), self.which)
        return val

    def backward(self, scale=1.0):
        if self._init is None:
            raise RuntimeError("backward before forward")
        drift, u_th, u0, ids, np2 = self._init
        t0 = time.perf_counter()
        lup, luf = self.sim.adjoint_reverse(self._lam * scale)
        self.timings["reverse"] = time.perf_counter() - t0
        valid, s, n = electron_parameters(u0, ids, np2, drift, u_th, self.p.drift_axis)
        lu = np.where(valid[None], lup[2:5, :, :, 1], 0.0)
        g_drift = float((s * lu[self.p.drift_axis]).sum())
        g_uth = float((n * lu).sum())
        g_amps = None
        if self.modes is not None and self.modes.count:
            g_amps = self.modes.grad(fold_ghosts(luf)[self.modes.comp])
        self.lam_up, self.lam_uf = lup, luf
        return g_drift, g_uth, g_amps


def _autograd_function():
    import torch

    class FieldEnergy(torch.autograd.Function):
        """L = field energy after the problem's steps, as a function of the electron beam drift,
        the electron thermal spread and the seed-mode amplitudes (float64 tensors)."""

        @staticmethod
        def forward(ctx, drift, u_th, amps, problem):
            a = None if amps is None else amps.detach().cpu().numpy().astype(np.float64)
            val = problem.forward(float(drift), float(u_th), a)
            ctx.problem = problem
            ctx.has_amps = amps is not None
            return torch.tensor(val, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            gd, gt, ga = ctx.problem.backward(float(grad))
            t = lambda v: torch.tensor(v, dtype=torch.float64)  # noqa: E731
            ga_t = torch.from_numpy(np.asarray(ga)) if ctx.has_amps and ga is not None else None
            return t(gd), t(gt), ga_t, None

    return FieldEnergy


_FN = None


def field_energy_fn(drift, u_th, amps, problem: FieldEnergyProblem):
    """torch entry: ``field_energy_fn(drift, u_th, amps, problem).backward()`` fills the
    .grad of the float64 tensors drift, u_th and amps."""
    global _FN
    if _FN is None:
        _FN = _autograd_function()
    return _FN.apply(drift, u_th, amps, problem)
