"""The discrete adjoint of the FP64 2D step against central finite differences.

Tolerances (stated per test):
  * transposed field operators, <L x, y> = <x, L^T y>: 1e-12 relative;
  * push, deposit and field -> push -> deposit Jacobians along random directions:
    1e-6 relative (central differences, steps 1e-3 and, for the piecewise-quadratic
    deposit weights, 1e-6);
  * whole steps (1 and 4) along random field and particle directions: 1e-6 relative;
  * gradients of the field energy with respect to beam drift, thermal spread and
    seed-mode amplitudes through the checkpointed reverse sweep: 1e-5 relative;
  * the checkpoint interval changes only the atomic summation order: 1e-12;
  * the mixed-precision adjoint (FP32 reverse push and deposit) against the FP64 adjoint:
    1e-4 relative on the parameter gradients.
The CG runs at a relative tolerance of 1e-13 so that finite differences resolve it.
"""
import math

import numpy as np
import pytest

from tests.helpers import small_case
from wumingpic_gb300.adjoint import FieldEnergyProblem, SeedModes, field_energy
from wumingpic_gb300.loader import Plasma2D
from wumingpic_gb300.pic2d import Pic2D

pytestmark = pytest.mark.gpu

RTOL_CG = 1e-13


def seeded_case(seed=5, nx=16, ny=16, ppc=4):
    p, st = small_case(nx=nx, ny=ny, ppc=ppc, seed=seed, u_the=0.1)
    rng = np.random.default_rng(seed)
    st.uf[...] = np.pad(0.01 * rng.standard_normal((6, p.nx, p.ny)), ((0, 0), (2, 2), (2, 2)), mode="wrap")
    return p, st


def sim(p, st):
    g = Pic2D(p, precision="fp64")
    g.cg_tolerance(RTOL_CG, 2000)
    g.put_state(st)
    return g


def test_transposed_field_operators(gpu_lib):
    p, st = seeded_case()
    g = sim(p, st)
    out = g.adjoint_selfcheck()
    g.close()
    assert np.all(out < 1e-12), out


@pytest.mark.parametrize("seed", [5, 6])
def test_push_deposit_chain_jacobians(gpu_lib, seed):
    p, st = seeded_case(seed)
    g = sim(p, st)
    # the spline weights are piecewise quadratic: the deposit's difference step stays small
    for check, h in ((g.adjoint_pushcheck, 1e-3), (g.adjoint_depositcheck, 1e-6), (g.adjoint_chaincheck, 1e-3)):
        fd, ad = check(h)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (check.__name__, fd, ad)
    g.close()


@pytest.mark.parametrize("nsteps", [1, 4])
def test_step_gradient_random_directions(gpu_lib, nsteps):
    p, st = seeded_case()

    def run(s):
        g = sim(p, s)
        g.step(nsteps)
        v = field_energy(g.get_fields(), "B")[0]
        g.close()
        return v

    g0 = sim(p, st)
    g0.step(nsteps)
    _, lam = field_energy(g0.get_fields(), "B")
    g0.close()
    g = sim(p, st)
    lup, luf = g.adjoint(nsteps, 2, lam)
    g.close()
    rng = np.random.default_rng(11)
    h = 1e-5

    def check(field, v, adj):
        sp, sm = st.copy(), st.copy()
        getattr(sp, field)[...] += h * v
        getattr(sm, field)[...] -= h * v
        fd = (run(sp) - run(sm)) / (2 * h)
        assert abs(adj - fd) <= 1e-6 * abs(fd), (field, fd, adj)

    vf = rng.standard_normal(st.uf.shape)
    for comps in (slice(0, 3), slice(3, 6)):  # B and E components, ghosts included
        v = np.zeros_like(vf)
        v[comps] = vf[comps]
        check("uf", v, (v * luf).sum())
    vp = rng.standard_normal(st.up.shape)
    for k, scale in ((0, 0.1), (1, 0.1), (2, 0.01), (3, 0.01), (4, 0.01)):  # x, y, ux, uy, uz
        v = np.zeros_like(vp)
        v[k] = scale * vp[k]
        check("up", v, (v[:5] * lup[:5]).sum())


def test_checkpoint_interval(gpu_lib):
    """The recomputation between checkpoints reproduces the recorded run: the gradients do
    not depend on K beyond the order of the adjoint's atomic sums."""
    p, st = seeded_case(6)
    g0 = sim(p, st)
    g0.step(5)
    _, lam = field_energy(g0.get_fields(), "EB")
    g0.close()
    res = []
    for every in (1, 2, 5):
        g = sim(p, st)
        res.append(g.adjoint(5, every, lam))
        g.close()
    for lup, luf in res[1:]:
        assert np.abs(luf - res[0][1]).max() <= 1e-12 * np.abs(res[0][1]).max()
        assert np.abs(lup[:5] - res[0][0][:5]).max() <= 1e-12 * np.abs(res[0][0][:5]).max()


@pytest.mark.parametrize("every", [2, 5])
def test_reverse_twice(gpu_lib, every):
    """The record keeps its last segment's step states; a second reverse sweep of the same
    record recomputes that segment and gives the same gradients."""
    p, st = seeded_case(6)
    g = sim(p, st)
    g.adjoint_record(5, every)
    _, lam = field_energy(g.get_fields(), "EB")
    lup1, luf1 = g.adjoint_reverse(lam)
    lup2, luf2 = g.adjoint_reverse(lam)
    g.close()
    assert np.abs(luf2 - luf1).max() <= 1e-12 * np.abs(luf1).max()
    assert np.abs(lup2[:5] - lup1[:5]).max() <= 1e-12 * np.abs(lup1[:5]).max()


@pytest.mark.parametrize("every", [2, 3])
def test_replayed_fields_match_full_recompute(gpu_lib, every):
    """With the recorded fields kept, the recompute of a segment pushes and sorts only; the
    gradients equal those of the full recompute (deposit and solve run again) to the order
    of the adjoint's atomic sums, for the same record and a second reverse sweep."""
    p, st = seeded_case(7)
    res = []
    for keep in (True, False):
        g = sim(p, st)
        g.adjoint_keep_fields(keep)
        g.adjoint_record(7, every)
        _, lam = field_energy(g.get_fields(), "EB")
        res.append(g.adjoint_reverse(lam) + g.adjoint_reverse(lam))
        g.close()
    # a record made with the store, which is then given back before the reverse sweeps
    g = sim(p, st)
    g.adjoint_record(7, every)
    g.adjoint_keep_fields(False)
    _, lam = field_energy(g.get_fields(), "EB")
    res.append(g.adjoint_reverse(lam) + g.adjoint_reverse(lam))
    g.close()
    for other in res[1:]:
        for a, b in zip(res[0], other):
            scale = np.abs(b[:5] if b.ndim == 4 else b).max()
            assert np.abs((a - b)[:5] if a.ndim == 4 else a - b).max() <= 1e-12 * scale


def small_problem(nsteps=10, every=4, which="B"):
    p = Plasma2D(nx=32, ny=32, ppc=8, drift=0.3, u_the=0.05, seed=21)
    modes = SeedModes.lowest(p.nx, p.ny, 8)
    amps = 1e-4 * np.random.default_rng(3).standard_normal(modes.count)
    return FieldEnergyProblem(p, nsteps, every, modes, which=which, cg_rtol=RTOL_CG), amps


@pytest.mark.parametrize("which", ["B", "EB"])
def test_parameter_gradients_vs_fd(gpu_lib, which):
    prob, amps = small_problem(which=which)
    drift, u_th = 0.3, 0.05
    val = prob.forward(drift, u_th, amps)
    g_drift, g_uth, g_amps = prob.backward()
    assert math.isclose(val, prob.value(drift, u_th, amps), rel_tol=1e-13)
    h = 1e-6
    fd_drift = (prob.value(drift + h, u_th, amps) - prob.value(drift - h, u_th, amps)) / (2 * h)
    fd_uth = (prob.value(drift, u_th + h, amps) - prob.value(drift, u_th - h, amps)) / (2 * h)
    assert abs(g_drift - fd_drift) <= 1e-5 * abs(fd_drift), (g_drift, fd_drift)
    assert abs(g_uth - fd_uth) <= 1e-5 * abs(fd_uth), (g_uth, fd_uth)
    for k in (0, 3, 7):
        da = np.zeros_like(amps)
        da[k] = 1e-8
        fd = (prob.value(drift, u_th, amps + da) - prob.value(drift, u_th, amps - da)) / 2e-8
        assert abs(g_amps[k] - fd) <= 1e-5 * abs(fd), (k, g_amps[k], fd)
    prob.close()


@pytest.mark.parametrize("which", ["B", "EB"])
def test_mixed_adjoint_vs_fp64_adjoint(gpu_lib, which):
    """FP32 reverse push and deposit along the same recorded FP64 run: the parameter gradients
    within 1e-4 relative of the FP64 adjoint's (the seed amplitudes as a vector norm)."""
    prob, amps = small_problem(which=which)
    drift, u_th = 0.3, 0.05
    prob.forward(drift, u_th, amps)
    g64 = prob.backward()
    prob.sim.adjoint_precision("mixed")
    prob.forward(drift, u_th, amps)
    g32 = prob.backward()
    prob.close()
    for a, b in zip(g32[:2], g64[:2]):
        assert abs(a - b) <= 1e-4 * abs(b), (a, b)
    assert np.linalg.norm(g32[2] - g64[2]) <= 1e-4 * np.linalg.norm(g64[2])


def test_torch_autograd(gpu_lib):
    torch = pytest.importorskip("torch")
    from wumingpic_gb300.adjoint import field_energy_fn
    prob, amps = small_problem(nsteps=6, every=3)
    d = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    t = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    a = torch.tensor(amps, dtype=torch.float64, requires_grad=True)
    loss = 2.0 * field_energy_fn(d, t, a, prob)
    loss.backward()
    prob2, _ = small_problem(nsteps=6, every=3)
    prob2.forward(0.3, 0.05, amps)
    g_drift, g_uth, g_amps = prob2.backward()
    assert math.isclose(d.grad.item(), 2 * g_drift, rel_tol=1e-12)
    assert math.isclose(t.grad.item(), 2 * g_uth, rel_tol=1e-12)
    assert np.allclose(a.grad.numpy(), 2 * g_amps, rtol=1e-12, atol=0)
    prob.close()
    prob2.close()
