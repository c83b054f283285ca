"""Host logic of the adjoint wrapper: the parameter maps and their transposes."""
import dataclasses
import math

import numpy as np

from wumingpic_gb300.adjoint import SeedModes, electron_parameters, field_energy, fold_ghosts, wrap_ghosts
from wumingpic_gb300.loader import Plasma2D, load_weibel2d


def test_fold_is_transpose_of_wrap():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((6, 16, 12))
    y = rng.standard_normal((6, 20, 16))
    assert abs((wrap_ghosts(x) * y).sum() - (x * fold_ghosts(y)).sum()) < 1e-12


def test_seed_modes():
    m = SeedModes.lowest(32, 24, 64)
    assert m.count == 64 and len({tuple(r) for r in m.modes}) == 64
    rng = np.random.default_rng(1)
    a = rng.standard_normal(64)
    g = rng.standard_normal((32, 24))
    assert abs((m.field(a) * g).sum() - (a * m.grad(g)).sum()) < 1e-10
    # cos and sin of one wave vector are orthogonal on the periodic grid
    assert abs((m.basis[0] * m.basis[1]).sum()) < 1e-10


def test_electron_parameters_recover_the_loader():
    """u = u_th n + s drift e_axis, with n the loader's normals (a load with u_th 1, drift 0)."""
    p = Plasma2D(nx=16, ny=12, ppc=4, drift=0.3, u_the=0.05, seed=7)
    st = load_weibel2d(p)
    st1 = load_weibel2d(dataclasses.replace(p, drift=0.0, u_the=1.0))
    valid, s, n = electron_parameters(st.up[2:5], st.up[5], st.np2, 0.3, 0.05, p.drift_axis)
    assert valid.sum() == p.nx * p.ppc * p.ny
    assert np.abs(np.where(valid[None], n - st1.up[2:5, :, :, 1], 0)).max() < 1e-12
    assert s[:, 0][:4].tolist() == [1.0, -1.0, 1.0, -1.0]
    assert abs(s[valid].sum()) == 0  # the beams carry no net current


def test_field_energy_gradient():
    rng = np.random.default_rng(2)
    uf = rng.standard_normal((6, 12, 10))
    for which in ("B", "E", "EB"):
        v, lam = field_energy(uf, which)
        d = rng.standard_normal(uf.shape)
        h = 1e-6
        fd = (field_energy(uf + h * d, which)[0] - field_energy(uf - h * d, which)[0]) / (2 * h)
        assert math.isclose(fd, (lam * d).sum(), rel_tol=1e-8)
