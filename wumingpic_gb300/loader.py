"""Seeded synthetic plasma loader writing WumingPIC's reference array layout.

The reference driver's loader seeds its RNG from OS entropy
(utils/wuming_utils.f90:39-56) and draws inside OpenMP loops
(2d/proj/weibel/app.f90:405-431), so its initial state cannot be reproduced.
This loader writes the same *kind* of state from a counter-based Philox stream
(numpy ``Generator(Philox(seed))``) so that the GPU library and the CPU oracle
start every comparison from an identical, recorded initial condition.

Conventions kept from the reference driver:
  * species 1 = ions (r = mass ratio), species 2 = electrons (r = 1)
    (2d/proj/weibel/app.f90:299-302);
  * charges q = +-sqrt(r / (4 pi n0 / dx^2)) * omega_p, omega_pi = omega_pe / sqrt(r_i);
  * positions in physical units with index origin nxgs = nygs = 2
    (2d/proj/weibel/app.f90:250-255); ions and electrons co-located so the
    initial charge density is zero (app.f90:410-411);
  * momenta are four-velocities u = gamma v (2d/common/particle.f90:158-160);
  * particle IDs are -pid bit-cast into the last real(8) slot (app.f90:468);
  * the state is bucket-sorted by x cell inside each row, cumcnt holding the
    prefix sums (2d/common/sort.f90:64-69).

A "drift" is applied to the four-velocity component, and beam particles
alternate +drift / -drift so that the net current vanishes.
"""
from dataclasses import dataclass, field
import math

import numpy as np

PI = 4.0 * math.atan(1.0)


@dataclass
class Plasma2D:
    """Physics/grid parameters of one 2D run (the scalar arguments of the
    reference's particle__init / field__init / bc__init calls)."""
    nx: int
    ny: int
    ppc: int                      # particles per cell per species (n0)
    mass_ratio: float = 25.0
    omega_pe: float = 0.1
    drift: float = 0.5            # electron beam four-velocity (units of c), +-drift along `drift_axis`
    drift_axis: int = 2           # 0 = x, 1 = y, 2 = z
    u_the: float = 0.05           # electron thermal spread (four-velocity, per component)
    u_thi: float = 0.0            # ion thermal spread
    delx: float = 1.0
    delt: float = 0.5
    c: float = 1.0
    gfac: float = 0.501
    np_slack: float = 1.5         # per-row capacity np = slack * ppc * nx (the reference uses 5)
    nsp: int = 2
    ndim: int = 6
    bc: str = "periodic"
    b0: tuple = (0.0, 0.0, 0.0)  # uniform initial B
    seed: int = 12345
    nxgs: int = 2
    nygs: int = 2
    window: int = 0               # shock: cells of the active window nxs..nxe from nxgs (0 = all)
    u0: float = 0.0               # shock: upstream four-velocity along x (the flow is -u0)

    @property
    def nxge(self):
        return self.nxgs + self.nx - 1

    @property
    def nxe(self):
        """right end of the active window (the shock driver's nxe)"""
        return self.nxgs + (self.window or self.nx) - 1

    @property
    def nyge(self):
        return self.nygs + self.ny - 1

    @property
    def np_cap(self):
        return int(math.ceil(self.np_slack * self.ppc * self.nx))

    def charges(self):
        r = np.array([self.mass_ratio, 1.0])
        wpe = self.omega_pe
        wpi = wpe / math.sqrt(self.mass_ratio)
        n0 = self.ppc
        q = np.array([+math.sqrt(r[0] / (4 * PI * n0 / self.delx ** 2)) * wpi,
                      -math.sqrt(r[1] / (4 * PI * n0 / self.delx ** 2)) * wpe])
        return q, r

    @property
    def n_particles(self):
        return self.nx * self.ny * self.ppc * self.nsp


@dataclass
class State2D:
    """Reference-layout host arrays (Fortran order), as the Fortran driver holds them."""
    up: np.ndarray      # (ndim, np, ny, nsp) float64
    gp: np.ndarray
    uf: np.ndarray      # (6, nx+4, ny+4) float64
    cumcnt: np.ndarray  # (nx+1, ny, nsp) int32
    np2: np.ndarray     # (ny, nsp) int32

    def copy(self):
        return State2D(*(np.array(a, order="F", copy=True) for a in (self.up, self.gp, self.uf, self.cumcnt,
                                                                    self.np2)))


def empty_state2d(p: Plasma2D) -> State2D:
    up = np.zeros((p.ndim, p.np_cap, p.ny, p.nsp), order="F")
    return State2D(up=up, gp=np.zeros_like(up, order="F"),
                   uf=np.zeros((6, p.nx + 4, p.ny + 4), order="F"),
                   cumcnt=np.zeros((p.nx + 1, p.ny, p.nsp), dtype=np.int32, order="F"),
                   np2=np.zeros((p.ny, p.nsp), dtype=np.int32, order="F"))


def load_weibel2d(p: Plasma2D) -> State2D:
    """Counter-streaming electron beams (+-drift along drift_axis) with isotropic
    thermal spread, cold (or warm) ions, uniform random positions in each cell,
    n0 = ppc particles per cell per species, zero fields except a uniform b0."""
    rng = np.random.Generator(np.random.Philox(p.seed))
    st = empty_state2d(p)
    nx, ny, n0 = p.nx, p.ny, p.ppc
    # cells that hold particles: all of them, or with conducting walls in x the
    # cells between the walls, [nxs+1, nxe-1) (2d/proj/reconnection/app.f90:418)
    # (the shock driver's upstream plasma fills its window likewise, drifting at -u0 along x)
    nw = p.window or nx
    c_lo, c_hi = (0, nx) if p.bc == "periodic" else (1, nw - 2)
    npr = (c_hi - c_lo) * n0  # particles per row per species
    # positions: cell-major inside each row, uniform in the cell
    ix = np.repeat(np.arange(c_lo, c_hi), n0)                # (npr,)
    rx = rng.random((ny, npr))
    ry = rng.random((ny, npr))
    xs = (p.nxgs + ix[None, :] + rx) * p.delx                 # (ny, npr)
    ys = (p.nygs + np.arange(ny)[:, None] + ry) * p.delx
    for isp in range(p.nsp):
        st.up[0, :npr, :, isp] = xs.T
        st.up[1, :npr, :, isp] = ys.T
    # momenta
    sd = (p.u_thi, p.u_the)
    for isp in range(p.nsp):
        u = rng.standard_normal((3, npr, ny)) * sd[isp]
        if isp == 1 and p.drift != 0.0:
            sign = np.where(np.arange(npr) % 2 == 0, 1.0, -1.0)
            u[p.drift_axis] += p.drift * sign[:, None]
        if p.u0 != 0.0:
            u[0] -= p.u0
        st.up[2:5, :npr, :, isp] = u
    # ids: -pid bit-cast to real(8), pid = running index per species over rows
    for isp in range(p.nsp):
        pid = (np.arange(ny)[None, :] * npr + np.arange(1, npr + 1)[:, None]).astype(np.int64)
        st.up[5, :npr, :, isp] = (-pid).view(np.float64)
    st.np2[:, :] = npr
    cc = (np.clip(np.arange(nx + 1), c_lo, c_hi) - c_lo).astype(np.int32) * n0
    st.cumcnt[:, :, :] = cc[:, None, None]
    st.uf[0, :, :] = p.b0[0]
    st.uf[1, :, :] = p.b0[1]
    st.uf[2, :, :] = p.b0[2]
    st.gp[...] = st.up
    return st


def config_weibel2d(size="small", seed=12345):
    """The 2D Weibel configurations: 'cfg0' (256^2, 16 ppc, +-0.5c, u_th 0.05c),
    'cfg1' (2048^2, 64 ppc, +-0.3c, u_th 0.1c), 'cfg4' (512^2, 32 ppc, 0.3c, 0.05c), or
    a small case for tests."""
    if size == "cfg0":
        return Plasma2D(nx=256, ny=256, ppc=16, drift=0.5, u_the=0.05, seed=seed)
    if size == "cfg1":
        return Plasma2D(nx=2048, ny=2048, ppc=64, drift=0.3, u_the=0.1, seed=seed, np_slack=1.25)
    if size == "cfg4":
        return Plasma2D(nx=512, ny=512, ppc=32, drift=0.3, u_the=0.05, seed=seed)
    return Plasma2D(nx=16, ny=12, ppc=4, drift=0.5, u_the=0.05, seed=seed)


@dataclass
class Harris2D(Plasma2D):
    """The reconnection driver's Harris current sheet (2d/proj/reconnection/app.f90:260-346,
    360-450): conducting walls in x, periodic in y, B_y = b0 tanh((x - x0) / lcs) with a
    localised X-point perturbation of relative amplitude e1, density ncs sech^2 + nbg
    particles per cell, drifting Maxwellians carrying the sheet current along z.

    Derived as the driver does: Debye length = dx, v_te = sqrt(rtemp) c / (sqrt(1 + rtemp)
    alpha) (pressure balance), v_ti = v_te sqrt(1 / r_i) / sqrt(rtemp), omega_pe = v_te /
    (dx sqrt 2), omega_ce = omega_pe / alpha, q from n0 = nbg + ncs, b0 = r_i c / q_i
    omega_ci, lcs in units of c / omega_pi.  Every row holds nbg (nx - 1) + int(2 ncs lcs)
    particles per species: nbg (nx - 3) uniform between the walls, the rest the sheet."""
    alpha: float = 2.0            # omega_pe / omega_ce
    rtemp: float = 0.2            # T_e / T_i
    lcs: float = 0.5              # sheet half-thickness in c / omega_pi
    nbg: int = 6                  # background particles per cell per species
    ncs: int = 32                 # sheet particles per cell per species at the centre
    e1: float = 0.1               # X-point perturbation B1 / B0 (the driver's constant is 0.12)
    bc: str = "reconnection"
    drift: float = 0.0
    u_the: float = 0.0

    def __post_init__(self):
        self.ppc = self.nbg + self.ncs  # n0 of the charge normalisation

    def derived(self):
        """(vte, vti, wpe, wpi, wge, wgi, q, b0, lcs in length units, x0, y0)"""
        r = np.array([self.mass_ratio, 1.0])
        c, dx = self.c, self.delx
        vte = math.sqrt(self.rtemp) * c / (math.sqrt(1 + self.rtemp) * self.alpha)
        vti = vte * math.sqrt(r[1] / r[0]) / math.sqrt(self.rtemp)
        wpe = vte / dx / math.sqrt(2.0)
        wpi = wpe * math.sqrt(r[1] / r[0])
        wge = wpe / self.alpha
        wgi = wge / self.mass_ratio
        n0 = self.nbg + self.ncs
        q = np.array([+math.sqrt(r[0] / (4 * PI * n0 / dx ** 2)) * wpi,
                      -math.sqrt(r[1] / (4 * PI * n0 / dx ** 2)) * wpe])
        b0 = r[0] * c / q[0] * wgi
        lcs = self.lcs * c / wpi
        x0 = 0.5 * (self.nxge + self.nxgs) * dx
        y0 = 0.5 * (self.nyge - self.nygs) * dx
        return dict(vte=vte, vti=vti, wpe=wpe, wpi=wpi, wge=wge, wgi=wgi, q=q, r=r, b0=b0, lcs=lcs, x0=x0, y0=y0)

    def charges(self):
        dv = self.derived()
        return dv["q"], dv["r"]

    @property
    def n_row(self):
        """particles per row per species (2d/proj/reconnection/app.f90:307, truncated)"""
        return int(self.nbg * (self.nxge - self.nxgs) + self.ncs * 2 * self.derived()["lcs"])

    @property
    def np_cap(self):
        return int(math.ceil(self.np_slack * self.n_row))

    @property
    def n_particles(self):
        return self.n_row * self.ny * self.nsp


def harris_fields(p: Harris2D, i, j):
    """(bx, by) at the node (i dx, j dx) (2d/proj/reconnection/app.f90:375-378, 393-401)."""
    dv = p.derived()
    b0, lcs, x0, y0 = dv["b0"], dv["lcs"], dv["x0"], dv["y0"]
    x, y = i * p.delx, j * p.delx
    g = np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2)
    bx = +p.e1 * b0 * ((y - y0) / lcs) * g
    by = b0 * np.tanh((x - x0) / lcs) - p.e1 * b0 * ((x - x0) / lcs) * g
    return bx, by


def harris_current(p: Harris2D, x, y):
    """(jz, density) at particle positions (2d/proj/reconnection/app.f90:380-384)."""
    dv = p.derived()
    b0, lcs, x0, y0 = dv["b0"], dv["lcs"], dv["x0"], dv["y0"]
    sech2 = np.cosh((x - x0) / lcs) ** (-2)
    r2 = ((x - x0) ** 2 + (y - y0) ** 2) / (2 * lcs) ** 2
    jz = b0 / (4 * PI * lcs) * sech2 - 2 * p.e1 * b0 / (4 * PI * lcs) * (1.0 - r2) * np.exp(-r2)
    return jz, p.ncs * sech2 + p.nbg


def load_harris2d(p: Harris2D) -> State2D:
    """The Harris sheet of the reconnection driver (set_initial_condition,
    2d/proj/reconnection/app.f90:360-450) from a seeded Philox stream, bucket-sorted as the
    driver does after loading (app.f90:337-340)."""
    rng = np.random.Generator(np.random.Philox(p.seed))
    dv = p.derived()
    st = empty_state2d(p)
    nx, ny, dx = p.nx, p.ny, p.delx
    n = p.n_row
    ibg = p.nbg * (p.nxge - p.nxgs - 2)
    jabs = (p.nygs + np.arange(ny))[:, None]
    xs = np.empty((ny, n))
    xs[:, :ibg] = (p.nxgs + 1) * dx + rng.random((ny, ibg)) * dx * (p.nxge - p.nxgs - 2)
    r1 = (2.0 * rng.random((ny, n - ibg)) - 1.0) * math.tanh(0.5 * (p.nxge - p.nxgs - 2) * dx / dv["lcs"])
    xs[:, ibg:] = dv["lcs"] * 0.5 * (np.log(1.0 + r1) - np.log(1.0 - r1)) + dv["x0"]
    ys = jabs * dx + rng.random((ny, n)) * dx
    # the driver's stable bucket sort by int(x) (ions and electrons share positions)
    cell = np.trunc(xs).astype(np.int64) - p.nxgs
    order = np.argsort(cell, axis=1, kind="stable")
    xs = np.take_along_axis(xs, order, axis=1)
    ys = np.take_along_axis(ys, order, axis=1)
    cell = np.take_along_axis(cell, order, axis=1)
    counts = np.bincount((np.arange(ny)[:, None] * nx + cell).ravel(), minlength=ny * nx).reshape(ny, nx)
    cc = np.zeros((nx + 1, ny), np.int32)
    cc[1:] = np.cumsum(counts, axis=1).T
    jz, dens = harris_current(p, xs, ys)
    f = (1.0 / ((1.0 + p.rtemp) * dv["q"][0]), p.rtemp / ((1.0 + p.rtemp) * dv["q"][1]))
    sd = (dv["vti"] / math.sqrt(2.0), dv["vte"] / math.sqrt(2.0))
    for isp in range(p.nsp):
        st.up[0, :n, :, isp] = xs.T
        st.up[1, :n, :, isp] = ys.T
        u = rng.standard_normal((3, n, ny)) * sd[isp]
        u[2] += (f[isp] * jz / dens).T
        st.up[2:5, :n, :, isp] = u
        pid = (np.arange(ny)[None, :] * n + np.arange(1, n + 1)[:, None]).astype(np.int64)
        st.up[5, :n, :, isp] = (-pid).view(np.float64)
        st.cumcnt[:, :, isp] = cc
    st.np2[:, :] = n
    i = np.arange(p.nxgs - 2, p.nxge + 3)[:, None]
    j = np.arange(p.nygs - 2, p.nyge + 3)[None, :]
    bx, by = harris_fields(p, i, j)
    st.uf[0] = bx
    st.uf[1] = by
    st.gp[...] = st.up
    return st


def config_harris2d(size="small", seed=12345):
    """'cfg3': 4096 x 2048 cells (2048 between the walls in x, 4096 periodic in y: the
    reference's orientation), 32 ppc/species at the sheet centre + 6 background (0.2 n0),
    m_i/m_e 25, omega_ce/omega_pe 0.5, T_i/T_e 5, sheet half-width 0.5 c/omega_pi, 10 %
    perturbation; or a small case for tests."""
    if size == "cfg3":
        return Harris2D(nx=2048, ny=4096, ppc=38, mass_ratio=25.0, seed=seed, np_slack=1.25)
    return Harris2D(nx=64, ny=48, ppc=20, mass_ratio=25.0, lcs=0.2, ncs=16, nbg=4, seed=seed, np_slack=1.5)


# ---------------------------------------------------------------------------
# 3D (3d/proj/weibel/app.f90 conventions: ndim = 7, (x, y, z, ux, uy, uz, id),
# rows (j, k) of x-sorted particles, uf(6, nxgs-2:nxge+2, nys-2:nye+2, nzs-2:nze+2))
# ---------------------------------------------------------------------------
@dataclass
class Plasma3D:
    """Physics/grid parameters of one 3D run (periodic in x, y, z)."""
    nx: int
    ny: int
    nz: int
    ppc: int
    mass_ratio: float = 16.0
    omega_pe: float = 0.1
    drift: float = 0.5
    drift_axis: int = 0           # 0 = x, 1 = y, 2 = z (the 3D Weibel configuration drifts along x)
    u_the: float = 0.05
    u_thi: float = 0.0
    delx: float = 1.0
    delt: float = 0.5
    c: float = 1.0
    gfac: float = 0.501
    np_slack: float = 1.5
    nsp: int = 2
    ndim: int = 7
    seed: int = 12345
    nxgs: int = 2
    nygs: int = 2
    nzgs: int = 2
    bc: str = "periodic"          # "reconnection": conducting walls in x (3d/proj/reconnection);
                                  # "shock": wall at nxs, open end at nxe of the window (3d/proj/shock)
    window: int = 0               # shock: cells of the active window nxs..nxe from nxgs (0 = all)
    u0: float = 0.0               # shock: upstream four-velocity along x (the flow is -u0)

    @property
    def nxge(self):
        return self.nxgs + self.nx - 1

    @property
    def nyge(self):
        return self.nygs + self.ny - 1

    @property
    def nzge(self):
        return self.nzgs + self.nz - 1

    @property
    def np_cap(self):
        return int(math.ceil(self.np_slack * self.ppc * self.nx))

    def charges(self):
        r = np.array([self.mass_ratio, 1.0])
        wpe = self.omega_pe
        wpi = wpe / math.sqrt(self.mass_ratio)
        n0 = self.ppc
        q = np.array([+math.sqrt(r[0] / (4 * PI * n0 / self.delx ** 3)) * wpi,
                      -math.sqrt(r[1] / (4 * PI * n0 / self.delx ** 3)) * wpe])
        return q, r

    @property
    def n_particles(self):
        cells_x = self.nx if self.bc == "periodic" else (self.window or self.nx) - 3
        return cells_x * self.ny * self.nz * self.ppc * self.nsp

    @property
    def nxe(self):
        """right end of the active window (the shock driver's nxe)"""
        return self.nxgs + (self.window or self.nx) - 1


@dataclass
class State3D:
    """Reference-layout host arrays of the 3D driver (Fortran order)."""
    up: np.ndarray      # (ndim, np, ny, nz, nsp) float64
    gp: np.ndarray
    uf: np.ndarray      # (6, nx+4, ny+4, nz+4) float64
    cumcnt: np.ndarray  # (nx+1, ny, nz, nsp) int32
    np2: np.ndarray     # (ny, nz, nsp) int32

    def copy(self):
        return State3D(*(np.array(a, order="F", copy=True) for a in (self.up, self.gp, self.uf, self.cumcnt,
                                                                    self.np2)))


def empty_state3d(p: Plasma3D) -> State3D:
    up = np.zeros((p.ndim, p.np_cap, p.ny, p.nz, p.nsp), order="F")
    return State3D(up=up, gp=np.zeros_like(up, order="F"),
                   uf=np.zeros((6, p.nx + 4, p.ny + 4, p.nz + 4), order="F"),
                   cumcnt=np.zeros((p.nx + 1, p.ny, p.nz, p.nsp), dtype=np.int32, order="F"),
                   np2=np.zeros((p.ny, p.nz, p.nsp), dtype=np.int32, order="F"))


def load_weibel3d(p: Plasma3D) -> State3D:
    """Counter-streaming electron beams (+-drift along drift_axis, alternating sign) with
    isotropic thermal spread, cold (or warm) ions co-located with the electrons, uniform
    random positions in each cell, ppc particles per cell per species, zero fields."""
    rng = np.random.Generator(np.random.Philox(p.seed))
    st = empty_state3d(p)
    nx, ny, nz, n0 = p.nx, p.ny, p.nz, p.ppc
    # with conducting walls in x the plasma fills the cells between them, [nxs+1, nxe-1); the shock
    # driver's upstream plasma fills its window likewise, drifting at -u0 along x
    nw = p.window or nx
    c_lo, c_hi = (0, nx) if p.bc == "periodic" else (1, nw - 2)
    npr = (c_hi - c_lo) * n0
    ix = np.repeat(np.arange(c_lo, c_hi), n0)
    rx = rng.random((nz, ny, npr))
    ry = rng.random((nz, ny, npr))
    rz = rng.random((nz, ny, npr))
    xs = (p.nxgs + ix[None, None, :] + rx) * p.delx
    ys = (p.nygs + np.arange(ny)[None, :, None] + ry) * p.delx
    zs = (p.nzgs + np.arange(nz)[:, None, None] + rz) * p.delx
    for isp in range(p.nsp):
        st.up[0, :npr, :, :, isp] = xs.transpose(2, 1, 0)
        st.up[1, :npr, :, :, isp] = ys.transpose(2, 1, 0)
        st.up[2, :npr, :, :, isp] = zs.transpose(2, 1, 0)
    sd = (p.u_thi, p.u_the)
    for isp in range(p.nsp):
        u = rng.standard_normal((3, npr, ny, nz)) * sd[isp]
        if isp == 1 and p.drift != 0.0:
            sign = np.where(np.arange(npr) % 2 == 0, 1.0, -1.0)
            u[p.drift_axis] += p.drift * sign[:, None, None]
        if p.u0 != 0.0:
            u[0] -= p.u0
        st.up[3:6, :npr, :, :, isp] = u
    for isp in range(p.nsp):
        row = (np.arange(ny)[:, None] + ny * np.arange(nz)[None, :]).astype(np.int64)  # (ny, nz)
        pid = row[None, :, :] * npr + np.arange(1, npr + 1, dtype=np.int64)[:, None, None]
        st.up[6, :npr, :, :, isp] = (-pid).view(np.float64)
    st.np2[:, :, :] = npr
    cc = (np.clip(np.arange(nx + 1), c_lo, c_hi) - c_lo).astype(np.int32) * n0
    st.cumcnt[:, :, :, :] = cc[:, None, None, None]
    st.gp[...] = st.up
    return st


def config_weibel3d(size="small", seed=12345):
    """The 3D Weibel configuration 'cfg2' (256^3, 16 ppc, m_i/m_e = 16, beams +-0.5c along x,
    u_th 0.05c), or a small case for tests."""
    if size == "cfg2":
        return Plasma3D(nx=256, ny=256, nz=256, ppc=16, drift=0.5, u_the=0.05, seed=seed)
    return Plasma3D(nx=8, ny=6, nz=5, ppc=3, drift=0.5, u_the=0.05, seed=seed)
