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
        return self.nx * self.ny * self.nz * self.ppc * self.nsp


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
    npr = nx * n0
    ix = np.repeat(np.arange(nx), n0)
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
        st.up[3:6, :npr, :, :, isp] = u
    for isp in range(p.nsp):
        row = (np.arange(ny)[:, None] + ny * np.arange(nz)[None, :]).astype(np.int64)  # (ny, nz)
        pid = row[None, :, :] * npr + np.arange(1, npr + 1, dtype=np.int64)[:, None, None]
        st.up[6, :npr, :, :, isp] = (-pid).view(np.float64)
    st.np2[:, :, :] = npr
    st.cumcnt[:, :, :, :] = (np.arange(nx + 1, dtype=np.int32) * n0)[:, None, None, None]
    st.gp[...] = st.up
    return st


def config_weibel3d(size="small", seed=12345):
    """The 3D Weibel configuration 'cfg2' (256^3, 16 ppc, m_i/m_e = 16, beams +-0.5c along x,
    u_th 0.05c), or a small case for tests."""
    if size == "cfg2":
        return Plasma3D(nx=256, ny=256, nz=256, ppc=16, drift=0.5, u_the=0.05, seed=seed)
    return Plasma3D(nx=8, ny=6, nz=5, ppc=3, drift=0.5, u_the=0.05, seed=seed)
