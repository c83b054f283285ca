"""Shared test helpers: small seeded cases, an independent charge-density
routine, and a literal pure-Python restatement of the reference's particle
migration used to cross-check both the C++ oracle and the closed-form plan the
GPU kernels implement."""
import numpy as np

from wumingpic_gb300.loader import Plasma2D, load_weibel2d


def small_plasma(nx=16, ny=12, ppc=6, seed=3, **kw):
    kw.setdefault("drift", 0.5)
    kw.setdefault("u_the", 0.05)
    return Plasma2D(nx=nx, ny=ny, ppc=ppc, seed=seed, **kw)


def small_case(**kw):
    p = small_plasma(**kw)
    return p, load_weibel2d(p)


def rho2d(p, up, np2, q):
    """Charge density sum_p q S(x_p) on the periodic interior grid (nx, ny),
    with the reference's quadratic spline and cell index int(x)."""
    R = np.zeros((p.nx, p.ny))
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = np2[jj, isp]
            x = up[0, :n, jj, isp] / p.delx
            y = up[1, :n, jj, isp] / p.delx
            i = np.floor(x).astype(int)
            j = np.floor(y).astype(int)
            dx = x - 0.5 - i
            dy = y - 0.5 - j
            sx = [0.5 * (0.5 - dx) ** 2, 0.75 - dx ** 2, 0.5 * (0.5 + dx) ** 2]
            sy = [0.5 * (0.5 - dy) ** 2, 0.75 - dy ** 2, 0.5 * (0.5 + dy) ** 2]
            for a in range(3):
                for b in range(3):
                    np.add.at(R, ((i + a - 1 - p.nxgs) % p.nx, (j + b - 1 - p.nygs) % p.ny), q[isp] * sx[a] * sy[b])
    return R


def continuity_residual(p, q, up0, gp1, np2, uj):
    """(rho1 - rho0) dx/dt + div J on the periodic interior; uj already folded."""
    r0 = rho2d(p, up0, np2, q)
    r1 = rho2d(p, gp1, np2, q)
    J = uj[:, 2:-2, 2:-2]
    res = (r1 - r0) * p.delx / p.delt + (np.roll(J[0], -1, 0) - J[0]) + (np.roll(J[1], -1, 1) - J[1])
    return np.abs(res).max(), np.abs(r1 - r0).max() * p.delx / p.delt


def literal_particle_y(up, np2, nys, nye, nygs, nyge, delx, ndim, npcap):
    """Pure-Python restatement of boundary_periodic__particle_y with one rank
    and one thread (2d/common/boundary_periodic.f90:99-248), round-down wraps
    omitted (callers use positions where the wrap is exact).  up is modified in
    place (Fortran layout (ndim, np, ny, nsp), 0-based here)."""
    ny = nye - nys + 1
    nsp = up.shape[3]
    for isp in range(nsp):
        bff = {j: [] for j in range(nys - 1, nye + 2)}
        flag = {j: [] for j in range(nys, nye + 1)}
        for j in range(nys, nye + 1):
            jj = j - nys
            for ii in range(np2[jj, isp]):
                jpos = int(up[1, ii, jj, isp] / delx)
                if jpos != j:
                    if jpos <= nygs - 1:
                        up[1, ii, jj, isp] += ny * delx
                    elif jpos >= nyge + 1:
                        up[1, ii, jj, isp] -= ny * delx
                    bff[jpos].append(up[:, ii, jj, isp].copy())
                    flag[j].append(ii)
        bff[nye] = bff[nye] + bff[nys - 1]
        bff[nys] = bff[nys] + bff[nye + 1]
        for j in range(nys, nye + 1):
            jj = j - nys
            n2 = int(np2[jj, isp])
            fl = flag[j]
            buf = bff[j]
            iii = 0
            cnt = len(buf)
            cnt_tmp = len(fl) - 1
            k = 0
            done = False
            while k < len(fl) and not done:
                if cnt == 0:
                    if n2 - 1 < fl[k]:
                        break
                    while n2 - 1 == fl[cnt_tmp]:
                        n2 -= 1
                        if n2 - 1 < fl[k]:
                            done = True
                            break
                        cnt_tmp -= 1
                    if done:
                        break
                    up[:, fl[k], jj, isp] = up[:, n2 - 1, jj, isp]
                    n2 -= 1
                else:
                    up[:, fl[k], jj, isp] = buf[iii]
                    iii += 1
                    cnt -= 1
                k += 1
            for m in range(cnt):
                up[:, n2 + m, jj, isp] = buf[iii + m]
            n2 += cnt
            if n2 > npcap:
                raise RuntimeError("capacity")
            np2[jj, isp] = n2
    return up, np2


def closed_form_plan(dirs, ny):
    """The closed-form post-migration order the GPU implements (see
    wumingpic_gb300/csrc/kernels_common.cu, k_migrate_plan), for one species.
    dirs[jj] = int array (n,) of 0 stay / 1 up / 2 down.  Returns, per row, the
    list of (source row, source slot)."""
    up = [np.nonzero(d == 1)[0] for d in dirs]
    dn = [np.nonzero(d == 2)[0] for d in dirs]
    out = []
    for jj in range(ny):
        d = dirs[jj]
        n = len(d)
        holes = np.nonzero(d != 0)[0]
        h = len(holes)
        if ny == 1:
            arr = [(jj, s) for s in dn[jj]] + [(jj, s) for s in up[jj]]
        elif jj == 0:
            arr = [(1, s) for s in dn[1]] + [(ny - 1, s) for s in up[ny - 1]]
        elif jj == ny - 1:
            arr = [(jj - 1, s) for s in up[jj - 1]] + [(0, s) for s in dn[0]]
        else:
            arr = [(jj - 1, s) for s in up[jj - 1]] + [(jj + 1, s) for s in dn[jj + 1]]
        b = len(arr)
        nn = n - h + b
        seq = []
        tail = [t for t in range(n - 1, nn - 1, -1) if d[t] == 0] if b < h else []
        m = 0
        for t in range(nn):
            if t >= n:
                seq.append(arr[h + t - n])
            elif d[t] == 0:
                seq.append((jj, t))
            else:
                seq.append(arr[m] if m < b else (jj, tail[m - b]))
                m += 1
        out.append(seq)
    return out


# ---------------------------------------------------------------------------
# 3D
# ---------------------------------------------------------------------------
def small_plasma3d(nx=8, ny=6, nz=5, ppc=4, seed=3, **kw):
    from wumingpic_gb300.loader import Plasma3D
    kw.setdefault("drift", 0.5)
    kw.setdefault("u_the", 0.05)
    return Plasma3D(nx=nx, ny=ny, nz=nz, ppc=ppc, seed=seed, **kw)


def small_case3d(**kw):
    from wumingpic_gb300.loader import load_weibel3d
    p = small_plasma3d(**kw)
    return p, load_weibel3d(p)


def rho3d(p, up, np2, q):
    """Charge density on the periodic interior grid (nx, ny, nz), quadratic spline, cell int(x)."""
    R = np.zeros((p.nx, p.ny, p.nz))
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = np2[jj, kk, isp]
                pos = [up[d, :n, jj, kk, isp] / p.delx for d in range(3)]
                idx = [np.floor(a).astype(int) for a in pos]
                sh = []
                for d in range(3):
                    h = pos[d] - 0.5 - idx[d]
                    sh.append([0.5 * (0.5 - h) ** 2, 0.75 - h ** 2, 0.5 * (0.5 + h) ** 2])
                org = (p.nxgs, p.nygs, p.nzgs)
                dims = (p.nx, p.ny, p.nz)
                for a in range(3):
                    for b in range(3):
                        for c in range(3):
                            np.add.at(R, tuple((idx[d] + (a, b, c)[d] - 1 - org[d]) % dims[d] for d in range(3)),
                                      q[isp] * sh[0][a] * sh[1][b] * sh[2][c])
    return R


def continuity_residual3d(p, q, up0, gp1, np2, uj):
    """(rho1 - rho0) dx/dt + div J on the periodic interior; uj already folded."""
    r0 = rho3d(p, up0, np2, q)
    r1 = rho3d(p, gp1, np2, q)
    J = uj[:, 2:-2, 2:-2, 2:-2]
    res = (r1 - r0) * p.delx / p.delt
    for d in range(3):
        res = res + (np.roll(J[d], -1, d) - J[d])
    return np.abs(res).max(), np.abs(r1 - r0).max() * p.delx / p.delt


def literal_particle_yz(up, np2, p):
    """Pure-Python restatement of boundary_periodic__particle_yz
    (3d/common/boundary_periodic.f90:104-455) on one rank, single thread: wrap, buffer per
    destination row (ghost rows included), y transfers for all z rows, then z transfers,
    then hole filling.  Operates in place on the reference-layout arrays."""
    nys, nye, nzs, nze = p.nygs, p.nyge, p.nzgs, p.nzge
    ndim = up.shape[0]
    for isp in range(p.nsp):
        bff = {}
        flags = {}
        for k in range(nzs, nze + 1):
            for j in range(nys, nye + 1):
                fl = []
                for ii in range(1, np2[j - nys, k - nzs, isp] + 1):
                    a = up[:, ii - 1, j - nys, k - nzs, isp]
                    jpos = int(a[1] / p.delx)
                    kpos = int(a[2] / p.delx)
                    if not (jpos == j and kpos == k):
                        if jpos <= p.nygs - 1:
                            a[1] = a[1] + (p.nyge - p.nygs + 1) * p.delx
                        elif jpos >= p.nyge + 1:
                            a[1] = a[1] - (p.nyge - p.nygs + 1) * p.delx
                        if kpos <= p.nzgs - 1:
                            a[2] = a[2] + (p.nzge - p.nzgs + 1) * p.delx
                        elif kpos >= p.nzge + 1:
                            a[2] = a[2] - (p.nzge - p.nzgs + 1) * p.delx
                        bff.setdefault((jpos, kpos), []).append(a.copy())
                        fl.append(ii)
                flags[(j, k)] = fl
        for k in range(nzs - 1, nze + 2):
            bff.setdefault((nye, k), []).extend(bff.pop((nys - 1, k), []))
        for k in range(nzs - 1, nze + 2):
            bff.setdefault((nys, k), []).extend(bff.pop((nye + 1, k), []))
        for j in range(nys, nye + 1):
            bff.setdefault((j, nze), []).extend(bff.pop((j, nzs - 1), []))
        for j in range(nys, nye + 1):
            bff.setdefault((j, nzs), []).extend(bff.pop((j, nze + 1), []))
        for k in range(nzs, nze + 1):
            for j in range(nys, nye + 1):
                row = up[:, :, j - nys, k - nzs, isp]
                n2 = int(np2[j - nys, k - nzs, isp])
                fl = flags[(j, k)]
                arr = bff.get((j, k), [])
                iii = 0
                cnt = len(arr)
                cnt_tmp = len(fl)
                ii = 1
                while ii <= len(fl):
                    if cnt == 0:
                        if n2 < fl[ii - 1]:
                            break
                        done = False
                        while n2 == fl[cnt_tmp - 1]:
                            n2 -= 1
                            if n2 < fl[ii - 1]:
                                done = True
                                break
                            cnt_tmp -= 1
                        if done:
                            break
                        row[:, fl[ii - 1] - 1] = row[:, n2 - 1]
                        n2 -= 1
                    else:
                        row[:, fl[ii - 1] - 1] = arr[iii]
                        iii += 1
                        cnt -= 1
                    ii += 1
                for m in range(cnt):
                    row[:, n2 + m] = arr[iii + m]
                np2[j - nys, k - nzs, isp] = n2 + cnt
    return np2


def literal_moments2d(p, gp, np2, bc="periodic"):
    """mom_calc__nvt + bc__mom (2d/common/mom_calc.f90:164-249,
    2d/common/boundary_periodic.f90:571-636) in numpy, independent of the oracle's
    loops: np.add.at per node offset, then the ghost folds.  Summation order differs
    from the reference's, so agreement is to round-off."""
    nxm, nym = p.nx + 2, p.ny + 2
    mom = np.zeros((7, nxm, nym, p.nsp))
    for isp in range(p.nsp):
        for jj in range(p.ny):
            n = np2[jj, isp]
            x = gp[0, :n, jj, isp] / p.delx
            y = gp[1, :n, jj, isp] / p.delx
            u = gp[2:5, :n, jj, isp]
            ih = np.trunc(x - 0.5).astype(int)
            jh = np.trunc(y - 0.5).astype(int)
            dx, dy = x - 0.5 - ih, y - 0.5 - jh
            gam = 1.0 / np.sqrt(1.0 + (u * u).sum(0) / (p.c * p.c))
            pre = [np.ones(n), u[0] * gam, u[1] * gam, u[2] * gam, u[0] ** 2 * gam, u[1] ** 2 * gam, u[2] ** 2 * gam]
            for a, wx in ((0, 1.0 - dx), (1, dx)):
                for b, wy in ((0, 1.0 - dy), (1, dy)):
                    for l in range(7):
                        np.add.at(mom[l, :, :, isp], (ih + a - (p.nxgs - 1), jh + b - (p.nygs - 1)), pre[l] * wx * wy)
    if bc == "reconnection":
        mom[:, 1] += mom[:, 0]
        mom[:, nxm - 2] += mom[:, nxm - 1]
    else:
        mom[:, 1] += mom[:, nxm - 1]
        mom[:, nxm - 2] += mom[:, 0]
    mom[:, :, nym - 2] += mom[:, :, 0]
    mom[:, :, 1] += mom[:, :, nym - 1]
    return mom


def literal_moments3d(p, gp, np2, bc="periodic"):
    """mom_calc__nvt + bc__mom in 3D (3d/common/mom_calc.f90:219-332,
    3d/common/boundary_periodic.f90:1102-1235; with walls the x ghosts fold onto the wall
    columns, 3d/proj/reconnection/boundary_reconnection.f90:1134-1137) in numpy."""
    nxm, nym, nzm = p.nx + 2, p.ny + 2, p.nz + 2
    mom = np.zeros((7, nxm, nym, nzm, p.nsp))
    for isp in range(p.nsp):
        for kk in range(p.nz):
            for jj in range(p.ny):
                n = np2[jj, kk, isp]
                r = gp[0:3, :n, jj, kk, isp]
                u = gp[3:6, :n, jj, kk, isp]
                h = np.floor(r / p.delx - 0.5).astype(int)
                d = r - 0.5 - h
                gam = 1.0 / np.sqrt(1.0 + (u * u).sum(0) / (p.c * p.c))
                pre = [np.ones(n), u[0] * gam, u[1] * gam, u[2] * gam, u[0] ** 2 * gam, u[1] ** 2 * gam,
                       u[2] ** 2 * gam]
                for a in (0, 1):
                    for b in (0, 1):
                        for cz in (0, 1):
                            w = (d[0] if a else 1 - d[0]) * (d[1] if b else 1 - d[1]) * (d[2] if cz else 1 - d[2])
                            idx = (h[0] + a - (p.nxgs - 1), h[1] + b - (p.nygs - 1), h[2] + cz - (p.nzgs - 1))
                            for l in range(7):
                                np.add.at(mom[l, :, :, :, isp], idx, pre[l] * w)
    if bc == "periodic":
        mom[:, 1] += mom[:, nxm - 1]
        mom[:, nxm - 2] += mom[:, 0]
    else:
        mom[:, 1] += mom[:, 0]
        mom[:, nxm - 2] += mom[:, nxm - 1]
    mom[:, :, nym - 2] += mom[:, :, 0]
    mom[:, :, 1] += mom[:, :, nym - 1]
    mom[:, :, 1:nym - 1, nzm - 2] += mom[:, :, 1:nym - 1, 0]
    mom[:, :, 1:nym - 1, 1] += mom[:, :, 1:nym - 1, nzm - 1]
    return mom
