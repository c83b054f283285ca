"""Restart snapshots in the reference's own file format.

A snapshot is the pair <prefix>.raw / <prefix>.json that paraio__output writes and
paraio__input reads (2d/common/paraio.f90:93-428, 3d/common/paraio.f90): a raw file of
little-endian records written back to back, and a JSON index (json-fortran's printer)
that gives every record's datatype, byte offset, byte size, shape and, for the scalar and
small-array attributes, the value itself.

Record order, one rank (nproc = 1):
  attributes  dummy_attribute(i4 = 8), it, nxs, nxe, ndim, np, nxgs, nxge, nygs, nyge,
              [nzgs, nzge,] nsp, nproc, delx, delt, c, r(nsp), q(nsp)
              (paraio.f90:150-160 and put_metadata, 2d/common/paraio.f90:956-1002)
  2D datasets up(ndim, np, nyl, nsp, 1) f8, np2(nyl, nsp, 1) i4,
              uf(6, nx+4, ny+4, 1) f8                      (2d/common/paraio.f90:172-225)
  3D datasets np2(nyl, nzl, nsp, 1) i4, upNN(ndim, npg) f8 per species holding the active
              particles of rows (j, k) in k-outer order, poffset(nsp, 1) i8,
              uf(6, nx+4, ny+4, nz+4, 1) f8                (3d/common/paraio.f90:183-270)

One extension, appended after uf and ignored by paraio__input (it reads datasets by name):
df, the SAVEd CG warm start of field__fdtd_i, so that a restarted run continues bit for
bit instead of restarting the solver from zero as the reference does.

cumcnt is not part of the snapshot; the drivers rebuild it with sort__bucket after
io__input (2d/proj/weibel/app.f90:351-352), and `load` does the same.
"""
import json
import os
import sys

import numpy as np

_DUMMY_ATTRIBUTE = 8  # MPI_OFFSET_KIND, the value paraio__output writes first (paraio.f90:150)


# ---------------------------------------------------------------------------
# json-fortran's printer: two-space indentation, one array element per line, and reals
# in the compact form of an E30.16E3 edit descriptor (0.1E+1 for 1.0).
# ---------------------------------------------------------------------------
def fortran_real(v):
    """A double as json-fortran prints it: the 16-digit mantissa 0.d1d2... of an
    E30.16E3 edit descriptor without trailing zeros, the exponent without leading zeros."""
    v = float(v)
    if v == 0.0:
        return "0.0E+0"
    sign = "-" if v < 0 else ""
    d, e = f"{abs(v):.15e}".split("e")  # d.ddddddddddddddd x 10^e, correctly rounded
    digits = d.replace(".", "").rstrip("0") or "0"
    exp = int(e) + 1
    return f"{sign}0.{digits}E{'+' if exp >= 0 else '-'}{abs(exp)}"


def _dump(v, level):
    pad = "  " * level
    if isinstance(v, dict):
        items = [f'{pad}  "{k}": {_dump(x, level + 1).lstrip()}' for k, x in v.items()]
        return pad + "{\n" + ",\n".join(items) + "\n" + pad + "}"
    if isinstance(v, (list, tuple)):
        items = [pad + "  " + _dump(x, level + 1).lstrip() for x in v]
        return pad + "[\n" + ",\n".join(items) + "\n" + pad + "]"
    if isinstance(v, str):
        return pad + json.dumps(v)
    if isinstance(v, (bool, np.bool_)):
        return pad + ("true" if v else "false")
    if isinstance(v, (int, np.integer)):
        return pad + str(int(v))
    return pad + fortran_real(v)


def dumps_json_fortran(obj):
    """The text json-fortran's json%print writes for `obj` (dicts keep insertion order)."""
    return _dump(obj, 0) + "\n"


# ---------------------------------------------------------------------------
# raw records
# ---------------------------------------------------------------------------
class _Writer:
    def __init__(self, fh):
        self.fh = fh
        self.disp = 0
        self.attribute = {}
        self.dataset = {}

    def attr(self, name, value, kind):
        arr = np.atleast_1d(np.asarray(value, dtype="<i4" if kind == "i4" else "<f8"))
        entry = {"datatype": kind, "offset": self.disp, "size": int(arr.nbytes), "ndim": 1,
                 "shape": [int(arr.size)], "description": ""}
        data = [int(x) if kind == "i4" else float(x) for x in arr]
        entry["data"] = data[0] if np.ndim(value) == 0 else data
        self.attribute[name] = entry
        self.fh.write(arr.tobytes())
        self.disp += arr.nbytes

    def data(self, name, arr, kind, shape, desc):
        dt = {"f8": "<f8", "i4": "<i4", "i8": "<i8"}[kind]
        raw = np.asarray(arr, dtype=dt).tobytes(order="F")
        self.dataset[name] = {"datatype": kind, "offset": self.disp, "size": len(raw), "ndim": len(shape),
                              "shape": [int(x) for x in shape], "description": desc}
        self.fh.write(raw)
        self.disp += len(raw)


def _endian_flag():
    return 1 if sys.byteorder == "little" else 16777216  # mpiio_get_endian_flag


def _common_attributes(w, it, nxs, nxe, p, ndim, three_d):
    q, r = p.charges()
    w.attr("dummy_attribute", _DUMMY_ATTRIBUTE, "i4")
    w.attr("it", it, "i4")
    w.attr("nxs", nxs, "i4")
    w.attr("nxe", nxe, "i4")
    w.attr("ndim", ndim, "i4")
    w.attr("np", p.np_cap, "i4")
    w.attr("nxgs", p.nxgs, "i4")
    w.attr("nxge", p.nxge, "i4")
    w.attr("nygs", p.nygs, "i4")
    w.attr("nyge", p.nyge, "i4")
    if three_d:
        w.attr("nzgs", p.nzgs, "i4")
        w.attr("nzge", p.nzge, "i4")
    w.attr("nsp", p.nsp, "i4")
    w.attr("nproc", 1, "i4")
    w.attr("delx", p.delx, "f8")
    w.attr("delt", p.delt, "f8")
    w.attr("c", p.c, "f8")
    w.attr("r", np.asarray(r, dtype=np.float64), "f8")
    w.attr("q", np.asarray(q, dtype=np.float64), "f8")


def _finish(prefix, w):
    index = {"meta": {"endian": _endian_flag(), "rawfile": os.path.basename(prefix) + ".raw"},
             "attribute": w.attribute, "dataset": w.dataset}
    with open(prefix + ".json", "w") as f:
        f.write(dumps_json_fortran(index))


def write_restart2d(prefix, p, up, uf, np2, it, df=None):
    """paraio__output(up, uf, np2, nxs, nxe, it, prefix) for one rank (2d/common/paraio.f90:93)."""
    ndim = up.shape[0]
    with open(prefix + ".raw", "wb") as fh:
        w = _Writer(fh)
        _common_attributes(w, it, p.nxgs, p.nxge, p, ndim, False)
        w.data("up", up, "f8", (ndim, up.shape[1], up.shape[2], up.shape[3], 1), "particles")
        w.data("np2", np2, "i4", (np2.shape[0], np2.shape[1], 1), "number of active particles")
        w.data("uf", uf, "f8", (6, uf.shape[1], uf.shape[2], 1), "electromagnetic fields including ghost cells")
        if df is not None:
            w.data("df", df, "f8", (6, df.shape[1], df.shape[2], 1), "CG warm start of field__fdtd_i (extension)")
    _finish(prefix, w)


def write_restart3d(prefix, p, up, uf, np2, it, df=None):
    """paraio__output of the 3D code for one rank: active particles packed per species."""
    ndim = up.shape[0]
    with open(prefix + ".raw", "wb") as fh:
        w = _Writer(fh)
        _common_attributes(w, it, p.nxgs, p.nxge, p, ndim, True)
        w.data("np2", np2, "i4", (np2.shape[0], np2.shape[1], np2.shape[2], 1), "number of active particles")
        for isp in range(p.nsp):
            packed = pack_species3d(up, np2, isp)
            w.data(f"up{isp + 1:02d}", packed, "f8", (ndim, packed.shape[1]), f"particle species #{isp + 1:02d}")
        w.data("poffset", np.zeros((p.nsp, 1), np.int64), "i8", (p.nsp, 1), "particle offset")
        w.data("uf", uf, "f8", (6, uf.shape[1], uf.shape[2], uf.shape[3], 1),
               "electromagnetic fields including ghost cells")
        if df is not None:
            w.data("df", df, "f8", (6, df.shape[1], df.shape[2], df.shape[3], 1),
                   "CG warm start of field__fdtd_i (extension)")
    _finish(prefix, w)


def pack_species3d(up, np2, isp):
    """get_particle_count mode 0 (3d/common/paraio.f90:1020-1037): the active particles of
    species isp, rows in (k outer, j inner) order, as an (ndim, n) array."""
    cols = [up[:, :np2[j, k, isp], j, k, isp] for k in range(np2.shape[1]) for j in range(np2.shape[0])]
    return np.concatenate(cols, axis=1) if cols else np.zeros((up.shape[0], 0))


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------
class Snapshot:
    """The records of a snapshot: .attribute[name] (scalars and small arrays) and
    .dataset[name] (arrays in the reference's Fortran order)."""

    def __init__(self, prefix):
        with open(prefix + ".json") as f:
            self.index = json.load(f)
        self.raw = prefix + ".raw"
        if self.index["meta"]["endian"] != 1:
            raise ValueError("big-endian snapshots are not supported")
        self.attribute = {k: self._read(v) for k, v in self.index["attribute"].items()}
        for k, v in list(self.attribute.items()):
            if self.index["attribute"][k]["shape"] == [1]:
                self.attribute[k] = v[0]

    def _read(self, meta):
        dt = {"f8": "<f8", "i4": "<i4", "i8": "<i8"}[meta["datatype"]]
        n = meta["size"] // np.dtype(dt).itemsize
        a = np.fromfile(self.raw, dtype=dt, count=n, offset=meta["offset"])
        if a.size != n:
            raise ValueError(f"snapshot {self.raw} is truncated")
        return a

    def has(self, name):
        return name in self.index["dataset"]

    def dataset(self, name):
        meta = self.index["dataset"][name]
        return self._read(meta).reshape(meta["shape"], order="F")


def _check(snap, p, three_d):
    """The consistency test of paraio__input (2d/common/paraio.f90:332-345)."""
    a = snap.attribute
    want = {"nxgs": p.nxgs, "nxge": p.nxge, "nygs": p.nygs, "nyge": p.nyge, "np": p.np_cap, "nsp": p.nsp, "nproc": 1}
    if three_d:
        want.update(nzgs=p.nzgs, nzge=p.nzge)
    bad = [k for k, v in want.items() if int(a[k]) != int(v)]
    if bad:
        raise ValueError(f"invalid input parameters: {', '.join(bad)}")


def read_restart2d(prefix, p):
    """paraio__input for one rank: (up, uf, np2, it, nxs, nxe, df or None)."""
    s = Snapshot(prefix)
    _check(s, p, False)
    up = np.asfortranarray(s.dataset("up")[..., 0])
    np2 = np.asfortranarray(s.dataset("np2")[..., 0])
    uf = np.asfortranarray(s.dataset("uf")[..., 0])
    df = np.asfortranarray(s.dataset("df")[..., 0]) if s.has("df") else None
    a = s.attribute
    return up, uf, np2, int(a["it"]), int(a["nxs"]), int(a["nxe"]), df


def read_restart3d(prefix, p):
    """paraio__input of the 3D code for one rank: the packed species unpacked into rows."""
    s = Snapshot(prefix)
    _check(s, p, True)
    a = s.attribute
    np2 = np.asfortranarray(s.dataset("np2")[..., 0])
    ndim = int(a["ndim"])
    up = np.zeros((ndim, p.np_cap, p.ny, p.nz, p.nsp), order="F")
    for isp in range(p.nsp):
        packed = s.dataset(f"up{isp + 1:02d}")
        ip = 0
        for k in range(p.nz):
            for j in range(p.ny):
                n = np2[j, k, isp]
                up[:, :n, j, k, isp] = packed[:, ip:ip + n]
                ip += n
    uf = np.asfortranarray(s.dataset("uf")[..., 0])
    df = np.asfortranarray(s.dataset("df")[..., 0]) if s.has("df") else None
    return up, uf, np2, int(a["it"]), int(a["nxs"]), int(a["nxe"]), df


# ---------------------------------------------------------------------------
# GPU contexts
# ---------------------------------------------------------------------------
def bucket_sort_rows(up, np2, p):
    """sort__bucket's stable counting sort by cell, int(x) - nxgs (2d/common/sort.f90:36-82;
    3d/common/sort.f90:40-88), applied to every row: returns (sorted up, cumcnt)."""
    out = np.zeros_like(up, order="F")
    rows = np2.shape[:-1]
    cumcnt = np.zeros((p.nx + 1,) + np2.shape, np.int32, order="F")
    for isp in range(np2.shape[-1]):
        for idx in np.ndindex(*rows):
            sel = (slice(None), slice(0, np2[idx + (isp,)])) + idx + (isp,)
            part = up[sel]
            cell = np.trunc(part[0]).astype(np.int64) - p.nxgs
            order = np.argsort(cell, kind="stable")
            out[sel] = part[:, order]
            counts = np.bincount(cell, minlength=p.nx)[:p.nx]
            cumcnt[(slice(1, None),) + idx + (isp,)] = np.cumsum(counts)
    return out, cumcnt


def save(g, prefix, it, with_df=True):
    """Snapshot of a Pic2D / Pic3D context in the reference's format (+ df)."""
    st = g.get_state()
    df = g.get_df() if with_df else None
    if st.up.ndim == 5:
        write_restart3d(prefix, g.p, st.up, st.uf, st.np2, it, df)
    else:
        write_restart2d(prefix, g.p, st.up, st.uf, st.np2, it, df)


def load(g, prefix):
    """io__input followed by sort__bucket, as the drivers restart; restores df when the
    snapshot carries it.  Returns the step number it."""
    three_d = hasattr(g.p, "nz")
    if three_d:
        from wumingpic_gb300.loader import empty_state3d as empty
        up, uf, np2, it, _, _, df = read_restart3d(prefix, g.p)
    else:
        from wumingpic_gb300.loader import empty_state2d as empty
        up, uf, np2, it, _, _, df = read_restart2d(prefix, g.p)
    st = empty(g.p)
    st.up[...], st.cumcnt[...] = bucket_sort_rows(up, np2, g.p)
    st.np2[...] = np2
    st.uf[...] = uf
    st.gp[...] = st.up
    g.put_state(st)
    if df is not None:
        g.put_df(df)
    return it
