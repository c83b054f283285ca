"""Restart snapshots in the reference's format (paraio__output / paraio__input).

CPU tests: the JSON index text against the reference's own fixture
(utils/iocore/jsonio_expected.json, copied to tests/golden/), and round trips of 2D and 3D
snapshots whose raw layout is checked independently of the writer (record by record,
offsets recomputed from the record sizes).  The GPU test continues a run from a snapshot
and compares it with the uninterrupted run.
"""
import json
import os

import numpy as np
import pytest

from tests.helpers import small_case, small_case3d
from wumingpic_gb300 import restart

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jsonio_expected.json")


def test_json_index_text_matches_reference_fixture():
    """The index that utils/iocore/jsonio_test.f90 writes, rebuilt with the restart writer's
    printer, is the fixture's text byte for byte."""
    def att(kind, off, size, shape, desc, data):
        return {"datatype": kind, "offset": off, "size": size, "ndim": 1, "shape": shape, "description": desc,
                "data": data}
    index = {
        "meta": {"endian": 1, "rawfile": "test.raw", "info": "some information", "large_int": 2 ** 32},
        "attribute": {
            "nx": att("i4", 0, 4, [1], "# grid in x", 16),
            "ny": att("i4", 4, 4, [1], "# grid in y", 32),
            "ns": att("i4", 8, 4, [1], "# species", 2),
            "mass": att("f8", 12, 16, [2], "mass", [1.0, 100.0]),
            "charge": att("f8", 28, 16, [2], "charge", [-1.0, 1.0]),
        },
        "dataset": {
            "emf": {"datatype": "f8", "offset": 44, "size": 24576, "ndim": 3, "shape": [6, 32, 16],
                    "description": "electromagnetic fields"},
            "mom": {"datatype": "f8", "offset": 24620, "size": 40960, "ndim": 3, "shape": [10, 32, 16],
                    "description": "moments"},
        },
    }
    with open(GOLDEN) as f:
        expected = f.read()
    assert restart.dumps_json_fortran(index) == expected


@pytest.mark.parametrize("v,s", [(1.0, "0.1E+1"), (100.0, "0.1E+3"), (-1.0, "-0.1E+1"), (0.5, "0.5E+0"),
                                 (0.0, "0.0E+0"), (0.01151647, "0.1151647E-1"), (2.5e-300, "0.25E-299")])
def test_fortran_real_format(v, s):
    assert restart.fortran_real(v) == s
    assert float(s) == v


def _records(index):
    recs = [(k, v) for sec in ("attribute", "dataset") for k, v in index[sec].items()]
    return sorted(recs, key=lambda kv: kv[1]["offset"])


def test_restart2d_round_trip_and_layout(tmp_path):
    p, st = small_case(nx=16, ny=12, ppc=4, seed=61)
    rng = np.random.default_rng(61)
    st.uf[...] = rng.standard_normal(st.uf.shape)
    df = np.asfortranarray(rng.standard_normal(st.uf.shape))
    prefix = str(tmp_path / "0000123_restart")
    restart.write_restart2d(prefix, p, st.up, st.uf, st.np2, 123, df=df)
    index = json.load(open(prefix + ".json"))
    # records are back to back from offset 0, in the reference's order
    names = [k for k, _ in _records(index)]
    assert names == ["dummy_attribute", "it", "nxs", "nxe", "ndim", "np", "nxgs", "nxge", "nygs", "nyge", "nsp",
                     "nproc", "delx", "delt", "c", "r", "q", "up", "np2", "uf", "df"]
    off = 0
    for _, v in _records(index):
        assert v["offset"] == off
        off += v["size"]
    assert os.path.getsize(prefix + ".raw") == off
    raw = open(prefix + ".raw", "rb").read()
    a = index["attribute"]
    assert np.frombuffer(raw, "<i4", 1, 0)[0] == 8 and a["it"]["data"] == 123
    assert a["nxs"]["data"] == p.nxgs and a["nxe"]["data"] == p.nxge and a["np"]["data"] == p.np_cap
    q, r = p.charges()
    np.testing.assert_array_equal(np.frombuffer(raw, "<f8", p.nsp, a["q"]["offset"]), q)
    d = index["dataset"]
    assert d["up"]["shape"] == [p.ndim, p.np_cap, p.ny, p.nsp, 1]
    up = np.frombuffer(raw, "<f8", st.up.size, d["up"]["offset"]).reshape(st.up.shape, order="F")
    np.testing.assert_array_equal(up, st.up)
    # reader
    up2, uf2, np22, it, nxs, nxe, df2 = restart.read_restart2d(prefix, p)
    np.testing.assert_array_equal(up2, st.up)
    np.testing.assert_array_equal(uf2, st.uf)
    np.testing.assert_array_equal(np22, st.np2)
    np.testing.assert_array_equal(df2, df)
    assert (it, nxs, nxe) == (123, p.nxgs, p.nxge)
    # the consistency test of paraio__input
    from wumingpic_gb300.loader import Plasma2D
    with pytest.raises(ValueError):
        restart.read_restart2d(prefix, Plasma2D(nx=16, ny=14, ppc=4))


def test_restart3d_packs_rows_in_reference_order(tmp_path):
    p, st = small_case3d(seed=62)
    prefix = str(tmp_path / "snap3d")
    restart.write_restart3d(prefix, p, st.up, st.uf, st.np2, 7)
    index = json.load(open(prefix + ".json"))
    names = [k for k, _ in _records(index)]
    assert names[-5:] == ["np2", "up01", "up02", "poffset", "uf"]
    d = index["dataset"]
    raw = open(prefix + ".raw", "rb").read()
    for isp in range(p.nsp):
        meta = d[f"up{isp + 1:02d}"]
        n = int(st.np2[:, :, isp].sum())
        assert meta["shape"] == [p.ndim, n]
        packed = np.frombuffer(raw, "<f8", p.ndim * n, meta["offset"]).reshape((p.ndim, n), order="F")
        ip = 0
        for k in range(p.nz):          # k outer, j inner (3d/common/paraio.f90:1025-1036)
            for j in range(p.ny):
                m = st.np2[j, k, isp]
                np.testing.assert_array_equal(packed[:, ip:ip + m], st.up[:, :m, j, k, isp])
                ip += m
    up2, uf2, np22, it, _, _, df2 = restart.read_restart3d(prefix, p)
    assert it == 7 and df2 is None
    np.testing.assert_array_equal(np22, st.np2)
    np.testing.assert_array_equal(uf2, st.uf)
    for isp in range(p.nsp):
        for k in range(p.nz):
            for j in range(p.ny):
                m = st.np2[j, k, isp]
                np.testing.assert_array_equal(up2[:, :m, j, k, isp], st.up[:, :m, j, k, isp])


def test_bucket_sort_rebuilds_cumcnt():
    """A sorted state comes back unchanged with its cumcnt; a shuffled row is sorted stably."""
    p, st = small_case(nx=16, ny=12, ppc=4, seed=63)
    up, cc = restart.bucket_sort_rows(st.up, st.np2, p)
    np.testing.assert_array_equal(cc, st.cumcnt)
    for isp in range(p.nsp):
        for j in range(p.ny):
            n = st.np2[j, isp]
            np.testing.assert_array_equal(up[:, :n, j, isp], st.up[:, :n, j, isp])
    sh = st.up.copy(order="F")
    n = st.np2[3, 0]
    perm = np.random.default_rng(0).permutation(n)
    sh[:, :n, 3, 0] = sh[:, perm, 3, 0]
    up2, cc2 = restart.bucket_sort_rows(sh, st.np2, p)
    np.testing.assert_array_equal(cc2, st.cumcnt)
    x = up2[0, :n, 3, 0]
    assert np.all(np.diff(np.trunc(x)) >= 0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64_exact", "mixed"])
def test_restart_continues_the_run(gpu_lib, tmp_path, precision):
    """Six steps straight, against three steps, a snapshot, a fresh context loaded from it and
    three more steps: identical particles, fields and CG warm start (the df extension)."""
    from wumingpic_gb300.pic2d import Pic2D
    p, st = small_case(nx=32, ny=32, ppc=6, seed=64, u_the=0.1)
    a = Pic2D(p, precision=precision)
    a.put_state(st)
    a.step(6)
    ref = a.get_state()
    b = Pic2D(p, precision=precision)
    b.put_state(st)
    b.step(3)
    prefix = str(tmp_path / "0000003_restart")
    restart.save(b, prefix, 3)
    c = Pic2D(p, precision=precision)
    assert restart.load(c, prefix) == 3
    c.step(3)
    out = c.get_state()
    if precision == "mixed":
        # the fixed-point current scales follow the bin depths, which a reload lays out
        # afresh, so the continued run agrees to FP32 round-off rather than bit for bit
        assert out.np2.sum() == ref.np2.sum()
        np.testing.assert_allclose(c.energy(), a.energy(), rtol=1e-5)
        return
    np.testing.assert_array_equal(out.np2, ref.np2)
    np.testing.assert_array_equal(out.cumcnt, ref.cumcnt)
    for isp in range(p.nsp):
        for j in range(p.ny):
            n = ref.np2[j, isp]
            np.testing.assert_array_equal(out.up[:, :n, j, isp], ref.up[:, :n, j, isp])
    np.testing.assert_array_equal(out.uf, ref.uf)
    np.testing.assert_array_equal(c.get_df(), a.get_df())
