"""Host-side pieces of bench.py that run without a GPU: the end-to-end timing around the C
ABI's synchronous calls (with a stand-in context and link figures) and the summary of the
bench line's legs."""
import json
import time
import types

import numpy as np

import bench


class _FakeContext:
    """put / step / get that take known times, like the C ABI's calls (each returns after its work)."""

    def __init__(self, st, put_s=0.004, step_s=0.002, get_s=0.006):
        self.st, self.put_s, self.step_s, self.get_s = st, put_s, step_s, get_s

    def get_state(self, st=None):
        time.sleep(self.get_s)
        return self.st

    def put_state(self, st):
        time.sleep(self.put_s)

    def step(self, n):
        time.sleep(self.step_s * n)


def test_measure_e2e_splits_the_step(monkeypatch):
    from wumingpic_gb300 import _lib
    monkeypatch.setattr(_lib, "host_register", lambda a: None)
    monkeypatch.setattr(_lib, "host_unregister", lambda a: None)
    monkeypatch.setattr(bench, "measure_link", lambda: {"h2d_gbs": 200.0, "d2h_gbs": 100.0})
    np2 = np.full((8, 2), 5, np.int32)
    st = types.SimpleNamespace(up=np.zeros((6, 9, 8, 2), order="F"), uf=np.zeros((6, 12, 12), order="F"),
                               cumcnt=np.zeros((9, 8, 2), np.int32, order="F"), np2=np2)
    out = bench.measure_e2e(_FakeContext(st), types.SimpleNamespace(ndim=6))
    nbytes = int(np2.sum()) * 6 * 8 + st.uf.nbytes + np2.nbytes + st.cumcnt.nbytes
    assert out["h2d_bytes_per_step"] == out["d2h_bytes_per_step"] == nbytes
    link = out["link"]
    split = link["split_ms_per_step"]
    assert split["put"] >= 4.0 and split["step"] >= 2.0 and split["get"] >= 6.0
    assert abs(split["put"] + split["step"] + split["get"] - link["e2e_ms_per_step"]) < 1.0
    floor = 1e3 * (nbytes / 200e9 + nbytes / 100e9)
    assert abs(link["exchange_floor_ms_per_step"] - floor) < 1e-12
    assert abs(link["frac"] - floor / link["e2e_ms_per_step"]) < 1e-12
    assert abs(link["put_gbs"] - nbytes / (split["put"] * 1e-3) / 1e9) < 1e-9 * link["put_gbs"]
    assert out["value"] == int(np2.sum()) * out["steps"] / (link["e2e_ms_per_step"] * out["steps"] / 1e3)
    json.dumps(out)


def _line():
    kern = {"ref_flops_over_fp64_peak": 0.67, "hbm_frac": 0.05}
    return {
        "fp64_path": {"value": 1.4e9, "ms_per_step": 384.0, "mixed_over_fp64": 32.6, "fp64_fma_peak_gflops": 1255.0,
                      "kernels": {"k_push2d": dict(kern), "k_deposit2d": dict(kern)}},
        "mixed_3d_path": {"value": 1.26e10, "ms_per_step": 42.4, "mixed_over_fp64": 50.3},
        "fp64_3d_path": {"value": 2.5e8, "ms_per_step": 2137.0},
        "reconnection": {"mixed": {"value": 1.1e10}, "fp64": {"value": 8.4e8}, "mixed_over_fp64": 13.2},
        "adjoint": {"cost_over_forward": 3.46, "fd_check": {"rel_err": 3.9e-11},
                    "mixed_adjoint": {"cost_over_mixed_forward": 17.1}},
        "growth_check": {"growth_rate_rel_err": 2.7e-8, "energy_max_rel_diff": 9.7e-10,
                         "workload": "2D Weibel 512^2 cells, 64 ppc/species"},
    }


def test_summary_of_every_leg():
    out = bench.summary(_line())
    assert set(out) == {"fp64_2d", "mixed_3d", "fp64_3d", "reconnection", "adjoint", "growth_check"}
    assert out["fp64_2d"]["k_push2d"]["fp64_pipe_active_ncu"] == bench.FP64_PIPE_ACTIVE_NCU["k_push2d"]
    assert out["adjoint"]["cost_over_forward"] == 3.46
    assert out["adjoint"]["mixed_cost_over_mixed_forward"] == 17.1
    assert out["growth_check"]["grid"] == "512^2"
    assert "mixed_over_fp64" not in out["fp64_3d"]
    assert len(json.dumps(out)) < 1500  # short enough to survive a truncated log


def test_summary_with_legs_skipped():
    line = _line()
    for key in ("fp64_path", "mixed_3d_path", "reconnection", "growth_check"):
        line[key] = None
    del line["adjoint"]["mixed_adjoint"]
    out = bench.summary(line)
    assert set(out) == {"fp64_3d", "adjoint"}
    assert "mixed_cost_over_mixed_forward" not in out["adjoint"]
