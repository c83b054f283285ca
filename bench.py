"""Benchmark of the 2D particle-in-cell step (particle-updates/s).

Default workload: the 2D Weibel configuration at scale -- 2048 x 2048 cells,
64 particles per cell per species (536,870,912 particles), beams +-0.3c,
u_th = 0.1c, c dt/dx = 0.5 -- loaded on the device from a seeded Philox
stream (synthetic data).  One step = push + deposition + implicit field solve
(CG) + particle boundaries + bucket sort/migration: one pass of the reference
driver loop body (2d/proj/weibel/app.f90:102-107).

The headline value is the mixed-precision path (FP32 particles, FP64 fields);
the FP64 path is timed beside it on the same workload.  Prints one JSON line.
``--impl reference`` times the CPU restatement of the reference (oracle/,
OpenMP over all host cores) on the same metric instead.
"""
import argparse
import dataclasses
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-updates/s on 1 GB300: mixed vs FP64 path at <=1% growth-rate error"
UNIT = "particle-updates/s"

# Algorithmic bytes of the dominant kernels (compulsory traffic, one launch):
#  k_mix_push2 (mixed push + deposit): per particle read its 32-byte state and write it back =
#    64 B, the per-update figure of the split representation (cell index 4 B + two FP32
#    offsets 8 B + three FP32 momenta 12 B + 64-bit id 8 B); here the cell is implicit in the
#    particle's column and those 4 bytes of the slot carry the arrival key of a particle that
#    changes cell.
#  k_push2d (FP64 push): per particle read x, y, ux, uy, uz, id (48 B) + write them (48 B) = 96 B.
#  k_deposit2d (FP64 deposit): per particle read old x, y (16 B) + new x, y, ux, uy, uz (40 B)
#    = 56 B, plus 600 B per cell for the cell's 5x5x3 current tile.
BYTES_MIX_PUSH = 64
# k_mix_push2's measured DRAM traffic per particle: dram__bytes_read.sum + dram__bytes_write.sum of
# one launch on the 512^2 x 64 ppc case of the same physics (1.135 + 1.037 GB for 33,554,432
# particles), scaled to the particles of a launch (an earlier build of the kernel moved 64.4 B per
# particle at 512^2 and 66.4 B on the 2048^2 workload)
TRAFFIC_MIX_PUSH_PER_PARTICLE = (1.135205e9 + 1.036641e9) / 33554432
BYTES_PUSH_FP64 = 96
BYTES_DEPOSIT_FP64 = 56
BYTES_DEPOSIT_CELL = 600
# FP64 floating-point operations per particle of the FP64 kernels, counted from the
# reference's statements (2d/common/particle.f90:99-163, 2d/common/field.f90:224-298) with
# each sqrt and divide counted as one operation: `ref_fp64_gflops` is that count over the launch
# time, a reference-equivalent rate (the FMA build's factored deposit executes fewer operations,
# the push's FP64 sqrt and divides more)
FLOP_PUSH_FP64 = 215
FLOP_DEPOSIT_FP64 = 600
# FP64 pipe utilisation of the same kernels measured by ncu (sm__inst_executed_pipe_fp64,
# pct_of_peak_sustained_active) on one launch at 512^2 x 64 ppc: what bounds them
FP64_PIPE_ACTIVE_NCU = {"k_push2d": 0.912, "k_deposit2d": 0.862}


def config(name):
    from wumingpic_gb300.loader import Plasma2D
    if name == "cfg1":
        return Plasma2D(nx=2048, ny=2048, ppc=64, drift=0.3, u_the=0.1, seed=20261203, np_slack=1.25)
    if name == "cfg0":
        return Plasma2D(nx=256, ny=256, ppc=16, drift=0.5, u_the=0.05, seed=20261203)
    if name.startswith("sq"):  # sqN_PPC: N x N cells, PPC per species, the cfg1 physics
        n, ppc = name[2:].split("_")
        return Plasma2D(nx=int(n), ny=int(n), ppc=int(ppc), drift=0.3, u_the=0.1, seed=20261203, np_slack=1.25)
    raise ValueError(name)


def workload_desc(p, name):
    return {"workload": f"2D Weibel {p.nx}x{p.ny} cells, {p.ppc} ppc/species, {p.n_particles} particles, "
                        f"drift +-{p.drift}c, u_th {p.u_the}c, c*dt/dx={p.c * p.delt / p.delx}",
            "name": name, "nx": p.nx, "ny": p.ny, "ppc_per_species": p.ppc, "particles": p.n_particles,
            "l2": "inputs larger than L2 (particle state >> 129 MB)", "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:  # noqa: BLE001
                pass
            self._stop.wait(0.2)

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        smax = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(self.rows)}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


def host_mem_available():
    """MemAvailable of this host in bytes (Linux), or None."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def oracle_grid(full):
    """The workload's grid if the oracle's state fits this host's memory (up and gp in the
    reference layout plus the migration buffers: about 2.6 x the up array), else the largest
    square grid of the same physics and particles per cell that does, and whether it is the
    full grid."""
    per_cell = full.np_slack * full.ppc * full.nsp * 6 * 8 * 2.6 / 2  # bytes per cell
    avail = host_mem_available()
    n = full.nx
    while avail is not None and n > 64 and n * n * per_cell * 2 > 0.85 * avail:
        n //= 2
    return n, n == full.nx


def oracle_state(full, n):
    """Oracle instance and reference-layout state of the workload's physics on n x n cells,
    written by the oracle's row-parallel loader (seeded counter hash)."""
    import ctypes
    import numpy as np
    from oracle.oracle import Oracle2D, lib as orc_lib
    from wumingpic_gb300.loader import Plasma2D, empty_state2d
    p = Plasma2D(nx=n, ny=n, ppc=full.ppc, drift=full.drift, u_the=full.u_the, seed=full.seed,
                 np_slack=full.np_slack)
    st = empty_state2d(p)
    L = orc_lib()
    L.orc2d_load_weibel.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 7 + [
        ctypes.c_double, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_ulonglong]
    sd = np.array([p.u_thi, p.u_the])
    rc = L.orc2d_load_weibel(st.up.ctypes.data, st.cumcnt.ctypes.data, st.np2.ctypes.data, p.nx, p.ny, p.np_cap,
                             p.nsp, p.ppc, p.nxgs, p.nygs, p.delx, sd.ctypes.data, p.drift, p.drift_axis, p.seed)
    if rc:
        raise RuntimeError(f"oracle loader status {rc}")
    q, r = p.charges()
    threads = len(os.sched_getaffinity(0))
    o = Oracle2D(nx=p.nx, ny=p.ny, np_cap=p.np_cap, q=q, r=r, delt=p.delt, gfac=p.gfac, threads=threads)
    return p, st, o, threads


def cpu_baseline(name, budget_s=15.0):
    """The oracle (C++ restatement of the reference, OpenMP over all host cores) on the
    workload itself when the host holds it: one untimed step (first touch of the state),
    then steps until about budget_s seconds have passed."""
    full = config(name)
    n, whole = oracle_grid(full)
    p, st, o, threads = oracle_state(full, n)
    rc = o.step(st)
    if rc:
        raise RuntimeError(f"oracle status {rc}")
    t0 = time.perf_counter()
    steps = 0
    while steps == 0 or (time.perf_counter() - t0 < budget_s and steps < 50):
        rc = o.step(st)
        if rc:
            raise RuntimeError(f"oracle status {rc}")
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": p.n_particles * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steps of {p.nx}^2 x {p.ppc} ppc/sp, {'the workload' if whole else 'reduced grid'}"}


def run_reference(args):
    """The reference arm: the oracle (the CPU restatement of the reference's step, OpenMP over
    all host cores) runs the workload's own steps: W untimed, then K timed, each one full step
    of the whole grid.  Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name = args.config
    full = config(name)
    n, whole = oracle_grid(full)
    t0 = time.perf_counter()
    p, st, o, threads = oracle_state(full, n)
    load_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        if o.step(st):
            raise RuntimeError("oracle step failed")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if o.step(st):
            raise RuntimeError("oracle step failed")
    dt = time.perf_counter() - t0
    v = p.n_particles * args.steps / dt
    cfg = workload_desc(p, name if whole else f"{name} on a reduced {n}x{n} grid (host memory)")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full steps of {p.nx}^2 x {p.ppc} ppc/sp after {args.warmup}"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "host_load_s": load_s}
    print(json.dumps(line), flush=True)


def rank_totals(ms, npart, dist, device):
    """Whole-job figures of a replica run: the slowest rank's timed region (MAX over the
    ranks) and the particles all ranks advanced (SUM); with no process group, the local ones."""
    if not dist:
        return float(ms), int(npart)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    n = torch.tensor([int(npart)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), int(n.item())


def time_path(p, precision, steps, warmup, rank, torch, dist, local):
    """Device-resident timing of `steps` fused steps on one context."""
    from wumingpic_gb300.pic2d import Pic2D
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = Pic2D(p, precision=precision, stream=stream.cuda_stream)
    g.load_weibel(seed=p.seed + 7919 * rank)
    npart = g.num_particles()
    for _ in range(warmup):
        g.step(1)
    g.timing(True)
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        g.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    stages = g.stage_times()
    g.timing(False)
    ms, ntotal = rank_totals(ms, npart, dist, "cuda")
    return g, ntotal, ms, stages, clocks


def time_moments(g, torch, reps=3):
    """mom_calc__accl + mom_calc__nvt + bc__mom on the device (wpic_moments with no host copy),
    averaged over `reps` calls after one warm-up call, and one call with the copy to the host."""
    stream = torch.cuda.current_stream()
    g.moments(to_host=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        g.moments(to_host=False)
    e1.record(stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mom = g.moments(to_host=True)
    host_ms = (time.perf_counter() - t0) * 1e3
    return {"device_ms": e0.elapsed_time(e1) / reps, "with_host_copy_ms": host_ms,
            "mom_bytes": int(mom.nbytes), "reps": reps}


def time_path3d(steps, rank, torch, dist, world, precision="fp64", n=256):
    """The 3D path (FP64, or mixed: FP32 push and deposit on split positions) on the 3D
    Weibel workload (256^3 cells, 16 ppc/species, m_i/m_e = 16, beams +-0.5c along x,
    u_th 0.05c), state resident in HBM, one warm-up step."""
    from wumingpic_gb300.loader import Plasma3D
    from wumingpic_gb300.pic3d import Pic3D
    p = Plasma3D(nx=n, ny=n, nz=n, ppc=16, mass_ratio=16.0, drift=0.5, drift_axis=0, u_the=0.05,
                 seed=20261203 + 7919 * rank, np_slack=1.5)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = Pic3D(p, precision=precision, stream=stream.cuda_stream)
    g.load_weibel()
    npart = g.num_particles()
    g.step(1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms, ntotal = rank_totals(e0.elapsed_time(e1), npart, dist, "cuda")
    cg = [int(x) for x in g.cg_iters()]
    moments = time_moments(g, torch, reps=2)
    g.close()
    return {"workload": f"3D Weibel {n}^3 cells, 16 ppc/species, {npart} particles, drift +-0.5c along x, "
                        f"u_th 0.05c, m_i/m_e 16, c*dt/dx=0.5",
            "value": ntotal * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
            "steps": steps, "warmup": 1, "dtype": "f64" if precision == "fp64" else "f32+f64",
            "cg_iterations": cg, "moments": moments}


def time_reconnection(steps, rank, torch, dist, ny=4096, nx=2048):
    """The reconnection configuration: a Harris sheet between conducting walls in x (2048
    cells) and periodic in y (4096 cells; the reference's orientation), 32 ppc/species at
    the sheet centre + 6 background, m_i/m_e 25, omega_ce/omega_pe 0.5, T_i/T_e 5, sheet
    half-width 0.5 c/omega_pi, 10 % X-point perturbation.  Mixed and FP64 paths from the
    same host-loaded state, each with one warm-up step and `steps` timed steps; energies
    compared after the same number of steps."""
    from wumingpic_gb300.loader import config_harris2d, load_harris2d
    from wumingpic_gb300.pic2d import Pic2D
    p = dataclasses.replace(config_harris2d("cfg3", seed=20261205 + 7919 * rank), nx=nx, ny=ny)
    t0 = time.perf_counter()
    st = load_harris2d(p)
    load_s = time.perf_counter() - t0
    out = {"workload": f"Harris sheet {ny} (periodic y) x {nx} (walls in x) cells, {p.ncs}+{p.nbg} ppc/species, "
                       f"{p.n_particles} particles, m_i/m_e 25, wce/wpe 0.5, Ti/Te 5, c*dt/dx=0.5",
           "host_load_s": load_s}
    energies = {}
    for precision in ("mixed", "fp64"):
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        g = Pic2D(p, precision=precision, stream=stream.cuda_stream)
        g.put_state(st)
        g.step(1)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms, ntotal = rank_totals(e0.elapsed_time(e1), g.num_particles(), dist, "cuda")
        energies[precision] = g.energy()
        out[precision] = {"value": ntotal * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                          "steps": steps, "warmup": 1, "cg_iterations": [int(x) for x in g.cg_iters()]}
        g.close()
    em, ed = energies["mixed"], energies["fp64"]
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["energy_rel_diff_mixed_vs_fp64"] = [float(abs(a - b) / abs(b)) if b else None for a, b in zip(em, ed)]
    return out


def time_growth_check(steps, rank, dist, n=512, every=10):
    """The metric's accuracy qualifier on the workload's physics: drift +-0.3c, u_th 0.1c,
    64 ppc/species, on n x n cells (the largest grid whose FP64 run saturates within about a
    minute).  Mixed and FP64 paths run the same `steps` from the same host-loaded state with
    energy_history every `every` steps (2d/proj/weibel/app.f90:479-545); the growth rate is
    the linear-phase fit of the magnetic energy (wumingpic_gb300.diagnostics.growth_rate)."""
    import numpy as np
    from wumingpic_gb300.diagnostics import energy_history, growth_rate
    from wumingpic_gb300.loader import Plasma2D, load_weibel2d
    from wumingpic_gb300.pic2d import Pic2D
    p = Plasma2D(nx=n, ny=n, ppc=64, drift=0.3, u_the=0.1, seed=20261211 + 7919 * rank, np_slack=3.0)
    st = load_weibel2d(p)
    runs, secs = {}, {}
    for precision in ("mixed", "fp64"):
        g = Pic2D(p, precision=precision)
        g.put_state(st)
        t0 = time.perf_counter()
        runs[precision] = energy_history(g.step, g.energy, steps, every, p.delt)
        secs[precision] = time.perf_counter() - t0
        g.close()
    t, em = runs["mixed"]
    _, ed = runs["fp64"]
    gm, wm, nm = growth_rate(t, em[:, 3])
    gd, wd, nd = growth_rate(t, ed[:, 3])
    tot_m, tot_d = em.sum(axis=1), ed.sum(axis=1)
    return {"workload": f"2D Weibel {n}^2 cells, 64 ppc/species ({p.n_particles} particles), drift +-0.3c, "
                        f"u_th 0.1c, {steps} steps, energy every {every}",
            "growth_rate_mixed": gm, "growth_rate_fp64": gd, "growth_rate_rel_err": abs(gm / gd - 1.0),
            "fit_window_mixed": wm, "fit_window_fp64": wd, "fit_points": [nm, nd],
            "b_energy_growth": float(ed[:, 3].max() / ed[1, 3]),
            "energy_max_rel_diff": float(np.max(np.abs(tot_m - tot_d) / np.abs(tot_d))),
            "run_s": secs}


def time_adjoint(steps, every, rank, dist, n=512):
    """The discrete adjoint on the 512^2 Weibel workload (32 ppc/species, drift 0.3c, u_th
    0.05c, 64 Bz seed modes of amplitude ~1e-4): the gradient of the final magnetic energy
    with respect to drift, u_th and the seed amplitudes through the checkpointed reverse
    sweep, its cost against the plain FP64 forward of the same steps, and one central
    difference (drift, h = 1e-6)."""
    import numpy as np
    from wumingpic_gb300.adjoint import FieldEnergyProblem, SeedModes
    from wumingpic_gb300.loader import config_weibel2d
    p = dataclasses.replace(config_weibel2d("cfg4", seed=20261204 + 7919 * rank), nx=n, ny=n)
    modes = SeedModes.lowest(p.nx, p.ny, 64)
    amps = 1e-4 * np.random.default_rng(3 + rank).standard_normal(modes.count)
    prob = FieldEnergyProblem(p, steps, every, modes, which="B", cg_rtol=1e-13)
    drift, u_th, h = 0.3, 0.05, 1e-6
    prob.value(drift, u_th, amps)
    t_fwd = prob.timings["forward"]
    val = prob.forward(drift, u_th, amps)
    g_drift, g_uth, g_amps = prob.backward()
    t_rec, t_rev = prob.timings["record"], prob.timings["reverse"]
    fd = (prob.value(drift + h, u_th, amps) - prob.value(drift - h, u_th, amps)) / (2 * h)
    # the mixed-precision adjoint (FP32 reverse push and deposit) on the same recorded run
    prob.sim.adjoint_precision("mixed")
    prob.forward(drift, u_th, amps)
    m_drift, m_uth, m_amps = prob.backward()
    m_rec, m_rev = prob.timings["record"], prob.timings["reverse"]
    prob.sim.adjoint_precision("fp64")
    npart = prob.sim.num_particles()
    val_mixed = prob.value_mixed(drift, u_th, amps)
    mix_ms, _ = rank_totals(prob.timings["forward_mixed"] * 1e3, npart, dist, "cuda")
    # the mixed forward's own sensitivity: central differences at a step where its FP32 rounding
    # (about 1e-7 of L) is far below the difference it resolves, beside the same differences of
    # the FP64 forward (their gap is the h^2 truncation, common to both)
    # (steps h and h/2, Richardson-extrapolated to remove the h^2 truncation)
    hm = 1e-3

    def cd(f, h):
        return (f(drift + h, u_th, amps) - f(drift - h, u_th, amps)) / (2 * h)

    fd_mixed_h, fd_mixed_h2 = cd(prob.value_mixed, hm), cd(prob.value_mixed, hm / 2)
    fd_fp64_h, fd_fp64_h2 = cd(prob.value, hm), cd(prob.value, hm / 2)
    fd_mixed = (4 * fd_mixed_h2 - fd_mixed_h) / 3
    fd_fp64_hm = (4 * fd_fp64_h2 - fd_fp64_h) / 3
    prob.close()
    fwd_ms, _ = rank_totals(t_fwd * 1e3, npart, dist, "cuda")
    rec_ms, _ = rank_totals(t_rec * 1e3, npart, dist, "cuda")
    rev_ms, _ = rank_totals(t_rev * 1e3, npart, dist, "cuda")
    m_rec_ms, _ = rank_totals(m_rec * 1e3, npart, dist, "cuda")
    m_rev_ms, _ = rank_totals(m_rev * 1e3, npart, dist, "cuda")
    rel = lambda a, b: abs(a - b) / abs(b) if b else None  # noqa: E731
    nfield = max(0, ((steps + every - 1) // every - 1) * every - 1)
    return {"workload": f"2D Weibel {n}^2 cells, 32 ppc/species ({npart} particles), drift +-0.3c, u_th 0.05c, "
                        f"64 Bz seed modes; L = final magnetic energy after {steps} steps",
            "steps": steps, "checkpoint_every": every, "dtype": "f64", "cg_rtol": 1e-13,
            "gradient_of": "L of the FP64 forward: both adjoints reverse the recorded FP64 trajectory",
            "recompute": f"the last segment's step states kept by the record; the other segments pushed and "
                         f"sorted again with the recorded fields replayed ({nfield} field states of "
                         f"{12 * (n + 4) * (n + 4) * 8 / 2**20:.0f} MiB kept on the device)",
            "forward_ms": fwd_ms, "record_ms": rec_ms, "reverse_ms": rev_ms,
            "cost_over_forward": (rec_ms + rev_ms) / fwd_ms, "reverse_over_forward": rev_ms / fwd_ms,
            "cost_over_mixed_forward": (rec_ms + rev_ms) / mix_ms, "L": val,
            "mixed_forward": {"L": val_mixed, "rel_diff_vs_fp64": abs(val_mixed - val) / abs(val),
                              "forward_ms": mix_ms, "fp64_over_mixed_time": fwd_ms / mix_ms,
                              "fd_drift": {"h": [hm, hm / 2], "richardson": True,
                                           "fd_mixed": fd_mixed, "fd_fp64": fd_fp64_hm,
                                           "fd_mixed_h": fd_mixed_h, "fd_fp64_h": fd_fp64_h,
                                           "mixed_fd_vs_fp64_fd": rel(fd_mixed, fd_fp64_hm),
                                           "mixed_adjoint_vs_mixed_fd": rel(m_drift, fd_mixed),
                                           "fp64_adjoint_vs_mixed_fd": rel(g_drift, fd_mixed)}},
            "grad": {"drift": g_drift, "u_th": g_uth, "amps_norm": float(np.linalg.norm(g_amps))},
            "fd_check": {"param": "drift", "h": h, "fd": fd, "adjoint": g_drift,
                         "rel_err": abs(g_drift - fd) / abs(fd) if fd else None},
            "mixed_adjoint": {"arithmetic": "FP32 reverse push and deposit per particle; FP64 trajectory, "
                                            "field adjoint, adjoint CG and sums",
                              "record_ms": m_rec_ms, "reverse_ms": m_rev_ms,
                              "cost_over_forward": (m_rec_ms + m_rev_ms) / fwd_ms,
                              "cost_over_mixed_forward": (m_rec_ms + m_rev_ms) / mix_ms,
                              "rel_diff_vs_fp64_adjoint": {
                                  "drift": rel(m_drift, g_drift), "u_th": rel(m_uth, g_uth),
                                  "amps": float(np.linalg.norm(m_amps - g_amps) / np.linalg.norm(g_amps))},
                              "rel_err_vs_fd_drift": rel(m_drift, fd)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg1")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the FP64 path (0 = skip)")
    ap.add_argument("--fp64-3d-steps", type=int, default=2,
                    help="timed steps of the 3D FP64 path on the 256^3 x 16 ppc Weibel workload (0 = skip)")
    ap.add_argument("--mixed-3d-steps", type=int, default=5,
                    help="timed steps of the 3D mixed path on the 256^3 x 16 ppc Weibel workload (0 = skip)")
    ap.add_argument("--grid3d", type=int, default=256, help="cells per edge of the 3D legs")
    ap.add_argument("--only-3d", action="store_true",
                    help="run only the 3D legs and print them (a profiling aid, not the bench line)")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="steps of the adjoint leg on the 512^2 workload (0 = skip)")
    ap.add_argument("--adjoint-every", type=int, default=20, help="checkpoint interval of the adjoint leg")
    ap.add_argument("--adjoint-grid", type=int, default=512, help="cells per edge of the adjoint leg")
    ap.add_argument("--only-adjoint", action="store_true", help="run the adjoint leg alone and print its JSON")
    ap.add_argument("--reconnection-steps", type=int, default=3,
                    help="timed steps of each path on the Harris-sheet workload (0 = skip)")
    ap.add_argument("--reconnection-grid", default="4096x2048", help="periodic y x walled x cells")
    ap.add_argument("--only-reconnection", action="store_true", help="run the reconnection leg alone")
    ap.add_argument("--growth-steps", type=int, default=1200,
                    help="steps of the growth-rate check (mixed against FP64, the workload's physics; 0 = skip)")
    ap.add_argument("--growth-grid", type=int, default=512, help="cells per edge of the growth-rate check")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--stages", action="store_true", help="print the per-stage breakdown to stderr")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from wumingpic_gb300 import _lib

    rny, rnx = (int(v) for v in args.reconnection_grid.lower().split("x"))
    if args.only_reconnection:
        out = time_reconnection(args.reconnection_steps, rank, torch, dist, ny=rny, nx=rnx)
        if rank == 0:
            print(json.dumps(out), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    if args.only_adjoint:
        out = time_adjoint(args.adjoint_steps, args.adjoint_every, rank, dist, n=args.adjoint_grid)
        if rank == 0:
            print(json.dumps(out), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    p = config(args.config)
    hbm_peak, hbm_src = measured_hbm_peak()
    if args.only_3d:
        out = {}
        if args.fp64_3d_steps > 0:
            out["fp64_3d_path"] = time_path3d(args.fp64_3d_steps, rank, torch, dist, world, n=args.grid3d)
        if args.mixed_3d_steps > 0:
            out["mixed_3d_path"] = time_path3d(args.mixed_3d_steps, rank, torch, dist, world, precision="mixed",
                                               n=args.grid3d)
        if rank == 0:
            print(json.dumps(out), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    # ---- mixed path: the headline ----
    g, npart, ms, stages, clocks = time_path(p, "mixed", args.steps, args.warmup, rank, torch, dist, local)
    value = npart * args.steps / (ms / 1e3)  # npart: all ranks' particles
    push_ms, push_n = stages["push"]
    per_launch = push_ms / max(1, push_n)
    achieved = BYTES_MIX_PUSH * (npart / world) / (per_launch / 1e3) / 1e9  # one GPU's launch
    roofline = {"bound": "hbm", "kernel": "k_mix_push2 (fused push + deposit + column compaction, mixed precision)",
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": TRAFFIC_MIX_PUSH_PER_PARTICLE * (npart / world),
                "traffic_unit": "bytes per launch (ncu dram read + write: 64.7 B per particle at 512^2 x 64 ppc, scaled)",
                "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)",
                "bytes_per_particle": BYTES_MIX_PUSH, "launch_ms": per_launch}
    launches = int(sum(v[1] for v in stages.values()))
    moments = time_moments(g, torch)
    e2e = None if args.no_e2e else measure_e2e(g, p, dist)
    g.close()

    # ---- FP64 path on the same workload ----
    fp64 = None
    if args.fp64_steps > 0:
        g64, n64, ms64, st64, clk64 = time_path(p, "fp64", args.fp64_steps, 1, rank, torch, dist, local)
        v64 = n64 * args.fp64_steps / (ms64 / 1e3)
        n64 = n64 // world  # one GPU's particles, for the per-launch kernel figures
        peak64 = _lib.fma_peak_gflops(True)
        dep_ms = st64["deposit"][0] / max(1, st64["deposit"][1] // 2)
        push64_ms = st64["push"][0] / max(1, st64["push"][1])
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps,
                "warmup": 1, "mixed_over_fp64": value / v64 if v64 else None,
                "fp64_fma_peak_gflops": peak64,
                "kernels": {
                    "k_deposit2d": {"launch_ms": dep_ms,
                                    "hbm_gbs": (BYTES_DEPOSIT_FP64 * n64 + BYTES_DEPOSIT_CELL * p.nx * p.ny)
                                    / (dep_ms / 1e3) / 1e9,
                                    "ref_fp64_gflops": FLOP_DEPOSIT_FP64 * n64 / (dep_ms / 1e3) / 1e9},
                    "k_push2d": {"launch_ms": push64_ms,
                                 "hbm_gbs": BYTES_PUSH_FP64 * n64 / (push64_ms / 1e3) / 1e9,
                                 "ref_fp64_gflops": FLOP_PUSH_FP64 * n64 / (push64_ms / 1e3) / 1e9}},
                "stages_ms_per_step": {k: v[0] / args.fp64_steps for k, v in st64.items()}, "clocks": clk64}
        for name, k in fp64["kernels"].items():
            k["hbm_frac"] = k["hbm_gbs"] / hbm_peak
            k["ref_flops_over_fp64_peak"] = k["ref_fp64_gflops"] / peak64
            k["fp64_pipe_active_ncu"] = FP64_PIPE_ACTIVE_NCU[name]
        fp64["moments"] = time_moments(g64, torch)
        g64.close()

    # ---- 3D FP64 path: 256^3 cells, 16 ppc/species (the 3D Weibel configuration) ----
    fp64_3d = None
    if args.fp64_3d_steps > 0:
        fp64_3d = time_path3d(args.fp64_3d_steps, rank, torch, dist, world, n=args.grid3d)
    mixed_3d = None
    if args.mixed_3d_steps > 0:
        mixed_3d = time_path3d(args.mixed_3d_steps, rank, torch, dist, world, precision="mixed", n=args.grid3d)
        if fp64_3d:
            mixed_3d["mixed_over_fp64"] = mixed_3d["value"] / fp64_3d["value"]

    reconnection = None
    if args.reconnection_steps > 0:
        reconnection = time_reconnection(args.reconnection_steps, rank, torch, dist, ny=rny, nx=rnx)

    adjoint = None
    if args.adjoint_steps > 0:
        adjoint = time_adjoint(args.adjoint_steps, args.adjoint_every, rank, dist, n=args.adjoint_grid)

    growth = None
    if args.growth_steps > 0:
        growth = time_growth_check(args.growth_steps, rank, dist, n=args.growth_grid)

    base = None
    if rank == 0 and not args.no_cpu:
        try:
            base = cpu_baseline(args.config)
        except Exception as ex:  # noqa: BLE001
            base = {"error": str(ex)}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": workload_desc(p, args.config),
                "path": "mixed: integer cell + FP32 offset, FP32 push/gather/deposition, FP64 fields and CG",
                "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "gpu_launches": launches,
                "clocks": clocks, "stages_ms_per_step": {k: v[0] / args.steps for k, v in stages.items()},
                "moments": moments, "fp64_path": fp64, "fp64_3d_path": fp64_3d, "mixed_3d_path": mixed_3d,
                "reconnection": reconnection, "adjoint": adjoint, "growth_check": growth}
        line["summary"] = summary(line)  # last, so that the tail of the line carries it
        print(json.dumps(line), flush=True)
        if args.stages:
            for k, (t, n) in stages.items():
                print(f"mixed {k:16s} {t / args.steps:10.3f} ms/step {n:8d} launches", file=sys.stderr)
            if fp64:
                for k, t in fp64["stages_ms_per_step"].items():
                    print(f"fp64  {k:16s} {t:10.3f} ms/step", file=sys.stderr)
    if dist:
        dist.destroy_process_group()


def summary(line):
    """The legs' headline figures in a few hundred characters."""
    def r(x, n=4):
        return None if x is None else float(f"{x:.{n}g}")
    out = {}
    f = line.get("fp64_path")
    if f:
        k = f["kernels"]
        out["fp64_2d"] = {"value": r(f["value"]), "ms_per_step": r(f["ms_per_step"]),
                          "mixed_over_fp64": r(f["mixed_over_fp64"]), "fp64_fma_peak_gflops": r(f["fp64_fma_peak_gflops"]),
                          "k_push2d": {"fp64_pipe_active_ncu": FP64_PIPE_ACTIVE_NCU["k_push2d"],
                                       "ref_flops_over_fp64_peak": r(k["k_push2d"]["ref_flops_over_fp64_peak"], 3),
                                       "hbm_frac": r(k["k_push2d"]["hbm_frac"], 3)},
                          "k_deposit2d": {"fp64_pipe_active_ncu": FP64_PIPE_ACTIVE_NCU["k_deposit2d"],
                                          "ref_flops_over_fp64_peak": r(k["k_deposit2d"]["ref_flops_over_fp64_peak"], 3),
                                          "hbm_frac": r(k["k_deposit2d"]["hbm_frac"], 3)}}
    for key, name in (("mixed_3d_path", "mixed_3d"), ("fp64_3d_path", "fp64_3d")):
        v = line.get(key)
        if v:
            out[name] = {"value": r(v["value"]), "ms_per_step": r(v["ms_per_step"])}
            if "mixed_over_fp64" in v:
                out[name]["mixed_over_fp64"] = r(v["mixed_over_fp64"])
    rc = line.get("reconnection")
    if rc:
        out["reconnection"] = {"mixed": r(rc["mixed"]["value"]), "fp64": r(rc["fp64"]["value"]),
                               "mixed_over_fp64": r(rc["mixed_over_fp64"])}
    a = line.get("adjoint")
    if a:
        out["adjoint"] = {"cost_over_forward": r(a["cost_over_forward"], 3), "fd_rel_err": r(a["fd_check"]["rel_err"], 3)}
        if "mixed_adjoint" in a:
            out["adjoint"]["mixed_cost_over_mixed_forward"] = r(a["mixed_adjoint"].get("cost_over_mixed_forward"), 3)
    gc = line.get("growth_check")
    if gc:
        out["growth_check"] = {"growth_rate_rel_err": r(gc["growth_rate_rel_err"], 3),
                               "energy_max_rel_diff": r(gc["energy_max_rel_diff"], 3),
                               "grid": gc["workload"].split(" cells")[0].replace("2D Weibel ", "")}
    return out


def measure_e2e(g, p, dist=None):
    """The same step through the C ABI with the reference-layout state in host memory:
    every step copies the state in (host -> device), runs the step and copies the new
    state back (device -> host).  With several ranks: all ranks' particles over the
    slowest rank's time."""
    from wumingpic_gb300 import _lib
    st = g.get_state()
    pinned = []
    for a in (st.up, st.uf, st.cumcnt, st.np2):
        try:
            _lib.host_register(a)
            pinned.append(a)
        except Exception:  # noqa: BLE001
            pass
    steps = 2
    g.put_state(st)
    g.step(1)
    g.get_state(st)
    # the three calls return after their work has finished (each synchronises its stream),
    # so marks between them split the step into the exchange in, the step and the exchange out
    split = [0.0, 0.0, 0.0]
    t0 = time.perf_counter()
    for _ in range(steps):
        ta = time.perf_counter()
        g.put_state(st)
        tb = time.perf_counter()
        g.step(1)
        tc = time.perf_counter()
        g.get_state(st)
        td = time.perf_counter()
        split[0] += tb - ta
        split[1] += tc - tb
        split[2] += td - tc
    dt = time.perf_counter() - t0
    for a in pinned:
        _lib.host_unregister(a)
    ms, n = rank_totals(dt * 1e3, int(st.np2.sum()), dist, "cuda")
    dt = ms / 1e3
    # what crosses the link: each row's valid prefix of up (np2 particles of ndim words), uf,
    # cumcnt and np2 (wpic_put_particles / wpic_get_particles copy the valid prefixes only)
    bytes_state = int(st.np2.sum()) * p.ndim * 8 + st.uf.nbytes + st.np2.nbytes + st.cumcnt.nbytes
    link = measure_link()
    ms_step = dt * 1e3 / steps
    floor_ms = 1e3 * (bytes_state / (link["h2d_gbs"] * 1e9) + bytes_state / (link["d2h_gbs"] * 1e9))
    put_s, step_s, get_s = (x / steps for x in split)
    link.update({"exchange_floor_ms_per_step": floor_ms, "e2e_ms_per_step": ms_step,
                 "frac": floor_ms / ms_step,
                 "split_ms_per_step": {"put": put_s * 1e3, "step": step_s * 1e3, "get": get_s * 1e3},
                 "put_gbs": bytes_state / put_s / 1e9, "get_gbs": bytes_state / get_s / 1e9})
    return {"value": n * steps / dt, "unit": UNIT, "h2d_bytes_per_step": int(bytes_state),
            "d2h_bytes_per_step": int(bytes_state), "steps": steps, "link": link,
            "note": "reference-layout host arrays (page-locked with wpic_host_register), the valid state in "
                    "and out every step"}


def measure_link(nbytes=1 << 30, reps=3):
    """The host link's copy bandwidth each way (one page-locked 1 GiB buffer, copy-engine
    copies timed with CUDA events): the bound of the end-to-end exchange.  The conversion
    kernels' in-place reads and writes of registered host memory reach the same figures."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dbuf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for key, dst, src in (("h2d_gbs", dbuf, h), ("d2h_gbs", h, dbuf)):
        dst.copy_(src, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        out[key] = nbytes * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del h, dbuf
    return out


if __name__ == "__main__":
    main()
