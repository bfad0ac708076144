#!/usr/bin/env python3
"""Benchmark: FEN projection step on GB300 — Mcell-steps/s.

Workload (default): 3D Taylor-Green vortex, periodic [0, 2 pi]^3, 256^3 MAC grid, FP64,
Re = 1600 (nu = 1/1600), dt from CFL = 0.5 (constant-CFL mode), fast direct Poisson solve
by FFT in all three directions.  A "step" is one navier_stokes_solver time step
(predictor, ghost fill, Poisson solve, correction, pressure update, diagnostics).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config tgv3d|tgv2d|channel]

One JSON line on rank 0.  `value` is device time (CUDA events on the library's stream, K
captured steps replayed back to back, inputs resident in HBM); `e2e` is the same metric
through the C ABI with pinned host buffers (upload of u, v, w, p, K advance_solution calls
each returning dt and the diagnostics to the host, download of u, v, w, p into pinned
buffers).  Defaults: K = 100 timed steps after W = 3 warm-up steps; nvidia-smi clocks and
throttle reasons are sampled every 50 ms during the timed region.  Inputs are larger than L2
(137 MB per field at 256^3).
Multi-GPU: the path does not shard (one grid per device); N ranks run N independent
replicas (weak scaling) and `value` sums their cells over the slowest rank's time.
`--impl reference` times the CPU restatement of the reference (the oracle port; the
Fortran/MPI/FFTW reference cannot be built on these machines) on rank 0's host cores.

At N=1 the line also carries `forms`: the mixed-precision form against the FP64 path on the
channel workload (throughput of each and the mixed form's relative L2 error after the same
steps), and the discrete adjoint on 2D decaying turbulence (backward/forward time ratio and
the gradient's agreement with central differences), and the batched ensemble of 512 2D
Kolmogorov runs in one persistent launch.  `--no-forms` skips them.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Algorithmic bytes per cell of each stage of one step: the compulsory reads and writes of
# the stage counted once, a complex half-spectrum as one real word per cell; the Poisson
# correction phi between the inverse transform and the correction is an intermediate of this
# implementation and is not counted.  FP64 words: 13 + 4 + 6 + 1 + 8 = 32 (3D) and
# 9 + 3 + 2 + 1 + 6 = 21 (2D).
STAGES = ["predictor", "ghost_vstar", "forward_x", "spectral", "inverse_x", "correct", "ghost", "checks"]
STAGE_WORDS = {
    3: {"predictor": 13,   # read u, v, w, p, dv_o(3); write v*(3), dv_o(3)
        "forward_x": 4,    # read v*(3); write the half spectrum
        "spectral": 6,     # y forward, z forward + solve + inverse, y inverse: 3 x (read + write)
        "inverse_x": 1,    # read the half spectrum
        "correct": 8},     # read v*(3), p; write v(3), p
    2: {"predictor": 9, "forward_x": 3, "spectral": 2, "inverse_x": 1, "correct": 6},
}
# The mixed form keeps u, v, w, p, v* and dv_o as double-float pairs (8 B per value): its
# predictor reads u, v, w, p, dv_o and writes v*, dv_o as pairs, 13 pair words = 104 B/cell.
MIXED_PREDICTOR_BYTES = {3: 104, 2: 72}
# ncu figures of one launch of the dominant kernel (the predictor), per cell: DRAM bytes read +
# written and FP64 thread instructions, from `--set full` captures of the named case.
NCU_PREDICTOR = {
    "fp64": {"dram_bytes_per_cell": 99.6, "fp64_instr_per_cell": 72.0,
             "source": "ncu --set full, k_predictor_tile, 3D TGV 192^3 FP64, one launch"},
    "mixed": {"dram_bytes_per_cell": 100.4, "fp64_instr_per_cell": 0.0,
              "source": "ncu --set full, k_predictor_df_tile, channel 256x128x192 mixed, one launch"},
}


def device_sms_and_clock():
    """SM count of device 0 and its maximum SM clock in GHz (nvidia-smi; 2.07 if unreadable)."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ghz = 2.07
    try:
        out = subprocess.run(["nvidia-smi", "-i", "0", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=10)
        ghz = float(out.stdout.strip().splitlines()[0]) / 1e3
    except Exception:
        pass
    return sms, ghz


def fp64_issue(instr_per_cell, cells, ms, sms=None, ghz=None):
    """Achieved FP64 instruction rate of a kernel with `instr_per_cell` FP64 thread
    instructions per cell against the issue peak of 2 FP64 thread instructions per SM per
    cycle (`sms` SMs at `ghz`)."""
    if not instr_per_cell or not ms:
        return None
    if sms is None or ghz is None:
        sms, ghz = device_sms_and_clock()
    peak = 2 * sms * ghz
    got = instr_per_cell * cells / (ms / 1e3) / 1e9
    return {"achieved": round(got, 1), "peak": round(peak, 1), "unit": "G FP64 instr/s", "frac": round(got / peak, 4),
            "instr_per_cell": instr_per_cell}


def roofline_block(dim, form, cells, stage_ms, peak, peak_kind, sms=None, ghz=None):
    """Roofline of the dominant kernel, the predictor (the largest single kernel of the step in
    both forms): algorithmic bytes per cell x cells / its CUDA-event time against the measured
    HBM copy bandwidth; the whole step's algorithmic bytes beside it."""
    words = STAGE_WORDS[dim]
    bpc = 8 * words["predictor"] if form == "fp64" else MIXED_PREDICTOR_BYTES[dim]
    ms = stage_ms["predictor"]
    achieved = bpc * cells / (ms / 1e3) / 1e9
    ncu = NCU_PREDICTOR[form]
    tr = ncu["dram_bytes_per_cell"]
    step_w = sum(words.values())
    step_ms = sum(stage_ms.values())
    kern = ("k_predictor_tile" if form == "fp64" else "k_predictor_df_tile") if dim == 3 else \
        ("k_predictor<2>" if form == "fp64" else "k_predictor_df<2>")
    out = {"bound": "hbm", "kernel": kern,
           "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
           "traffic": int(tr * cells) if tr and dim == 3 else None, "peak_source": peak_kind,
           "bytes_per_cell": bpc, "stage_ms": {k: round(v, 4) for k, v in stage_ms.items()},
           "step_algorithmic_bytes_per_cell": 8 * step_w if form == "fp64" else None,
           "step_achieved_gbs": round(8 * step_w * cells / (step_ms / 1e3) / 1e9, 1) if form == "fp64" else None}
    if tr:
        out["traffic_source"] = ncu["source"] + f" ({tr} B/cell), scaled by cells"
    if form == "fp64" and dim == 3:
        out["fp64_issue"] = fp64_issue(ncu["fp64_instr_per_cell"], cells, ms, sms, ghz)
        out["fp64_issue_source"] = ncu["source"]
        out["note"] = "FP64 kernels are bound by FP64 issue on GB300, not by HBM"
    return out


CONFIGS = {
    "tgv3d": dict(dim=3, n=(256, 256, 256), L=(2 * np.pi,) * 3, nu=1.0 / 1600, cfl=0.5, constant_cfl=True,
                  bc=["Periodic"] * 6, desc="3D Taylor-Green vortex 256^3, Re=1600, CFL=0.5, FP64, FFT x/y/z"),
    "tgv2d": dict(dim=2, n=(128, 128, 1), L=(2 * np.pi, 2 * np.pi, 2 * np.pi / 128), nu=0.01, dt=1e-3,
                  bc=["Periodic"] * 4, desc="2D Taylor-Green vortex 128^2, nu=0.01, dt=1e-3, FP64"),
    "channel": dict(dim=3, n=(512, 256, 384), L=(4 * np.pi, 2.0, 4 * np.pi / 3), nu=1.0 / 180, cfl=0.5,
                    constant_cfl=True, g=(1.0, 0.0, 0.0), aniso=True,
                    bc=["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"],
                    desc="channel 512x256x384, Re_tau=180, walls in y, CFL=0.5, FP64, FFT x/z + Thomas y"),
}


def max_over_ranks(x, dist, device):
    """The slowest rank's value (replicas are timed independently; the job ends with the last)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, cells, steps, ms):
    """Whole-job Mcell-steps/s of `world` replicas of `cells` cells, `steps` steps each, all
    finished within `ms` milliseconds (weak scaling: per-GPU work fixed)."""
    return world * cells * steps / (ms / 1e3) / 1e6


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init_fields(name, cfg, n, shape):
    """Initial fields of workload `name` on an n-cell grid, Fortran layout (k, j, i) with ghosts."""
    from tests import cases as C

    L = cfg["L"]
    if name == "tgv3d":
        return dict(zip("uvwp", C.tgv3d_fields(n[0], L[0])))
    if name == "tgv2d":
        u, v, p = C.tgv2d_fields(n[0], L[0])
        return {"u": u, "v": v, "p": p}
    # channel: laminar Poiseuille u = (1 - y^2)/(2 nu) plus seeded uniform noise of 5% of
    # the centreline velocity on u, v, w (PCG64 seed 1234, Fortran order)
    assert shape == (n[2] + 2, n[1] + 2, n[0] + 2)
    return dict(zip("uvwp", C.channel_fields(n, L, cfg["nu"])))


def start_velocity(name, cfg):
    """Velocity scale given to set_timestep (navier_stokes.f90:641): U = 1 for the TGV,
    the centreline velocity 1/(2 nu) for the channel."""
    return 1.0 if name == "tgv3d" else 1.0 / (2 * cfg["nu"])


def make_oracle(name, cfg, n, nthreads):
    from oracle import oracle as O

    bcmap = {"Periodic": O.PERIODIC, "Wall": O.WALL}
    L = list(cfg["L"])
    if name == "tgv2d":
        L[2] = L[0] / n[0]
    o = O.Oracle(cfg["dim"], n, L, bc=[bcmap[b] for b in cfg["bc"]], viscosity=cfg["nu"],
                 g=cfg.get("g", (0, 0, 0)), cfl=cfg.get("cfl", 1.0), constant_cfl=cfg.get("constant_cfl", False),
                 aniso=cfg.get("aniso", False), nthreads=nthreads)
    f = init_fields(name, cfg, n, o.shape)
    for key, fid in (("u", O.U), ("v", O.V), ("w", O.W), ("p", O.P)):
        if key in f:
            o.field(fid)[...] = f[key]
            o.update_ghost_nodes(fid)
    if cfg.get("constant_cfl"):
        dt = o.set_timestep(start_velocity(name, cfg))
    else:
        dt = cfg["dt"]
        o.dt_o = dt
    return o, dt


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.05)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_baseline(name, cfg, max_seconds=20.0):
    """Time the oracle port on the host cores on a bounded sample of the workload: the full
    grid when a step fits the budget, else the same configuration on a coarser grid (the
    metric is per cell)."""
    nthreads = os.cpu_count() or 1
    n = list(cfg["n"])
    est = n[0] * n[1] * n[2] / (2e6 * nthreads)  # ~2 Mcell-steps/s per core
    while est > max_seconds / 3 and n[0] > 32:
        n = [x // 2 for x in n[:2]] + [n[2] // 2 if cfg["dim"] == 3 else 1]
        est /= 8 if cfg["dim"] == 3 else 4
    o, dt = make_oracle(name, cfg, n, nthreads)
    steps, t0 = 0, time.perf_counter()
    while True:
        dt = o.step(dt)
        steps += 1
        el = time.perf_counter() - t0
        if el > max_seconds or steps >= 50:
            break
    cells = n[0] * n[1] * n[2]
    return {"value": round(cells * steps / el / 1e6, 3), "unit": "Mcell-steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{steps} steps of {name} at {n[0]}x{n[1]}x{n[2]} ({el:.1f} s), CPU restatement (not FFTW)"}


def form_mixed(F, steps, scale=1):
    """Channel flow (512x256x384, Re_tau = 180, CFL = 0.5): the mixed form against the FP64
    path over the same `steps` steps from the same initial field.  Returns both throughputs
    and the mixed form's relative L2 error per field (p mean-free)."""
    cfg = CONFIGS["channel"]
    n, L = tuple(x // scale for x in cfg["n"]), cfg["L"]
    cells = n[0] * n[1] * n[2]
    out, ref = {}, {}
    for prec, name in ((F.FP64, "fp64"), (F.MIXED, "mixed")):
        g = F.Grid(n[0], n[1], n[2], L[0], L[1], L[2], bc=cfg["bc"], aniso=True)
        s = F.Solver(g, viscosity=cfg["nu"], g=cfg["g"], CFL=cfg["cfl"], constant_CFL=True, precision=prec)
        fields = init_fields("channel", cfg, n, g.shape)
        for k, fid in (("u", F.U), ("v", F.V), ("w", F.W), ("p", F.P)):
            s.set_field(fid, fields[k])
            s.update_ghost_nodes(fid)
        dt = s.set_timestep(start_velocity("channel", cfg))
        ms = s.time_steps(steps, dt)
        out[name] = round(cells * steps / (ms / 1e3) / 1e6, 3)
        res = {k: s.get_field(fid)[1:-1, 1:-1, 1:-1] for k, fid in (("u", F.U), ("v", F.V), ("w", F.W), ("p", F.P))}
        if name == "mixed":
            # stage times after the fields are read (profile_step advances the state)
            peak, peak_kind = measured_peaks()
            stage = dict(zip(STAGES, s.profile_step(3, s.status()["dt"])))
            out["roofline"] = roofline_block(3, "mixed", cells, stage, peak, peak_kind)
        if name == "fp64":
            ref = res
        else:
            err = {}
            for k in "uvwp":
                a, b = res[k], ref[k]
                if k == "p":
                    a, b = a - a.mean(), b - b.mean()
                err[k] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
            out["rel_l2_vs_fp64"] = err
        s.destroy_solver()
        del s
    out["speedup"] = round(out["mixed"] / out["fp64"], 3)
    out["unit"] = "Mcell-steps/s"
    out["workload"] = f"channel {n[0]}x{n[1]}x{n[2]}, {steps} steps from Poiseuille + 5% noise, CFL 0.5"
    return out


def form_adjoint(F, ndir=16, nsteps=500, every=50):
    """Adjoint of a 2D decaying-turbulence rollout (256^2 periodic, nu = 2e-3, dt = 2e-3 =
    dt_o, 500 steps, checkpoints every 50): backward/forward time ratio and the agreement
    of the gradient with central differences along `ndir` seeded unit directions,
    eps = 1e-6 |u0|."""
    from tests import cases as C

    n, L, nu, dt = 256, 2 * np.pi, 2e-3, 2e-3
    u0, v0 = C.decaying_turbulence_2d(n, L, 1)
    tu, tv = C.decaying_turbulence_2d(n, L, 2)
    g = F.Grid(n, n, 1, L, L, L / n)

    def load(s, u, v):
        for fid, a in ((F.U, u), (F.V, v), (F.P, None), (F.DVO_X, None), (F.DVO_Y, None)):
            f = s.zeros(fid)
            if a is not None:
                f[1, 1:-1, 1:-1] = a
            s.set_field(fid, f)
            if fid in (F.U, F.V, F.P):
                s.update_ghost_nodes(fid)
        s.set_dt_o(dt)

    def loss(s):
        uT, vT = s.get_field(F.U)[1, 1:-1, 1:-1], s.get_field(F.V)[1, 1:-1, 1:-1]
        return 0.5 * (np.sum((uT - tu) ** 2) + np.sum((vT - tv) ** 2)), uT, vT

    s = F.Solver(g, viscosity=nu)
    s.adjoint_setup(nsteps, every)
    ratios = []
    for _ in range(3):
        load(s, u0, v0)
        s.adjoint_forward(dt)
        J, uT, vT = loss(s)
        lu, lv = s.zeros(), s.zeros()
        lu[1, 1:-1, 1:-1], lv[1, 1:-1, 1:-1] = uT - tu, vT - tv
        gu, gv, ms = s.adjoint_backward(lu, lv)
        ratios.append(ms[0] / ms[1])
    gu, gv = gu[1, 1:-1, 1:-1], gv[1, 1:-1, 1:-1]
    f = F.Solver(g, viscosity=nu)
    rng = np.random.Generator(np.random.PCG64(3))
    eps = 1e-6 * np.sqrt(np.sum(u0 ** 2) + np.sum(v0 ** 2))
    worst = 0.0
    for _ in range(ndir):
        du, dv = rng.standard_normal((n, n)), rng.standard_normal((n, n))
        nrm = np.sqrt(np.sum(du ** 2) + np.sum(dv ** 2))
        du, dv = du / nrm, dv / nrm
        Jpm = []
        for sgn in (1.0, -1.0):
            load(f, u0 + sgn * eps * du, v0 + sgn * eps * dv)
            f.advance_n(nsteps, dt)
            Jpm.append(loss(f)[0])
        fd = (Jpm[0] - Jpm[1]) / (2 * eps)
        ad = float(np.sum(gu * du) + np.sum(gv * dv))
        worst = max(worst, abs(fd - ad) / abs(ad))
    return {"ratio_backward_over_forward": round(statistics.median(ratios), 3), "forward_ms": round(ms[1], 3),
            "backward_ms": round(ms[0], 3), "fd_directions": ndir, "fd_max_rel_err": worst,
            "workload": "2D decaying turbulence 256^2, nu=2e-3, dt=2e-3, 500 steps, checkpoints every 50, FP64",
            "tgv3d_64": form_adjoint3d(F)}


def form_adjoint3d(F, ndir=4, nsteps=100, every=10):
    """Adjoint of a 3D rollout: Taylor-Green 64^3 (ppp), nu = 1/1600, fixed dt = 5e-3 = dt_o,
    100 steps, checkpoints every 10, loss 1/2 |v_T - v_target|^2 with a seeded smooth target:
    backward/forward time ratio (median of 3) and central differences along `ndir` seeded
    smooth directions, eps = 1e-6 |v_0|."""
    from tests import cases as C

    N, L, dt = 64, 2 * np.pi, 5e-3
    g = F.Grid(N, N, N, L, L, L)
    x0 = [C.interior(a, 3) for a in C.tgv3d_fields(N, L)]
    rng = np.random.Generator(np.random.PCG64(31))
    grid = np.meshgrid(*[np.arange(N) / N] * 3, indexing="ij")

    def smooth(kmax=3):
        f = np.zeros((N, N, N))
        for _ in range(6):
            k = rng.integers(0, kmax + 1, size=3)
            ph = rng.uniform(0, 2 * np.pi, size=3)
            term = rng.uniform(-1, 1) * np.ones((N, N, N))
            for d in range(3):
                term = term * np.cos(2 * np.pi * k[d] * grid[d] + ph[d])
            f += term
        return f

    target = [smooth() for _ in range(3)]
    vel = (F.U, F.V, F.W)

    def load(s, x):
        for fid, a in zip(vel + (F.P,), x):
            f = s.zeros(fid)
            f[1:-1, 1:-1, 1:-1] = a
            s.set_field(fid, f)
            s.update_ghost_nodes(fid)
        for q in range(3):
            s.set_field(F.DVO_X + q, s.zeros(F.DVO_X + q))
        s.set_dt_o(dt)

    def final(s):
        return [C.interior(s.get_field(fid), 3) for fid in vel]

    def loss(vT):
        return 0.5 * sum(np.sum((a - b) ** 2) for a, b in zip(vT, target))

    s = F.Solver(g, viscosity=1.0 / 1600)
    s.adjoint_setup(nsteps, every)
    ratios = []
    for _ in range(3):
        load(s, x0)
        s.adjoint_forward(dt)
        vT = final(s)
        lam = []
        for a, b in zip(vT, target):
            f = s.zeros()
            f[1:-1, 1:-1, 1:-1] = a - b
            lam.append(f)
        out = s.adjoint_backward(*lam)
        ms = out[-1]
        ratios.append(ms[0] / ms[1])
    grads = [C.interior(a, 3) for a in out[:-1]]
    f = F.Solver(g, viscosity=1.0 / 1600)
    norm = np.sqrt(sum(np.sum(a ** 2) for a in x0[:-1]))
    eps = 1e-6
    worst = 0.0
    for _ in range(ndir):
        d = [smooth(kmax=6) for _ in range(3)]
        dn = np.sqrt(sum(np.sum(a ** 2) for a in d))
        d = [a * norm / dn for a in d]
        Js = []
        for sgn in (1.0, -1.0):
            load(f, [a + sgn * eps * b for a, b in zip(x0[:-1], d)] + [x0[-1]])
            f.advance_n(nsteps, dt)
            Js.append(loss(final(f)))
        fd = (Js[0] - Js[1]) / (2 * eps)
        ad = sum(float(np.sum(gq * b)) for gq, b in zip(grads, d))
        worst = max(worst, abs(fd - ad) / abs(ad))
    return {"ratio_backward_over_forward": round(statistics.median(ratios), 3), "forward_ms": round(ms[1], 3),
            "backward_ms": round(ms[0], 3), "fd_directions": ndir, "fd_max_rel_err": worst,
            "workload": "3D Taylor-Green 64^3, nu=1/1600, dt=5e-3, 100 steps, checkpoints every 10, FP64"}


def form_ensemble(F, steps=2000, nruns=512, tune_steps=10, sizes=(64, 96, 128, 192, 256), adjoint=True):
    """Batched ensemble: 512 independent 2D Kolmogorov runs (N ~ U{64, 96, 128, 192, 256},
    Re ~ U[50, 500], forcing sin(4y), noise 1e-2, CFL 0.4) advanced `steps` steps in one
    persistent launch, FP32 with FP64 reductions, tile shapes from the autotuner."""
    from tests import cases as C

    n, nu, init = C.kolmogorov_ensemble(nruns, sizes=tuple(sizes))
    e = F.Ensemble(n, nu, length=2 * np.pi, CFL=0.4, forcing=(1.0, 4))
    for q in range(nruns):
        e.upload(q, *init(q))
    e.set_timestep(1.0)
    t0 = time.perf_counter()
    cfg = e.tune(steps=tune_steps)
    tune_s = time.perf_counter() - t0
    l0 = e.launches()
    ms = e.advance(steps)
    launches = e.launches() - l0
    cells = int(np.sum(n.astype(np.int64) ** 2))
    st = [e.status(q) for q in range(nruns)]
    # forward/adjoint pair of every run: loss 1/2 |u_T|^2 per run, checkpoints every 50 steps
    adj = None
    if adjoint:
        e.adjoint_setup(steps, min(50, steps))
        fwd_ms = e.adjoint_forward()
        for q in range(nruns):
            uT, vT, _ = e.download(q)
            e.adjoint_seed(q, uT, vT)
        bwd_ms = e.adjoint_backward()
        g = [e.adjoint_gradient(q) for q in range(min(nruns, 4))]
        adj = {"forward_ms": round(fwd_ms, 3), "backward_ms": round(bwd_ms, 3),
               "ratio_backward_over_forward": round(bwd_ms / fwd_ms, 3), "checkpoint_every": min(50, steps),
               "finite": bool(all(np.isfinite(x).all() for pair in g for x in pair))}
    e.destroy()
    return {"value": round(cells * steps / (ms / 1e3) / 1e6, 3), "unit": "Mcell-steps/s", "ms": round(ms, 3),
            "runs": nruns, "cells": cells, "steps": steps, "launches": launches, "config": cfg,
            "tune_s": round(tune_s, 2), "max_maxdiv": max(abs(s["maxdiv"]) for s in st),
            "any_nan": any(s["nan"] for s in st), "adjoint_pair": adj,
            "workload": f"{nruns} 2D Kolmogorov runs, N~U{{64..256}}, Re~U[50,500], CFL 0.4, {steps} steps, FP32"}


def run_reference(args, name, cfg):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    n = cfg["n"]
    o, dt = make_oracle(name, cfg, n, nthreads)
    for _ in range(args.warmup):
        dt = o.step(dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt = o.step(dt)
    el = time.perf_counter() - t0
    cells = n[0] * n[1] * n[2]
    v = cells * args.steps / el / 1e6
    line = {"impl": "reference", "metric": "Mcell-steps/s", "value": round(v, 3), "unit": "Mcell-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["desc"], "cells": cells, "flush": "inputs larger than L2"},
            "cpu_baseline": {"value": round(v, 3), "unit": "Mcell-steps/s", "cores": nthreads, "kind": "port",
                             "sample": f"{args.steps} timed steps of the full {n[0]}x{n[1]}x{n[2]} grid; FEN's "
                                       "Fortran/MPI/FFTW build is not available here, so the oracle port runs"},
            "e2e": {"value": round(v, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="tgv3d", choices=list(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=0, help="cubic/square override of the grid (profiling runs)")
    ap.add_argument("--no-forms", action="store_true", help="skip the mixed-precision and adjoint measurements")
    ap.add_argument("--form-steps", type=int, default=500, help="channel steps of the mixed-vs-FP64 comparison")
    ap.add_argument("--form", default="", choices=["", "mixed", "adjoint", "ensemble"],
                    help="run one form alone and print its JSON (profiling; --grid divides the channel, "
                         "--ensemble-runs/--ensemble-sizes/--ensemble-steps size the ensemble)")
    ap.add_argument("--ensemble-runs", type=int, default=512)
    ap.add_argument("--ensemble-steps", type=int, default=2000)
    ap.add_argument("--ensemble-sizes", default="64,96,128,192,256")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="arithmetic form of the headline run (mixed: FP32 stencils/transforms, FP64 "
                         "tridiagonal, zero mode, refinement residual and reductions)")
    ap.add_argument("--shape", default="", help="grid override NXxNYxNZ of the headline run (profiling runs)")
    args = ap.parse_args()
    cfg_name = args.config
    cfg = dict(CONFIGS[cfg_name])
    if args.shape:
        cfg["n"] = tuple(int(x) for x in args.shape.lower().split("x"))
        cfg["desc"] = cfg["desc"] + f" (grid override {cfg['n']})"
    elif args.grid:
        g0 = args.grid
        cfg["n"] = (g0, g0, g0 if cfg["dim"] == 3 else 1) if cfg_name != "channel" else (2 * g0, g0, (3 * g0) // 2)
        cfg["desc"] = cfg["desc"] + f" (grid override {cfg['n']})"
    rank, world, local = env_rank()
    if args.form and args.impl == "ours":
        import fen_gb300 as F

        if args.form == "mixed":
            res = form_mixed(F, args.form_steps, scale=max(1, args.grid and 256 // args.grid or 1))
        elif args.form == "adjoint":
            res = form_adjoint(F)
        else:
            res = form_ensemble(F, steps=args.ensemble_steps, nruns=args.ensemble_runs,
                                sizes=[int(x) for x in args.ensemble_sizes.split(",")])
        print(json.dumps({"form": args.form, **res}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, cfg_name, cfg)
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    import fen_gb300 as F

    n, L = cfg["n"], cfg["L"]
    g = F.Grid(n[0], n[1], n[2], L[0], L[1], L[2], bc=cfg["bc"], dim=cfg["dim"], aniso=cfg.get("aniso", False))
    s = F.Solver(g, viscosity=cfg["nu"], g=cfg.get("g", (0, 0, 0)), CFL=cfg.get("cfl", 1.0),
                 constant_CFL=cfg.get("constant_cfl", False), precision=F.MIXED if args.precision == "mixed" else F.FP64)
    fields = init_fields(cfg_name, cfg, n, g.shape)
    fid = {"u": F.U, "v": F.V, "w": F.W, "p": F.P}
    keys = [k for k in "uvwp" if k in fields]

    def upload_all(src):
        for k in keys:
            s.set_field(fid[k], src[k])
            s.update_ghost_nodes(fid[k])

    def start_dt():
        if cfg.get("constant_cfl"):
            return s.set_timestep(start_velocity(cfg_name, cfg))
        s.set_dt_o(cfg["dt"])
        return cfg["dt"]

    upload_all(fields)
    dt = start_dt()
    dt = s.advance_n(args.warmup, dt)
    cells = n[0] * n[1] * n[2]

    # ---- device-timed throughput (graph replay, inputs resident in HBM) ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    s.sync()
    l0 = s.kernel_launches()
    with ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]) if world == 1 else local) as clk:
        ms = s.time_steps(args.steps, dt)
    launches = s.kernel_launches() - l0
    s.sync()
    torch.cuda.synchronize()
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    value = replica_throughput(world, cells, args.steps, ms)
    ms_per_step = ms / args.steps

    # ---- per-stage device times for the roofline ----
    st = s.profile_step(3, s.status()["dt"])
    stage = dict(zip(STAGES, st))
    peak, peak_kind = measured_peaks()
    sms, ghz = device_sms_and_clock()
    roofline = roofline_block(cfg["dim"], args.precision, cells, stage, peak, peak_kind, sms, ghz)

    # ---- end to end through the C ABI with pinned host buffers ----
    host = {k: torch.from_numpy(np.ascontiguousarray(fields[k])).pin_memory() for k in keys}
    outb = {k: torch.empty(fields[k].shape, dtype=torch.float64).pin_memory() for k in keys}
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in keys:
        s.set_field(fid[k], host[k].numpy())
        s.update_ghost_nodes(fid[k])
    dt2 = start_dt()
    for step in range(1, args.steps + 1):
        dt2 = s.advance_solution(step, dt2)
    for k in keys:
        s.get_field(fid[k], out=outb[k].numpy())
    s.sync()
    el = time.perf_counter() - t0
    if dist:
        el = max_over_ranks(el, dist, "cuda")
    field_bytes = 8 * int(np.prod(g.shape)) if cfg["dim"] == 3 else 8 * (n[0] + 2) * (n[1] + 2)
    e2e = {"value": round(world * cells * args.steps / el / 1e6, 3), "unit": "Mcell-steps/s",
           "h2d_bytes_per_step": int(len(keys) * field_bytes / args.steps + 8),
           "d2h_bytes_per_step": int(len(keys) * field_bytes / args.steps + 160)}

    if rank == 0:
        line = {"metric": "Mcell-steps/s", "value": round(value, 3), "unit": "Mcell-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "f32 stencils/transforms + f64 solve/reductions",
                "data": "synthetic",
                "config": {"workload": cfg["desc"] if args.precision == "fp64" else cfg["desc"].replace("FP64", "mixed"),
                           "cells": cells, "grid": list(n), "form": args.precision,
                           "flush": f"inputs larger than L2 (fields {8 * int(np.prod(g.shape)) / 1e6:.0f} MB each)"
                           if cells > 1e6 else "L2-resident",
                           "parallelism": f"replicas{world}"},
                "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "clocks": clk.summary()}
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(cfg_name, cfg)
        if world == 1 and not args.no_forms:
            s.destroy_solver()
            line["forms"] = {"mixed": form_mixed(F, args.form_steps), "adjoint": form_adjoint(F),
                             "ensemble": form_ensemble(F)}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
