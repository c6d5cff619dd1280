"""Benchmark of the forward model on the crossing-bundle workload.

One step = the forward model of one volume: voxelize 2 x 1000 fibers of 50
points into a 512x512x120 volume at 0.2 µm (generate_tissue) and march it at
5 tilts ((0,0) and 5.5° at phi = 0/90/180/270°) x 9 polarizer angles with
Slerp interpolation (run_simulation), epa fused.  Synthetic seeded fibers
(``fastpli_gb300.synth.crossing``); the label + vector volume (503 MB) is
larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  ``value`` is ray-voxel steps per second of
the whole step, device-resident; ``e2e`` the same metric through the
drop-in host API (host numpy in and out, copies inside the timed region).
``--impl reference`` times the CPU forward model (the oracle's C
restatement of the reference, all host threads) on the same workload.
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
sys.path.insert(0, ROOT)

METRIC = "ray-voxel steps/s (forward model: voxelize + 5 tilts x 9 angles, Slerp)"
UNIT = "steps/s"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _workload(rank=0):
    from fastpli_gb300 import synth
    # every rank voxelizes and marches its own seeded volume (weak scaling)
    return synth.crossing(seed=2 + rank)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while the
    timed region runs (a streaming nvidia-smi child, stopped afterwards)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._p = None
        self._t = None

    def _reader(self):
        for line in self._p.stdout:
            parts = [c.strip() for c in line.strip().split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __enter__(self):
        try:
            self._p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._reader, daemon=True)
            self._t.start()
            time.sleep(0.3)  # first sample before the timed region starts
        except Exception:
            self._p = None
        return self

    def __exit__(self, *a):
        if self._p:
            time.sleep(0.15)
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
            if self._t:
                self._t.join(timeout=5)

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[0]) for r in self.rows) if v is not None]
        mx = [v for v in (num(r[1]) for r in self.rows) if v is not None]
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        reasons = sorted({n for r in self.rows for n, v in zip(self.NAMES, r[3:7])
                          if v == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _ncu_metric(summary, name):
    """(value, unit) of a metric of the first launch in a committed ncu
    summary under profiles/ (None when absent)."""
    import re
    try:
        text = open(os.path.join(ROOT, "profiles", summary)).read()
    except OSError:
        return None
    m = re.search(r"`" + re.escape(name) + r"`\) \| ([0-9.]+) ?(\S*) \|", text)
    return (float(m.group(1)), m.group(2)) if m else None


def _ncu_traffic(summary):
    """DRAM bytes (read + write) per launch of the first launch listed in a
    committed ncu summary under profiles/ (None when absent)."""
    unit = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    total = 0.0
    for name in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
        v = _ncu_metric(summary, name)
        if v is None:
            return None
        total += v[0] * unit.get(v[1], 1)
    return total


def _ncu_limiter(summary):
    """What bounds a kernel that is not HBM-bound, from the same summary:
    the fraction of cycles the schedulers issued and the FMA-pipe load."""
    issue = _ncu_metric(summary, "smsp__issue_active.avg.pct_of_peak_sustained_active")
    fma = _ncu_metric(summary, "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active")
    if issue is None:
        return None
    return {"kind": "instruction issue / latency (ncu)", "issue_active_frac": issue[0] / 100,
            "fma_pipe_frac": None if fma is None else fma[0] / 100}


# Per-step operation counts of the reference formulas for the march's
# FP32 / SFU roofs (ray-voxel step with rho collapsed; background steps cost
# one multiply): NN 50 FP32 + 4 SFU (sqrt, rcp, sin, cos); Slerp adds the 8
# neighbour label compares and 7 interpolations of ~30 FP32 + acos + 2 sin +
# rcp.  A vertical ray's interpolation collapses, so untilted steps count as NN.
OPS_NN = (50, 4)
OPS_SLERP = (50 + 8 + 7 * 30, 4 + 7 * 4)
# voxelizer: one candidate test (a voxel of a segment's clipped box) is ~25
# FP64 operations and one FP64 division in the reference
FP64_PER_CANDIDATE = 26


def measure_peaks():
    """FP32 flop/s, SFU op/s, FP64 flop/s and L2 atomics/s of this GPU from the
    microbenchmarks in fastpli_gb300/csrc/peaks (None if unavailable)."""
    import ctypes
    from fastpli_gb300 import build as fb
    try:
        lib = ctypes.CDLL(fb.PEAKS_LIB)
    except OSError:
        return None
    lib.fpgb_measure_peaks.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    out = (ctypes.c_double * 4)()
    if lib.fpgb_measure_peaks(out, None) != 0:
        return None
    return {"fp32_flops": out[0], "sfu_ops": out[1], "fp64_flops": out[2],
            "l2_atomics": out[3]}


def candidate_tests(w):
    """Voxels of every segment's clipped box (generator.cpp:295-312), the
    voxelizer's algorithmic unit, from the fiber table on the host."""
    X, Y, Z = (int(v) for v in w.dim)
    total = 0
    for fibers, layers in zip(w.bundles, w.layers):
        smax = np.sqrt(max(l[0] for l in layers) ** 2)
        for f in fibers:
            p = (np.asarray(f[:, :3], np.float64) - np.asarray(w.origin)) * (1.0 / w.voxel_size)
            r = np.asarray(f[:, 3], np.float64) * (1.0 / w.voxel_size)
            rmax = np.maximum(r[:-1], r[1:]) * smax
            lo = np.minimum(p[:-1], p[1:]) - rmax[:, None]
            hi = np.maximum(p[:-1], p[1:]) + rmax[:, None]
            lo = np.clip(lo, 0, [X, Y, Z])
            hi = np.clip(hi, 0, [X, Y, Z])
            ext = np.maximum(np.floor(hi + 0.5) - np.trunc(lo), 0)
            total += int(np.prod(ext, axis=1).sum())
    return total


def roofline_model(peaks, hbm_gbs, w, n_steps_untilted, n_steps_tilted, tissue_frac,
                   march_steps_per_s, candidates, voxelize_s):
    """The march against min(HBM, FP32, SFU) steps/s and the voxelizer against
    the FP64 rate at the reference's per-candidate work."""
    if peaks is None:
        return None
    f = tissue_frac
    fp32 = ((f * OPS_NN[0] + 1 - f) * n_steps_untilted +
            (f * OPS_SLERP[0] + 1 - f) * n_steps_tilted) / (n_steps_untilted + n_steps_tilted)
    sfu = (f * OPS_NN[1] * n_steps_untilted + f * OPS_SLERP[1] * n_steps_tilted) / (
        n_steps_untilted + n_steps_tilted)
    roofs = {"hbm": hbm_gbs * 1e9 / 16, "fp32": peaks["fp32_flops"] / fp32,
             "sfu": peaks["sfu_ops"] / sfu}
    bound = min(roofs, key=roofs.get)
    vox_roof = peaks["fp64_flops"] / FP64_PER_CANDIDATE
    vox_rate = candidates / voxelize_s
    return {
        "measured_peaks": peaks,
        "march": {"unit": "ray-voxel steps/s", "achieved": march_steps_per_s,
                  "roofs": roofs, "bound": bound, "frac": march_steps_per_s / roofs[bound],
                  "ops_per_step": {"fp32": fp32, "sfu": sfu}, "tissue_step_frac": f},
        "voxelizer": {"unit": "candidate tests/s", "achieved": vox_rate,
                      "candidates": candidates, "roof_fp64": vox_roof, "bound": "fp64",
                      "frac": vox_rate / vox_roof},
    }


# kernels of one device-resident step: the voxelizer's segment binning (count,
# scan, fill) and brick kernel, then one march per tilt
VOXELIZER_LAUNCHES = 4


def _setup_args(w):
    kw = w.setup_kwargs()
    return (kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
            kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
            kw["flip_z"], kw["filter_rotations"])


# ---------------------------------------------------------------- CPU arm ---
def cpu_forward(w, n_threads, tilts=None):
    """The oracle's C restatement of the reference forward model; returns
    (seconds, ray-voxel steps)."""
    import oracle
    oracle.build(ref=False)
    from fastpli_gb300 import _native as N
    tilts = w.tilts if tilts is None else tilts
    t0 = time.perf_counter()
    lab, vec, props, _ = oracle.generate(w.dim, w.origin, w.voxel_size, w.bundles, w.layers,
                                         n_threads=n_threads)
    for theta, phi in tilts:
        oracle.simulate(lab, vec, props, theta, phi, n_threads=n_threads, **w.setup_kwargs())
    dt = time.perf_counter() - t0
    s = N.SetupBlock(*_setup_args(w))
    d = np.asarray(w.dim, np.int64)
    steps = sum(int(N.load(build_if_missing=False).fpgb_count_steps(
        N.byref(s.struct), N.ptr(d), float(t), float(p))) for t, p in tilts)
    return dt, steps


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    w = _workload(0)
    from fastpli_gb300 import build as nb
    nb.build()
    threads = os.cpu_count() or 1
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_forward(w, threads, tilts=w.tilts[:1])
    times, steps = [], 0
    for _ in range(args.steps):
        dt, steps = cpu_forward(w, threads)
        times.append(dt)
    value = steps / (sum(times) / len(times))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": dict(w.describe(), inputs="fibers (host)",
                           parallelism=f"OpenMP {threads} threads"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "full forward-model steps of the workload"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm ---
def run_gpu(args):
    import torch
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from fastpli_gb300.simulation import _Generator, _Simulator
    import fastpli_gb300
    fastpli_gb300.native_library()

    w = _workload(rank)
    X, Y, Z = (int(v) for v in w.dim)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    sim = _Simulator()
    sim.set_pli_setup(*_setup_args(w))
    steps_per = sum(sim.count_steps(w.dim, float(t), float(p)) for t, p in w.tilts)
    n_rho = sim.n_rho
    dev = torch.device("cuda", local)
    label = torch.empty((X, Y, Z), dtype=torch.int32, device=dev)
    vector = torch.empty((X, Y, Z, 3), dtype=torch.float32, device=dev)
    images = [torch.empty((X, Y, n_rho), dtype=torch.float64, device=dev) for _ in w.tilts]
    wsp = torch.empty(g.workspace_size(), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    _, _, props, _ = g.run_generation_device(label=label, vector=vector, workspace=wsp)
    tissue_voxels = int((label > 0).sum().item())

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        g.run_generation_device(label=label, vector=vector, workspace=wsp,
                                sync_warnings=False)
        if ev:
            ev[1].record(stream)
        sim.run_tilts_device(w.dim, label, vector, props, w.tilts, images=images,
                             sync_warnings=False)
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            step(evs[i])
        t1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_total = t0.elapsed_time(t1)
    gen_ms = [e[0].elapsed_time(e[1]) for e in evs]
    march_ms = [e[1].elapsed_time(e[2]) for e in evs]
    if dist:
        tt = torch.tensor([ms_total], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_total = float(tt.item())
    ms_step = ms_total / args.steps
    value = ws * steps_per / (ms_step * 1e-3)

    # ----- e2e through the drop-in host API (numpy in/out) ---------------
    # three full untimed steps first: the first host-API steps after the
    # device loop pay one-off costs (pool growth, page-locked host blocks)
    e2e_steps = max(3, min(args.steps, 10))
    # (the warm-up steps keep their results alive exactly as the timed steps
    # do, so the host allocator's cache holds the blocks the timed loop needs)
    for _ in range(3):
        lab_h, vec_h, props_h = g.run_generation()
        imgs = [sim.run_simulation(w.dim, lab_h, vec_h, props_h, float(t), float(p))
                for t, p in w.tilts]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_step_s = []
    for _ in range(e2e_steps):
        t_e2e = time.perf_counter()
        lab_h, vec_h, props_h = g.run_generation()
        imgs = [sim.run_simulation(w.dim, lab_h, vec_h, props_h, float(t), float(p))
                for t, p in w.tilts]
        e2e_step_s.append(time.perf_counter() - t_e2e)
    e2e_s = sum(e2e_step_s) / e2e_steps
    if dist:
        tt = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    vol_bytes = X * Y * Z * 16
    img_bytes = X * Y * n_rho * 8
    fib_bytes = int(sum(f.nbytes for b in w.bundles for f in b))
    h2d = fib_bytes + len(w.tilts) * vol_bytes
    d2h = vol_bytes + len(w.tilts) * img_bytes
    del imgs

    # ----- roofline of the dominant kernel ------------------------------
    hbm_peak, peak_kind = _peaks()
    gen_avg = sum(gen_ms) / len(gen_ms)
    march_avg = sum(march_ms) / len(march_ms)
    n_untilted = sum(sim.count_steps(w.dim, float(t), float(p))
                     for t, p in w.tilts if float(t) == 0.0)
    model = roofline_model(measure_peaks(), hbm_peak, w, n_untilted, steps_per - n_untilted,
                           tissue_voxels / float(X * Y * Z), steps_per / (march_avg * 1e-3),
                           candidate_tests(w), gen_avg * 1e-3)
    # march: one label (4 B) and one axis (12 B) per ray-voxel step
    march_bytes = 16 * steps_per
    march_gbs = march_bytes / (march_avg * 1e-3) / 1e9
    # voxelizer: label + vector written once per voxel (16 B); the winner keys
    # stay in shared memory, the segment table (280 B per segment) is noise
    gen_bytes = 16 * X * Y * Z
    gen_gbs = gen_bytes / (gen_avg * 1e-3) / 1e9
    if march_avg >= gen_avg:
        prof = "march_rays_slerp_tilted_crossing512x512x120.md"
        traffic = _ncu_traffic(prof)
        roof = {"kernel": "march_rays (5 tilts)", "bound": "hbm", "achieved": march_gbs,
                "peak": hbm_peak, "unit": "GB/s", "frac": march_gbs / hbm_peak,
                "traffic": traffic, "traffic_per": "one tilted launch (ncu)",
                "limiter": _ncu_limiter(prof),
                "algorithmic_bytes_per_launch": march_bytes / len(w.tilts),
                "algorithmic_bytes_per_step": 16, "peak_source": peak_kind}
    else:
        prof = "voxel_bricks_crossing512x512x120.md"
        traffic = _ncu_traffic(prof)
        roof = {"kernel": "voxel_bricks (+ binning)", "bound": "hbm", "achieved": gen_gbs,
                "peak": hbm_peak, "unit": "GB/s", "frac": gen_gbs / hbm_peak,
                "traffic": traffic, "traffic_per": "one launch (ncu)",
                "limiter": _ncu_limiter(prof),
                "algorithmic_bytes_per_launch": gen_bytes,
                "algorithmic_bytes_per_voxel": 16, "peak_source": peak_kind}

    line = None
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu:
            threads = os.cpu_count() or 1
            dt, st = cpu_forward(w, threads)
            cpu = {"value": st / dt, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "one full forward-model step of the workload (oracle C "
                             "restatement, OpenMP)"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": dict(w.describe(), l2="inputs larger than L2 (503 MB volume)",
                           parallelism=f"replicas x{ws}"),
            "tissue_voxels_per_s": tissue_voxels / (gen_avg * 1e-3),
            "voxelize_ms": gen_avg, "march_ms": march_avg,
            "march_steps_per_s": steps_per / (march_avg * 1e-3),
            "roofline": roof, "roofline_model": model, "cpu_baseline": cpu,
            "e2e": {"value": ws * steps_per / e2e_s, "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps, "step_ms_mean": 1e3 * e2e_s,
                    "step_ms_min": 1e3 * min(e2e_step_s),
                    "step_ms_max": 1e3 * max(e2e_step_s)},
            "gpu_launches": args.steps * (VOXELIZER_LAUNCHES + len(w.tilts)),
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------- tiles mode ---
def run_tiles(args):
    """Batched uneven tiles (``--workload tiles``): N tiles of the uneven-tile
    mixture (xy 64-512, z 30-120 voxels at 0.2 um, 50-2000 fibers, per-tile
    dn/mu), 5 tilts x 9 angles each, Slerp.  One step = the whole batch
    (voxelize all tiles + march all pairs) replayed from a CUDA graph; the
    plain per-call path (per tile: voxelize, then one march per tilt) is timed
    on the same tiles for comparison."""
    import torch
    from fastpli_gb300 import autotune, synth
    from fastpli_gb300.batch import TileBatch
    from fastpli_gb300.simulation import _Generator, _Simulator
    import fastpli_gb300
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    fastpli_gb300.native_library()
    from fastpli_gb300.shard import rank_units
    tiles_all = synth.tiles(args.tiles)
    mine = rank_units([t.n_voxels for t in tiles_all], ws, rank)
    tiles = [tiles_all[i] for i in mine]
    kw = tiles[0].setup_kwargs()
    b = TileBatch(tiles, kw).allocate()
    cfg, _, _ = autotune.tune(b, reps=1)
    b.capture()
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        e0.record()
        for _ in range(args.steps):
            b.replay()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    w = b.warnings()
    steps = b.steps
    vox = int(b.info.total_voxels)
    # plain per-call path on the same tiles (device resident, no host copies)
    sim = _Simulator()
    sim.set_pli_setup(*_setup_args(tiles[0]))
    gens = []
    for t in tiles:
        g = _Generator()
        g.set_volume(t.dim, t.origin, t.voxel_size)
        g.set_fiber_bundles(t.bundles, t.layers)
        X, Y, Z = (int(v) for v in t.dim)
        lab = torch.empty((X, Y, Z), dtype=torch.int32, device="cuda")
        vec = torch.empty((X, Y, Z, 3), dtype=torch.float32, device="cuda")
        img = torch.empty((X, Y, sim.n_rho), dtype=torch.float64, device="cuda")
        wsp = torch.empty(g.workspace_size(), dtype=torch.uint8, device="cuda")
        gens.append((g, t, lab, vec, img, wsp))

    def plain():
        for g, t, lab, vec, img, wsp in gens:
            _, _, props, _ = g.run_generation_device(label=lab, vector=vec, workspace=wsp,
                                                     sync_warnings=False)
            for th, ph in t.tilts:
                sim.run_simulation_device(t.dim, lab, vec, props, float(th), float(ph),
                                          image=img, sync_warnings=False)
    import warnings as _w
    with _w.catch_warnings():
        _w.simplefilter("ignore")
        plain()
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        e0.record()
        plain()
        e1.record()
        torch.cuda.synchronize()
        plain_wall = time.perf_counter() - p0
    plain_ms = e0.elapsed_time(e1)
    ms = max_over_ranks_ms(ms, ws, local)
    if rank == 0:
        line = {"metric": "ray-voxel steps/s (uneven tile batch, voxelize + 5 tilts x 9 angles, "
                          "Slerp)", "value": ws * steps / (ms * 1e-3), "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"{len(tiles)} uneven tiles (64-512 xy, 30-120 z)",
                           "voxels": vox, "pairs": int(b.info.n_pairs),
                           "graph": "CUDA graph replay", "march_config": list(cfg),
                           "l2": "inputs larger than L2"},
                "tissue_voxels_per_s": None,
                "plain_per_call": {"ms_per_batch_device": plain_ms,
                                   "ms_per_batch_wall": plain_wall * 1e3,
                                   "steps_per_s": steps / (plain_ms * 1e-3)},
                "fp64_replays": w["fp64_replays"], "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    b.close()
    return 0


# ----------------------------------------------------------- serve mode ---
def run_serve(args):
    """Serving (``--workload serve``): Poisson arrivals at each rate of
    ``--rates``; every request is a tile of the uneven-tile mixture (a pool of
    ``--pool`` seeded tiles) with 1 or 5 tilts (Bernoulli 1/2), Slerp, epa on
    the device; HBM admission budget 150 GB.  The continuous-batching server
    is compared with the plain per-call path serving the same arrival stream
    one request at a time.  Reports p50/p99 arrival-to-result latency and
    throughput per rate."""
    import torch
    import warnings as _w
    from fastpli_gb300 import serving, synth
    import fastpli_gb300
    ws, rank, local = _dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    fastpli_gb300.native_library()
    pool = [synth.tile(i) for i in range(args.pool)]
    kw = pool[0].setup_kwargs()
    rng = np.random.default_rng(5)

    def stream_of(lam, n):
        gaps = rng.exponential(1.0 / lam, n)
        picks = rng.integers(0, len(pool), n)
        five = rng.random(n) < 0.5
        return np.cumsum(gaps), [(pool[i], synth.TILTS_5 if f else synth.TILTS_5[:1])
                                 for i, f in zip(picks, five)]

    def serve(server, arrivals, specs):
        t0 = time.perf_counter()
        reqs = []
        with server:
            for a, (tile, tilts) in zip(arrivals, specs):
                d = t0 + a - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                reqs.append(server.submit(tile, tilts))
            for r in reqs:
                r.wait(600)
        wall = time.perf_counter() - t0
        st = serving.latency_stats(reqs)
        st["throughput_rps"] = len(reqs) / wall
        st["batches"] = server.batches
        return st

    with _w.catch_warnings():
        _w.simplefilter("ignore")
        # warm both paths (module load, autotune cache)
        warm_a, warm_s = stream_of(1000.0, 8)
        serve(serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=32, n_slots=2), warm_a, warm_s)
        serve(serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=1, n_slots=1,
                                    runner=serving.PlainRunner(kw)), warm_a, warm_s)
        results = []
        with ClockSampler(local) as clocks:
            for lam in args.rates:
                n = int(min(args.max_requests, max(40, lam * args.seconds)))
                arrivals, specs = stream_of(lam, n)
                batched = serve(serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=32,
                                                      n_slots=2), arrivals, specs)
                plain = serve(serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=1, n_slots=1,
                                                    runner=serving.PlainRunner(kw)),
                              arrivals, specs)
                results.append({"rate_rps": lam, "requests": n, "batched": batched,
                                "plain": plain})
    best = max(r["batched"]["throughput_rps"] for r in results)
    line = {"metric": "serving: requests/s and p50/p99 latency under Poisson load "
                      "(uneven tiles, 1 or 5 tilts, Slerp, epa)",
            "value": best, "unit": "requests/s", "n_gpus": 1, "steps": len(results),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"tile pool of {len(pool)} (64-512 xy, 30-120 z)",
                       "hbm_budget_gb": 150, "max_tiles_per_batch": 32, "streams": 2},
            "sweep": results, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks_ms(ms, ws, local):
    if ws <= 1:
        return ms
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from fastpli_gb300.shard import max_over_ranks
    return max_over_ranks(ms, dist, device=torch.device("cuda", local))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="crossing", choices=["crossing", "tiles", "serve"])
    ap.add_argument("--rates", type=float, nargs="+", default=[10, 50, 200, 500],
                    help="serve: Poisson arrival rates (requests/s)")
    ap.add_argument("--seconds", type=float, default=4.0, help="serve: seconds per rate")
    ap.add_argument("--max-requests", type=int, default=600, help="serve: cap per rate")
    ap.add_argument("--pool", type=int, default=48, help="serve: distinct tiles")
    ap.add_argument("--tiles", type=int, default=256, help="tiles of the tiles workload")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "tiles":
        return run_tiles(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
