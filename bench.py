"""Benchmark of the forward model.

Default workload (the headline line): the uneven-tile batch — 256 independent
tissue tiles, xy sides uniform 64-512 voxels, z 30-120 voxels at 0.2 µm, 50-2000
fibers of uniformly random direction per tile with the tile's own dn in
[-0.004, 0.004] and mu in [0, 20] (``fastpli_gb300.synth.tiles``, seeds
1000 + i), each tile voxelized and marched at 5 tilts ((0,0) and 5.5° at
phi = 0/90/180/270°) x 9 polarizer angles with Slerp interpolation.  One step
= the whole batch (voxelize every tile + march every (tile, tilt) pair) as one
CUDA-graph replay.  The 26 GB of label + vector fields are far larger than
L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload tiles|crossing|serve]

Prints one JSON line (rank 0):
  value       ray-voxel steps/s of the batch, device-resident (fiber tables
              already in HBM; CUDA-graph replays timed with CUDA events);
  e2e         the same metric through the batch's C ABI with HOST buffers:
              host planning from the flat fiber arrays, upload of the tables,
              the batch, and one device-to-host copy of every image into
              page-locked memory, per step (wall clock);
  plain_per_call / e2e_plain_host_api
              the same tiles through the plain per-call path (one voxelizer
              call + 5 march calls per tile), device-resident and through the
              drop-in host API (numpy label/vector out of run_generation and
              back into each run_simulation, as Simpli does);
  roofline    the dominant kernel (voxelizer or march, timed stage by stage)
              against the measured HBM copy rate;
  cpu_baseline / parity
              the oracle (the C restatement of the reference, all host
              threads) on a bounded sample of the same tiles, and the GPU
              results of those tiles compared with it;
  crossing / watson / serving
              the 512x512x120 crossing-bundle volume (5 tilts), the
              1024x1024x240 voxelization-heavy Watson volume (1 tilt) and a
              short Poisson serving sweep (batched vs plain, p50/p99).

``--impl reference`` times the CPU forward model (the oracle's C restatement
of the reference, all host threads) on rotating samples of the same tiles; it
loads nothing of this package's native library.
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

METRIC = "ray-voxel steps/s (uneven tile batch: voxelize + 5 tilts x 9 angles, Slerp)"
UNIT = "steps/s"
N_TILES = 256
CPU_SAMPLE_STRIDE = 8      # GPU arm's CPU baseline / parity: every 8th tile (32 tiles)
ONE_THREAD_TILES = (0, 128)  # the CPU baseline's 1-thread figure
REF_TILES_PER_STEP = 8     # reference arm: 8 consecutive tiles per step, rotating
VOXELIZER_LAUNCHES = 4     # brick_bin (count), brick_scan, brick_bin (fill), voxel_bricks
MARCH_LAUNCHES = 2         # batch_march untilted, tilted
E2E_GROUPS = 16            # host-buffer e2e: tile groups pipelined by run_tiles_host (16: 228 ms, 8: 232, 4: 244, 2: 271)
# units of the committed ncu captures (profiles/*_tiles16.md): the first 16 tiles
PROFILED_TILTED_STEPS = 268946100   # batch_march, tilted launch
PROFILED_VOXELS = 67210825          # voxel_bricks


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
        return float(p["hbm_gbs"]), "measured", float(p.get("sm_max_mhz", 2070.0))
    except Exception:
        return 6800.0, "fallback", 2070.0


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
    """What bounds a kernel that is not HBM-bound, from the same summary."""
    issue = _ncu_metric(summary, "smsp__issue_active.avg.pct_of_peak_sustained_active")
    if issue is None:
        return None
    out = {"kind": "instruction issue / latency (ncu)", "issue_active_frac": issue[0] / 100,
           "source": "profiles/" + summary}
    dram = _ncu_metric(summary, "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed")
    if dram is not None:
        out["dram_frac"] = dram[0] / 100
    return out


# Minimal thread instructions of one voxelizer candidate test (a voxel of a
# segment's clipped box): the FP32 estimate of its distance to the segment
# (about 10 FMAs: w = c - p, c1 = w.v, t = clamp(c1 / c2), |w - t v|^2),
# the threshold compare and one shared-memory atomicMin of the winner key:
# 16.  The issue roof is the GPU's thread-instruction rate over that count.
VOXEL_MIN_INST = 16


def candidate_tests(tiles):
    """Voxels of every segment's clipped box (generator.cpp:295-312), the
    voxelizer's algorithmic unit, from the fiber tables on the host."""
    total = 0
    for w in tiles:
        X, Y, Z = (int(v) for v in w.dim)
        for fibers, layers in zip(w.bundles, w.layers):
            smax = np.sqrt(max(l[0] for l in layers) ** 2)
            if not len(fibers):
                continue
            pts = [np.asarray(f, np.float64) for f in fibers if len(f) > 1]
            for f in pts:
                p = (f[:, :3] - np.asarray(w.origin)) * (1.0 / w.voxel_size)
                r = f[:, 3] * (1.0 / w.voxel_size)
                rmax = np.maximum(r[:-1], r[1:]) * smax
                lo = np.clip(np.minimum(p[:-1], p[1:]) - rmax[:, None], 0, [X, Y, Z])
                hi = np.clip(np.maximum(p[:-1], p[1:]) + rmax[:, None], 0, [X, Y, Z])
                ext = np.maximum(np.floor(hi + 0.5) - np.trunc(lo), 0)
                total += int(np.prod(ext, axis=1).sum())
    return total


def _setup_args(w):
    kw = w.setup_kwargs()
    return (kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
            kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
            kw["flip_z"], kw["filter_rotations"])


def _simulator(w):
    from fastpli_gb300.simulation import _Simulator
    sim = _Simulator()
    sim.set_pli_setup(*_setup_args(w))
    return sim


# ---------------------------------------------------------------- CPU arm ---
def cpu_forward(tiles, n_threads, keep=False):
    """The oracle's C restatement of the reference forward model over
    ``tiles`` (voxelize, then every tilt); returns (seconds, ray-voxel steps,
    outputs).  Steps are counted on the host with the reference's z loop
    (oracle.count_steps), so nothing of the product library is loaded."""
    import oracle
    t0 = time.perf_counter()
    steps, outs = 0, []
    for w in tiles:
        lab, vec, props, _ = oracle.generate(w.dim, w.origin, w.voxel_size, w.bundles, w.layers,
                                             n_threads=n_threads)
        imgs = [oracle.simulate(lab, vec, props, th, ph, n_threads=n_threads,
                                **w.setup_kwargs())[0] for th, ph in w.tilts]
        steps += sum(oracle.count_steps(w.dim, th, w.setup_kwargs()["step_size"])
                     for th, _ in w.tilts)
        if keep:
            outs.append((lab, vec, imgs))
    return time.perf_counter() - t0, steps, outs


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    import oracle
    from fastpli_gb300 import synth
    oracle.build(ref=False)
    threads = os.cpu_count() or 1
    k = REF_TILES_PER_STEP

    def sample(step):
        return [synth.tile((step * k + j) % N_TILES) for j in range(k)]

    for i in range(min(args.warmup, 2)):
        cpu_forward(sample(N_TILES // k - 1 - i), threads)
    times, steps = [], []
    for i in range(args.steps):
        tiles = sample(i)  # generating the fibers is not timed
        dt, st, _ = cpu_forward(tiles, threads)
        times.append(dt)
        steps.append(st)
    value = sum(steps) / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"uneven tile batch, {N_TILES} tiles (xy 64-512, z 30-120 "
                                   f"@ 0.2 um, 50-2000 fibers, 5 tilts x 9 angles, Slerp)",
                       "inputs": "fibers (host)", "parallelism": f"OpenMP {threads} threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{k} consecutive tiles of the {N_TILES}-tile mixture "
                                       f"per step, rotating ({args.steps * k} tiles timed); "
                                       "voxelize + 5 tilts each"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm ---
def _events(n):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def measure_stages(b, reps, stream):
    """Voxelizer and march of the batch timed separately (CUDA events on the
    launching stream): average ms of each."""
    import torch
    ev = [_events(3) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for e in ev:
            e[0].record(stream)
            b.run(stages=1, stream=stream)
            e[1].record(stream)
            b.run(stages=2, stream=stream)
            e[2].record(stream)
    torch.cuda.synchronize()
    vox = sum(e[0].elapsed_time(e[1]) for e in ev) / reps
    march = sum(e[1].elapsed_time(e[2]) for e in ev) / reps
    return vox, march


def plain_device_pass(tiles, sim, bufs):
    """The plain per-call path over the tiles, device-resident: one
    voxelizer call and 5 march calls per tile."""
    for (g, t, lab, vec, img, wsp) in bufs:
        _, _, props, _ = g.run_generation_device(label=lab, vector=vec, workspace=wsp,
                                                 sync_warnings=False)
        for th, ph in t.tilts:
            sim.run_simulation_device(t.dim, lab, vec, props, float(th), float(ph), image=img,
                                      sync_warnings=False)


def plain_host_pass(tiles, sim, gens):
    """The drop-in host API over the tiles, as Simpli drives it: numpy label /
    vector fields out of run_generation, passed back into run_simulation for
    every tilt; images returned as numpy."""
    for g, t in zip(gens, tiles):
        lab, vec, props = g.run_generation()
        for th, ph in t.tilts:
            sim.run_simulation(t.dim, lab, vec, props, float(th), float(ph))


def run_gpu(args):
    import warnings as _w
    import torch
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import fastpli_gb300
    from fastpli_gb300 import autotune, synth
    from fastpli_gb300 import batch as B
    from fastpli_gb300.shard import rank_units
    from fastpli_gb300.simulation import _Generator
    fastpli_gb300.native_library()
    _w.simplefilter("ignore")  # "objects overlap" etc.: the tiles overlap by design
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()

    all_params = [synth.tile_params(i) for i in range(args.tiles)]
    mine = rank_units([int(np.prod(p[0])) for p in all_params], ws, rank)
    tiles = [synth.tile(i) for i in mine]
    kw = tiles[0].setup_kwargs()
    flats = B.flatten(tiles)
    b = B.TileBatch(tiles, kw, flat_fibers=flats).allocate()
    if args.no_tune:
        cfg = b.config = (0, 2, 1, 0)
    else:
        cfg, _, _ = autotune.tune(b, reps=1)
    b.capture()
    steps = b.steps
    n_pairs = int(b.info.n_pairs)
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        e0, e1 = _events(2)
        e0.record(stream)
        for _ in range(args.steps):
            b.replay()
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_step = e0.elapsed_time(e1) / args.steps
    if dist:
        from fastpli_gb300.shard import max_over_ranks
        ms_step = max_over_ranks(ms_step, dist, device=dev)
    value = ws * steps / (ms_step * 1e-3)

    # ----- stage split (voxelizer | march), for the roofline --------------
    vox_ms, march_ms = measure_stages(b, 3, stream)

    # ----- parity sample: GPU results of the CPU-baseline tiles -----------
    b.replay()
    torch.cuda.synchronize()
    sample_idx = list(range(0, len(tiles), CPU_SAMPLE_STRIDE))
    gpu_sample = [(b.label(t).cpu().numpy(), b.vector(t).cpu().numpy(),
                   [b.image(p).cpu().numpy() for p in b.pairs_of(t)]) for t in sample_idx]

    # ----- e2e through the batch C ABI with host buffers --------------------
    # (a) one batch: plan, upload, run, one copy of every image down
    host_out = torch.empty(b.output_bytes, dtype=torch.uint8, pin_memory=True)
    arena, wsp = b.arena, b.workspace

    def one_batch_step():
        bb = B.TileBatch(tiles, kw, flat_fibers=flats)
        bb.allocate(arena=arena, workspace=wsp)
        bb.config = cfg
        bb.run()
        bb.outputs_host(out=host_out)
        return bb

    for _ in range(2):
        one_batch_step().close()
    torch.cuda.synchronize()
    one_s = []
    for _ in range(3):
        t0 = time.perf_counter()
        one_batch_step().close()
        one_s.append(time.perf_counter() - t0)
    b.close()  # the graph and the handle
    del arena, wsp, host_out
    b = None
    torch.cuda.empty_cache()

    # (b) the pipelined host call (run_tiles_host): groups planned on a host
    # thread while the previous group runs, images copied down meanwhile
    e2e_n = max(3, min(args.steps, 10))
    bufs = None
    for _ in range(2):
        _, st = B.run_tiles_host(tiles, kw, chunks=E2E_GROUPS, config=cfg, flat_fibers=flats,
                                 host_buffers=bufs)
        bufs = st["host_buffers"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_s = []
    for _ in range(e2e_n):
        t0 = time.perf_counter()
        _, st = B.run_tiles_host(tiles, kw, chunks=E2E_GROUPS, config=cfg, flat_fibers=flats,
                                 host_buffers=bufs)
        e2e_s.append(time.perf_counter() - t0)
    e2e_mean = sum(e2e_s) / len(e2e_s)
    if dist:
        from fastpli_gb300.shard import max_over_ranks
        e2e_mean = max_over_ranks(e2e_mean, dist, device=dev)
    h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
    del bufs, st
    torch.cuda.empty_cache()

    # ----- the plain per-call path on the same tiles ------------------------
    sim = _simulator(tiles[0])
    gens, bufs = [], []
    for t in tiles:
        g = _Generator()
        g.set_volume(t.dim, t.origin, t.voxel_size)
        g.set_fiber_bundles(t.bundles, t.layers)
        gens.append(g)
    for g, t in zip(gens, tiles):
        X, Y, Z = (int(v) for v in t.dim)
        bufs.append((g, t, torch.empty((X, Y, Z), dtype=torch.int32, device=dev),
                     torch.empty((X, Y, Z, 3), dtype=torch.float32, device=dev),
                     torch.empty((X, Y, sim.n_rho), dtype=torch.float64, device=dev),
                     torch.empty(g.workspace_size(), dtype=torch.uint8, device=dev)))
    plain_device_pass(tiles, sim, bufs)
    torch.cuda.synchronize()
    p0, p1 = _events(2)
    p0.record(stream)
    plain_device_pass(tiles, sim, bufs)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    del bufs
    torch.cuda.empty_cache()
    plain_host_pass(tiles[:8], sim, gens[:8])  # warm the host allocator
    t0 = time.perf_counter()
    plain_host_pass(tiles, sim, gens)
    plain_host_s = time.perf_counter() - t0
    vol_bytes = sum(int(np.prod(t.dim)) * 16 for t in tiles)
    img_bytes = sum(int(t.dim[0] * t.dim[1]) * sim.n_rho * 8 * len(t.tilts) for t in tiles)
    fib_bytes = sum(f.nbytes for t in tiles for bnd in t.bundles for f in bnd)
    plain_h2d = fib_bytes + sum(int(np.prod(t.dim)) * 16 * len(t.tilts) for t in tiles)

    # ----- roofline of the dominant kernel ----------------------------------
    hbm, peak_kind, sm_mhz = _peaks()
    vox = sum(int(np.prod(t.dim)) for t in tiles)
    march_bytes = 16 * steps
    vox_bytes = 16 * vox
    march_gbs = march_bytes / (march_ms * 1e-3) / 1e9
    vox_gbs = vox_bytes / (vox_ms * 1e-3) / 1e9
    # DRAM traffic from the committed ncu captures of the same kernels on the
    # first 16 tiles (a --set full capture of the whole batch is too large),
    # scaled to this batch by the units processed: the tilted march by its
    # steps (the untilted column march reads each voxel once per tilt: 16 B a
    # step), the voxelizer by its voxels
    import oracle
    tilted = sum(oracle.count_steps(t.dim, th, t.setup_kwargs()["step_size"])
                 for t in tiles for th, _ in t.tilts if float(th) != 0.0)
    if march_ms >= vox_ms:
        prof = "batch_march_tiles16.md"
        t16 = _ncu_traffic(prof)
        traffic = (None if t16 is None
                   else t16 * tilted / PROFILED_TILTED_STEPS + 16.0 * (steps - tilted))
        roof = {"kernel": "batch_march (2 launches: untilted, tilted)", "bound": "hbm",
                "achieved": march_gbs, "peak": hbm, "unit": "GB/s", "frac": march_gbs / hbm,
                "traffic": traffic, "traffic_per": "batch: ncu of 16 tiles scaled by steps",
                "limiter": _ncu_limiter(prof), "algorithmic_bytes_per_launch": march_bytes,
                "algorithmic_bytes_per_step": 16, "peak_source": peak_kind}
    else:
        prof = "voxel_bricks_tiles16.md"
        t16 = _ncu_traffic(prof)
        roof = {"kernel": "voxel_bricks (+ binning)", "bound": "hbm", "achieved": vox_gbs,
                "peak": hbm, "unit": "GB/s", "frac": vox_gbs / hbm,
                "traffic": None if t16 is None else t16 * vox / PROFILED_VOXELS,
                "traffic_per": "one launch: ncu of 16 tiles scaled by voxels",
                "limiter": _ncu_limiter(prof), "algorithmic_bytes_per_launch": vox_bytes,
                "algorithmic_bytes_per_voxel": 16, "peak_source": peak_kind}
    cands = candidate_tests(tiles)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    issue_rate = sms * 4 * 32 * sm_mhz * 1e6  # thread instructions per second
    hbm_steps = hbm * 1e9 / 16
    model = {
        "march": {"unit": "ray-voxel steps/s", "achieved": steps / (march_ms * 1e-3),
                  "roof_hbm": hbm_steps, "frac_hbm": steps / (march_ms * 1e-3) / hbm_steps,
                  "ms": march_ms, "bytes_per_step": 16},
        "voxelizer": {"unit": "candidate tests/s", "candidates": cands,
                      "achieved": cands / (vox_ms * 1e-3), "ms": vox_ms,
                      "roof_issue": issue_rate / VOXEL_MIN_INST,
                      "frac_issue": cands / (vox_ms * 1e-3) / (issue_rate / VOXEL_MIN_INST),
                      "min_thread_inst_per_candidate": VOXEL_MIN_INST,
                      "frac_hbm": vox_gbs / hbm, "bytes_per_voxel": 16},
        "batch": {"unit": "ray-voxel steps/s", "achieved": steps / (ms_step * 1e-3),
                  "roof_hbm": hbm_steps, "frac_hbm": steps / (ms_step * 1e-3) / hbm_steps,
                  "target_frac": 0.6,
                  "note": "voxelizer + march of the batch against the march's HBM roof "
                          "(16 B per ray-voxel step)"},
    }

    line = None
    if rank == 0:
        # the GPU extras first: the CPU legs below load every host core
        extra = {}
        if not args.quick:
            extra["crossing"] = measure_crossing(dev)
            extra["watson"] = measure_watson(dev)
            if args.serve_seconds > 0:
                extra["serving"] = serve_sweep(args.rates, args.serve_seconds,
                                               args.max_requests, 20, local, pool=tiles)
        cpu, par = None, None
        if ws == 1 and not args.no_cpu:
            import oracle
            oracle.build(ref=False)
            threads = os.cpu_count() or 1
            sample = [tiles[t] for t in sample_idx]
            dt, st, outs = cpu_forward(sample, threads, keep=True)
            one = [tiles[t] for t in ONE_THREAD_TILES]
            dt1, st1, _ = cpu_forward(one, 1)
            cpu = {"value": st / dt, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"{len(sample)} of the {len(tiles)} tiles (every "
                             f"{CPU_SAMPLE_STRIDE}th), voxelize + 5 tilts each "
                             "(oracle C restatement, OpenMP)",
                   "one_thread": {"value": st1 / dt1, "unit": UNIT, "cores": 1,
                                  "sample": f"tiles {list(ONE_THREAD_TILES)}, voxelize + 5 "
                                            "tilts each"}}
            par = parity_of(gpu_sample, outs)
            del outs
        del gpu_sample
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"uneven tile batch, {args.tiles} tiles (xy 64-512, z 30-120 "
                                   f"@ 0.2 um, 50-2000 fibers, 5 tilts x 9 angles, Slerp)",
                       "tiles": len(tiles), "voxels": vox, "pairs": n_pairs,
                       "ray_voxel_steps": steps, "graph": "CUDA graph replay",
                       "march_config": {"ctas_per_sm": cfg[0], "items_per_grab": cfg[1],
                                        "coop": cfg[2], "ray_block": B.TileBatch.SHAPES[cfg[3]]},
                       "l2": f"inputs larger than L2 ({vox_bytes / 1e9:.1f} GB of fields)",
                       "parallelism": f"replicas x{ws} (tiles sharded)"},
            "tissue_voxels_per_s": vox / (vox_ms * 1e-3),
            "voxelize_ms": vox_ms, "march_ms": march_ms,
            "plain_per_call": {"ms_per_batch": plain_ms, "steps_per_s": steps / (plain_ms * 1e-3),
                               "batched_speedup": plain_ms / ms_step},
            "roofline": roof, "roofline_model": model, "cpu_baseline": cpu, "parity": par,
            "e2e": {"value": ws * steps / e2e_mean, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_n, "step_ms_mean": 1e3 * e2e_mean,
                    "step_ms_min": 1e3 * min(e2e_s), "step_ms_max": 1e3 * max(e2e_s),
                    "path": f"batch.run_tiles_host: {E2E_GROUPS} groups, each "
                            "fpgb_batch_create (host thread) / upload / run / one D2H copy of "
                            "its images, overlapped"},
            "e2e_one_batch": {"value": ws * steps / (sum(one_s) / len(one_s)), "unit": UNIT,
                              "step_ms_mean": 1e3 * sum(one_s) / len(one_s),
                              "path": "one fpgb_batch_create / upload / run / D2H, in order"},
            "e2e_plain_host_api": {"value": steps / plain_host_s, "unit": UNIT,
                                   "ms_per_batch": 1e3 * plain_host_s,
                                   "h2d_bytes_per_step": plain_h2d,
                                   "d2h_bytes_per_step": vol_bytes + img_bytes},
            "gpu_launches": args.steps * (VOXELIZER_LAUNCHES + MARCH_LAUNCHES),
            "clocks": clocks.summary(),
            **extra,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def parity_of(gpu, cpu):
    """Label / vector mismatches and image errors of the GPU results against
    the oracle's, over the sampled tiles."""
    n_lab = n_vec = 0
    rel = rel_mean = 0.0
    pixels = 0
    for (gl, gv, gi), (cl, cv, ci) in zip(gpu, cpu):
        n_lab += int((gl != cl).sum())
        n_vec += int((gv.view(np.uint32) != cv.view(np.uint32)).sum())
        for a, r in zip(gi, ci):
            rel = max(rel, float(np.max(np.abs(a - r) / np.maximum(np.abs(r), 1e-300))))
            m = np.maximum(np.abs(r.mean(-1, keepdims=True)), 1e-300)
            rel_mean = max(rel_mean, float(np.max(np.abs(a - r) / m)))
            pixels += r.size
    return {"against": "oracle (FP64 C restatement, pinned to the reference build)",
            "tiles": len(gpu), "label_mismatches": n_lab, "vector_mismatches": n_vec,
            "image_max_rel": rel, "image_max_rel_to_pixel_mean": rel_mean,
            "image_values": pixels, "bars": {"labels": 0, "vectors": 0, "image_rel": 1e-4}}


# ------------------------------------------------- the other workloads ---
def measure_crossing(dev, steps=10, warmup=3):
    """The 512x512x120 crossing-bundle volume: voxelize + 5 tilts per step,
    device-resident, and through the drop-in host API."""
    import torch
    from fastpli_gb300 import synth
    from fastpli_gb300.simulation import _Generator
    w = synth.crossing(seed=2)
    X, Y, Z = (int(v) for v in w.dim)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    sim = _simulator(w)
    n_steps = sum(sim.count_steps(w.dim, float(t), float(p)) for t, p in w.tilts)
    label = torch.empty((X, Y, Z), dtype=torch.int32, device=dev)
    vector = torch.empty((X, Y, Z, 3), dtype=torch.float32, device=dev)
    images = [torch.empty((X, Y, sim.n_rho), dtype=torch.float64, device=dev) for _ in w.tilts]
    wsp = torch.empty(g.workspace_size(), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    _, _, props, _ = g.run_generation_device(label=label, vector=vector, workspace=wsp)
    tissue = int((label > 0).sum().item())
    ev = [_events(3) for _ in range(steps)]

    def step(e=None):
        if e:
            e[0].record(stream)
        g.run_generation_device(label=label, vector=vector, workspace=wsp, sync_warnings=False)
        if e:
            e[1].record(stream)
        sim.run_tilts_device(w.dim, label, vector, props, w.tilts, images=images,
                             sync_warnings=False)
        if e:
            e[2].record(stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    t0, t1 = _events(2)
    t0.record(stream)
    for e in ev:
        step(e)
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    gen_ms = sum(e[0].elapsed_time(e[1]) for e in ev) / steps
    march_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / steps
    for _ in range(3):
        lab_h, vec_h, props_h = g.run_generation()
        imgs = [sim.run_simulation(w.dim, lab_h, vec_h, props_h, float(t), float(p))
                for t, p in w.tilts]
    e2e = []
    for _ in range(5):
        t_e = time.perf_counter()
        lab_h, vec_h, props_h = g.run_generation()
        imgs = [sim.run_simulation(w.dim, lab_h, vec_h, props_h, float(t), float(p))
                for t, p in w.tilts]
        e2e.append(time.perf_counter() - t_e)
    del imgs
    rofl = measure_rofl(w, label, images, stream)
    hbm, _, _ = _peaks()
    return {"workload": "crossing 512x512x120 @ 0.2 um, 2 x 1000 fibers, 5 tilts x 9 angles, "
                        "Slerp",
            "rofl": rofl,
            "steps_per_s": n_steps / (ms * 1e-3), "ms_per_step": ms, "voxelize_ms": gen_ms,
            "march_ms": march_ms, "tissue_voxels_per_s": tissue / (gen_ms * 1e-3),
            "march_frac_hbm": 16 * n_steps / (march_ms * 1e-3) / (hbm * 1e9),
            "e2e_host_api": {"steps_per_s": n_steps / (sum(e2e) / len(e2e)),
                             "ms_per_step": 1e3 * sum(e2e) / len(e2e),
                             "h2d_bytes_per_step": len(w.tilts) * X * Y * Z * 16,
                             "d2h_bytes_per_step": X * Y * Z * 16 +
                             len(w.tilts) * X * Y * sim.n_rho * 8}}


def measure_rofl(w, label, images, stream, reps=3, cpu_pixels=48, side=None):
    """ROFL (Simpli.apply_rofl's fit) of the crossing volume's 5-tilt image
    series, every tissue pixel, on the device (MINPACK, one thread per
    pixel), and the oracle (scipy's MINPACK, as the reference) on a sample
    of the same pixels on one host core (cpu_pixels = 0: no CPU leg).
    ``side``: only the first side x side pixels (a small case for ncu)."""
    import torch
    from fastpli_gb300 import analysis
    data = torch.stack(images)                        # [5, X, Y, n_rho]
    mask = (label > 0).any(dim=2)
    if side:
        data = data[:, :side, :side].contiguous()
        mask = mask[:side, :side].contiguous()
    n_pix = int(mask.sum().item())
    out = {"workload": f"rofl of the crossing images: {n_pix} tissue pixels x 5 tilts x "
                       f"{data.shape[-1]} angles"}
    import warnings
    warnings.simplefilter("ignore")  # pixels at the evaluation limit (grad_mode)
    for grad in (False, True):
        analysis.rofl_device(data, mask=mask, grad_mode=grad)
        torch.cuda.synchronize()
        t0, t1 = _events(2)
        t0.record(stream)
        for _ in range(reps):
            res = analysis.rofl_device(data, mask=mask, grad_mode=grad)
        t1.record(stream)
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / reps
        key = "grad_mode" if grad else "forward_differences"
        out[key] = {"ms": ms, "pixels_per_s": n_pix / (ms * 1e-3)}
    if not cpu_pixels or n_pix == 0:
        return out
    # the CPU baseline leg: the oracle on a bounded sample of the same pixels
    from oracle import rofl as O
    idx = torch.nonzero(mask).cpu().numpy()
    pick = idx[np.linspace(0, len(idx) - 1, cpu_pixels).astype(int)]
    host = data.cpu().numpy()
    t_c = time.perf_counter()
    for x, y in pick:
        O.rofl(host[:, x, y, :])
    dt = time.perf_counter() - t_c
    out["cpu_baseline"] = {"value": cpu_pixels / dt, "unit": "pixels/s", "cores": 1,
                           "kind": "port", "sample": f"{cpu_pixels} of the tissue pixels "
                           "(oracle.rofl: scipy leastsq, forward differences)"}
    return out


def run_rofl(args):
    """``--workload rofl``: ROFL alone on the crossing volume's 5-tilt images
    (the first ``--rofl-side``^2 pixels), as its own line; the small case the
    ncu summary of rofl_fit is taken on."""
    import torch
    import fastpli_gb300
    from fastpli_gb300 import synth
    from fastpli_gb300.simulation import _Generator
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    fastpli_gb300.native_library()
    w = synth.crossing(seed=2)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    sim = _simulator(w)
    label, vector, props, _ = g.run_generation_device(sync_warnings=False)
    images = sim.run_tilts_device(w.dim, label, vector, props, w.tilts, sync_warnings=False)
    stream = torch.cuda.current_stream()
    with ClockSampler(local) as clocks:
        res = measure_rofl(w, label, images, stream, reps=max(1, args.steps),
                           cpu_pixels=0 if args.no_cpu else 48, side=args.rofl_side)
    if rank == 0:
        fd = res["forward_differences"]
        line = {"metric": "ROFL pixels/s (MINPACK fit of 5 tilts x 9 angles per pixel, "
                          "forward differences)", "value": fd["pixels_per_s"],
                "unit": "pixels/s", "n_gpus": ws, "steps": args.steps, "warmup": 1,
                "ms_per_step": fd["ms"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": res["workload"]}, "detail": res,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    return 0


def measure_watson(dev, steps=3):
    """The voxelization-heavy volume: 1024x1024x240 at 0.1 um, 20,000 fibers
    of 50 points (Watson kappa = 5), 3 layers; voxelize + 1 tilt."""
    import torch
    from fastpli_gb300 import synth
    from fastpli_gb300.simulation import _Generator
    w = synth.watson()
    X, Y, Z = (int(v) for v in w.dim)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    sim = _simulator(w)
    label = torch.empty((X, Y, Z), dtype=torch.int32, device=dev)
    vector = torch.empty((X, Y, Z, 3), dtype=torch.float32, device=dev)
    image = torch.empty((X, Y, sim.n_rho), dtype=torch.float64, device=dev)
    wsp = torch.empty(g.workspace_size(), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    _, _, props, _ = g.run_generation_device(label=label, vector=vector, workspace=wsp)
    tissue = int((label > 0).sum().item())
    n_steps = sim.count_steps(w.dim, 0.0, 0.0)
    ev = [_events(3) for _ in range(steps)]
    for e in [None] + ev:
        if e:
            e[0].record(stream)
        g.run_generation_device(label=label, vector=vector, workspace=wsp, sync_warnings=False)
        if e:
            e[1].record(stream)
        sim.run_simulation_device(w.dim, label, vector, props, 0.0, 0.0, image=image,
                                  sync_warnings=False)
        if e:
            e[2].record(stream)
    torch.cuda.synchronize()
    gen_ms = sum(e[0].elapsed_time(e[1]) for e in ev) / steps
    march_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / steps
    del label, vector, image, wsp
    torch.cuda.empty_cache()
    return {"workload": "watson 1024x1024x240 @ 0.1 um, 20000 fibers, 3 layers, 1 tilt",
            "voxelize_ms": gen_ms, "march_ms": march_ms,
            "tissue_voxels_per_s": tissue / (gen_ms * 1e-3), "voxels": X * Y * Z,
            "steps_per_s": n_steps / (march_ms * 1e-3),
            "forward_ms": gen_ms + march_ms}


def serve_sweep(rates, seconds, max_requests, min_requests, local, pool_n=N_TILES, pool=None):
    """Poisson arrivals at each rate; every request a tile of the uneven-tile
    mixture with 1 or 5 tilts (Bernoulli 1/2), Slerp, epa on the device; the
    continuous-batching server against the plain per-call path serving the
    same stream one request at a time."""
    import warnings as _w
    import torch
    from fastpli_gb300 import serving, synth
    torch.cuda.set_device(local)
    pool = [synth.tile(i) for i in range(pool_n)] if pool is None else list(pool)
    pool_n = len(pool)
    kw = pool[0].setup_kwargs()
    rng = np.random.default_rng(5)

    def stream_of(lam, n):
        gaps = rng.exponential(1.0 / lam, n)
        picks = rng.integers(0, len(pool), n)
        five = rng.random(n) < 0.5
        return np.cumsum(gaps), [(pool[i], synth.TILTS_5 if f else synth.TILTS_5[:1])
                                 for i, f in zip(picks, five)]

    # every server instance is warmed before its timed stream
    # (ForwardServer.start(warm=...)): the pool's 4 largest tiles with 5 tilts
    # through each of its paths on each stream slot, so that its worker's
    # cached device buffers have grown (growing one synchronises the device)
    warm = sorted(pool, key=lambda t: -t.n_voxels)[:4]

    def serve(server, arrivals, specs):
        reqs = []
        server.start(warm=warm, warm_tilts=synth.TILTS_5)
        try:
            t0 = time.perf_counter()
            for a, (tile, tilts) in zip(arrivals, specs):
                d = t0 + a - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                reqs.append(server.submit(tile, tilts))
            for r in reqs:
                r.wait(600)
        finally:
            server.stop()
        wall = time.perf_counter() - t0
        st = serving.latency_stats(reqs)
        st["throughput_rps"] = len(reqs) / wall
        st["batches"] = server.batches
        st["mean_batch"] = float(np.mean([r.batch_size for r in reqs]))
        return st

    results = []
    with _w.catch_warnings():
        _w.simplefilter("ignore")
        warm_a, warm_s = stream_of(1000.0, 8)
        serve(serving.ForwardServer(kw, hbm_budget=150e9), warm_a, warm_s)
        serve(serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=1, n_slots=1,
                                    runner=serving.PlainRunner(kw)), warm_a, warm_s)
        for i, lam in enumerate(rates):
            n = int(min(max_requests, max(min_requests, lam * seconds)))
            arrivals, specs = stream_of(lam, n)
            runs = {}
            # the two servers take turns going first (the GPU warms over a run)
            for which in (("batched", "plain") if i % 2 == 0 else ("plain", "batched")):
                srv = (serving.ForwardServer(kw, hbm_budget=150e9) if which == "batched" else
                       serving.ForwardServer(kw, hbm_budget=150e9, max_tiles=1, n_slots=1,
                                             runner=serving.PlainRunner(kw)))
                runs[which] = serve(srv, arrivals, specs)
            batched, plain = runs["batched"], runs["plain"]
            results.append({"rate_rps": lam, "requests": n, "batched": batched,
                            "plain": plain})
    return {"workload": f"Poisson arrivals, requests drawn from the first {pool_n} tiles of the "
                        "uneven-tile mixture, 1 or 5 tilts, Slerp, epa; HBM budget 150 GB",
            "sweep": results}


def run_serve(args):
    """``--workload serve``: the serving sweep alone, as its own JSON line."""
    import torch
    import fastpli_gb300
    ws, rank, local = _dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    fastpli_gb300.native_library()
    with ClockSampler(local) as clocks:
        res = serve_sweep(args.rates, args.seconds, args.max_requests, args.min_requests,
                          local, pool_n=args.pool)
    best = max(r["batched"]["throughput_rps"] for r in res["sweep"])
    line = {"metric": "serving: requests/s and p50/p99 latency under Poisson load "
                      "(uneven tiles, 1 or 5 tilts, Slerp, epa)",
            "value": best, "unit": "requests/s", "n_gpus": 1, "steps": len(res["sweep"]),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": res["workload"], "hbm_budget_gb": 150},
            "sweep": res["sweep"], "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_crossing(args):
    """``--workload crossing``: the 512x512x120 volume alone, as its own line."""
    import torch
    import fastpli_gb300
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    fastpli_gb300.native_library()
    import warnings as _w
    _w.simplefilter("ignore")
    with ClockSampler(local) as clocks:
        res = measure_crossing(torch.device("cuda", local), steps=args.steps,
                               warmup=args.warmup)
    if rank == 0:
        line = {"metric": "ray-voxel steps/s (crossing 512x512x120: voxelize + 5 tilts x 9 "
                          "angles, Slerp)", "value": res["steps_per_s"], "unit": UNIT,
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": res["workload"]}, "detail": res,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="tiles",
                    choices=["tiles", "crossing", "serve", "rofl"])
    ap.add_argument("--rofl-side", type=int, default=0,
                    help="rofl: fit only the first n x n pixels (0: all)")
    ap.add_argument("--rates", type=float, nargs="+", default=[10, 20, 50, 100, 200, 500],
                    help="serving: Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-seconds", type=float, default=3.0,
                    help="tiles line: seconds of arrivals per rate of the short serving sweep "
                         "(0 = skip)")
    ap.add_argument("--seconds", type=float, default=20.0, help="serve: seconds per rate")
    ap.add_argument("--min-requests", type=int, default=40, help="serve: requests per rate, min")
    ap.add_argument("--max-requests", type=int, default=2000, help="serve: requests per rate, max")
    ap.add_argument("--pool", type=int, default=N_TILES, help="serving: distinct tiles")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--tiles", type=int, default=N_TILES,
                    help="tiles of the batch (the first n of the mixture; smaller for profiling)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (fixed launch configuration; for profiling)")
    ap.add_argument("--quick", action="store_true",
                    help="tiles line only (no crossing / watson / serving keys)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "crossing":
        return run_crossing(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "rofl":
        return run_rofl(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
