"""Continuous-batching server for forward-model requests.

A request is one tissue tile (fibers, layers, volume) plus a tilt set; its
result is the epa modalities (transmittance, direction, retardation) of every
tilt, computed from the images while the tissue stays in HBM across tilts and
analysis.  The server thread

  * admits pending requests in arrival order while their device bytes fit the
    HBM budget (bytes of every batch in flight are counted until it retires);
  * groups admitted requests into one ``TileBatch`` (batched voxelizer + one
    persistent march over all (tile, tilt) pairs) and launches it on a free
    stream slot, so new batches start while earlier ones still run (the GPU
    overlaps them).  While fewer than ``min_batch`` requests wait, they go one
    at a time through the single-volume kernels instead (no batch planning
    and upload: lower latency at light and moderate load; two lone requests
    still overlap on two slots); both paths give the same bits;
  * retires finished batches (CUDA event), copies each request's epa maps to
    the host and completes it.

Every tile is computed with the arithmetic of the single-volume path, so a
request's result does not depend on what it was batched with (tested).
Host-side failures (a planning error, an allocation refusal, an exception in
a batch) complete the affected requests with the error and the server keeps
serving.  There is no device-side wait anywhere: the GPU only runs the
batch's fixed launch sequence.
"""

import collections
import threading
import time
import types

import numpy as np

_BYTES_PER_VOXEL = 4 + 12  # label, vector (the voxelizer keeps its keys on chip)


def estimate_bytes(tile, tilts, n_rho, epa=True):
    """Device bytes of one request (arena + workspace), from its shape."""
    X, Y, Z = (int(v) for v in tile.dim)
    n_seg = sum(max(0, len(f) - 1) for b in tile.bundles for f in b)
    per_pair = X * Y * 8 * (n_rho + (3 if epa else 0)) + 1472 + 64 * 1024
    return X * Y * Z * _BYTES_PER_VOXEL + n_seg * 400 + len(tilts) * per_pair + (1 << 20)


class Request:
    __slots__ = ("rid", "tile", "tilts", "arrival", "nbytes", "done", "result", "error",
                 "t_start", "t_done", "batch_size")

    def __init__(self, rid, tile, tilts, nbytes):
        self.rid = rid
        self.tile = tile
        self.tilts = np.asarray(tilts, np.float64).reshape(-1, 2)
        self.arrival = time.perf_counter()
        self.nbytes = nbytes
        self.done = threading.Event()
        self.result = None
        self.error = None
        self.t_start = None
        self.t_done = None
        self.batch_size = 0

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival

    def wait(self, timeout=None):
        if not self.done.wait(timeout):
            raise TimeoutError(f"request {self.rid} not done after {timeout} s")
        if self.error is not None:
            raise self.error
        return self.result


def form_batch(pending, budget_free, max_tiles):
    """Requests to launch now: the longest arrival-order prefix of ``pending``
    whose bytes fit ``budget_free`` (at most ``max_tiles``)."""
    out, used = [], 0
    for r in pending:
        if len(out) >= max_tiles or used + r.nbytes > budget_free:
            break
        out.append(r)
        used += r.nbytes
    return out


class GpuRunner:
    """Launches a batch of requests on a stream (TileBatch) and collects the
    results once its event has completed."""

    def __init__(self, setup, epa=True, keep_images=False, tune=True):
        self.setup = dict(setup)
        self.epa = epa
        self.keep_images = keep_images
        self.tune = tune
        self.n_rho = len(np.asarray(setup["filter_rotations"]).reshape(-1))

    def launch(self, reqs, stream):
        import torch
        from .batch import TileBatch
        tiles = [types.SimpleNamespace(dim=r.tile.dim, origin=r.tile.origin,
                                       voxel_size=r.tile.voxel_size, bundles=r.tile.bundles,
                                       layers=r.tile.layers, tilts=r.tilts) for r in reqs]
        b = TileBatch(tiles, self.setup, epa=True)
        if self.tune:
            from . import autotune
            cache = autotune._load()
            k = autotune.key(b)
            if k in cache:
                b.config = tuple(cache[k]["config"])
                if len(b.config) > 3:
                    b.set_shape(b.config[3])  # before the upload: no extra copy
        with torch.cuda.stream(stream):
            b.allocate(stream=stream)
            b.run(stream=stream)
            ev = torch.cuda.Event()
            ev.record(stream)
        return b, ev

    def collect(self, b, reqs, stream):
        import torch
        with torch.cuda.stream(stream):
            b.warnings(stream=stream)  # raises on a label range error
            # every pair's epa maps gathered on the device, then one copy down
            blocks = [b.epa_block(p) for p in range(int(b.info.n_pairs))]
            host = torch.cat([e.reshape(-1) for e in blocks]).cpu().numpy()
            at = 0
            for t, r in enumerate(reqs):
                maps = []
                for p in b.pairs_of(t):
                    n = blocks[p].numel()
                    e = host[at: at + n].reshape(blocks[p].shape)
                    at += n
                    maps.append((e[0], e[1], e[2]))
                images = [b.image(p).clone() for p in b.pairs_of(t)] if self.keep_images else None
                r.result = {"epa": maps, "images": images}
        b.close()


class ForwardServer:
    """Continuous batching over ``n_slots`` CUDA streams under an HBM budget."""

    def __init__(self, setup, hbm_budget=150e9, max_tiles=32, n_slots=2, runner=None,
                 streams=None, single_runner=None, min_batch=4):
        self.budget = float(hbm_budget)
        self.max_tiles = int(max_tiles)
        # fewer requests than this waiting: launch them one by one on the
        # single-request path (no batch planning and upload); a TileBatch pays
        # off once the queue is this long (measured: a batch of 2-3 took
        # 6.4 ms against 2.6 ms per lone request at 200 requests/s)
        self.min_batch = int(min_batch)
        self.runner = runner if runner is not None else GpuRunner(setup)
        # batches of one request: the single-volume kernels, the request's
        # tilts overlapped on the library's streams (same results)
        self.single = single_runner if single_runner is not None else (
            PlainRunner(setup, overlap_tilts=True) if runner is None else None)
        self.n_rho = self.runner.n_rho
        self._streams = streams
        self.n_slots = int(n_slots)
        self._pending = collections.deque()
        self._inflight = []  # (runner, handle, reqs, event, stream, nbytes)
        self._in_bytes = 0
        self._lock = threading.Condition()
        self._run = False
        self._thread = None
        self._next_id = 0
        self._warm = ([], None)
        self._warm_error = None
        self._warm_done = threading.Event()
        self.completed = []
        self.batches = 0

    # --------------------------------------------------------- client API ---
    def submit(self, tile, tilts):
        with self._lock:
            rid = self._next_id
            self._next_id += 1
        r = Request(rid, tile, tilts, estimate_bytes(tile, np.asarray(tilts).reshape(-1, 2),
                                                      self.n_rho))
        if r.nbytes > self.budget:
            r.error = MemoryError(f"request {rid} needs {r.nbytes} bytes, more than the "
                                  f"HBM budget {self.budget:.0f}")
            r.t_done = time.perf_counter()
            r.done.set()
            return r
        with self._lock:
            self._pending.append(r)
            self._lock.notify()
        return r

    def start(self, warm=None, warm_tilts=None):
        """Starts the worker.  ``warm``: tiles (the largest requests expected)
        that the worker runs once through every path on every stream slot
        before it serves: the device buffers a slot caches between requests
        then have grown, since growing one synchronises the device and under
        load would stall the other slot's work.  Returns when the warm-up is
        done."""
        if self._streams is None:
            import torch
            self._streams = [torch.cuda.Stream() for _ in range(self.n_slots)]
        self._run = True
        self._warm = (list(warm or []), warm_tilts)
        self._warm_done = threading.Event()
        self._thread = threading.Thread(target=self._loop, name="fpgb-server", daemon=True)
        self._thread.start()
        self._warm_done.wait()
        if self._warm_error is not None:
            self.stop()
            raise self._warm_error
        return self

    def stop(self, timeout=60.0):
        with self._lock:
            self._run = False
            self._lock.notify()
        if self._thread:
            self._thread.join(timeout)
            if self._thread.is_alive():
                raise TimeoutError("server thread did not stop")

    def __enter__(self):
        return self.start()

    def __exit__(self, *a):
        self.stop()

    # ------------------------------------------------------------ worker ---
    def _free_stream(self):
        busy = {id(s) for _, _, _, _, s, _ in self._inflight}
        for s in self._streams:
            if id(s) not in busy:
                return s
        return None

    def _finish(self, reqs, error=None):
        t = time.perf_counter()
        for r in reqs:
            if error is not None:
                r.error = error
            r.t_done = t
            r.done.set()
        self.completed.extend(reqs)

    def _retire(self):
        still = []
        for run, h, reqs, ev, s, nb in self._inflight:
            if ev.query():
                try:
                    run.collect(h, reqs, s)
                    self._finish(reqs)
                except Exception as e:  # noqa: BLE001 - reported per request
                    self._finish(reqs, e)
                self._in_bytes -= nb
            else:
                still.append((run, h, reqs, ev, s, nb))
        self._inflight = still

    def _warm_up(self):
        tiles, tilts = self._warm
        if not tiles:
            return
        tilts = np.asarray(tilts if tilts is not None else [(0.0, 0.0)], np.float64)

        def run(runner, group, s):
            reqs = [Request(-1, t, tilts, 0) for t in group]
            h, ev = runner.launch(reqs, s)
            ev.synchronize()
            runner.collect(h, reqs, s)

        for s in self._streams:
            if self.single is not None:
                for t in tiles:
                    run(self.single, [t], s)
            if self.max_tiles > 1:
                run(self.runner, tiles[:self.max_tiles], s)
            else:
                for t in tiles:
                    run(self.runner, [t], s)

    def _loop(self):
        self._warm_error = None
        try:
            self._warm_up()
        except Exception as e:  # noqa: BLE001 - raised by start()
            self._warm_error = e
        finally:
            self._warm_done.set()
        try:
            if self._warm_error is None:
                self._serve()
        finally:
            if self._streams and not isinstance(self._streams[0], str):
                # the library's cached buffers of this worker thread
                from . import _native
                _native.load().fpgb_release_thread_pool()

    def _serve(self):
        while True:
            with self._lock:
                if not self._run and not self._pending and not self._inflight:
                    return
                if not self._pending and not self._inflight:
                    self._lock.wait(0.05)
                    continue
            self._retire()
            s = self._free_stream()
            reqs = []
            if s is not None:
                with self._lock:
                    cap = self.max_tiles
                    if self.single is not None and len(self._pending) < self.min_batch:
                        cap = 1
                    reqs = form_batch(self._pending, self.budget - self._in_bytes, cap)
                    for _ in reqs:
                        self._pending.popleft()
            if reqs:
                nb = sum(r.nbytes for r in reqs)
                t0 = time.perf_counter()
                for r in reqs:
                    r.t_start = t0
                    r.batch_size = len(reqs)
                run = self.single if (len(reqs) == 1 and self.single is not None) else self.runner
                try:
                    h, ev = run.launch(reqs, s)
                except Exception as e:  # noqa: BLE001 - reported per request
                    self._finish(reqs, e)
                    continue
                self._inflight.append((run, h, reqs, ev, s, nb))
                self._in_bytes += nb
                self.batches += 1
            elif self._inflight:
                time.sleep(0.0002)


def latency_stats(reqs):
    """p50 / p99 / mean arrival-to-result latency of the completed requests,
    and its two parts: waiting for admission (arrival to launch) and service
    (launch to result on the host)."""
    ok = [r for r in reqs if r.latency is not None and r.error is None]
    lat = np.array([r.latency for r in ok])
    if lat.size == 0:
        return {"n": 0}
    wait = np.array([r.t_start - r.arrival for r in ok if r.t_start is not None])
    serv = np.array([r.t_done - r.t_start for r in ok if r.t_start is not None])
    out = {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
           "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3)}
    if wait.size:
        out.update(wait_p50_ms=float(np.percentile(wait, 50) * 1e3),
                   service_p50_ms=float(np.percentile(serv, 50) * 1e3))
    return out


class PlainRunner:
    """The plain per-call path as a runner (one request at a time): voxelize
    with ``_Generator.run_generation_device``, then one
    ``_Simulator.run_simulation_device(epa=True)`` per tilt, each tilt's
    maps copied to the host on their own.  Used as the baseline the batched
    server is compared with.  With ``overlap_tilts`` (the batched server's
    path for a lone request) the tilts run through ``run_tilts_device`` on
    the library's streams and all maps come back in one copy; the results
    are the same bits."""

    def __init__(self, setup, overlap_tilts=False):
        from .simulation import _Simulator
        self.overlap_tilts = bool(overlap_tilts)
        self.setup = dict(setup)
        self.n_rho = len(np.asarray(setup["filter_rotations"]).reshape(-1))
        self.sim = _Simulator()
        kw = self.setup
        self.sim.set_pli_setup(kw.get("step_size", 1.0), kw["light_intensity"],
                               kw["voxel_size"], kw["wavelength"],
                               kw.get("tissue_refrection", 1.0), kw.get("interpolate", "Slerp"),
                               kw.get("untilt_sensor_view", True), kw.get("flip_z", False),
                               kw["filter_rotations"])

    def launch(self, reqs, stream):
        import torch
        from .simulation import _Generator
        out = []
        with torch.cuda.stream(stream):
            for r in reqs:
                g = _Generator()
                g.set_volume(r.tile.dim, r.tile.origin, r.tile.voxel_size)
                g.set_fiber_bundles(r.tile.bundles, r.tile.layers)
                lab, vec, props, _ = g.run_generation_device(stream=stream, sync_warnings=False)
                if self.overlap_tilts:
                    res = self.sim.run_tilts_device(r.tile.dim, lab, vec, props, r.tilts,
                                                    epa=True, stream=stream, sync_warnings=False)
                    out.append(torch.stack([torch.stack(x[1:]) for x in res]))  # [k, 3, X, Y]
                    continue
                maps = [self.sim.run_simulation_device(r.tile.dim, lab, vec, props, float(t),
                                                       float(p), epa=True, stream=stream,
                                                       sync_warnings=False)[1:]
                        for t, p in r.tilts]
                out.append(maps)
            ev = torch.cuda.Event()
            ev.record(stream)
        return out, ev

    def collect(self, h, reqs, stream):
        import torch
        # the copies go on the request's own stream, whose work is complete:
        # on the legacy default stream they would wait for whatever the
        # library's blocking streams run for other requests
        with torch.cuda.stream(stream):
            for maps, r in zip(h, reqs):
                if isinstance(maps, list):
                    epa = [tuple(m.cpu().numpy() for m in tdr) for tdr in maps]
                else:  # one block of every tilt's maps: one copy
                    a = maps.cpu().numpy()
                    epa = [(a[i, 0], a[i, 1], a[i, 2]) for i in range(a.shape[0])]
                r.result = {"epa": epa, "images": None}
