"""Batched forward model of many uneven tissue tiles (``include/fastpli_gb300_batch.h``).

One ``TileBatch`` voxelizes every tile and marches every (tile, tilt) pair
with one fixed launch sequence: the voxelizer key and write passes over all
tiles, then a persistent march kernel that pulls blocks of rays from a queue
ordered by cost.  The sequence allocates nothing and never synchronises, so it
is captured once into a CUDA graph (``capture()``) and replayed
(``replay()``).  Each tile's labels, vectors and images are bit-identical to
the single-volume ``_Generator`` / ``_Simulator`` results.

The launch configuration (resident CTAs per SM, work items per queue grab) is
chosen by ``fastpli_gb300.autotune``.
"""

import ctypes

import numpy as np

from . import _native as N


class BatchSizes(ctypes.Structure):
    _fields_ = [("n_tiles", ctypes.c_int64), ("n_pairs", ctypes.c_int64),
                ("n_items", ctypes.c_int64), ("n_segments", ctypes.c_int64),
                ("total_voxels", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("arena_bytes", ctypes.c_size_t), ("workspace_bytes", ctypes.c_size_t),
                ("upload_bytes", ctypes.c_size_t)]


_P = ctypes.c_void_p
_SIGS = {
    "fpgb_batch_create": ([ctypes.c_int64, _P, _P, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int,
                           _P], ctypes.c_int),
    "fpgb_batch_info": ([_P, _P], ctypes.c_int),
    "fpgb_batch_layout": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
    "fpgb_batch_props": ([_P, ctypes.c_int64, _P, ctypes.c_int64], ctypes.c_int),
    "fpgb_batch_upload": ([_P, _P, _P, _P], ctypes.c_int),
    "fpgb_batch_run": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P], ctypes.c_int),
    "fpgb_batch_run_stages": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P],
                              ctypes.c_int),
    "fpgb_batch_set_shape": ([_P, ctypes.c_int, _P], ctypes.c_int),
    "fpgb_batch_warnings": ([_P, _P, _P, _P], ctypes.c_int),
    "fpgb_batch_destroy": ([_P], ctypes.c_int),
}


def lib():
    L = N.load()
    if not getattr(L, "_fpgb_batch_bound", False):
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        L._fpgb_batch_bound = True
    return L


def exported_symbols():
    return tuple(_SIGS)


class TileBatch:
    """Plan of a batch of tiles (host side).  ``tiles`` are objects with
    ``dim``, ``origin``, ``voxel_size``, ``bundles``, ``layers``, ``tilts``
    (e.g. ``fastpli_gb300.synth.Workload``); ``setup`` holds the keyword
    arguments of ``_Simulator.set_pli_setup``."""

    def __init__(self, tiles, setup, background_mu=None, epa=False, flat_fibers=None):
        L = lib()
        self.tiles = list(tiles)
        n = len(self.tiles)
        if n == 0:
            raise ValueError("empty batch")
        # flat_fibers: the tiles' fibers already in the C ABI's flat host
        # layout (``flatten(tiles)``), e.g. kept between batches of the same tiles
        self._flats = (list(flat_fibers) if flat_fibers is not None
                       else [N.FlatFibers(t.bundles, t.layers) for t in self.tiles])
        self._vols = (N.Volume * n)(*[N.make_volume(t.dim, t.origin, t.voxel_size)
                                      for t in self.tiles])
        self._fibers = (N.Fibers * n)(*[f.struct for f in self._flats])
        self._setup = N.SetupBlock(setup.get("step_size", 1.0), setup["light_intensity"],
                                   setup["voxel_size"], setup["wavelength"],
                                   setup.get("tissue_refrection", 1.0),
                                   setup.get("interpolate", "Slerp"),
                                   setup.get("untilt_sensor_view", True),
                                   setup.get("flip_z", False), setup["filter_rotations"])
        tilts = [np.asarray(t.tilts, np.float64).reshape(-1, 2) for t in self.tiles]
        self.tilt_off = np.concatenate([[0], np.cumsum([len(t) for t in tilts])]).astype(np.int64)
        self.tilts = np.ascontiguousarray(np.concatenate(tilts), np.float64)
        self._bg = None if background_mu is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(background_mu, np.float64), (n,)))
        h = ctypes.c_void_p()
        N.check(L.fpgb_batch_create(n, ctypes.addressof(self._vols), ctypes.addressof(self._fibers),
                                    N.ptr(self._bg), N.byref(self._setup.struct),
                                    N.ptr(self.tilt_off), N.ptr(self.tilts), int(bool(epa)), 0,
                                    ctypes.byref(h)))
        self._h = h
        self.epa = bool(epa)
        info = BatchSizes()
        N.check(L.fpgb_batch_info(self._h, ctypes.byref(info)))
        self.info = info
        self.label_off = np.zeros(n, np.int64)
        self.vector_off = np.zeros(n, np.int64)
        self.n_props = np.zeros(n, np.int64)
        self.image_off = np.zeros(info.n_pairs, np.int64)
        self.epa_off = np.zeros(info.n_pairs, np.int64)
        N.check(L.fpgb_batch_layout(self._h, N.ptr(self.label_off), N.ptr(self.vector_off),
                                    N.ptr(self.image_off), N.ptr(self.epa_off),
                                    N.ptr(self.n_props)))
        self.pair_tile = np.repeat(np.arange(n), np.diff(self.tilt_off))
        self.n_rho = self._setup.n_rho
        self.arena = None
        self.workspace = None
        self._graph = None
        self.shape = 0
        self.config = (0, 0, 1, 0)

    # ------------------------------------------------------------ sizes ---
    @property
    def steps(self):
        return int(self.info.steps)

    @property
    def device_bytes(self):
        return int(self.info.arena_bytes + self.info.workspace_bytes)

    def props(self, t):
        out = np.zeros((int(self.n_props[t]), 2))
        N.check(lib().fpgb_batch_props(self._h, t, N.ptr(out), out.shape[0]))
        return out

    # ----------------------------------------------------------- device ---
    def allocate(self, device="cuda", arena=None, workspace=None, stream=None):
        """Bind device memory (torch uint8 tensors, allocated unless given) and
        upload the tables."""
        import torch
        self.arena = arena if arena is not None else torch.empty(
            int(self.info.arena_bytes), dtype=torch.uint8, device=device)
        self.workspace = workspace if workspace is not None else torch.empty(
            int(self.info.workspace_bytes), dtype=torch.uint8, device=device)
        N.check(lib().fpgb_batch_upload(self._h, self.arena.data_ptr(),
                                        self.workspace.data_ptr(), _stream(stream)))
        return self

    SHAPES = ("128 consecutive rays", "2 x 64 rays", "4 x 32 rays", "8 x 16 rays",
              "16 x 8 rays")

    def set_shape(self, shape, stream=None):
        """Ray-block shape of the march's work items (``SHAPES``); results do
        not depend on it.  A captured graph is dropped (capture again)."""
        shape = int(shape)
        if shape != self.shape:
            N.check(lib().fpgb_batch_set_shape(self._h, shape, _stream(stream)))
            self.shape = shape
            self._graph = None

    def run(self, ctas_per_sm=None, items_per_grab=None, coop=None, stream=None, stages=3,
            shape=None):
        """Voxelize every tile and march every pair (stages=3), or only the
        voxelizer (1) or only the march (2).  Launch knobs default to
        ``config`` = (ctas_per_sm, items_per_grab, coop, shape)."""
        cfg = list(self.config) + [0, 0, 1, 0][len(self.config):]
        c, g, k, sh = cfg[:4]
        c = c if ctas_per_sm is None else ctas_per_sm
        g = g if items_per_grab is None else items_per_grab
        k = k if coop is None else coop
        self.set_shape(sh if shape is None else shape, stream)
        if stages == 3:
            N.check(lib().fpgb_batch_run(self._h, int(c), int(g), int(k), _stream(stream)))
        else:
            N.check(lib().fpgb_batch_run_stages(self._h, int(stages), int(c), int(g), int(k),
                                                _stream(stream)))

    def capture(self):
        """Capture the batch's launch sequence into a CUDA graph."""
        import torch
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(stream=s)  # warm module loading outside the capture
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self.run()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()

    def warnings(self, stream=None):
        w = N.Warnings()
        replays = np.zeros(1, np.int64)
        N.check(lib().fpgb_batch_warnings(self._h, N.byref(w), N.ptr(replays), _stream(stream)))
        d = w.as_dict()
        d["fp64_replays"] = int(replays[0])
        return d

    # ---------------------------------------------------------- results ---
    def _view(self, off, count, dtype, shape):
        import torch
        nbytes = count * torch.empty((), dtype=dtype).element_size()
        return self.arena[int(off): int(off) + nbytes].view(dtype).view(*shape)

    def label(self, t):
        import torch
        X, Y, Z = (int(v) for v in self.tiles[t].dim)
        return self._view(self.label_off[t], X * Y * Z, torch.int32, (X, Y, Z))

    def vector(self, t):
        import torch
        X, Y, Z = (int(v) for v in self.tiles[t].dim)
        return self._view(self.vector_off[t], 3 * X * Y * Z, torch.float32, (X, Y, Z, 3))

    def image(self, p):
        import torch
        X, Y = (int(v) for v in self.tiles[self.pair_tile[p]].dim[:2])
        return self._view(self.image_off[p], X * Y * self.n_rho, torch.float64,
                          (X, Y, self.n_rho))

    def epa_block(self, p):
        """transmittance, direction, retardation of pair p as one
        [3, X, Y] float64 device view."""
        import torch
        if not self.epa:
            raise ValueError("batch planned without epa")
        X, Y = (int(v) for v in self.tiles[self.pair_tile[p]].dim[:2])
        return self._view(self.epa_off[p], 3 * X * Y, torch.float64, (3, X, Y))

    def epa_maps(self, p):
        e = self.epa_block(p)
        return e[0], e[1], e[2]

    def outputs_host(self, out=None, stream=None):
        """Copies every pair's image (and epa maps) to the host in ONE
        device-to-host copy of the arena's output region (the pairs' buffers
        follow the tiles' volumes in the arena) into ``out`` (a page-locked
        uint8 torch tensor of at least ``output_bytes`` bytes, allocated when
        None), and returns (out, per-pair numpy image views)."""
        import torch
        lo = int(self.image_off[0])
        nbytes = int(self.info.arena_bytes) - lo
        if out is None:
            out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        st = torch.cuda.current_stream() if stream is None else stream
        with torch.cuda.stream(st):
            out[:nbytes].copy_(self.arena[lo: lo + nbytes], non_blocking=True)
        st.synchronize()
        return out, self.host_views(out)

    def host_views(self, out):
        """Per-pair numpy image views into a host copy of the output region."""
        lo = int(self.image_off[0])
        base = out.numpy()
        views = []
        for p in range(int(self.info.n_pairs)):
            X, Y = (int(v) for v in self.tiles[self.pair_tile[p]].dim[:2])
            o = int(self.image_off[p]) - lo
            views.append(base[o: o + 8 * X * Y * self.n_rho].view(np.float64)
                         .reshape(X, Y, self.n_rho))
        return views

    @property
    def output_bytes(self):
        """Bytes of the arena's image (+ epa) region that ``outputs_host`` copies."""
        return int(self.info.arena_bytes) - int(self.image_off[0])

    @property
    def upload_bytes(self):
        """Host-to-device bytes of ``allocate`` (segment, layer, tile and
        march tables)."""
        return int(self.info.upload_bytes)

    def pairs_of(self, t):
        return list(range(int(self.tilt_off[t]), int(self.tilt_off[t + 1])))

    def close(self):
        if getattr(self, "_h", None):
            lib().fpgb_batch_destroy(self._h)
            self._h = None
        self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_tiles_host(tiles, setup, chunks=4, config=None, flat_fibers=None, host_buffers=None):
    """The forward model of many tiles from host fibers to host images,
    pipelined: the tiles are cut into ``chunks`` contiguous groups of about
    equal voxel count; while the GPU voxelizes and marches group c, a host
    thread plans group c + 1 (``fpgb_batch_create`` releases the GIL), and
    group c's images go down on a copy stream while group c + 1 runs.
    Returns (images, stats): one float64 [X, Y, n_rho] numpy array per
    (tile, tilt) pair in tile order, views into page-locked buffers (pass
    the ``host_buffers`` list of an earlier call to reuse them), and the bytes
    moved each way.  ``config`` is the march configuration (``TileBatch.config``,
    e.g. from ``autotune``).  Each image is the one the single-volume path
    gives for that tile and tilt."""
    import concurrent.futures as cf
    import torch
    tiles = list(tiles)
    flats = list(flat_fibers) if flat_fibers is not None else flatten(tiles)
    vox = np.array([float(np.prod(t.dim)) for t in tiles])
    cut = np.searchsorted(np.cumsum(vox), vox.sum() * np.arange(1, chunks) / chunks)
    bounds = [0] + sorted(set(int(c) + 1 for c in cut if 0 <= c < len(tiles) - 1)) + [len(tiles)]
    groups = [list(range(a, b)) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]
    comp = torch.cuda.current_stream()
    up = torch.cuda.Stream()
    down = torch.cuda.Stream()
    host = list(host_buffers) if host_buffers is not None else []
    batches, images, h2d, d2h = [], [], 0, 0

    def plan(g):
        b = TileBatch([tiles[i] for i in g], setup, flat_fibers=[flats[i] for i in g])
        if config is not None:
            b.config = tuple(config)
            if len(b.config) > 3:
                b.set_shape(b.config[3])  # before the upload: no extra copy
        return b

    with cf.ThreadPoolExecutor(1) as ex:
        fut = ex.submit(plan, groups[0])
        for ci in range(len(groups)):
            b = fut.result()
            if ci + 1 < len(groups):
                fut = ex.submit(plan, groups[ci + 1])
            b.allocate(stream=up)  # synchronises `up` only
            comp.wait_stream(up)
            b.run(stream=comp)
            done = torch.cuda.Event()
            done.record(comp)
            down.wait_event(done)
            n = b.output_bytes
            if ci >= len(host) or host[ci].numel() < n:
                buf = torch.empty(n, dtype=torch.uint8, pin_memory=True)
                host[ci:ci + 1] = [buf]
            lo = int(b.image_off[0])
            with torch.cuda.stream(down):
                host[ci][:n].copy_(b.arena[lo: lo + n], non_blocking=True)
                b.arena.record_stream(down)
            batches.append(b)
            h2d += b.upload_bytes
            d2h += n
    down.synchronize()
    for ci, b in enumerate(batches):
        images.extend(b.host_views(host[ci]))
        b.close()
    return images, {"h2d_bytes": h2d, "d2h_bytes": d2h, "groups": len(groups),
                    "host_buffers": host}


def flatten(tiles):
    """The tiles' fibers in the C ABI's flat host layout (for ``flat_fibers``)."""
    return [N.FlatFibers(t.bundles, t.layers) for t in tiles]


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
