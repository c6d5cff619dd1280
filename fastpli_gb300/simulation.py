"""Drop-in host classes for fastpli's compiled simulation modules.

``_Generator`` mirrors ``fastpli.simulation.__generation._Generator``
(src/simulation/bindings/generator_module.cpp:23-140) and ``_Simulator``
mirrors ``fastpli.simulation.__simulation._Simulator``
(src/simulation/bindings/simulator_module.cpp:18-157): same method names,
argument order, dtypes and return shapes.  Both run on the GPU through the C
ABI of ``libfastpli_gb300.so``; there is no CPU path.

Differences, all deliberate:
  * input inconsistencies the reference answers with ``exit(EXIT_FAILURE)``
    (simulator.cpp:131-176) raise ``ValueError`` instead;
  * ``set_mpi_comm`` / ``set_cell_populations`` raise ``NotImplementedError``
    (one GPU per process; cell populations are not reachable from Simpli);
  * ``set_omp_num_threads`` is accepted and returns 1 (no CPU threads);
  * the GIL is released around device work (ctypes releases it), warnings
    are raised after the call from device counters.

``*_device`` methods keep everything in device memory (torch CUDA tensors)
and take an optional CUDA stream.
"""

import ctypes
import warnings

import numpy as np

from . import _native as N

_GEN_WARN = {
    "overlap": "objects overlap",
    "single_point": "fiber object with only single point",
    "layer_overflow": "voxel beyond the outermost layer (reference reads past "
                      "its layer table here)",
}
_SIM_WARN = {
    "zero_axis": "optical_axis is 0 for tissue > 0",
    "not_normalized": "optical_axis not normalized",
}


def _emit(w, table):
    for key, msg in table.items():
        if w.get(key, 0):
            warnings.warn(msg, UserWarning)


def _torch():
    import torch
    return torch


_TORCH_DTYPES = {np.dtype(np.int32): "int32", np.dtype(np.float32): "float32",
                 np.dtype(np.float64): "float64"}


_PINNED_MIN_BYTES = 8 << 20


def _host_empty(shape, dtype):
    """An uninitialised numpy array for an output of the host-buffer calls.
    From 8 MiB up it lives in page-locked host memory: the device->host copy
    into it runs at the link's rate with no page faulting, and an array passed
    back in (the label / vector fields to run_simulation) is copied up at the
    same rate.  That memory comes from torch's caching host allocator, so
    arrays that are dropped return their blocks for the next call.  Either
    way the result is an ordinary numpy array (its base keeps the block
    alive)."""
    shape = tuple(int(v) for v in shape)
    dt = np.dtype(dtype)
    if int(np.prod(shape)) * dt.itemsize < _PINNED_MIN_BYTES:
        return np.empty(shape, dt)
    try:
        torch = _torch()
    except ImportError:  # no torch: ordinary pageable memory (one-copy path)
        return np.empty(shape, dt)
    t = torch.empty(shape, dtype=getattr(torch, _TORCH_DTYPES[dt]), pin_memory=True)
    return t.numpy()


def _stream_handle(stream):
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class _Generator:
    """GPU voxelizer with the interface of the reference's ``_Generator``."""

    def __init__(self):
        self._vol = None
        self._flat = None
        self._dim = None

    def set_omp_num_threads(self, i):
        return 1

    def set_mpi_comm(self, comm_address, n):
        raise NotImplementedError("MPI domain decomposition is not supported: "
                                  "one GPU per process")

    def set_cell_populations(self, cell_pops, cell_prop):
        raise NotImplementedError("cell populations are not supported")

    def set_volume(self, global_dim, origin, voxel_size):
        """generator.cpp:45-124 (single rank: local == global, offset 0)."""
        d = np.asarray(global_dim)
        if d.size != 3:
            raise TypeError("global_dim must have 3 entries")
        d = d.astype(np.int64)
        if np.any(d <= 0):
            raise ValueError(f"dim.global[any] <= 0: [{d[0]},{d[1]},{d[2]}]")
        if not voxel_size > 0:
            raise ValueError(f"voxel_size <= 0: {voxel_size}")
        self._dim = d
        self._vol = N.make_volume(d, origin, voxel_size)

    def set_fiber_bundles(self, fbs, prs):
        """generator_module.cpp:37-66: list of bundles of (n,4) float arrays
        and per-bundle lists of (scale, dn, mu, model) tuples."""
        self._flat = N.FlatFibers(fbs, prs)

    def dim_local(self):
        return list(map(int, self._dim))

    def dim_offset(self):
        return [0, 0, 0]

    def _check(self):
        if self._vol is None:
            raise ValueError("volume not set")
        if self._flat is None:
            raise ValueError("fiber_bundles not set")

    def n_props(self):
        self._check()
        return self._flat.n_props

    def run_generation(self, only_label=False):
        """-> (label int32 [X,Y,Z], vector float32 [X,Y,Z,3] or shape (0,),
        properties float64 [n,2])."""
        self._check()
        lib = N.load()
        X, Y, Z = (int(v) for v in self._dim)
        label = _host_empty((X, Y, Z), np.int32)
        vector = (np.zeros((0,), np.float32) if only_label
                  else _host_empty((X, Y, Z, 3), np.float32))
        cap = self._flat.n_props
        props = np.zeros((cap, 2), np.float64)
        n_props = np.zeros(1, np.int64)
        w = N.Warnings()
        N.check(lib.fpgb_generate_tissue(
            N.byref(self._vol), N.byref(self._flat.struct), int(bool(only_label)),
            N.ptr(label), None if only_label else N.ptr(vector), N.ptr(props),
            cap, N.ptr(n_props), N.byref(w)))
        _emit(w.as_dict(), _GEN_WARN)
        return label, vector, props[: int(n_props[0])]

    def run_generation_device(self, only_label=False, stream=None, label=None,
                              vector=None, workspace=None, sync_warnings=True):
        """Voxelize into device memory.  Returns (label, vector, props,
        warnings) with label/vector torch CUDA tensors (allocated unless
        given) and props a float64 numpy array.  With ``sync_warnings=False``
        the call does not synchronise and warnings are not collected."""
        self._check()
        torch = _torch()
        lib = N.load()
        X, Y, Z = (int(v) for v in self._dim)
        dev = torch.device("cuda", torch.cuda.current_device())
        if label is None:
            label = torch.empty((X, Y, Z), dtype=torch.int32, device=dev)
        if vector is None and not only_label:
            vector = torch.empty((X, Y, Z, 3), dtype=torch.float32, device=dev)
        cap = self._flat.n_props
        props = np.zeros((cap, 2), np.float64)
        n_props = np.zeros(1, np.int64)
        w = N.Warnings()
        ws_ptr, ws_bytes = None, 0
        if workspace is not None:
            ws_ptr, ws_bytes = workspace.data_ptr(), workspace.numel() * workspace.element_size()
        N.check(lib.fpgb_generate_tissue_device(
            N.byref(self._vol), N.byref(self._flat.struct), int(bool(only_label)),
            N.ptr(label), None if only_label else N.ptr(vector), N.ptr(props), cap,
            N.ptr(n_props), ws_ptr, ws_bytes, N.byref(w) if sync_warnings else None,
            _stream_handle(stream)))
        if sync_warnings:
            _emit(w.as_dict(), _GEN_WARN)
        return label, vector, props[: int(n_props[0])], w.as_dict()

    def workspace_size(self):
        self._check()
        return int(N.load().fpgb_generate_workspace_size(
            N.byref(self._vol), N.byref(self._flat.struct)))


class _Simulator:
    """GPU ray march with the interface of the reference's ``_Simulator``."""

    def __init__(self):
        self._setup = None

    def set_omp_num_threads(self, i):
        return 1

    def set_mpi_comm(self, comm_address, n):
        raise NotImplementedError("MPI domain decomposition is not supported: "
                                  "one GPU per process")

    def set_pli_setup(self, step_size, light_intensity, voxel_size, wavelength,
                      tissue_refrection, interpolate, untilt_sensor_view, flip_z,
                      filter_rotations):
        """simulator_module.cpp:23-54."""
        self._setup = N.SetupBlock(step_size, light_intensity, voxel_size,
                                   wavelength, tissue_refrection, interpolate,
                                   untilt_sensor_view, flip_z, filter_rotations)

    @property
    def n_rho(self):
        return self._setup.n_rho

    def _need_setup(self):
        if self._setup is None:
            raise ValueError("pli_setup not set yet")

    @staticmethod
    def _dim(dim, shape):
        d = np.asarray(dim, np.int64).reshape(-1)
        if d.size != 3:
            raise TypeError("dim must have 3 entries")
        return np.ascontiguousarray(d)

    def run_simulation(self, dim, label_field, vector_field, properties,
                       theta=0.0, phi=0.0):
        """-> image float64 [X, Y, n_rho]."""
        self._need_setup()
        lib = N.load()
        d = self._dim(dim, None)
        label = np.ascontiguousarray(label_field, dtype=np.int32)
        vector = np.ascontiguousarray(vector_field, dtype=np.float32)
        props = np.ascontiguousarray(properties, dtype=np.float64)
        n = int(np.prod(d))
        if label.size == 0:
            raise ValueError("label_field.size() == 0")
        if label.size * 3 != vector.size:
            raise ValueError("label_field_.size()*3 != vector_field_.size()")
        if label.size != n:
            raise ValueError("dim_.local.x() * dim_.local.y() * dim_.local.z() "
                             "!= label_field_.size()")
        if props.size % 2 != 0:
            raise ValueError("properties must be (n, 2)")
        self.count_steps(d, theta, phi)  # setup / tilt errors before any allocation
        image = _host_empty((int(d[0]), int(d[1]), self.n_rho), np.float64)
        w = N.Warnings()
        N.check(lib.fpgb_run_simulation(
            N.byref(self._setup.struct), N.ptr(d), N.ptr(label), N.ptr(vector),
            N.ptr(props), props.size // 2, float(theta), float(phi), N.ptr(image),
            N.byref(w)))
        _emit(w.as_dict(), _SIM_WARN)
        return image

    def run_simulation_device(self, dim, label_field, vector_field, properties,
                              theta=0.0, phi=0.0, image=None, epa=False,
                              stream=None, sync_warnings=True):
        """Device-resident march on torch CUDA tensors.  Returns the image
        tensor (float64 [X,Y,n_rho]) or (image, t, d, r) when ``epa``."""
        self._need_setup()
        torch = _torch()
        lib = N.load()
        d = self._dim(dim, None)
        props = np.ascontiguousarray(properties, dtype=np.float64)
        for t, dt in ((label_field, torch.int32), (vector_field, torch.float32)):
            if not t.is_cuda or t.dtype != dt or not t.is_contiguous():
                raise ValueError("label/vector must be contiguous CUDA tensors "
                                 "of int32/float32")
        n = int(np.prod(d))
        if label_field.numel() != n or vector_field.numel() != 3 * n:
            raise ValueError("label/vector sizes do not match dim")
        X, Y = int(d[0]), int(d[1])
        if image is None:
            image = torch.empty((X, Y, self.n_rho), dtype=torch.float64,
                                device=label_field.device)
        w = N.Warnings()
        wp = N.byref(w) if sync_warnings else None
        if epa:
            t = torch.empty((X, Y), dtype=torch.float64, device=label_field.device)
            dd = torch.empty_like(t)
            r = torch.empty_like(t)
            N.check(lib.fpgb_run_simulation_epa_device(
                N.byref(self._setup.struct), N.ptr(d), N.ptr(label_field),
                N.ptr(vector_field), N.ptr(props), props.size // 2, float(theta),
                float(phi), N.ptr(image), N.ptr(t), N.ptr(dd), N.ptr(r), wp,
                _stream_handle(stream)))
        else:
            N.check(lib.fpgb_run_simulation_device(
                N.byref(self._setup.struct), N.ptr(d), N.ptr(label_field),
                N.ptr(vector_field), N.ptr(props), props.size // 2, float(theta),
                float(phi), N.ptr(image), wp, _stream_handle(stream)))
        if sync_warnings:
            _emit(w.as_dict(), _SIM_WARN)
        if epa:
            return image, t, dd, r
        return image

    def run_tilts_device(self, dim, label_field, vector_field, properties, tilts,
                         images=None, epa=False, stream=None, sync_warnings=True):
        """Every (theta, phi) of ``tilts`` on one device-resident volume, the
        marches spread over the library's own streams (joined back to
        ``stream``) so that one tilt's last rays share the GPU with the next
        tilt's first.  Each result is the one run_simulation_device gives for
        that tilt.  Returns a list with one image tensor per tilt, or
        (image, t, d, r) per tilt when ``epa``; ``images`` may hold the
        output tensors."""
        self._need_setup()
        torch = _torch()
        lib = N.load()
        d = self._dim(dim, None)
        props = np.ascontiguousarray(properties, dtype=np.float64)
        for t, dt in ((label_field, torch.int32), (vector_field, torch.float32)):
            if not t.is_cuda or t.dtype != dt or not t.is_contiguous():
                raise ValueError("label/vector must be contiguous CUDA tensors "
                                 "of int32/float32")
        n = int(np.prod(d))
        if label_field.numel() != n or vector_field.numel() != 3 * n:
            raise ValueError("label/vector sizes do not match dim")
        tl = np.ascontiguousarray(np.asarray(tilts, np.float64).reshape(-1, 2))
        k = tl.shape[0]
        X, Y = int(d[0]), int(d[1])
        dev = label_field.device
        if images is None:
            images = [torch.empty((X, Y, self.n_rho), dtype=torch.float64, device=dev)
                      for _ in range(k)]
        if len(images) != k or any(not im.is_cuda or im.dtype != torch.float64 or
                                   not im.is_contiguous() or im.numel() != X * Y * self.n_rho
                                   for im in images):
            raise ValueError("images must be one contiguous float64 CUDA tensor "
                             "[X, Y, n_rho] per tilt")
        def ptrs(ts):  # a C array of device pointers
            return (ctypes.c_void_p * k)(*[t.data_ptr() for t in ts])

        epa_out = [None, None, None]
        if epa:
            epa_out = [[torch.empty((X, Y), dtype=torch.float64, device=dev) for _ in range(k)]
                       for _ in range(3)]
        epa_ptrs = [ptrs(e) if epa else None for e in epa_out]
        theta = np.ascontiguousarray(tl[:, 0])
        phi = np.ascontiguousarray(tl[:, 1])
        w = (N.Warnings * max(k, 1))()
        N.check(lib.fpgb_run_simulations_device(
            N.byref(self._setup.struct), N.ptr(d), N.ptr(label_field), N.ptr(vector_field),
            N.ptr(props), props.size // 2, k, N.ptr(theta), N.ptr(phi), ptrs(images),
            *epa_ptrs, w if sync_warnings else None, _stream_handle(stream)))
        if sync_warnings:
            for i in range(k):
                _emit(w[i].as_dict(), _SIM_WARN)
        if epa:
            return [(images[i], epa_out[0][i], epa_out[1][i], epa_out[2][i]) for i in range(k)]
        return list(images)

    def count_steps(self, dim, theta=0.0, phi=0.0):
        """Ray-voxel steps one call marches (X*Y rays x steps per ray)."""
        self._need_setup()
        d = self._dim(dim, None)
        n = N.load().fpgb_count_steps(N.byref(self._setup.struct), N.ptr(d),
                                      float(theta), float(phi))
        if n < 0:
            N.check(N.FPGB_EINVAL)
        return int(n)
