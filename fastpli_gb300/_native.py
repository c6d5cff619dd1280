"""ctypes binding of the C ABI in ``include/fastpli_gb300.h``.

The shared library is built in-tree (``fastpli_gb300/build.py``).  There is
no CPU fallback: if the library is missing or fails to load, every call
raises.  Error codes become Python exceptions with the library's message:
FPGB_EINVAL -> ValueError (the reference raises ValueError for argument
errors and exits the process for inconsistent input; both are ValueError
here), FPGB_ENOMEM -> MemoryError, anything else -> RuntimeError.
"""

import ctypes
import os
import threading

import numpy as np

from . import build as _build

FPGB_OK = 0
FPGB_EINVAL = -1
FPGB_ECUDA = -2
FPGB_ENOMEM = -3
FPGB_ETIMEOUT = -4

INTERP = {"NN": 0, "Lerp": 1, "Slerp": 2}
WARNING_FIELDS = ("overlap", "single_point", "zero_axis", "not_normalized",
                  "empty_light", "layer_overflow")


class Warnings(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in WARNING_FIELDS]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n in WARNING_FIELDS}


class Volume(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int64 * 3), ("origin", ctypes.c_double * 3),
                ("voxel_size", ctypes.c_double)]


class Fibers(ctypes.Structure):
    _fields_ = [("n_bundles", ctypes.c_int64),
                ("bundle_fiber_off", ctypes.c_void_p),
                ("fiber_point_off", ctypes.c_void_p),
                ("points", ctypes.c_void_p),
                ("bundle_layer_off", ctypes.c_void_p),
                ("layer_scale", ctypes.c_void_p),
                ("layer_dn", ctypes.c_void_p),
                ("layer_mu", ctypes.c_void_p),
                ("layer_model", ctypes.c_void_p)]


class Setup(ctypes.Structure):
    _fields_ = [("step_size", ctypes.c_double),
                ("light_intensity", ctypes.c_double),
                ("voxel_size", ctypes.c_double),
                ("wavelength", ctypes.c_double),
                ("tissue_refrection", ctypes.c_double),
                ("interpolate", ctypes.c_int32),
                ("untilt_sensor_view", ctypes.c_int32),
                ("flip_z", ctypes.c_int32),
                ("n_rho", ctypes.c_int32),
                ("filter_rotations", ctypes.c_void_p)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_SIGS = {
    "fpgb_last_error": ([], ctypes.c_char_p),
    "fpgb_version": ([], ctypes.c_char_p),
    "fpgb_release_pool": ([], ctypes.c_int),
    "fpgb_release_thread_pool": ([], ctypes.c_int),
    "fpgb_generate_tissue": ([_P, _P, ctypes.c_int, _P, _P, _P, _I64, _P, _P],
                             ctypes.c_int),
    "fpgb_generate_workspace_size": ([_P, _P], ctypes.c_size_t),
    "fpgb_generate_tissue_device": ([_P, _P, ctypes.c_int, _P, _P, _P, _I64, _P,
                                     _P, ctypes.c_size_t, _P, _P], ctypes.c_int),
    "fpgb_generate_tissue_noalloc": ([_P, _P, ctypes.c_int, _P, _P, _P, _I64, _P, _P, _P],
                                     ctypes.c_int),
    "fpgb_run_simulation": ([_P, _P, _P, _P, _P, _I64, _D, _D, _P, _P],
                            ctypes.c_int),
    "fpgb_run_simulation_device": ([_P, _P, _P, _P, _P, _I64, _D, _D, _P, _P, _P],
                                   ctypes.c_int),
    "fpgb_run_simulation_epa_device": ([_P, _P, _P, _P, _P, _I64, _D, _D, _P, _P,
                                        _P, _P, _P, _P], ctypes.c_int),
    "fpgb_run_simulations_device": ([_P, _P, _P, _P, _P, _I64, _I64, _P, _P, _P, _P, _P,
                                     _P, _P, _P], ctypes.c_int),
    "fpgb_count_steps": ([_P, _P, _D, _D], ctypes.c_int64),
    "fpgb_optic_resample_size": ([_I64, _I64, _D, _P], ctypes.c_int),
    "fpgb_optic_filter_resample_device": ([_P, _I64, _I64, _I64, _D, _D, _P, _P],
                                          ctypes.c_int),
    "fpgb_optic_filter_resample": ([_P, _I64, _I64, _I64, _D, _D, _P], ctypes.c_int),
    "fpgb_optic_noise_device": ([_P, _I64, _D, ctypes.c_uint64, ctypes.c_uint64, _P, _P, _P],
                                ctypes.c_int),
    "fpgb_epa_device": ([_P, _I64, _I64, _P, _P, _P, _P], ctypes.c_int),
    "fpgb_rofl_device": ([_P, _I64, _I64, _D, _D, _D, ctypes.c_int, _P, _P, _P, _P],
                         ctypes.c_int),
}

_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load (building first if needed) the native library; raises on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"fastpli_gb300 native library missing: {path}")
        lib = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def exported_symbols():
    return tuple(_SIGS)


def check(rc):
    if rc == FPGB_OK:
        return
    msg = load().fpgb_last_error().decode(errors="replace")
    if rc == FPGB_EINVAL:
        raise ValueError(msg)
    if rc == FPGB_ENOMEM:
        raise MemoryError(msg)
    if rc == FPGB_ETIMEOUT:
        raise TimeoutError(msg)
    raise RuntimeError(msg)


def ptr(a):
    """Address of a numpy array, torch tensor, or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")


class FlatFibers:
    """Fiber bundles flattened for ``fpgb_fibers`` (arrays kept alive here)."""

    def __init__(self, fiber_bundles, layers):
        if len(fiber_bundles) != len(layers):
            raise ValueError("fbs and prs not the same size")
        b_off, f_off, pts = [0], [0], []
        l_off, sc, dn, mu, md = [0], [], [], [], []
        for fb, lys in zip(fiber_bundles, layers):
            for f in fb:
                f = np.ascontiguousarray(f, dtype=np.float64)
                if f.size % 4 != 0:
                    raise ValueError("fiber data has to be of shape nx4")
                f = f.reshape(-1, 4)
                pts.append(f)
                f_off.append(f_off[-1] + f.shape[0])
            b_off.append(len(f_off) - 1)
            for ly in lys:
                m = ly[3]
                m = m.encode() if isinstance(m, str) else bytes([int(m)])
                if len(m) != 1 or m not in (b"b", b"p", b"r"):
                    raise ValueError('Orientation must be "b", "p", or "r"')
                sc.append(float(ly[0]))
                dn.append(float(ly[1]))
                mu.append(float(ly[2]))
                md.append(m[0])
            l_off.append(len(sc))
        self.bundle_fiber_off = np.asarray(b_off, np.int64)
        self.fiber_point_off = np.asarray(f_off, np.int64)
        self.points = np.ascontiguousarray(
            np.concatenate(pts) if pts else np.zeros((0, 4)), np.float64)
        self.bundle_layer_off = np.asarray(l_off, np.int64)
        self.layer_scale = np.asarray(sc + [0.0], np.float64)
        self.layer_dn = np.asarray(dn + [0.0], np.float64)
        self.layer_mu = np.asarray(mu + [0.0], np.float64)
        self.layer_model = np.asarray(md + [0], np.uint8)
        self.n_bundles = len(fiber_bundles)
        self.max_layer = max([len(l) for l in layers] + [0])
        self.n_fibers = int(self.fiber_point_off.size - 1)
        self.n_points = int(self.points.shape[0])
        self.struct = Fibers(
            self.n_bundles, ptr(self.bundle_fiber_off), ptr(self.fiber_point_off),
            ptr(self.points), ptr(self.bundle_layer_off), ptr(self.layer_scale),
            ptr(self.layer_dn), ptr(self.layer_mu), ptr(self.layer_model))

    @property
    def n_props(self):
        return self.n_bundles * self.max_layer + 1


def make_volume(dim, origin, voxel_size):
    d = np.asarray(dim, np.int64).reshape(3)
    o = np.asarray(origin, np.float64).reshape(3)
    return Volume((ctypes.c_int64 * 3)(*d.tolist()),
                  (ctypes.c_double * 3)(*o.tolist()), float(voxel_size))


class SetupBlock:
    """``fpgb_setup`` plus the filter-rotation array it points to."""

    def __init__(self, step_size, light_intensity, voxel_size, wavelength,
                 tissue_refrection, interpolate, untilt_sensor_view, flip_z,
                 filter_rotations):
        if interpolate not in INTERP:
            raise ValueError("Only NN, Lerp or Slerp are supported")
        self.rot = np.ascontiguousarray(filter_rotations, np.float64).reshape(-1)
        self.struct = Setup(float(step_size), float(light_intensity),
                            float(voxel_size), float(wavelength),
                            float(tissue_refrection), INTERP[interpolate],
                            int(bool(untilt_sensor_view)), int(bool(flip_z)),
                            int(self.rot.size), ptr(self.rot))

    @property
    def n_rho(self):
        return int(self.rot.size)


def byref(s):
    return ctypes.addressof(s)
