"""The oracle — TEST INFRASTRUCTURE ONLY.

Two CPU implementations of fastpli's simulation forward model, both reached
through ctypes with the same argument lists:

* ``impl="port"``  — ``oracle/pli_oracle.c``: this project's double-precision
  C restatement of ``PliGenerator::RunTissueGeneration``
  (src/simulation/generator.cpp:163-383) and ``PliSimulator::RunSimulation``
  (src/simulation/simulator.cpp:182-411).  Built by ``make -C oracle`` into
  ``oracle/_lib/liboracle.so``; it exists wherever the repository is built.
* ``impl="ref"``   — the reference's own unmodified C++ compiled from its
  sources by ``make -C oracle ref`` into ``oracle/_ref/libpliref.so``.  Only
  buildable where the reference sources are present; used to pin the port
  and to generate the golden fixtures in ``tests/golden``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker / the timed CPU
baseline; the product (``fastpli_gb300``) never does.
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(_HERE, "_lib", "liboracle.so")
REF_LIB = os.path.join(_HERE, "_ref", "libpliref.so")
# Checkout of the reference project (read only, never needed at run time on a
# machine without it): FPGB_REFERENCE_ROOT, else the build container's path.
REF_ROOT_DEFAULT = os.environ.get("FPGB_REFERENCE_ROOT", "/root/reference")


def reference_file(*parts):
    """Path of a file of the reference checkout, or None when it is absent."""
    path = os.path.join(REF_ROOT_DEFAULT, *parts)
    return path if os.path.exists(path) else None

WARNING_NAMES = ("overlap", "single_point", "zero_axis", "not_normalized",
                 "empty_light", "layer_overflow")

_libs = {}

_P = ctypes.c_void_p
_GEN_ARGS = [_P, _P, ctypes.c_double, ctypes.c_int64, _P, _P, _P, _P, _P, _P,
             _P, _P, ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int64,
             _P, _P]
_SIM_ARGS = [_P, _P, _P, _P, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
             ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
             ctypes.c_int, ctypes.c_int, _P, ctypes.c_int64, ctypes.c_double,
             ctypes.c_double, ctypes.c_int, _P, _P]


def build(ref=False, ref_root=REF_ROOT_DEFAULT):
    """Compile the port (and, when ``ref`` and the sources exist, the
    reference harness).  Returns the list of libraries that exist after."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    if ref and os.path.isdir(os.path.join(ref_root, "src", "simulation")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref",
                        f"REF_ROOT={ref_root}"], check=True)
    return [p for p in (PORT_LIB, REF_LIB) if os.path.exists(p)]


def available(impl):
    return os.path.exists(PORT_LIB if impl == "port" else REF_LIB)


def _lib(impl):
    if impl in _libs:
        return _libs[impl]
    path = PORT_LIB if impl == "port" else REF_LIB
    if not os.path.exists(path):
        raise RuntimeError(f"oracle library missing: {path} (run make -C oracle"
                           f"{' ref' if impl == 'ref' else ''})")
    lib = ctypes.CDLL(path)
    pre = "orc_" if impl == "port" else "ref_"
    gen = getattr(lib, pre + "generate")
    gen.argtypes = _GEN_ARGS
    gen.restype = ctypes.c_int
    sim = getattr(lib, pre + "simulate")
    sim.argtypes = _SIM_ARGS
    sim.restype = ctypes.c_int
    err = getattr(lib, pre + "last_error")
    err.restype = ctypes.c_char_p
    _libs[impl] = (gen, sim, err)
    return _libs[impl]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def flatten_bundles(fiber_bundles, layers):
    """(list of bundles of (n,4) arrays, list of per-bundle layer tuples) ->
    the flat arrays of the C-ABI."""
    if len(fiber_bundles) != len(layers):
        raise ValueError("fbs and prs not the same size")
    b_off, f_off, pts = [0], [0], []
    l_off, sc, dn, mu, md = [0], [], [], [], []
    for fb, lys in zip(fiber_bundles, layers):
        for f in fb:
            f = np.asarray(f, dtype=np.float64).reshape(-1, 4)
            pts.append(f)
            f_off.append(f_off[-1] + f.shape[0])
        b_off.append(len(f_off) - 1)
        for ly in lys:
            sc.append(float(ly[0]))
            dn.append(float(ly[1]))
            mu.append(float(ly[2]))
            md.append(ord(ly[3]) if isinstance(ly[3], str) else int(ly[3]))
        l_off.append(len(sc))
    points = (np.concatenate(pts) if pts else np.zeros((0, 4)))
    return dict(
        bundle_fiber_off=np.asarray(b_off, np.int64),
        fiber_point_off=np.asarray(f_off, np.int64),
        points=np.ascontiguousarray(points, np.float64),
        bundle_layer_off=np.asarray(l_off, np.int64),
        layer_scale=np.asarray(sc, np.float64),
        layer_dn=np.asarray(dn, np.float64),
        layer_mu=np.asarray(mu, np.float64),
        layer_model=np.asarray(md, np.uint8),
        n_bundles=len(fiber_bundles),
        max_layer=max([len(l) for l in layers] + [0]))


def generate(dim, origin, voxel_size, fiber_bundles, layers, only_label=False,
             n_threads=1, impl="port"):
    """Voxelize fiber bundles.  Returns (label int32 [X,Y,Z],
    vector float32 [X,Y,Z,3] or empty, props float64 [n,2], warnings dict)."""
    gen, _, err = _lib(impl)
    dim = np.asarray(dim, np.int64).reshape(3)
    origin = np.asarray(origin, np.float64).reshape(3)
    fl = flatten_bundles(fiber_bundles, layers)
    n = int(np.prod(dim))
    label = np.empty(tuple(dim), np.int32)
    vector = None if only_label else np.empty(tuple(dim) + (3,), np.float32)
    cap = fl["n_bundles"] * fl["max_layer"] + 1
    props = np.zeros((cap, 2), np.float64)
    n_props = np.zeros(1, np.int64)
    warn = np.zeros(6, np.int64)
    rc = gen(_ptr(dim), _ptr(origin), float(voxel_size), fl["n_bundles"],
             _ptr(fl["bundle_fiber_off"]), _ptr(fl["fiber_point_off"]),
             _ptr(fl["points"]), _ptr(fl["bundle_layer_off"]),
             _ptr(fl["layer_scale"]), _ptr(fl["layer_dn"]),
             _ptr(fl["layer_mu"]), _ptr(fl["layer_model"]), int(only_label),
             int(n_threads), _ptr(label), _ptr(vector), _ptr(props), cap,
             _ptr(n_props), _ptr(warn))
    if rc != 0:
        raise ValueError(err().decode())
    assert n_props[0] == cap and label.size == n
    if vector is None:
        vector = np.zeros((0,), np.float32)
    return label, vector, props, dict(zip(WARNING_NAMES, warn.tolist()))


_INTERP = {"NN": 0, "Lerp": 1, "Slerp": 2}


def _pi_case_cos(v):
    """vm::rot_pi_cases::cos (src/include/vemath.hpp:510-520)."""
    import math
    v = math.fmod(v, 2 * math.pi)
    if v == 0:
        return 1.0
    if v in (math.pi / 2, math.pi + math.pi / 2, -math.pi / 2, -(math.pi + math.pi / 2)):
        return 0.0
    if v in (math.pi, -math.pi):
        return -1.0
    return math.cos(v)


def count_steps(dim, theta, step_size=1.0):
    """Ray-voxel steps of one run_simulation call, on the host: X * Y rays,
    each stepping from z = step_z / 2 in steps of step_z = cos(theta) *
    step_size while floor(z) lies in [0, Z) (src/simulation/simulator.cpp:
    216-231 with LightDirectionUnitVector :585-590, and the loop :259-261)."""
    import math
    X, Y, Z = (int(v) for v in np.asarray(dim).reshape(3))
    dz = _pi_case_cos(float(theta)) * float(step_size)
    if not dz > 0:
        raise ValueError("light direction has no positive z component")
    n = 0
    z = 0.0 + dz * 0.5
    while math.floor(z) >= 0 and math.floor(z) < Z:
        n += 1
        z = z + dz
    return X * Y * n


def simulate(label, vector, props, theta=0.0, phi=0.0, *, step_size=1.0,
             light_intensity=26000.0, voxel_size=1.0, wavelength=525.0,
             tissue_refrection=1.0, interpolate="Slerp",
             untilt_sensor_view=True, flip_z=False, filter_rotations=None,
             n_threads=1, impl="port"):
    """Ray-march one tilt.  Returns (image float64 [X,Y,n_rho], warnings)."""
    _, sim, err = _lib(impl)
    label = np.ascontiguousarray(label, np.int32)
    vector = np.ascontiguousarray(vector, np.float32)
    props = np.ascontiguousarray(props, np.float64).reshape(-1, 2)
    if filter_rotations is None:
        filter_rotations = np.deg2rad([0, 30, 60, 90, 120, 150])
    rot = np.ascontiguousarray(filter_rotations, np.float64).reshape(-1)
    dim = np.asarray(label.shape, np.int64)
    if vector.size != 3 * label.size:
        raise ValueError("label_field_.size()*3 != vector_field_.size()")
    image = np.empty((dim[0], dim[1], rot.size), np.float64)
    warn = np.zeros(6, np.int64)
    rc = sim(_ptr(dim), _ptr(label), _ptr(vector), _ptr(props), props.shape[0],
             float(step_size), float(light_intensity), float(voxel_size),
             float(wavelength), float(tissue_refrection),
             _INTERP[interpolate], int(bool(untilt_sensor_view)),
             int(bool(flip_z)), _ptr(rot), rot.size, float(theta), float(phi),
             int(n_threads), _ptr(image), _ptr(warn))
    if rc != 0:
        raise ValueError(err().decode())
    return image, dict(zip(WARNING_NAMES, warn.tolist()))


def epa(data):
    """fastpli.analysis.epa.epa restated (src/fastpli/analysis/epa.py:9-45):
    transmittance, direction, retardation from the first Fourier harmonic over
    equidistant polarizer angles in [0, pi)."""
    data = np.asarray(data)
    dtype = np.float32 if data.itemsize <= 4 else np.float64
    data = data.astype(dtype)
    n = data.shape[-1]
    rho_2 = 2 * np.linspace(0, np.pi, n, False, dtype=dtype)
    a0 = np.sum(data, -1) / n
    a1 = 2 * np.sum(data * np.sin(rho_2), -1) / n
    b1 = 2 * np.sum(data * np.cos(rho_2), -1) / n
    t = 2 * a0
    d = 0.5 * np.arctan2(-b1, a1) + np.pi
    a0[a0 < np.finfo(dtype).eps * 100] = 1
    r = np.sqrt(a1 * a1 + b1 * b1) / a0
    d = d % np.pi
    return t, d, r
