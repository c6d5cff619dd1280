"""C-ABI checks that need no GPU: the library builds, loads and exports every
symbol the header declares; host-side planning and argument validation."""

import ctypes
import os
import re

import numpy as np
import pytest

import fastpli_gb300
from fastpli_gb300 import _native as N
from fastpli_gb300.simulation import _Generator, _Simulator

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name):
    src = open(os.path.join(ROOT, "include", name)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fpgb_[a-z0-9_]+)\s*\(", src)))


def test_library_loads_and_exports_header_symbols():
    from fastpli_gb300 import batch
    lib = fastpli_gb300.native_library()
    headers = sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h"))
    assert headers == ["fastpli_gb300.h", "fastpli_gb300_batch.h"]
    tables = {"fastpli_gb300.h": N.exported_symbols(),
              "fastpli_gb300_batch.h": batch.exported_symbols()}
    for h in headers:
        names = header_functions(h)
        assert names
        for n in names:
            assert hasattr(lib, n), f"{n} declared in include/{h} but not exported"
        assert set(names) == set(tables[h]), f"ctypes table out of sync with {h}"
    assert b"sm_103a" in lib.fpgb_version()


def _setup(**kw):
    base = dict(step_size=1.0, light_intensity=26000.0, voxel_size=0.2, wavelength=525.0,
                tissue_refrection=1.0, interpolate="Slerp", untilt_sensor_view=True,
                flip_z=False, filter_rotations=np.deg2rad(np.arange(0, 180, 20)))
    base.update(kw)
    return N.SetupBlock(**base)


def _steps_reference_loop(Z, theta, phi, step):
    """Replays simulator.cpp:230-231,259-261 for the z coordinate."""
    dz = np.cos(theta) * step if theta != 0 else step
    z, n = 0.0 + dz * 0.5, 0
    while 0 <= np.floor(z) < Z:
        n += 1
        z = z + dz
    return n


@pytest.mark.parametrize("theta,step", [(0.0, 1.0), (np.deg2rad(5.5), 1.0),
                                        (np.deg2rad(30), 0.37), (0.0, 2.5)])
def test_count_steps_matches_reference_loop(theta, step):
    s = _setup(step_size=step)
    dim = np.array([7, 5, 120], np.int64)
    n = N.load().fpgb_count_steps(N.byref(s.struct), N.ptr(dim), theta, 0.3)
    assert n == 7 * 5 * _steps_reference_loop(120, theta, 0.3, step)


@pytest.mark.parametrize("bad,msg", [
    (dict(step_size=0.0), "step_size"), (dict(light_intensity=-1.0), "light"),
    (dict(voxel_size=0.0), "voxel_size"), (dict(wavelength=0.0), "wavelength"),
    (dict(tissue_refrection=0.5), "tissue_refrection"),
    (dict(filter_rotations=[]), "filter_rotations")])
def test_setup_validation_raises_before_any_device_work(bad, msg):
    sim = _Simulator()
    kw = dict(step_size=1.0, light_intensity=1.0, voxel_size=1.0, wavelength=525.0,
              tissue_refrection=1.0, interpolate="NN", untilt_sensor_view=True, flip_z=False,
              filter_rotations=[0.0])
    kw.update(bad)
    sim.set_pli_setup(**kw)
    lab = np.zeros((2, 2, 2), np.int32)
    vec = np.zeros((2, 2, 2, 3), np.float32)
    with pytest.raises(ValueError, match=msg):
        sim.run_simulation([2, 2, 2], lab, vec, np.zeros((1, 2)), 0.0, 0.0)


def test_interpolate_string_checked():
    with pytest.raises(ValueError, match="NN, Lerp or Slerp"):
        _Simulator().set_pli_setup(1, 1, 1, 525, 1, "Cubic", True, False, [0.0])


def test_background_birefringence_rejected():
    sim = _Simulator()
    sim.set_pli_setup(1, 1, 1, 525, 1, "NN", True, False, [0.0])
    with pytest.raises(ValueError, match="background birefringence"):
        sim.run_simulation([1, 1, 1], np.zeros((1, 1, 1), np.int32),
                           np.zeros((1, 1, 1, 3), np.float32), np.array([[0.1, 0.0]]), 0, 0)


def test_generator_volume_validation():
    g = _Generator()
    with pytest.raises(ValueError, match="dim.global"):
        g.set_volume([0, 4, 4], [0, 0, 0], 1.0)
    with pytest.raises(ValueError, match="voxel_size"):
        g.set_volume([4, 4, 4], [0, 0, 0], 0.0)
    with pytest.raises(ValueError, match="Orientation"):
        g.set_fiber_bundles([[np.zeros((2, 4))]], [[(1.0, 0.0, 0.0, "x")]])
    with pytest.raises(ValueError, match="not the same size"):
        g.set_fiber_bundles([[np.zeros((2, 4))]], [])


def test_workspace_size_is_host_planned():
    g = _Generator()
    g.set_volume([10, 12, 14], [0, 0, 0], 0.5)
    g.set_fiber_bundles([[np.array([[0, 0, 0, 1], [5, 6, 7, 1]], float)],
                         [np.array([[5, 0, 0, 1], [5, 6, 7, 1.5]], float)]],
                        [[(1.0, 0.004, 1.0, "r")], [(0.5, 0.0, 1.0, "b"), (1.0, 0.004, 1.0, "p")]])
    ws = g.workspace_size()
    assert ws > 0
    assert g.n_props() == 1 + 2 * 2
    # keys live in shared memory per 8x8x32 brick: the workspace holds the
    # segment table, the brick lists and three words per brick, nothing per voxel
    g.set_volume([400, 400, 320], [0, 0, 0], 0.5)
    n_bricks = 50 * 50 * 10
    assert g.workspace_size() - ws <= 3 * 4 * n_bricks + 4096


def test_stage_entry_points_validate_before_device_work():
    """The optic, noise, epa and ROFL entry points refuse bad arguments with
    FPGB_EINVAL before any CUDA call (runs without a GPU)."""
    lib = N.load()
    one = np.zeros(8, np.float64)
    # sigma < 0, scale <= 0, n_rho <= 0, null buffers
    assert lib.fpgb_optic_filter_resample_device(N.ptr(one), 2, 2, 2, -1.0, 0.5, N.ptr(one),
                                                 None) == N.FPGB_EINVAL
    assert lib.fpgb_optic_filter_resample_device(N.ptr(one), 2, 2, 2, 0.7, 0.0, N.ptr(one),
                                                 None) == N.FPGB_EINVAL
    assert lib.fpgb_optic_filter_resample_device(None, 2, 2, 2, 0.7, 0.5, N.ptr(one),
                                                 None) == N.FPGB_EINVAL
    assert lib.fpgb_optic_filter_resample_device(N.ptr(one), 2, 2, 0, 0.7, 0.5, N.ptr(one),
                                                 None) == N.FPGB_EINVAL
    # a scale that leaves no output pixel
    assert lib.fpgb_optic_filter_resample_device(N.ptr(one), 2, 2, 2, 0.7, 0.1, N.ptr(one),
                                                 None) == N.FPGB_EINVAL
    assert b"empty" in lib.fpgb_last_error()
    # noise: gain <= 1
    assert lib.fpgb_optic_noise_device(N.ptr(one), 8, 1.0, 1, 0, N.ptr(one), None,
                                       None) == N.FPGB_EINVAL
    # epa: n_rho outside 1..64
    assert lib.fpgb_epa_device(N.ptr(one), 1, 0, N.ptr(one), N.ptr(one), N.ptr(one),
                               None) == N.FPGB_EINVAL
    assert lib.fpgb_epa_device(N.ptr(one), 1, 65, N.ptr(one), N.ptr(one), N.ptr(one),
                               None) == N.FPGB_EINVAL
    # rofl: n_rot <= 3, n_rot > 32, gain <= 1
    out = np.zeros(8)
    assert lib.fpgb_rofl_device(N.ptr(one), 1, 3, 0.1, 3.0, 0.0, 0, None, N.ptr(out), None,
                                None) == N.FPGB_EINVAL
    assert lib.fpgb_rofl_device(N.ptr(one), 1, 33, 0.1, 3.0, 0.0, 0, None, N.ptr(out), None,
                                None) == N.FPGB_EINVAL
    assert lib.fpgb_rofl_device(N.ptr(one), 1, 6, 0.1, 1.0, 0.0, 0, None, N.ptr(out), None,
                                None) == N.FPGB_EINVAL
    assert b"gain" in lib.fpgb_last_error()


def test_multi_tilt_entry_validates_before_device_work():
    """fpgb_run_simulations_device refuses missing tilt arrays, a negative
    tilt count and a tilt the setup rejects (theta = 90 deg: no positive z
    step) with FPGB_EINVAL, and takes an empty tilt list as a no-op, all
    before any CUDA call (runs without a GPU; the buffer addresses are never
    dereferenced)."""
    lib = N.load()
    s = _setup()
    dim = np.array([4, 4, 4], np.int64)
    props = np.zeros((1, 2))
    buf = np.zeros(4, np.int64)  # stands in for device buffers
    imgs = (ctypes.c_void_p * 2)(buf.ctypes.data, buf.ctypes.data)

    def call(n, theta, phi):
        return lib.fpgb_run_simulations_device(
            N.byref(s.struct), N.ptr(dim), N.ptr(buf), N.ptr(buf), N.ptr(props), 1, n,
            N.ptr(theta), N.ptr(phi), imgs, None, None, None, None, None)

    ph = np.zeros(2)
    assert call(2, None, ph) == N.FPGB_EINVAL
    assert call(-1, ph, ph) == N.FPGB_EINVAL
    assert call(2, np.array([0.0, np.pi / 2]), ph) == N.FPGB_EINVAL
    assert b"theta" in lib.fpgb_last_error()
    assert call(0, None, None) == 0
