"""The host-buffer calls on page-locked arrays take a pipelined path:
run_generation voxelizes in x-slabs and copies each slab down while the next
ones run; run_simulation copies the volume up in x-slabs and launches the
rays in chunks as soon as the slabs they can reach are on the device.  Both
must give exactly the bits of the plain paths: the device-resident calls and
the host-buffer calls on ordinary (pageable) numpy arrays.

The volume is large enough (label field > 8 MiB) for run_generation to hand
out page-locked arrays; tilts up to 60 degrees make the rays cross many
slabs."""

import warnings

import numpy as np
import pytest

from fastpli_gb300 import synth
from fastpli_gb300.simulation import _Generator, _Simulator

pytestmark = pytest.mark.gpu

TILTS = [(0.0, 0.0), (5.5, 0.0), (5.5, 90.0), (30.0, 45.0), (60.0, 200.0), (45.0, 300.0)]


def _volume():
    w = synth.crossing(seed=7, n_per_bundle=250, dim=(176, 160, 96), n_points=20)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    return w, g


def _sim(interp, untilt, flip_z, voxel_size):
    s = _Simulator()
    s.set_pli_setup(1.0, 26000.0, voxel_size, 525.0, 1.0, interp, untilt, flip_z,
                    np.deg2rad([0.0, 30.0, 60.0, 90.0, 120.0, 150.0]))
    return s


@pytest.fixture(scope="module")
def volume(cuda):
    torch = cuda
    w, g = _volume()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = g.run_generation()
        d_lab, d_vec, d_props, _ = g.run_generation_device()
    torch.cuda.synchronize()
    return w, lab, vec, props, d_lab, d_vec


def test_generation_outputs_are_page_locked_and_match_device(volume, cuda):
    torch = cuda
    w, lab, vec, props, d_lab, d_vec = volume
    # the arrays are numpy arrays backed by page-locked memory
    assert isinstance(lab, np.ndarray) and isinstance(vec, np.ndarray)
    assert torch.from_numpy(lab).is_pinned() and torch.from_numpy(vec).is_pinned()
    assert np.array_equal(lab, d_lab.cpu().numpy())
    assert np.array_equal(vec.view(np.uint32), d_vec.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("interp,untilt,flip_z", [("Slerp", True, False), ("NN", False, True),
                                                  ("Lerp", False, False)])
def test_pipelined_march_matches_plain_paths(volume, cuda, interp, untilt, flip_z):
    torch = cuda
    w, lab, vec, props, d_lab, d_vec = volume
    lab_pageable, vec_pageable = np.array(lab), np.array(vec)
    assert not torch.from_numpy(lab_pageable).is_pinned()
    sim = _sim(interp, untilt, flip_z, w.voxel_size)
    for t, p in TILTS:
        th, ph = np.deg2rad(t), np.deg2rad(p)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            img_pipe = sim.run_simulation(w.dim, lab, vec, props, th, ph)
            img_plain = sim.run_simulation(w.dim, lab_pageable, vec_pageable, props, th, ph)
            img_dev = sim.run_simulation_device(w.dim, d_lab, d_vec, props, th, ph)
        torch.cuda.synchronize()
        assert np.all(np.isfinite(img_pipe))
        assert np.array_equal(img_pipe.view(np.uint64), img_plain.view(np.uint64)), (t, p)
        assert np.array_equal(img_pipe.view(np.uint64),
                              img_dev.cpu().numpy().view(np.uint64)), (t, p)


@pytest.mark.parametrize("interp", ["Slerp", "NN"])
def test_wide_index_march_matches_narrow(volume, cuda, interp, monkeypatch):
    """Volumes with 3 X Y Z >= 2^32 voxels march with 64-bit index arithmetic;
    forced onto this volume (FPGB_WIDE_INDEX=1) those kernels give the bits of
    the 32-bit ones (the batched path: tests/test_batch.py)."""
    torch = cuda
    w, lab, vec, props, d_lab, d_vec = volume
    sim = _sim(interp, False, False, w.voxel_size)
    for t, p in TILTS:
        th, ph = np.deg2rad(t), np.deg2rad(p)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            monkeypatch.delenv("FPGB_WIDE_INDEX", raising=False)
            narrow = sim.run_simulation_device(w.dim, d_lab, d_vec, props, th, ph, epa=True)
            monkeypatch.setenv("FPGB_WIDE_INDEX", "1")
            wide = sim.run_simulation_device(w.dim, d_lab, d_vec, props, th, ph, epa=True)
            monkeypatch.delenv("FPGB_WIDE_INDEX")
        torch.cuda.synchronize()
        for x, y in zip(narrow, wide):
            assert torch.equal(x.view(torch.int64), y.view(torch.int64)), (t, p)


@pytest.mark.parametrize("interp,untilt", [("Slerp", True), ("NN", False)])
def test_pipelined_march_page_locked_image(cuda, interp, untilt):
    """An image of 8 MiB and more is page-locked, and the pipelined march
    copies its rows down as each launch completes them.  446 x 418 pixels:
    the last 4-row ray tile is partial, and 418 rows of 32 rays split the
    chunk boundaries inside ray tiles.  Bits equal the device-resident
    march's at every tilt (theta = 0 takes the column path)."""
    torch = cuda
    w = synth.crossing(seed=8, n_per_bundle=120, dim=(446, 418, 24), n_points=20)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    sim = _sim(interp, untilt, False, w.voxel_size)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = g.run_generation()
        d_lab, d_vec, _, _ = g.run_generation_device()
        for t, p in TILTS:
            th, ph = np.deg2rad(t), np.deg2rad(p)
            img = sim.run_simulation(w.dim, lab, vec, props, th, ph)
            ref = sim.run_simulation_device(w.dim, d_lab, d_vec, props, th, ph)
            torch.cuda.synchronize()
            assert torch.from_numpy(img).is_pinned()
            assert np.array_equal(img.view(np.uint64), ref.cpu().numpy().view(np.uint64)), (t, p)


def test_pipelined_march_rejects_bad_labels(volume, cuda):
    """A label outside the property table raises, as on the one-copy path
    (simulator.cpp:149-167), also when the volume goes up in slabs."""
    w, lab, vec, props, d_lab, d_vec = volume
    sim = _sim("Slerp", True, False, w.voxel_size)
    bad = _host_empty_like(lab)
    bad[...] = lab
    bad[w.dim[0] - 1, 3, 4] = props.shape[0] + 5  # in the last slab
    with pytest.raises(ValueError, match="label"):
        sim.run_simulation(w.dim, bad, vec, props, np.deg2rad(5.5), 0.0)
    bad[...] = lab
    bad[0, 0, 0] = -1
    with pytest.raises(ValueError, match="label"):
        sim.run_simulation(w.dim, bad, vec, props, np.deg2rad(5.5), 0.0)


def _host_empty_like(a):
    from fastpli_gb300.simulation import _host_empty
    out = _host_empty(a.shape, a.dtype)
    import torch
    assert torch.from_numpy(out).is_pinned()
    return out
