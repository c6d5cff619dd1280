"""Parity at the benchmarks' full sizes against the reference's own output
(tests/golden/full_manifest.json and full_images.npz, made by
tests/golden/make_full_golden.py from the reference's C++):

  crossing  512 x 512 x 120, 2 x 1000 fibers (the bench volume), 3 tilts
  watson    1024 x 1024 x 240, 20000 fibers, 3 layers (252 M voxels), 1 tilt

Labels and vectors: sha256 of the whole fields equal to the reference's
(bit-exact at full size).  Images (Slerp, 9 angles): every 16th / 32nd row
and column within 1e-4 relative per pixel, the mean of the full stack within
1e-5."""

import hashlib
import json
import os
import warnings

import numpy as np
import pytest

from fastpli_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MAKERS = {"crossing": synth.crossing, "watson": synth.watson}


def manifest():
    with open(os.path.join(GOLDEN, "full_manifest.json")) as f:
        return json.load(f)


def test_full_size_fixtures_are_consistent():
    man = manifest()
    imgs = np.load(os.path.join(GOLDEN, "full_images.npz"))
    for name, e in man.items():
        w = MAKERS[name]()
        X, Y = (int(v) for v in w.dim[:2])
        s = e["stride"]
        for k in range(len(e["tilts"])):
            img = imgs[f"{name}|{k}"]
            assert img.shape == ((X + s - 1) // s, (Y + s - 1) // s, len(w.rotations))
            assert np.all(np.isfinite(img))
        assert 0 < e["tissue_voxels"] <= int(np.prod(w.dim))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["crossing", "watson"])
def test_full_size_matches_reference(cuda, name):
    torch = cuda
    from fastpli_gb300.simulation import _Generator, _Simulator
    e = manifest()[name]
    imgs = np.load(os.path.join(GOLDEN, "full_images.npz"))
    w = MAKERS[name]()
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props, _ = g.run_generation_device()
    torch.cuda.synchronize()
    lab_h = lab.cpu().numpy()
    assert hashlib.sha256(lab_h.tobytes()).hexdigest() == e["label_sha256"]
    assert int((lab_h > 0).sum()) == e["tissue_voxels"]
    del lab_h
    assert hashlib.sha256(vec.cpu().numpy().tobytes()).hexdigest() == e["vector_sha256"]
    kw = w.setup_kwargs()
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    s = e["stride"]
    for k, (t, p) in enumerate(e["tilts"]):
        img = sim.run_simulation_device(w.dim, lab, vec, props, t, p)
        sub = img[::s, ::s].cpu().numpy()
        ref = imgs[f"{name}|{k}"]
        rel = np.abs(sub - ref) / np.abs(ref)
        assert rel.max() < 1e-4, (name, k, rel.max())
        assert abs(float(img.mean()) / e["image_mean"][k] - 1) < 1e-5


@pytest.mark.gpu
def test_crossing_every_pixel_of_every_bench_tilt_vs_oracle(cuda, oracle_port):
    """The bench volume (512 x 512 x 120, 2 x 1000 fibers) at all 5 bench
    tilts, every pixel and polarizer angle, against the FP64 oracle run in
    the test (the oracle is pinned bit for bit to the reference's build)."""
    import parity
    torch = cuda
    from fastpli_gb300.simulation import _Generator, _Simulator
    threads = os.cpu_count() or 1
    w = synth.crossing()
    olab, ovec, oprops, _ = oracle_port.generate(w.dim, w.origin, w.voxel_size, w.bundles,
                                                 w.layers, n_threads=threads)
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props, _ = g.run_generation_device()
    torch.cuda.synchronize()
    n_lab = int((lab.cpu().numpy() != olab).sum())
    n_vec = int((vec.cpu().numpy().view(np.uint32) != ovec.view(np.uint32)).sum())
    assert n_lab == 0 and n_vec == 0
    kw = w.setup_kwargs()
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    for k, (t, p) in enumerate(w.tilts):
        img = sim.run_simulation_device(w.dim, lab, vec, props, float(t), float(p))
        ref, _ = oracle_port.simulate(olab, ovec, oprops, float(t), float(p), n_threads=threads,
                                      **kw)
        e = parity.image_errors(img.cpu().numpy(), ref)
        parity.record(f"crossing512/tilt{k}", label_mismatch=n_lab, vector_mismatch=n_vec,
                      pixels=int(ref.size), **e)
        assert e["max_rel"] <= parity.IMG_RTOL, (k, e)
