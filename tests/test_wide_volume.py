"""A volume past the 32-bit index range, against the reference's own output.

fastpli_gb300.synth.wide_strip(): 5504 x 16384 x 16 voxels (1.44e9;
3 X Y Z >= 2^32), so the march takes its 64-bit index arithmetic by itself
(no FPGB_WIDE_INDEX), with all tissue in the last 32 x-columns, where the
vector field's linear index 3 ((x Y + y) Z + z) is past 2^32.  Golden
digests: tests/golden/wide_manifest.json and wide_images.npz, made by
tests/golden/make_wide_golden.py from the reference's C++.

* Labels and vectors of the strip bit-exact (sha256), the rest background.
  (The reference works in volume-local coordinates, so the same fibers
  shifted into a small volume give 17 different 'r' vectors: rounding at
  x ~ 5490 differs from rounding at x ~ 18.  Only the full-size reference
  pins this volume.)
* Images at theta = 0 and at 10 degrees towards +y: five rows at every 64th
  y within 1e-4 relative per pixel, the mean of the whole stack within 1e-5.
* The strip marched as a volume of its own (32-bit path) gives the same
  float64 image bits as the strip of the whole volume (64-bit path): rays
  there start at their pixel centre in x and move only in y (phi = 90 deg,
  whose cosine the reference takes as exactly 0, vemath.hpp:498-520), and
  Y = 16384 sets the same fixed-point format for both volumes.

Device memory: ~30 GB (label 5.8 GB, vectors 17.3 GB, image 6.5 GB)."""

import hashlib
import json
import os
import warnings

import numpy as np
import pytest

from fastpli_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "wide_manifest.json")) as f:
        return json.load(f)["wide"]


def test_wide_fixtures_are_consistent():
    e = manifest()
    w = synth.wide_strip()
    X, Y, Z = (int(v) for v in w.dim)
    assert 3 * X * Y * Z >= 2 ** 32 > 3 * synth.WIDE_STRIP * Y * Z
    assert e["strip_x0"] == X - synth.WIDE_STRIP and e["outside_strip_zero"]
    for b in w.bundles:  # all tissue inside the strip, away from its edges
        for f in b:
            assert f[:, 0].min() - f[:, 3].max() > e["strip_x0"] + 4
            assert f[:, 0].max() + f[:, 3].max() < X - 4
    assert np.allclose(np.asarray(e["tilts"]), w.tilts)
    imgs = np.load(os.path.join(GOLDEN, "wide_images.npz"))
    for k in range(len(e["tilts"])):
        img = imgs[f"wide|{k}"]
        assert img.shape == (len(e["rows"]), (Y + e["y_stride"] - 1) // e["y_stride"],
                             len(w.rotations))
        assert np.all(np.isfinite(img)) and np.all(img > 0)


@pytest.mark.gpu
def test_wide_volume_matches_reference(cuda):
    torch = cuda
    from fastpli_gb300.simulation import _Generator, _Simulator
    e = manifest()
    imgs = np.load(os.path.join(GOLDEN, "wide_images.npz"))
    w = synth.wide_strip()
    X, Y, Z = (int(v) for v in w.dim)
    x0 = e["strip_x0"]
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props, _ = g.run_generation_device()
    torch.cuda.synchronize()
    assert np.array_equal(props, np.asarray(e["props"]))
    assert hashlib.sha256(lab[x0:].cpu().numpy().tobytes()).hexdigest() == \
        e["strip_label_sha256"]
    assert hashlib.sha256(vec[x0:].cpu().numpy().tobytes()).hexdigest() == \
        e["strip_vector_sha256"]
    assert int(lab.count_nonzero()) == e["tissue_voxels"]
    assert not bool(lab[:x0].any())
    assert not bool(vec[:x0].view(torch.int32).any())

    kw = w.setup_kwargs()
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    img = torch.empty((X, Y, len(w.rotations)), dtype=torch.float64, device=lab.device)
    for k, (t, p) in enumerate(e["tilts"]):
        sim.run_simulation_device(w.dim, lab, vec, props, t, p, image=img)
        sub = img[e["rows"], ::e["y_stride"]].cpu().numpy()
        ref = imgs[f"wide|{k}"]
        rel = np.abs(sub - ref) / np.abs(ref)
        assert rel.max() < 1e-4, (k, rel.max())
        assert abs(float(img.mean()) / e["image_mean"][k] - 1) < 1e-5
        strip = sim.run_simulation_device((X - x0, Y, Z), lab[x0:], vec[x0:], props, t, p)
        assert torch.equal(img[x0:], strip), k
    del lab, vec, img, strip
    torch.cuda.empty_cache()
