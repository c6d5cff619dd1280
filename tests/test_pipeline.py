"""Fiber-bundle file I/O (fastpli.io.fiber_bundles) and the Simpli pipelines
(simpli.py:189-510) that write results to an h5py-like sink.

CPU: text-format round trip and the reference's own cube.dat (where the
reference tree is present) against the committed fiber fixture; the FOM
colour map against a per-pixel restatement of images.py:22-56; the tilt-halo
helpers.
GPU: run_pipeline on the reference's regression scenario (simpli_rep.py)
with an in-memory sink: the dataset names, dtypes and shapes the reference
writes, the tissue and the noise-free images of the reference's own
simpli_rep.h5."""

import io as _io
import os
import warnings

import numpy as np
import pytest

import cases
from fastpli_gb300 import analysis, io, objects
from fastpli_gb300.simpli import Simpli



def test_dat_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    fbs = [[rng.normal(size=(n, 4)) for n in (2, 5)], [rng.normal(size=(3, 4))]]
    path = str(tmp_path / "f.dat")
    io.save(path, fbs)
    with pytest.raises(FileExistsError):  # mode "w-" refuses to overwrite
        io.save(path, fbs)
    back = io.load(path)
    assert len(back) == 2 and [len(b) for b in back] == [2, 1]
    for b0, b1 in zip(fbs, back):
        for f0, f1 in zip(b0, b1):
            assert np.array_equal(f0, f1)  # str() of a float64 round-trips
    with pytest.raises(TypeError):
        io.load(str(tmp_path / "f.xyz"))


def test_dat_blank_line_rules():
    text = "1 2 3 4\n5 6 7 8\n\n9 9 9 1\n\n\n0 0 0 1\n"
    fbs = io.load_dat(_io.StringIO(text))
    assert [len(b) for b in fbs] == [2, 1]
    assert np.array_equal(list(fbs)[1][0], [[0, 0, 0, 1]])


def test_reference_cube_dat_matches_fixture():
    import oracle
    path = oracle.reference_file("tests", "cube.dat")
    if path is None:
        pytest.skip("reference checkout not present (set FPGB_REFERENCE_ROOT)")
    fbs = io.load(path)
    ref = cases.load_cube()
    assert len(fbs) == 1 and len(list(fbs)[0]) == len(ref[0])
    for a, b in zip(list(fbs)[0], ref[0]):
        assert np.array_equal(a, b)


def _fom_px(d, i):
    h = (360.0 * abs(d) / np.pi + 360) % 360
    v = 1.0 - 2 * abs(i) / np.pi
    hi = np.floor(h / 60)
    f = h / 60.0 - hi
    p, q, t = 0.0, v * (1 - f), v * f
    r, g, b = {1: (q, v, p), 2: (p, v, t), 3: (p, q, v), 4: (t, p, v),
               5: (v, p, q)}.get(int(hi), (v, t, p))
    return np.array((r * 255, g * 255, b * 255), np.int64)


def test_fom_hsv_black_matches_per_pixel():
    rng = np.random.default_rng(5)
    d = rng.uniform(-np.pi, np.pi, (17, 9))
    i = rng.uniform(-np.pi / 2, np.pi / 2, (17, 9))
    m = rng.uniform(size=(17, 9)) > 0.3
    ref = np.zeros((17, 9, 3), np.uint8)
    for x in range(17):
        for y in range(9):
            if m[x, y]:
                ref[x, y] = _fom_px(d[x, y], i[x, y])
    assert np.array_equal(analysis.fom_hsv_black(d, i, m), ref)


def test_crop_tilt_halo():
    s = Simpli()
    s.voxel_size = 2.0
    s.set_voi([-40] * 3, [40] * 3)
    s.pixel_size = 4.0
    s.tilts = np.deg2rad([(0, 0), (5.5, 0), (5.5, 90)])
    # ceil(tan(5.5 deg) * 40 / 2 * 2 / 4)
    assert s.crop_tilt_pixel() == int(np.ceil(np.tan(np.deg2rad(5.5)) * 40 / 2 * 0.5))
    assert s.crop_tilt_voxel() == int(np.round(s.crop_tilt_pixel() * 2))
    img = np.zeros((40, 40, 3))
    d = s.crop_tilt_voxel()
    assert s.rm_crop_tilt_halo(img).shape == (40 - 2 * d, 40 - 2 * d, 3)


class _Dataset:
    def __init__(self, value=None, shape=None, dtype=None):
        self.value = None if value is None else np.asarray(value)
        self.shape, self.dtype = shape, dtype
        self.attrs = {}

    def __setitem__(self, key, value):
        self.value = np.asarray(value).astype(self.dtype)

    def __getitem__(self, key):
        return self.value[key]


class _Sink:
    """The part of h5py.File the pipelines use, in memory."""

    def __init__(self):
        self.items, self.attrs = {}, {}

    def create_dataset(self, name, shape, dtype=None, **kw):
        self.items[name] = _Dataset(shape=shape, dtype=dtype)
        return self.items[name]

    def __setitem__(self, name, value):
        self.items[name] = _Dataset(value)

    def __getitem__(self, name):
        return self.items[name]

    def __bool__(self):
        return True


def _rep_simpli():
    """The scenario of the reference's regression file (simpli_rep.py)."""
    s = Simpli()
    s.voxel_size = 5
    s.set_voi([-60] * 3, [60] * 3)
    s.fiber_bundles = objects.FiberBundles(
        cases.load_cube(), [[(0.333, -0.004, 10, "p"), (0.666, 0, 5, "b"), (1.0, 0.004, 1, "r")]])
    s.filter_rotations = np.deg2rad([0, 30, 60, 90, 120, 150])
    s.light_intensity = 26000
    s.interpolate = "Slerp"
    s.wavelength = 525
    s.pixel_size = 20
    s.optical_sigma = 0.71
    s.tilts = np.deg2rad([(0, 0), (5.5, 0), (5.5, 90), (5.5, 180), (5.5, 270)])
    return s


@pytest.mark.gpu
def test_simpli_tilts_device_on_reference_regression(cuda):
    """Simpli.generate_tissue_device + run_tilts_device (the tilts overlapped
    on the library's streams) reproduce the regression file's images within
    1e-4, and each equals its own run_simulation_device call bit for bit."""
    torch = cuda
    g = np.load(os.path.join(cases.GOLDEN, "simpli_rep_h5.npz"))
    s = _rep_simpli()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = s.generate_tissue_device()
        res = s.run_tilts_device(lab, vec, props)
        assert len(res) == 5
        for k, (t, p) in enumerate(s.tilts):
            ref = g[f"simulation.data.{k}"]
            img = res[k].cpu().numpy()
            assert (np.abs(img - ref) / np.abs(ref)).max() < 1e-4, k
            one = s.run_simulation_device(lab, vec, props, t, p)
            assert torch.equal(res[k], one), k


@pytest.mark.gpu
def test_run_pipeline_on_reference_regression(cuda):
    g = np.load(os.path.join(cases.GOLDEN, "simpli_rep_h5.npz"))
    s = _rep_simpli()
    from fastpli_gb300 import optic
    s.noise_model = optic.NegativeBinomialNoise(3.0, seed=1)
    h5f = _Sink()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        (tissue, axis, props), stack, rofl, fom = s.run_pipeline(h5f=h5f, script="x = 1")
    assert h5f.attrs["script"] == "x = 1" and "fastpli/simpli" in h5f.attrs
    t = h5f["tissue/tissue"]
    assert t.dtype == np.uint16 and np.array_equal(t.value, g["tissue.tissue"])
    assert np.array_equal(h5f["tissue/optical_axis"].value.view(np.uint32),
                          g["tissue.optical_axis"].view(np.uint32))
    assert np.array_equal(h5f["tissue/properties"].value, g["tissue.tissue_properties"])
    for k in range(5):
        d = h5f[f"simulation/data/{k}"]
        ref = g[f"simulation.data.{k}"]
        assert (np.abs(d.value - ref) / np.abs(ref)).max() < 1e-4
        assert d.attrs["theta"] == s.tilts[k, 0] and d.attrs["phi"] == s.tilts[k, 1]
        assert h5f[f"simulation/optic/{k}"].value.shape == g[f"simulation.optic.{k}"].shape
        for name in ("transmittance", "direction", "retardation"):
            assert h5f[f"analysis/epa/{k}/{name}"].value.shape == (6, 6)
    assert np.array_equal(h5f["simulation/optic/mask"].value, g["simulation.optic.mask"])
    for name in ("direction", "inclination", "t_rel"):
        assert h5f[f"analysis/rofl/{name}"].value.shape == (6, 6)
    assert stack.shape == (5, 6, 6, 6)
    assert fom.shape == (6, 6, 3) and fom.dtype == np.uint8
