"""GPU parity: the CUDA voxelizer and ray march, called through the C ABI,
against the reference's golden fixtures and the oracle.

Bars (tests/parity.py; the max error of every result is recorded and printed
at the end of the run):
  * labels: bit-exact; vectors: bit-exact (float32 bits);
  * images: relative error <= 1e-4 per pixel (FP32 march vs FP64 reference);
  * epa transmittance/retardation <= 1e-3 relative, direction <= 1e-3 rad
    (mod pi).
"""

import hashlib
import json
import os
import warnings

import numpy as np
import pytest

import cases
from fastpli_gb300.simulation import _Generator, _Simulator

pytestmark = pytest.mark.gpu

from parity import EPA_TOL, IMG_RTOL, REPORT  # noqa: E402


def _gold(name):
    return np.load(os.path.join(cases.GOLDEN, name))


def _generator(c):
    g = _Generator()
    g.set_volume(c["dim"], c["origin"], c["voxel_size"])
    g.set_fiber_bundles(c["bundles"], c["layers"])
    return g


def _simulator(kw):
    s = _Simulator()
    base = dict(step_size=1.0, light_intensity=26000.0, voxel_size=1.0, wavelength=525.0,
                tissue_refrection=1.0, interpolate="Slerp", untilt_sensor_view=True,
                flip_z=False)
    base.update(kw)
    s.set_pli_setup(base["step_size"], base["light_intensity"], base["voxel_size"],
                    base["wavelength"], base["tissue_refrection"], base["interpolate"],
                    base["untilt_sensor_view"], base["flip_z"], base["filter_rotations"])
    return s


from parity import rel as _rel  # noqa: E402


def _check_images(key, got, ref):
    assert got.shape == ref.shape
    assert np.all(np.isfinite(got))
    rel = _rel(got, ref)
    mean_rel = float(np.max(np.abs(got - ref) / np.maximum(ref.mean(-1, keepdims=True), 1e-300)))
    REPORT[key] = {"max_rel": rel, "max_rel_to_pixel_mean": mean_rel}
    assert rel <= IMG_RTOL, f"{key}: max relative error {rel:.3e} > {IMG_RTOL}"


@pytest.mark.parametrize("name", sorted(cases.gen_cases()) + ["cube"])
def test_generation_bit_exact(cuda, name):
    c = cases.cube_case() if name == "cube" else cases.gen_cases()[name]
    g = _generator(c)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = g.run_generation()
    gold = _gold(f"gen_{name}.npz")
    n_lab = int(np.sum(lab != gold["label"]))
    n_vec = int(np.sum(vec.view(np.uint32) != gold["vector"].view(np.uint32)))
    REPORT[f"gen/{name}"] = {"label_mismatch": n_lab, "vector_mismatch": n_vec}
    assert n_lab == 0 and n_vec == 0
    assert np.array_equal(props, gold["props"])


def test_generation_only_label_and_warnings(cuda):
    c = cases.gen_cases()["edges"]
    g = _generator(c)
    with pytest.warns(UserWarning) as rec:
        lab, vec, _ = g.run_generation(only_label=True)
    msgs = {str(r.message) for r in rec}
    assert "fiber object with only single point" in msgs
    assert "objects overlap" in msgs
    assert vec.size == 0
    assert np.array_equal(lab, _gold("gen_edges.npz")["label"])


def test_generation_device_path_matches_host_path(cuda):
    torch = cuda
    c = cases.gen_cases()["edges"]
    g = _generator(c)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props, w = g.run_generation_device()
        ws = torch.empty(g.workspace_size(), dtype=torch.uint8, device="cuda")
        lab2, vec2, _, _ = g.run_generation_device(workspace=ws)
    torch.cuda.synchronize()
    gold = _gold("gen_edges.npz")
    for lb, vc in ((lab, vec), (lab2, vec2)):
        assert np.array_equal(lb.cpu().numpy(), gold["label"])
        assert np.array_equal(vc.cpu().numpy().view(np.uint32), gold["vector"].view(np.uint32))


@pytest.mark.parametrize("wname", ["parallel_x", "crossing_small"])
def test_synthetic_generation_digest(cuda, wname):
    man = json.load(open(os.path.join(cases.GOLDEN, "manifest.json")))["generation"][wname]
    w = cases.synth.parallel_x() if wname == "parallel_x" else cases.crossing_small()
    g = _generator(cases.synth_case(w))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = g.run_generation()
    assert hashlib.sha256(lab.tobytes()).hexdigest() == man["label_sha256"]
    assert hashlib.sha256(vec.tobytes()).hexdigest() == man["vector_sha256"]
    assert int((lab > 0).sum()) == man["tissue_voxels"]


@pytest.mark.parametrize("name", sorted(cases.sim_cases()))
def test_simulation_matches_reference(cuda, name):
    gname, kw, tilts = cases.sim_cases()[name]
    g = _gold(f"gen_{gname}.npz")
    ref = _gold(f"sim_{name}.npz")["images"]
    sim = _simulator(kw)
    dim = g["label"].shape
    for k, (t, p) in enumerate(tilts):
        img = sim.run_simulation(dim, g["label"], g["vector"], g["props"], t, p)
        _check_images(f"sim/{name}/{k}", img, ref[k])


@pytest.mark.parametrize("wname", ["parallel_x", "crossing_small"])
def test_synthetic_simulation_matches_reference(cuda, wname):
    sub = np.load(os.path.join(cases.GOLDEN, "synth_images.npz"))
    w = cases.synth.parallel_x() if wname == "parallel_x" else cases.crossing_small()
    g = _generator(cases.synth_case(w))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lab, vec, props = g.run_generation()
    for key in sub.files:
        name, interp, t, p = key.split("|")
        if name != wname:
            continue
        sim = _simulator(dict(w.setup_kwargs(), interpolate=interp))
        img = sim.run_simulation(lab.shape, lab, vec, props, float(t), float(p))
        _check_images(f"synth/{key}", img[::7, ::7], sub[key])


def test_rofl_voxel(cuda):
    tissue, axis, props, tilts, setups = cases.rofl_voxel()
    ref = _gold("rofl_voxel.npz")["images"]
    for k, ((t, p), kw) in enumerate(zip(tilts, setups)):
        img = _simulator(kw).run_simulation(tissue.shape, tissue, axis, props, t, p)
        _check_images(f"rofl/{k}", img, ref[k])


def test_device_path_and_fused_epa(cuda, oracle_port):
    torch = cuda
    name = "cube-Slerp"
    gname, kw, tilts = cases.sim_cases()[name]
    g = _gold(f"gen_{gname}.npz")
    ref = _gold(f"sim_{name}.npz")["images"]
    sim = _simulator(kw)
    lab = torch.from_numpy(g["label"]).cuda()
    vec = torch.from_numpy(g["vector"]).cuda()
    for k, (t, p) in enumerate(tilts):
        img, tt, dd, rr = sim.run_simulation_device(lab.shape, lab, vec, g["props"], t, p,
                                                    epa=True)
        torch.cuda.synchronize()
        _check_images(f"device/{name}/{k}", img.cpu().numpy(), ref[k])
        et, ed, er = oracle_port.epa(ref[k])
        trel = _rel(tt.cpu().numpy(), et)
        rrel = float(np.max(np.abs(rr.cpu().numpy() - er) / np.maximum(np.abs(er), 1e-3)))
        # direction is only defined where the pixel has retardation: on
        # uniform (background) pixels a1 = b1 = 0 up to rounding and
        # atan2 returns noise in both implementations
        defined = er > 1e-2
        dd_ = np.abs(dd.cpu().numpy() - ed)[defined]
        derr = float(np.max(np.minimum(dd_, np.pi - dd_))) if dd_.size else 0.0
        REPORT[f"epa/{name}/{k}"] = {"t_rel": trel, "r_rel": rrel, "d_abs": derr}
        assert trel <= EPA_TOL and rrel <= EPA_TOL and derr <= EPA_TOL


def test_tilts_on_streams_match_single_calls(cuda):
    """run_tilts_device spreads the tilts of one resident volume over the
    library's streams (7 tilts: the streams are shared).  Every image and
    epa map is bit-identical to that tilt's own run_simulation_device call,
    warnings come per tilt, and a label outside the property table raises."""
    torch = cuda
    gname, kw, tilts = cases.sim_cases()["cube-Slerp"]
    g = _gold(f"gen_{gname}.npz")
    sim = _simulator(kw)
    lab = torch.from_numpy(g["label"]).cuda()
    vec = torch.from_numpy(g["vector"]).cuda()
    many = [tuple(t) for t in tilts] + [(np.deg2rad(30.0), np.deg2rad(45.0)),
                                        (np.deg2rad(60.0), np.deg2rad(200.0))]
    res = sim.run_tilts_device(lab.shape, lab, vec, g["props"], many, epa=True)
    for k, (t, p) in enumerate(many):
        one = sim.run_simulation_device(lab.shape, lab, vec, g["props"], t, p, epa=True)
        for a, b in zip(res[k], one):
            assert torch.equal(a.view(torch.int64), b.view(torch.int64)), k
    plain = sim.run_tilts_device(lab.shape, lab, vec, g["props"], many)
    assert all(torch.equal(a, r[0]) for a, r in zip(plain, res))
    scaled = vec.clone()
    scaled[lab > 0] *= 1.0001
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        sim.run_tilts_device(lab.shape, lab, scaled, g["props"], many[:2])
    assert sum("not normalized" in str(x.message) for x in w) == 2
    with pytest.raises(ValueError, match="label"):
        sim.run_tilts_device(lab.shape, lab, vec, g["props"][:2], many)
    again = sim.run_tilts_device(lab.shape, lab, vec, g["props"], many[:1])
    assert torch.equal(again[0], res[0][0])


def test_axis_warnings(cuda):
    """simpli_test.py:327-358: no warning for unit axes, UserWarning for a
    1.0001-scaled axis and for a zero axis."""
    g = _gold("gen_layered_x.npz")
    sim = _simulator(dict(voxel_size=1.0, untilt_sensor_view=False,
                          filter_rotations=cases.ROT6))
    lab, vec, props = g["label"], g["vector"].copy(), g["props"]
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        sim.run_simulation(lab.shape, lab, vec, props, 0, 0)
        assert len(w) == 0
    vec[lab > 0, :] *= 1.0001
    with pytest.warns(UserWarning, match="not normalized"):
        sim.run_simulation(lab.shape, lab, vec, props, 0, 0)
    vec[:] = 0
    with pytest.warns(UserWarning, match="optical_axis is 0"):
        sim.run_simulation(lab.shape, lab, vec, props, 0, 0)


def test_label_range_errors(cuda):
    g = _gold("gen_layered_x.npz")
    sim = _simulator(dict(filter_rotations=cases.ROT6))
    with pytest.raises(ValueError, match="label exceed"):
        sim.run_simulation(g["label"].shape, g["label"], g["vector"], g["props"][:2], 0, 0)
    bad = g["label"].copy()
    bad[3, 3, 3] = -1
    with pytest.raises(ValueError, match="label < 0"):
        sim.run_simulation(bad.shape, bad, g["vector"], g["props"], 0, 0)
    # the library stays usable afterwards
    img = sim.run_simulation(g["label"].shape, g["label"], g["vector"], g["props"], 0, 0)
    assert np.all(np.isfinite(img))


def test_results_are_deterministic(cuda):
    w = cases.crossing_small()
    g = _generator(cases.synth_case(w))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        a = g.run_generation()
        b = g.run_generation()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    sim = _simulator(w.setup_kwargs())
    i1 = sim.run_simulation(a[0].shape, a[0], a[1], a[2], np.deg2rad(5.5), np.deg2rad(90))
    i2 = sim.run_simulation(a[0].shape, a[0], a[1], a[2], np.deg2rad(5.5), np.deg2rad(90))
    assert np.array_equal(i1, i2)
