"""Pins the oracle (the C restatement in oracle/pli_oracle.c) against the
reference: golden fixtures produced by the reference's own C++
(tests/golden/make_golden.py) and the analytic known-answer checks of the
reference's tests (tests/simulation/simpli_test.py:31-218)."""

import hashlib
import json
import os

import numpy as np
import pytest

import cases

GOLD = cases.GOLDEN


def _gold(name):
    return np.load(os.path.join(GOLD, name))


def _gen(oracle_port, c, **kw):
    return oracle_port.generate(c["dim"], c["origin"], c["voxel_size"], c["bundles"],
                                c["layers"], **kw)


@pytest.mark.parametrize("name", sorted(cases.gen_cases()) + ["cube"])
def test_port_generation_matches_reference(oracle_port, name):
    c = cases.cube_case() if name == "cube" else cases.gen_cases()[name]
    lab, vec, props, warn = _gen(oracle_port, c)
    g = _gold(f"gen_{name}.npz")
    assert np.array_equal(lab, g["label"])
    assert np.array_equal(vec.view(np.uint32), g["vector"].view(np.uint32))
    assert np.array_equal(props, g["props"])
    assert warn["overlap"] == int(g["warnings"][0] > 0)
    assert warn["single_point"] == int(g["warnings"][1])


def test_port_only_label_matches(oracle_port):
    c = cases.gen_cases()["polyline"]
    l0, v0, p0, _ = _gen(oracle_port, c, only_label=True)
    l1, v1, p1, _ = _gen(oracle_port, c)
    assert v0.size == 0
    assert np.array_equal(l0, l1)
    assert p1.shape == (4, 2)  # simpli_test.py:61


def test_port_multithreaded_generation_is_deterministic(oracle_port):
    c = cases.gen_cases()["edges"]
    a = _gen(oracle_port, c, n_threads=1)
    b = _gen(oracle_port, c, n_threads=4)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[1], b[1])


def test_kat_radial(oracle_port):
    """simpli_test.py:65-103: label 1 iff inside the circle; radial vector."""
    c = cases.gen_cases()["radial"]
    lab, vec, _, _ = _gen(oracle_port, c)
    x, y, r = 0 / 0.1, 0.25 / 0.1, 1 / 0.1
    for k in range(lab.shape[2]):
        assert np.array_equal(lab[:, :, 0], lab[:, :, k])
    for i in range(lab.shape[0]):
        for j in range(lab.shape[1]):
            t = 0 if (x - (i + 0.5)) ** 2 + (y - (j + 0.5)) ** 2 > r ** 2 else 1
            assert lab[i, j, 0] == t
            if t:
                phi = np.arctan2((j + 0.5) - y, (i + 0.5) - x)
                np.testing.assert_array_almost_equal(vec[i, j, 0], [np.cos(phi), np.sin(phi), 0],
                                                     decimal=6)


def test_kat_layered(oracle_port):
    """simpli_test.py:143-196: layer radii 0.3/0.6/1.0 r -> labels 1/2/3."""
    c = cases.gen_cases()["layered"]
    lab, vec, _, _ = _gen(oracle_port, c)
    x, y, r = 0.0, 2.5, 10.0
    for i in range(lab.shape[0]):
        for j in range(lab.shape[1]):
            rr = (x - (i + 0.5)) ** 2 + (y - (j + 0.5)) ** 2
            if rr > r ** 2:
                assert lab[i, j, 0] == 0
            elif np.sqrt(rr) < 0.3 * r:
                assert lab[i, j, 0] == 1
                np.testing.assert_array_almost_equal(vec[i, j, 0], [0, 0, 1], decimal=6)
            elif np.sqrt(rr) < 0.6 * r:
                assert lab[i, j, 0] == 2
                assert np.array_equal(vec[i, j, 0], [0, 0, 0])
            else:
                assert lab[i, j, 0] == 3


def test_kat_dimension(oracle_port):
    """simpli_test.py:31-46: tissue == int(optical_axis[..., 2])."""
    c = cases.gen_cases()["dimension"]
    lab, vec, props, _ = _gen(oracle_port, c)
    assert lab.shape == (3, 5, 7) and vec.shape == (3, 5, 7, 3)
    assert props.shape == (2, 2)
    assert np.array_equal(lab, np.array(vec[..., 2], dtype=int))


@pytest.mark.parametrize("name", sorted(cases.sim_cases()))
def test_port_simulation_matches_reference(oracle_port, name):
    gname, kw, tilts = cases.sim_cases()[name]
    g = _gold(f"gen_{gname}.npz")
    ref = _gold(f"sim_{name}.npz")["images"]
    for k, (t, p) in enumerate(tilts):
        img, _ = oracle_port.simulate(g["label"], g["vector"], g["props"], t, p, **kw)
        np.testing.assert_allclose(img, ref[k], rtol=1e-12, atol=0)


def test_port_rofl_voxel_matches_reference_and_known_answer(oracle_port):
    tissue, axis, props, tilts, setups = cases.rofl_voxel()
    ref = _gold("rofl_voxel.npz")["images"]
    for k, ((t, p), kw) in enumerate(zip(tilts, setups)):
        img, _ = oracle_port.simulate(tissue, axis, props, t, p, **kw)
        np.testing.assert_allclose(img, ref[k], rtol=1e-12)
    # theta = 0: one voxel of retardance ret = pi/2 * d_rel * cos^2(45°)
    t, d, r = oracle_port.epa(ref[0])
    v = axis[0, 0, 0].astype(np.float64)
    n = np.sqrt(v @ v)
    d_rel = 0.001 * 4 * 60e-6 / 525e-9 * n
    ret = np.pi / 2 * d_rel * (v[0] ** 2 + v[1] ** 2) / n ** 2
    assert abs(t[0, 0] - 13000.0) < 1e-8
    assert abs(r[0, 0] - abs(np.sin(ret))) < 1e-12
    assert min(d[0, 0], np.pi - d[0, 0]) < 1e-12


@pytest.mark.parametrize("wname", ["parallel_x", "crossing_small"])
def test_port_synthetic_digests(oracle_port, wname):
    man = json.load(open(os.path.join(GOLD, "manifest.json")))
    sub = np.load(os.path.join(GOLD, "synth_images.npz"))
    w = cases.synth.parallel_x() if wname == "parallel_x" else cases.crossing_small()
    lab, vec, props, warn = _gen(oracle_port, cases.synth_case(w), n_threads=4)
    m = man["generation"][wname]
    assert hashlib.sha256(lab.tobytes()).hexdigest() == m["label_sha256"]
    assert hashlib.sha256(vec.tobytes()).hexdigest() == m["vector_sha256"]
    assert np.array_equal(props, np.array(m["props"]))
    for key in sub.files:
        name, interp, t, p = key.split("|")
        if name != wname:
            continue
        kw = dict(w.setup_kwargs(), interpolate=interp)
        img, _ = oracle_port.simulate(lab, vec, props, float(t), float(p), n_threads=4, **kw)
        np.testing.assert_allclose(img[::7, ::7], sub[key], rtol=1e-12)


def test_port_rejects_invalid_input(oracle_port):
    g = _gold("gen_layered_x.npz")
    with pytest.raises(ValueError, match="background birefringence"):
        bad = g["props"].copy()
        bad[0, 0] = 0.1
        oracle_port.simulate(g["label"], g["vector"], bad, 0, 0)
    with pytest.raises(ValueError, match="label exceed"):
        oracle_port.simulate(g["label"], g["vector"], g["props"][:2], 0, 0)
    with pytest.raises(ValueError, match="step_size"):
        oracle_port.simulate(g["label"], g["vector"], g["props"], 0, 0, step_size=0)


def test_step_count_on_the_host_matches_the_library():
    """oracle.count_steps (the reference's z loop replayed in Python, used by
    the CPU arm of bench.py, which loads nothing of the product) agrees with
    the library's planner."""
    import oracle
    from fastpli_gb300 import _native as N
    lib = N.load()
    for dim in ((512, 512, 120), (64, 80, 30), (3, 5, 7), (100, 7, 119)):
        for step in (1.0, 0.7, 1.0 / np.cos(np.deg2rad(5.5))):
            for th, ph in np.deg2rad([(0, 0), (5.5, 0), (5.5, 270), (30, 45), (60, 200)]):
                s = N.SetupBlock(step, 26000.0, 0.2, 525.0, 1.0, "Slerp", True, False,
                                 np.deg2rad([0, 90]))
                d = np.asarray(dim, np.int64)
                want = int(lib.fpgb_count_steps(N.byref(s.struct), N.ptr(d), float(th), float(ph)))
                assert oracle.count_steps(dim, th, step) == want, (dim, step, th)
