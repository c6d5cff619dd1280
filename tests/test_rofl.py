"""ROFL tilt analysis (src/fastpli/analysis/rofl.py, _ROFL_with_jacobi.py).

CPU: the oracle (oracle/rofl.py, scipy's MINPACK as the reference calls it)
is pinned bit for bit to the reference's own ROFL code on the golden pixels
(tests/golden/rofl.npz, made by tests/golden/make_rofl_golden.py), and
reproduces the known answer of tests/analysis/rofl_test.py.
GPU (rofl.cu, one thread per pixel, FP64, MINPACK's lmdif / lmder restated
with the reference's tolerances, scaling and evaluation budget):
  * the rofl_test voxel: direction 0/180 deg within 1e-10, inclination
    +-45 deg within 1e-9, t_rel within 1e-8 of the analytic value (the
    reference test's own bounds);
  * noise-free pixels: the true parameters within 1e-12, the reference within
    1e-10;
  * noisy pixels, forward differences (grad_mode=False): parameters within
    1e-5 of the reference, chi^2 within 1e-9 relative, standard deviations
    within 1e-4 relative, the same evaluation count on at least 95% of the
    pixels.  The forward-difference Jacobian divides last-bit differences
    between CUDA's and numpy's FP64 trigonometry by h ~ 1.5e-8, so the
    iterates part at the 1e-8 level and MINPACK's stopping tests
    (xtol = ftol = 1.49e-8) may end one step apart; measured on GB300:
    2.3e-6, 7.6e-11, 8.9e-6, 1 pixel of 192;
  * grad_mode=True (the reference's own Jacobian, lmder): no finite
    differences, so the fit follows the reference's to rounding: parameters
    within 1e-12, chi^2 and deviations within 1e-11 relative on the noisy
    sets, the same evaluation count on every pixel;
  * 18 rotations (the kernel's instantiation for more than 10), against the
    oracle run in the test: measured 1.2e-7 (forward differences) and
    1.5e-14 (grad_mode), every evaluation count equal.
"""

import os
import warnings

import numpy as np
import pytest

from oracle import rofl as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rofl.npz")
SETS = ["voxel", "clean6", "noisy6", "clean9", "noisy9"]
TAU = np.deg2rad(5.5)


def gold():
    return np.load(GOLDEN)


def angdist(a, b, period):
    d = np.abs(np.asarray(a) - np.asarray(b)) % period
    return np.minimum(d, period - d)


# ---------------------------------------------------------------- CPU ---
@pytest.mark.parametrize("name", SETS)
@pytest.mark.parametrize("grad", [0, 1])
def test_oracle_matches_reference_rofl(name, grad):
    g = gold()
    got = np.array([O.rofl(d, TAU, 3, 0, bool(grad)) for d in g[name + "|in"]])
    assert np.array_equal(got, g[f"{name}|grad{grad}|out"])


def test_oracle_known_answer_voxel():
    d, a, t = O.rofl(gold()["voxel|in"][0], TAU, 3, 0, False)[:3]
    t_ref = 4 * 60 * 0.001 / 0.525  # rofl_test.py:49-50
    assert min(abs(d), abs(d - np.pi)) < 1e-10
    assert min(abs(a - np.pi / 4), abs(a + np.pi / 4)) < 1e-9
    assert abs(t - t_ref) < 1e-8


# ---------------------------------------------------------------- GPU ---
def _device(torch, data, grad=False):
    from fastpli_gb300 import analysis
    d = torch.from_numpy(np.ascontiguousarray(data.transpose(1, 0, 2)[:, :, None, :])).cuda()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return analysis.rofl_device(d, TAU, 3, 0, grad)[:, 0].cpu().numpy()


@pytest.mark.gpu
def test_device_known_answer_voxel(cuda):
    """tests/analysis/rofl_test.py through Simpli.apply_rofl."""
    torch = cuda
    from fastpli_gb300.simpli import Simpli
    s = Simpli()
    s.tilts = np.deg2rad([(0, 0), (5.5, 0), (5.5, 90), (5.5, 180), (5.5, 270)])
    imgs = gold()["voxel|in"][0][:, None, None, :]
    d, a, t, (dd, ad, td, chi, nfev) = s.apply_rofl(imgs)
    t_ref = 4 * 60 * 0.001 / 0.525
    assert min(abs(d[0, 0]), abs(d[0, 0] - np.pi)) < 1e-10
    assert min(abs(a[0, 0] - np.pi / 4), abs(a[0, 0] + np.pi / 4)) < 1e-9
    assert abs(t[0, 0] - t_ref) < 1e-8
    with pytest.raises(ValueError, match="not suitable"):
        s.tilts = np.deg2rad([(0, 0), (5.5, 0)])
        s.apply_rofl(imgs)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["clean6", "clean9"])
def test_device_noise_free_pixels(cuda, name):
    g = gold()
    out = _device(cuda, g[name + "|in"])
    truth, ref = g[name + "|truth"], g[name + "|grad0|out"]
    assert angdist(out[:, 0], truth[:, 0], np.pi).max() < 1e-12
    assert np.abs(out[:, 2] - truth[:, 2]).max() < 1e-12
    assert angdist(out[:, 0], ref[:, 0], np.pi).max() < 1e-10
    assert np.abs(out[:, 1] - ref[:, 1]).max() < 1e-10
    assert np.abs(out[:, 2] - ref[:, 2]).max() < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["noisy6", "noisy9"])
def test_device_noisy_pixels(cuda, name):
    import parity
    g = gold()
    out = _device(cuda, g[name + "|in"])
    ref = g[name + "|grad0|out"]
    dev = max(angdist(out[:, 0], ref[:, 0], np.pi).max(), np.abs(out[:, 1] - ref[:, 1]).max(),
              np.abs(out[:, 2] - ref[:, 2]).max())
    chi = (np.abs(out[:, 6] - ref[:, 6]) / ref[:, 6]).max()
    std = (np.abs(out[:, 3:6] - ref[:, 3:6]) / np.abs(ref[:, 3:6])).max()
    same_nfev = float(np.mean(out[:, 7] == ref[:, 7]))
    parity.record(f"rofl/{name}/lmdif", param_abs=float(dev), chi2_rel=float(chi),
                  std_rel=float(std), nfev_equal_frac=same_nfev)
    assert dev < 1e-5
    assert chi < 1e-9
    assert std < 1e-4
    assert same_nfev >= 0.95


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["clean6", "noisy6", "clean9", "noisy9"])
def test_device_grad_mode_matches_reference(cuda, name):
    import parity
    g = gold()
    out = _device(cuda, g[name + "|in"], grad=True)
    ref = g[name + "|grad1|out"]
    dev = max(angdist(out[:, 0], ref[:, 0], np.pi).max(), np.abs(out[:, 1] - ref[:, 1]).max(),
              np.abs(out[:, 2] - ref[:, 2]).max())
    assert np.array_equal(out[:, 7], ref[:, 7])
    assert dev < 1e-12
    if name.startswith("noisy"):  # noise-free chi^2 and deviations are rounding noise
        chi = (np.abs(out[:, 6] - ref[:, 6]) / ref[:, 6]).max()
        std = (np.abs(out[:, 3:6] - ref[:, 3:6]) / np.abs(ref[:, 3:6])).max()
        parity.record(f"rofl/{name}/lmder", param_abs=float(dev), chi2_rel=float(chi),
                      std_rel=float(std))
        assert chi < 1e-11 and std < 1e-11


@pytest.mark.gpu
def test_device_many_rotations_match_oracle(cuda):
    """18 rotations (the kernel's instantiation for more than 10): seeded
    noisy pixels of the model, the device fit against the oracle's scipy
    MINPACK fit of the same pixels, both Jacobian modes, at the bars of the
    6- and 9-rotation goldens."""
    import parity
    rng = np.random.default_rng(91)
    R, n = 18, 24
    mats = O.tilt_matrices(4, TAU)
    data = np.empty((n, 5, R))
    for i in range(n):
        p = (rng.uniform(0, np.pi), rng.uniform(-0.45 * np.pi, 0.45 * np.pi),
             rng.uniform(0.05, 0.8))
        m = O.model(*O.tilted_params(*p, mats, TAU), R, 0).reshape(5, R)
        data[i] = rng.negative_binomial(6500.0 * (1.0 + m) / 2, 1 / 3)
    for grad in (False, True):
        out = _device(cuda, data, grad=grad)
        ref = np.array([O.rofl(d, TAU, 3, 0, grad) for d in data], dtype=np.float64)
        dev = max(angdist(out[:, 0], ref[:, 0], np.pi).max(),
                  np.abs(out[:, 1:3] - ref[:, 1:3]).max())
        same_nfev = float(np.mean(out[:, 7] == ref[:, 7]))
        parity.record(f"rofl/rot18/grad{int(grad)}", param_abs=float(dev),
                      nfev_equal_frac=same_nfev)
        if grad:
            assert dev < 1e-12 and same_nfev == 1.0
        else:
            assert dev < 1e-5 and same_nfev >= 0.9


@pytest.mark.gpu
def test_device_maps_and_mask(cuda):
    """Whole maps [5, X, Y, R] with a mask: masked pixels are NaN, the rest
    equal the per-pixel results."""
    torch = cuda
    from fastpli_gb300 import analysis
    g = gold()
    data = g["noisy6|in"][:12]                      # [12, 5, 6]
    maps = data.transpose(1, 0, 2).reshape(5, 3, 4, 6)
    mask = np.ones((3, 4), bool)
    mask[1, 2] = False
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out = analysis.rofl_device(torch.from_numpy(np.ascontiguousarray(maps)).cuda(),
                                   mask=mask).cpu().numpy()
    single = _device(torch, data).reshape(3, 4, 8)
    assert np.all(np.isnan(out[1, 2]))
    keep = mask
    assert np.array_equal(out[keep], single[keep])
