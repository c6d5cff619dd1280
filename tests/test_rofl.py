"""ROFL tilt analysis (src/fastpli/analysis/rofl.py, _ROFL_with_jacobi.py).

CPU: the oracle (oracle/rofl.py, scipy's MINPACK as the reference calls it)
is pinned bit for bit to the reference's own ROFL code on the golden pixels
(tests/golden/rofl.npz, made by tests/golden/make_rofl_golden.py), and
reproduces the known answer of tests/analysis/rofl_test.py.
GPU (rofl.cu, one warp per pixel, FP64, its own Levenberg-Marquardt on the
same objective with its exact Jacobian):
  * the rofl_test voxel: direction 0/180 deg within 1e-10, inclination
    +-45 deg within 1e-9, t_rel within 1e-8 of the analytic value (the
    reference test's own bounds);
  * noise-free pixels: the true parameters within 1e-12, the reference within
    1e-10;
  * noisy pixels: chi^2 no worse than the reference's by more than 1e-12
    relative (the fit converges at least as far), parameters within 1e-3 of
    the reference (MINPACK's xtol/ftol stop leaves it up to ~5e-4 away from
    the minimum along flat directions), standard deviations within 1e-2.
grad_mode=True uses the reference's approximate Jacobian (derivatives with
respect to each tilt's own angles, not the fit parameters); where that
iteration ends depends on the optimizer's path, so only finiteness is tested
for it."""

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
    g = gold()
    out = _device(cuda, g[name + "|in"])
    ref = g[name + "|grad0|out"]
    assert np.all(out[:, 6] <= ref[:, 6] * (1 + 1e-12))
    assert angdist(out[:, 0], ref[:, 0], np.pi).max() < 1e-3
    assert np.abs(out[:, 1] - ref[:, 1]).max() < 1e-3
    assert np.abs(out[:, 2] - ref[:, 2]).max() < 1e-3
    rel = np.abs(out[:, 3:6] - ref[:, 3:6]) / np.abs(ref[:, 3:6])
    assert rel.max() < 1e-2
    assert np.all(out[:, 7] > 0)


@pytest.mark.gpu
def test_device_grad_mode_runs(cuda):
    g = gold()
    out = _device(cuda, g["noisy9|in"], grad=True)
    assert np.all(np.isfinite(out))
    assert np.all((out[:, 0] >= 0) & (out[:, 0] < np.pi))


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
