"""Optic stage (src/fastpli/simulation/optic.py) and epa on image stacks.

CPU: the oracle (oracle/optic.py) is pinned bit for bit to scipy's
gaussian_filter and to the reference's own filter_resample
(tests/golden/optic.npz, made by tests/golden/make_optic_golden.py); the
output-size rounding of the C ABI follows Python's round.
GPU: the device kernels (optic.cu) against the oracle — filter + resample
within 1e-13 relative (FP64 in scipy's summation order; the Gaussian weights
come from the host's exp), epa within 1e-12, the negative-binomial noise
against numpy's sampler in distribution, and the whole chain march ->
resample -> epa against the oracle within the march's 1e-4."""

import os

import numpy as np
import pytest
import scipy.ndimage

from fastpli_gb300 import _native as N
from fastpli_gb300 import optic
from oracle import optic as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "optic.npz")


def golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("|")[0] for k in g.files})
    return [(n, g[n + "|in"], g[n + "|out"], float(g[n + "|par"][0]), float(g[n + "|par"][1]))
            for n in names]


# ---------------------------------------------------------------- CPU ---
@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c[0])
def test_oracle_matches_reference_filter_resample(case):
    _, img, ref, sigma, scale = case
    got = O.filter_resample(img, sigma, scale)
    assert np.array_equal(got, ref, equal_nan=True)


@pytest.mark.parametrize("shape,sd", [((37, 23), 1.42), ((5, 3), 2.5), ((64, 64, 3), 0.71),
                                      ((11, 29), 7.3), ((1, 9), 1.0)])
def test_oracle_gaussian_is_scipy(shape, sd):
    a = np.random.default_rng(1).uniform(0, 26000, shape)
    ref = scipy.ndimage.gaussian_filter(a, sd, axes=(0, 1)) if len(shape) == 3 else \
        scipy.ndimage.gaussian_filter(a, sd)
    assert np.array_equal(O.gaussian_filter(a, sd), ref)


def test_resample_size_rounds_half_to_even():
    for n in (1, 2, 3, 5, 7, 40, 511, 512, 1023):
        for scale in (0.5, 0.25, 0.2 / 1.33, 1.0, 1.5, 1.7, 0.1):
            assert optic.resample_size((n, n + 1), scale) == (int(round(n * scale)),
                                                              int(round((n + 1) * scale)))
    with pytest.raises(ValueError):
        optic.resample_size((4, 4), 0.0)


def test_noise_model_arguments_checked():
    with pytest.raises(ValueError):
        optic.NegativeBinomialNoise(gain=1.0)
    with pytest.raises(ValueError):
        optic.NegativeBinomialNoise(gain=float("nan"))


def test_add_noise_mask_semantics():
    img = np.array([[1.0, np.nan], [3.0, 4.0]])
    mask = np.array([[True, True], [False, True]])
    out = optic.add_noise(img, lambda x: x + 10, mask)
    assert out[0, 0] == 11 and np.isnan(out[0, 1]) and out[1, 0] == 3 and out[1, 1] == 14


# ---------------------------------------------------------------- GPU ---
@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c[0])
def test_device_filter_resample_matches_golden(cuda, case):
    torch = cuda
    _, img, ref, sigma, scale = case
    got = optic.filter_resample_device(torch.from_numpy(img).cuda(), sigma, scale).cpu().numpy()
    assert got.shape == ref.shape
    nan = np.isnan(ref)
    assert np.array_equal(nan, np.isnan(got))
    rel = np.abs(got[~nan] - ref[~nan]) / np.abs(ref[~nan])
    assert rel.max(initial=0) <= 1e-13, rel.max()
    # host-buffer entry point and 2-D input
    host = optic.filter_resample(img, sigma, scale)
    assert np.array_equal(host, got, equal_nan=True)
    one = optic.filter_resample(img[:, :, 0], sigma, scale)
    assert np.array_equal(one, got[:, :, 0], equal_nan=True)


@pytest.mark.gpu
def test_device_epa_matches_oracle(cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    rho = np.linspace(0, np.pi, 9, False)
    phi = rng.uniform(0, np.pi, (33, 21, 1))
    img = 5000 + 3000 * rng.uniform(0, 1, (33, 21, 1)) * np.sin(2 * (rho - phi)) \
        + rng.normal(0, 10, (33, 21, 9))
    img[0, 0] = 0.0  # a0 < 100 eps branch
    t, d, r = (x.cpu().numpy() for x in optic.epa_device(torch.from_numpy(img).cuda()))
    rt, rd, rr = O.epa(img)
    assert np.allclose(t, rt, rtol=1e-12, atol=0)
    assert np.allclose(r, rr, rtol=1e-12, atol=1e-15)
    dd = np.abs(d - rd)
    assert np.minimum(dd, np.pi - dd).max() < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("x", [0.4, 3.0, 25.0, 6500.0])
def test_noise_distribution_matches_numpy(cuda, x):
    torch = cuda
    gain, n = 3.0, 400_000
    model = optic.NegativeBinomialNoise(gain, seed=11)
    got = model.device(torch.full((n,), x, dtype=torch.float64, device="cuda")).cpu().numpy()
    ref = np.random.default_rng(5).negative_binomial(x / (gain - 1), 1 / gain, n).astype(float)
    assert np.all(got == np.round(got)) and got.min() >= 0
    # mean x, variance gain * x: 6 standard errors
    se_mean = np.sqrt(gain * x / n)
    assert abs(got.mean() - x) < 6 * se_mean
    var = gain * x
    assert abs(got.var() / var - 1) < 6 * np.sqrt(2.0 / n) * 3
    # two-sample Kolmogorov-Smirnov distance of the discrete distributions
    grid = np.arange(0, max(got.max(), ref.max()) + 1)
    cg = np.searchsorted(np.sort(got), grid, side="right") / n
    cr = np.searchsorted(np.sort(ref), grid, side="right") / n
    assert np.abs(cg - cr).max() < 0.01


@pytest.mark.gpu
def test_noise_is_reproducible_and_offset_addressed(cuda):
    torch = cuda
    img = torch.linspace(100.0, 9000.0, 10_000, dtype=torch.float64, device="cuda")
    a = optic.NegativeBinomialNoise(3.0, seed=7).device(img)
    b = optic.NegativeBinomialNoise(3.0, seed=7).device(img)
    assert torch.equal(a, b)
    # pixel e's draw depends on (seed, offset + e): a shifted window reproduces it
    m = optic.NegativeBinomialNoise(3.0, seed=7)
    full = m.device(img, offset=0)
    m._calls -= 1  # same call index -> same seed
    part = m.device(img[100:], offset=100)
    assert torch.equal(full[100:], part)
    with pytest.raises(ValueError, match="n <= 0"):
        optic.NegativeBinomialNoise(3.0, seed=1).device(torch.zeros(4, dtype=torch.float64,
                                                                    device="cuda"))


@pytest.mark.gpu
def test_march_resample_epa_chain_matches_oracle(cuda):
    """Simpli-style pipeline on the device: march -> apply_optic_resample ->
    epa, against the oracle's FP64 march -> oracle optic -> oracle epa."""
    torch = cuda
    import cases
    import oracle
    from fastpli_gb300.simpli import Simpli
    from fastpli_gb300.simulation import _Simulator
    w = cases.crossing_small()
    kw = w.setup_kwargs()
    lab, vec, props, _ = oracle.generate(w.dim, w.origin, w.voxel_size, w.bundles, w.layers)
    ref, _ = oracle.simulate(lab, vec, props, 0.0, 0.0, **kw)
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"],
                      kw["wavelength"], kw["tissue_refrection"], kw["interpolate"],
                      kw["untilt_sensor_view"], kw["flip_z"], kw["filter_rotations"])
    img = sim.run_simulation_device(w.dim, torch.from_numpy(lab).cuda(),
                                    torch.from_numpy(vec).cuda(), props, 0.0, 0.0)
    s = Simpli()
    s.voxel_size = w.voxel_size
    s.optical_sigma = 0.71
    s.pixel_size = 2 * w.voxel_size
    res = s.apply_optic_resample(img)
    ref_res = O.filter_resample(ref, 0.71, 0.5)
    got = res.cpu().numpy()
    assert got.shape == ref_res.shape
    assert (np.abs(got - ref_res) / np.abs(ref_res)).max() < 1e-4
    t, d, r = (x.cpu().numpy() for x in s.apply_epa_device(res))
    rt, rd, rr = O.epa(ref_res)
    assert np.allclose(t, rt, rtol=1e-4)
    assert np.allclose(r, rr, rtol=1e-3, atol=1e-3)
    # host arrays through the same method give the same result
    host = s.apply_optic_resample(img.cpu().numpy())
    assert np.array_equal(host, got)
    # noise on the device through apply_optic
    s.noise_model = optic.NegativeBinomialNoise(3.0, seed=3)
    resampled, noisy = s.apply_optic(img)
    assert torch.equal(resampled, res)
    assert noisy.shape == res.shape and bool((noisy >= 0).all())
