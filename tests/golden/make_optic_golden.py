"""Generates tests/golden/optic.npz by running the REFERENCE's own optic code
(src/fastpli/simulation/optic.py: filter, resample, filter_resample) on
seeded image stacks, the way Simpli.apply_optic_resample applies it
(__simpli.py:529-548: every polarizer angle separately).

numba is not installed here, so the reference module is executed from its
source text with the ``@numba.njit(cache=True)`` decorator removed (the
function body is plain Python; numba only compiles it).  scipy provides the
Gaussian filter exactly as the reference calls it.

    python tests/golden/make_optic_golden.py [--ref-root /root/reference]
"""

import argparse
import os
import types

import numpy as np
import scipy.ndimage

HERE = os.path.dirname(os.path.abspath(__file__))

# (name, X, Y, n_rho, sigma, scale): the reference pipeline test
# (simpli_test.py:261-280: optical_sigma 0.71, voxel 1 um, pixel 2 um), the
# configs' voxel = pixel case, non-integer scales, a half-way size (5 * 0.5
# rounds to 2), a wide kernel on a short axis (repeated reflection), no
# filter, and scale > 1 (output pixels that receive no input are NaN)
CASES = [
    ("pipeline", 40, 36, 6, 0.71, 0.5),
    ("same_size", 33, 17, 9, 0.71, 1.0),
    ("scale_0.15", 61, 47, 3, 0.71, 0.2 / 1.33),
    ("half_round", 5, 7, 2, 0.71, 0.5),
    ("wide_kernel", 6, 40, 2, 3.0, 0.25),
    ("no_filter", 20, 18, 4, 0.0, 0.5),
    ("upscale", 9, 8, 2, 0.5, 1.7),
]


def reference_optic(ref_root):
    path = os.path.join(ref_root, "src", "fastpli", "simulation", "optic.py")
    src = open(path).read()
    src = src.replace("import numba\n", "").replace("@numba.njit(cache=True)\n", "")
    mod = types.ModuleType("reference_optic")
    # the reference calls scipy.ndimage.filters.gaussian_filter
    scipy_ns = types.SimpleNamespace(ndimage=types.SimpleNamespace(
        filters=types.SimpleNamespace(gaussian_filter=scipy.ndimage.gaussian_filter),
        fourier_gaussian=scipy.ndimage.fourier_gaussian, zoom=scipy.ndimage.zoom))
    exec(compile(src, path, "exec"), mod.__dict__)
    mod.scipy = scipy_ns
    return mod


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default="/root/reference")
    args = ap.parse_args()
    optic = reference_optic(args.ref_root)
    out = {}
    rng = np.random.default_rng(2024)
    for name, X, Y, R, sigma, scale in CASES:
        img = rng.uniform(3000.0, 9000.0, (X, Y, R))
        res = np.stack([optic.filter_resample(img[:, :, i], sigma, scale) for i in range(R)], -1)
        out[f"{name}|in"] = img
        out[f"{name}|out"] = res
        out[f"{name}|par"] = np.array([sigma, scale])
    np.savez_compressed(os.path.join(HERE, "optic.npz"), **out)
    print("wrote", os.path.join(HERE, "optic.npz"), len(CASES), "cases")


if __name__ == "__main__":
    main()
