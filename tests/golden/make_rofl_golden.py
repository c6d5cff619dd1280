"""Generates tests/golden/rofl.npz by running the REFERENCE's own ROFL code
(src/fastpli/analysis/rofl.py, _ROFL_with_jacobi.py, epa.py) on
  * the single-voxel tilt series of tests/analysis/rofl_test.py (the images
    in rofl_voxel.npz, themselves made by the reference's simulator), and
  * seeded synthetic pixels: the ROFL intensity model of random
    (direction, inclination, t_rel) at 6500 counts, without noise and with
    the pipelines' negative-binomial noise (gain 3), for 6 and 9 rotations,
with grad_mode False (the default) and True.

numba is not installed here, so the reference modules are executed from
their source text with the ``@numba.njit(cache=True)`` decorators removed.

    python tests/golden/make_rofl_golden.py [--ref-root /root/reference]
"""

import argparse
import os
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(path, name, extra=None):
    src = open(path).read()
    src = src.replace("import numba\n", "").replace("@numba.njit(cache=True)\n", "")
    for a, b in (extra or {}).items():
        src = src.replace(a, b)
    mod = types.ModuleType(name)
    exec(compile(src, path, "exec"), mod.__dict__)
    return mod


def reference_rofl(ref_root):
    base = os.path.join(ref_root, "src", "fastpli", "analysis")
    jac = _load(os.path.join(base, "_ROFL_with_jacobi.py"), "ref_rofl_jacobi")
    epa = _load(os.path.join(base, "epa.py"), "ref_epa")
    rofl = _load(os.path.join(base, "rofl.py"), "ref_rofl", {
        "from ._ROFL_with_jacobi import _execute_fit as rofl_fit\n": "",
        "from . import epa\n": ""})
    rofl.rofl_fit = jac._execute_fit
    rofl.epa = epa
    return rofl, jac


def synth_pixels(jac, rng, n, n_rot, noise, tau=np.deg2rad(5.5)):
    mats = jac._list_all_tilt_matrices(4, tau)
    data = np.empty((n, 5, n_rot))
    truth = np.empty((n, 3))
    for i in range(n):
        phi = rng.uniform(0, np.pi)
        alpha = rng.uniform(-0.45 * np.pi, 0.45 * np.pi)
        trel = rng.uniform(0.05, 0.8)
        m = jac._model(np.array([phi, alpha, trel]), mats, tau, n_rot, 0).reshape(5, n_rot)
        img = 6500.0 * (1.0 + m)
        if noise:
            img = rng.negative_binomial(img / (3 - 1), 1 / 3).astype(np.float64)
        data[i] = img
        truth[i] = (phi, alpha, trel)
    return data, truth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default="/root/reference")
    args = ap.parse_args()
    rofl, jac = reference_rofl(args.ref_root)
    rng = np.random.default_rng(77)
    out = {}
    voxel = np.load(os.path.join(HERE, "rofl_voxel.npz"))["images"][:, 0, 0, :]
    sets = {"voxel": (voxel[None], None)}
    for n_rot in (6, 9):
        sets[f"clean{n_rot}"] = synth_pixels(jac, rng, 48, n_rot, False)
        sets[f"noisy{n_rot}"] = synth_pixels(jac, rng, 96, n_rot, True)
    for name, (data, truth) in sets.items():
        for grad in (False, True):
            res = np.array([rofl.rofl(d, np.deg2rad(5.5), 3, 0, grad) for d in data],
                           dtype=np.float64)
            out[f"{name}|grad{int(grad)}|out"] = res
        out[f"{name}|in"] = data
        if truth is not None:
            out[f"{name}|truth"] = truth
    np.savez_compressed(os.path.join(HERE, "rofl.npz"), **out)
    print("wrote", os.path.join(HERE, "rofl.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
