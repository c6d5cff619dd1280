"""Generates the golden fixtures in this directory by running the REFERENCE's
own C++ (oracle/_ref/libpliref.so, built from the reference sources by
``make -C oracle ref``) on the scenarios of ``tests/cases.py``.

Run in a checkout that has the reference tree (default /root/reference):

    python tests/golden/make_golden.py [--ref-root /root/reference]

Outputs:
  cube_fibers.npz    fibers parsed from the reference's tests/cube.dat
  gen_<case>.npz     label / vector / props of small generation scenarios
  sim_<case>.npz     images per tilt of the simulation scenarios
  rofl_voxel.npz     the single-voxel tilt series of rofl_test.py
  manifest.json      sha256 digests of label/vector for the larger synthetic
                     volumes and mean reference images
  synth_images.npz   every 7th row/column of those reference images
The GPU machine has no reference tree; the tests only read these files.
"""

import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402


def parse_dat(path):
    """.dat fiber format of fastpli.io.fiber_bundles.load_dat
    (src/fastpli/io/fiber_bundles.py:44-80): one 'x y z r' line per point,
    one blank line ends a fiber, two end a bundle."""
    bundles, fiber, blank = [[]], [], 0
    with open(path) as f:
        for line in f:
            if line.strip():
                blank = 0
                fiber.append(list(map(float, line.split()))[:4])
            else:
                blank += 1
                if blank == 1 and fiber:
                    bundles[-1].append(np.array(fiber, float))
                    fiber = []
                elif blank == 2 and bundles[-1]:
                    bundles.append([])
    if fiber:
        bundles[-1].append(np.array(fiber, float))
    return [b for b in bundles if b]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=oracle.REF_ROOT_DEFAULT)
    args = ap.parse_args()
    oracle.build(ref=True, ref_root=args.ref_root)
    if not oracle.available("ref"):
        sys.exit("reference harness could not be built")

    cube = parse_dat(os.path.join(args.ref_root, "tests", "cube.dat"))
    assert len(cube) == 1
    np.savez_compressed(os.path.join(HERE, "cube_fibers.npz"),
                        **{f"f{i}": f for i, f in enumerate(cube[0])})

    import cases  # noqa: E402  (reads cube_fibers.npz)
    gens = cases.gen_cases()
    gens["cube"] = cases.cube_case()
    tissue = {}
    for name, c in gens.items():
        lab, vec, props, warn = oracle.generate(c["dim"], c["origin"], c["voxel_size"],
                                                c["bundles"], c["layers"], impl="ref")
        tissue[name] = (lab, vec, props)
        np.savez_compressed(os.path.join(HERE, f"gen_{name}.npz"), label=lab,
                            vector=vec, props=props,
                            warnings=np.array([warn[k] for k in oracle.WARNING_NAMES]))
        print("gen", name, lab.shape, int((lab > 0).sum()), warn)

    manifest = {"generation": {}, "simulation": {}}
    sub_images = {}
    for name, w in (("parallel_x", cases.synth.parallel_x()),
                    ("crossing_small", cases.crossing_small())):
        c = cases.synth_case(w)
        lab, vec, props, warn = oracle.generate(c["dim"], c["origin"], c["voxel_size"],
                                                c["bundles"], c["layers"], impl="ref")
        manifest["generation"][name] = {
            "label_sha256": digest(lab), "vector_sha256": digest(vec),
            "props": props.tolist(), "tissue_voxels": int((lab > 0).sum()),
            "warnings": warn}
        tilts = [(0.0, 0.0), (float(np.deg2rad(5.5)), 0.0),
                 (float(np.deg2rad(5.5)), float(np.deg2rad(90)))]
        for interp in ("NN", "Slerp"):
            kw = dict(w.setup_kwargs(), interpolate=interp)
            for t, p in tilts:
                img, _ = oracle.simulate(lab, vec, props, t, p, impl="ref", n_threads=8,
                                         **kw)
                key = f"{name}|{interp}|{t!r}|{p!r}"
                sub_images[key] = img[::7, ::7]
                manifest["simulation"][key] = {"mean": float(img.mean())}
        print("synth", name, manifest["generation"][name]["tissue_voxels"], warn)

    for name, (gname, kw, tilts) in cases.sim_cases().items():
        lab, vec, props = tissue[gname]
        imgs = []
        for t, p in tilts:
            img, warn = oracle.simulate(lab, vec, props, t, p, impl="ref", **kw)
            imgs.append(img)
        np.savez_compressed(os.path.join(HERE, f"sim_{name}.npz"),
                            images=np.stack(imgs), tilts=np.array(tilts, float))
        print("sim", name, imgs[0].shape)

    tissue_r, axis, props, tilts, setups = cases.rofl_voxel()
    imgs = [oracle.simulate(tissue_r, axis, props, t, p, impl="ref", **kw)[0]
            for (t, p), kw in zip(tilts, setups)]
    np.savez_compressed(os.path.join(HERE, "rofl_voxel.npz"), images=np.stack(imgs))

    np.savez_compressed(os.path.join(HERE, "synth_images.npz"), **sub_images)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("done")


if __name__ == "__main__":
    main()
