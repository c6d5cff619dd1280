"""Full-size reference digests for the two volumes the benchmarks use, made
by running the REFERENCE's own C++ (oracle/_ref/libpliref.so, built from the
reference sources by ``make -C oracle ref``) on the seeded synthetic inputs
of fastpli_gb300/synth.py:

  crossing  512 x 512 x 120 at 0.2 um, two crossing bundles of 1000 fibers
            (the bench workload); tilts (0, 0), (5.5, 0), (5.5, 90) degrees
  watson    1024 x 1024 x 240 at 0.1 um, 20000 fibers around a Watson axis,
            three layers (the voxelization-heavy volume); tilt (0, 0)

For each: sha256 of the label and vector fields, the tissue voxel count, and
per tilt the mean image and every 16th (crossing) / 32nd (watson) row and
column of the image stack.  Outputs full_manifest.json and full_images.npz.

    python tests/golden/make_full_golden.py [--threads 8]
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

import oracle  # noqa: E402
from fastpli_gb300 import synth  # noqa: E402

VOLUMES = {
    "crossing": (synth.crossing, 16, [(0.0, 0.0), (np.deg2rad(5.5), 0.0),
                                      (np.deg2rad(5.5), np.deg2rad(90.0))]),
    "watson": (synth.watson, 32, [(0.0, 0.0)]),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    oracle.build(ref=True)
    manifest, images = {}, {}
    for name, (make, stride, tilts) in VOLUMES.items():
        w = make()
        lab, vec, props, warn = oracle.generate(w.dim, w.origin, w.voxel_size, w.bundles,
                                                w.layers, n_threads=args.threads, impl="ref")
        entry = {"label_sha256": hashlib.sha256(lab.tobytes()).hexdigest(),
                 "vector_sha256": hashlib.sha256(vec.tobytes()).hexdigest(),
                 "tissue_voxels": int((lab > 0).sum()), "warnings": warn,
                 "stride": stride, "tilts": [list(map(float, t)) for t in tilts],
                 "image_mean": []}
        kw = w.setup_kwargs()
        for k, (t, p) in enumerate(tilts):
            img, _ = oracle.simulate(lab, vec, props, t, p, n_threads=args.threads, impl="ref",
                                     **kw)
            entry["image_mean"].append(float(img.mean()))
            images[f"{name}|{k}"] = np.ascontiguousarray(img[::stride, ::stride])
        manifest[name] = entry
        print(name, entry["label_sha256"][:16], entry["tissue_voxels"], flush=True)
        del lab, vec
    with open(os.path.join(HERE, "full_manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "full_images.npz"), **images)


if __name__ == "__main__":
    main()
