"""Reference digests for a volume past the 32-bit index range, made by running
the REFERENCE's own C++ (oracle/_ref/libpliref.so, built from the reference
sources by ``make -C oracle ref``) on fastpli_gb300.synth.wide_strip():
5504 x 16384 x 16 voxels at 1 um, all tissue in the last 32 x-columns.

Recorded (wide_manifest.json, wide_images.npz):
  * sha256 of the label and vector fields of the last 32 x-columns, the
    tissue voxel count of the whole volume, and that every voxel outside the
    strip is background (label 0, vector 0);
  * per tilt, the mean of the whole image stack and the image rows x = 0 and
    x = x0, x0 + 8, x0 + 16, x0 + 24 (x0 = 5472) at every 64th y.

Needs ~32 GB of host memory and ~2 minutes on 8 cores.

    python tests/golden/make_wide_golden.py [--threads 8]
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

Y_STRIDE = 64
ROW_OFFSETS = (0, 8, 16, 24)


def sample_rows(x0):
    return [0] + [x0 + k for k in ROW_OFFSETS]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    oracle.build(ref=True)
    w = synth.wide_strip()
    x0 = int(w.dim[0]) - synth.WIDE_STRIP
    lab, vec, props, warn = oracle.generate(w.dim, w.origin, w.voxel_size, w.bundles, w.layers,
                                            n_threads=args.threads, impl="ref")
    outside_zero = not lab[:x0].any() and not vec[:x0].view(np.int32).any()
    entry = {"strip_x0": x0,
             "strip_label_sha256": hashlib.sha256(lab[x0:].tobytes()).hexdigest(),
             "strip_vector_sha256": hashlib.sha256(vec[x0:].tobytes()).hexdigest(),
             "tissue_voxels": int(np.count_nonzero(lab)), "outside_strip_zero": outside_zero,
             "warnings": warn, "props": props.tolist(), "y_stride": Y_STRIDE,
             "rows": sample_rows(x0), "tilts": [list(map(float, t)) for t in w.tilts],
             "image_mean": []}
    images = {}
    kw = w.setup_kwargs()
    for k, (t, p) in enumerate(w.tilts):
        img, _ = oracle.simulate(lab, vec, props, t, p, n_threads=args.threads, impl="ref", **kw)
        entry["image_mean"].append(float(img.mean()))
        images[f"wide|{k}"] = np.ascontiguousarray(img[entry["rows"], ::Y_STRIDE])
        del img
    with open(os.path.join(HERE, "wide_manifest.json"), "w") as f:
        json.dump({"wide": entry}, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "wide_images.npz"), **images)
    print(entry["strip_label_sha256"][:16], entry["tissue_voxels"], outside_zero)


if __name__ == "__main__":
    main()
