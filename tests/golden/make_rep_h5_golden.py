"""The reference's own golden regression file, as a numpy fixture.

Reads tests/simulation/simpli_rep.h5 of the reference tree — the output of
its tests/simulation/simpli_rep.py (cube.dat fibers, 5 µm voxels, three
layers, Slerp, 5 tilts, optic with a seeded negative-binomial noise, epa and
ROFL), which the reference's simpli_test.py compares with h5diff at
1e-5 relative — with the minimal reader fastpli_gb300/h5read.py (no h5py
here), and
writes every dataset to simpli_rep_h5.npz, "/" in names replaced by ".".

    python tests/golden/make_rep_h5_golden.py [reference root]
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from fastpli_gb300 import h5read  # noqa: E402

REF_ROOT = os.environ.get("FPGB_REFERENCE_ROOT", "/root/reference")


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT
    src = os.path.join(root, "tests", "simulation", "simpli_rep.h5")
    data = h5read.read_all(src)
    out = {k.replace("/", "."): np.ascontiguousarray(v) for k, v in sorted(data.items())}
    np.savez_compressed(os.path.join(HERE, "simpli_rep_h5.npz"), **out)
    for k, v in out.items():
        print(k, v.dtype, v.shape)


if __name__ == "__main__":
    main()
