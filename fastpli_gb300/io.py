"""Fiber-bundle files: the .dat / .txt text format and .h5 groups of
fastpli.io.fiber_bundles (src/fastpli/io/fiber_bundles.py:13-179), same
function names, arguments and file layouts.

Text: one fiber point per line ("x y z radius"), one empty line ends a fiber,
two end a bundle.  HDF5: group "<bundle>" holding datasets "<fiber>" of shape
(n, 4).  .h5 files are read with h5py when it is installed and otherwise with
this package's minimal reader (h5read: files in h5py's default format);
writing .h5 needs h5py.
"""

import os

import numpy as np

from . import objects


def load(file_name, group_name="/"):
    """list(list((n, 4) fiber)) of a .dat / .txt / .h5 file
    (fiber_bundles.py:13-38)."""
    _, ext = os.path.splitext(file_name)
    if ext in (".dat", ".txt"):
        with open(file_name, "r") as f:
            return load_dat(f)
    if ext == ".h5":
        try:
            import h5py
        except ImportError:
            return _load_h5_file(file_name, group_name)
        with h5py.File(file_name, "r") as h5f:
            return load_h5(h5f[group_name])
    raise TypeError(ext + " is not implemented yet")


def load_dat(file):
    """Fiber bundles of an open text file (fiber_bundles.py:41-77)."""
    fiber, bundles = [], [[]]
    empty = 0
    for line in file:
        if line.strip():
            empty = 0
            fiber.append([float(v) for v in line.split()][:4])
            continue
        empty += 1
        if empty == 1 and fiber:  # end of a fiber
            bundles[-1].append(np.array(fiber, float))
            fiber = []
        elif empty == 2 and bundles[-1]:  # end of a bundle
            bundles.append([])
    if fiber:
        bundles[-1].append(np.array(fiber, float))
    return objects.FiberBundles(bundles)


def load_h5(h5f):
    """Fiber bundles of an h5py file or group (fiber_bundles.py:80-103):
    groups named by bundle index, datasets by fiber index."""
    bundles = []
    for b in sorted(int(k) for k in h5f.keys()):
        grp = h5f[str(b)]
        bundles.append([np.asarray(grp[str(f)][:], float)
                        for f in sorted(int(k) for k in grp.keys())])
    return objects.FiberBundles(bundles)


def _load_h5_file(file_name, group_name):
    from . import h5read
    prefix = group_name.strip("/")
    data = h5read.read_all(file_name)
    tree = {}
    for path, arr in data.items():
        if prefix:
            if not path.startswith(prefix + "/"):
                continue
            path = path[len(prefix) + 1:]
        parts = path.split("/")
        if len(parts) != 2:
            continue
        tree.setdefault(int(parts[0]), {})[int(parts[1])] = np.asarray(arr, float)
    return objects.FiberBundles([[tree[b][f] for f in sorted(tree[b])] for b in sorted(tree)])


def save(file_name, fiber_bundles, group_name="/", mode="w-"):
    """Write fiber bundles to a .dat / .txt / .h5 file (fiber_bundles.py:
    106-136); mode "w-" refuses to overwrite."""
    _, ext = os.path.splitext(file_name)
    if ext in (".dat", ".txt"):
        with open(file_name, "x" if mode == "w-" else mode) as f:
            save_dat(f, fiber_bundles)
    elif ext == ".h5":
        import h5py  # writing HDF5 needs h5py
        with h5py.File(file_name, mode) as h5f:
            if not group_name or group_name == "/":
                save_h5(h5f, fiber_bundles)
            else:
                save_h5(h5f.create_group(group_name), fiber_bundles)
    else:
        raise TypeError(ext + " is not implemented yet")


def save_dat(file, fiber_bundles):
    """Text format (fiber_bundles.py:139-160): str() of each coordinate."""
    fbs = objects.FiberBundles(fiber_bundles)
    n = len(fbs)
    for b, bundle in enumerate(fbs):
        for fiber in bundle:
            for p in fiber:
                file.write(f"{str(p[0])} {str(p[1])} {str(p[2])} {str(p[3])}\n")
            file.write("\n")
        if b != n - 1:
            file.write("\n")


def save_h5(h5f, fiber_bundles):
    """h5py file or group (fiber_bundles.py:163-179)."""
    for b, bundle in enumerate(objects.FiberBundles(fiber_bundles)):
        grp = h5f.create_group(str(b))
        for i, f in enumerate(bundle):
            grp[str(i)] = np.asarray(f)[:, :]
