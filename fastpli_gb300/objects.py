"""Input marshalling for fiber bundles and layers.

Mirrors the validation of fastpli.objects (src/fastpli/objects/layers.py:9-18,
76-99 and src/fastpli/objects/fibers.py:740-810) for the forms the forward
model consumes: a fiber is an (n, 4) float array of (x, y, z, radius) in µm,
a bundle is a list of fibers, and every bundle carries a list of layers
(scale, dn, mu, model) with model 'b' (background, no axis), 'p' (parallel)
or 'r' (radial).  Geometry transforms of the reference's object classes are
not part of the forward model and are not reproduced.
"""

import warnings

import numpy as np


def check_layer(ly):
    """layers.py:9-18."""
    if len(ly) != 4:
        raise TypeError("layer != (float, float, float, char)")
    if ly[1] < 0 and ly[-1] == "r":
        warnings.warn("birefringence negative and radial")
    if ly[1] > 0 and ly[-1] == "p":
        warnings.warn("birefringence positive and parallel")
    if ly[1] != 0 and ly[-1] == "b":
        raise ValueError("birefringence != 0 for background.")
    return (float(ly[0]), float(ly[1]), float(ly[2]), ly[3])


def check_layers(lys):
    """layers.py:76-99: validates, sorts by scale (warning), rejects equal
    scales."""
    if lys is None:
        return None
    if hasattr(lys, "data") and callable(lys.data):
        lys = lys.data()
    if len(lys) == 4 and not isinstance(lys[0], (list, tuple)):
        lys = [lys]
    lys = [check_layer(tuple(ly)) for ly in lys]
    if any(ly[0] > 1 for ly in lys):
        warnings.warn("layer scale > 1 detected")
    keys = sorted(range(len(lys)), key=lambda i: lys[i][0])
    if any(keys[i] > keys[i + 1] for i in range(len(keys) - 1)):
        warnings.warn("layers had to be sorted")
        lys = [lys[i] for i in keys]
    if any(lys[i][0] == lys[i + 1][0] for i in range(len(lys) - 1)):
        raise ValueError("detected layers of same radii")
    return lys


def as_fiber(f):
    f = np.array(f, dtype=np.float64, ndmin=2)
    if f.ndim != 2 or f.shape[1] != 4:
        raise TypeError("fiber is not a (n,4)-array")
    return np.ascontiguousarray(f)


class FiberBundles:
    """List of bundles plus per-bundle layers (fibers.py:740-810 surface:
    ``as_array()``, ``layers``, iteration, ``len``)."""

    def __init__(self, data=None, layers=None):
        if isinstance(data, FiberBundles):
            self._bundles = [list(b) for b in data._bundles]
            self._layers = list(data._layers) if layers is None else None
        elif hasattr(data, "as_array") and hasattr(data, "layers"):
            self._bundles = [[as_fiber(f) for f in fb] for fb in data.as_array()]
            self._layers = [check_layers(l) for l in data.layers]
        else:
            data = [] if data is None else data
            self._bundles = [[as_fiber(f) for f in fb] for fb in data]
            self._layers = [None] * len(self._bundles)
        if layers is not None:
            self.layers = layers

    def as_array(self):
        return [[f.copy() for f in fb] for fb in self._bundles]

    @property
    def layers(self):
        return list(self._layers)

    @layers.setter
    def layers(self, value):
        if len(value) != len(self._bundles):
            raise ValueError("Wrong number of [layers]")
        self._layers = [check_layers(l) for l in value]

    def __len__(self):
        return len(self._bundles)

    def __iter__(self):
        return iter(self._bundles)

    def __getitem__(self, i):
        return self._bundles[i]
