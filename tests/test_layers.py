"""Layer lists as the reference validates them (src/fastpli/objects/layers.py:
9-18,76-99) and as its C++ bundle re-sorts them (src/simulation/
fiber_bundle.cpp:76-92): unsorted layers are sorted with a warning, equal
scales are refused, and the voxelizer gives unsorted layers exactly the
labels, vectors and properties of the sorted list (GPU, against the oracle)."""

import warnings

import numpy as np
import pytest

from fastpli_gb300 import objects
from fastpli_gb300.simpli import Simpli
from fastpli_gb300.simulation import _Generator

SORTED = [(0.4, -0.003, 4.0, "p"), (0.7, 0.0, 2.0, "b"), (1.0, 0.004, 1.0, "r")]
UNSORTED = [SORTED[2], SORTED[0], SORTED[1]]
FIBERS = [[np.array([[-2.0, 1.1, 1.3, 1.0], [6.0, 1.4, 0.9, 1.0], [9.0, 3.0, 1.0, 0.8]])],
          [np.array([[1.6, -1.0, 1.2, 0.7], [1.9, 9.0, 1.5, 0.9]])]]


def _simpli(layers):
    s = Simpli()
    s.voxel_size = 0.25
    s.set_voi([0, 0, 0], [8, 6, 3])
    s.fiber_bundles = objects.FiberBundles(FIBERS, layers=[layers, SORTED])
    return s


def test_unsorted_layers_are_sorted_with_a_warning():
    with pytest.warns(UserWarning, match="layers had to be sorted"):
        out = objects.check_layers(UNSORTED)
    assert out == [tuple(map(lambda v: v, ly)) for ly in SORTED]
    with pytest.warns(UserWarning, match="layers had to be sorted"):
        s = _simpli(UNSORTED)
    assert s.fiber_bundles.layers[0] == SORTED


def test_sorted_layers_give_no_warning():
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        objects.check_layers(SORTED)


def test_equal_scales_are_refused():
    dup = [(0.5, 0.0, 1.0, "b"), (0.5, 0.004, 1.0, "r")]
    with pytest.raises(ValueError, match="same radii"):
        objects.check_layers(dup)
    with pytest.raises(ValueError, match="same radii"):
        objects.FiberBundles(FIBERS, layers=[dup, SORTED])
    # unsorted with a duplicate: sorted first (warning), then refused
    with pytest.warns(UserWarning, match="layers had to be sorted"):
        with pytest.raises(ValueError, match="same radii"):
            objects.check_layers([(1.0, 0.004, 1.0, "r"), (0.5, 0.0, 1.0, "b"),
                                  (0.5, 0.0, 2.0, "b")])


def test_background_with_birefringence_is_refused():
    with pytest.raises(ValueError, match="background"):
        objects.check_layers([(1.0, 0.001, 1.0, "b")])


@pytest.mark.gpu
def test_generator_sorts_unsorted_layers_like_the_reference(cuda, oracle_port):
    """_Generator takes the layer lists as given (the reference's C++ bundle
    sorts them itself, fiber_bundle.cpp:83-86): unsorted lists must give the
    oracle's result for the same input and the sorted list's result."""
    dim, origin, vs = np.array([32, 24, 12]), np.zeros(3), 0.25
    out = {}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for name, lys in (("unsorted", UNSORTED), ("sorted", SORTED)):
            g = _Generator()
            g.set_volume(dim, origin, vs)
            g.set_fiber_bundles(FIBERS, [lys, SORTED])
            out[name] = g.run_generation()
        olab, ovec, oprops, _ = oracle_port.generate(dim, origin, vs, FIBERS, [UNSORTED, SORTED])
    lab, vec, props = out["unsorted"]
    assert np.array_equal(lab, olab)
    assert np.array_equal(vec.view(np.uint32), ovec.view(np.uint32))
    assert np.array_equal(props, oprops)
    assert np.array_equal(lab, out["sorted"][0])
    assert np.array_equal(vec.view(np.uint32), out["sorted"][1].view(np.uint32))
    assert np.array_equal(props, out["sorted"][2])
    assert set(np.unique(lab)) >= {1, 2, 3, 4, 5, 6}  # every layer of both bundles is hit
