"""Parity scenarios shared by the golden-fixture script, the oracle tests and
the GPU tests.

The small scenarios restate the setups of the reference's own tests
(tests/simulation/simpli_test.py:31-63,65-218,220-260; tests/analysis/
rofl_test.py:15-45; the golden regression tests/simulation/simpli_rep.py with
fibers from tests/cube.dat), plus edge cases of the voxelizer (single-point
fibers, empty bundles, fibers outside the volume, a non-zero origin, layer
quotients past the outermost layer) and seeded synthetic workloads.
"""

import os

import numpy as np

from fastpli_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

LY3 = [(0.333, -0.004, 10.0, "p"), (0.666, 0.0, 5.0, "b"), (1.0, 0.004, 1.0, "r")]
ROT6 = np.deg2rad([0, 30, 60, 90, 120, 150])


def _vol(v_min, v_max, vs):
    v_min = np.asarray(v_min, float)
    v_max = np.asarray(v_max, float)
    dim = np.array(np.round((v_max - v_min) / vs), dtype=np.int64)
    return dim, v_min


def gen_cases():
    """name -> dict(dim, origin, voxel_size, bundles, layers)."""
    z_fiber = [np.array([[0, 0.25, -500, 1], [0, 0.25, 500, 1]], float)]
    dim15, o15 = _vol([0, 0, 0], [1.5, 1.5, 1.5], 0.1)
    dim20, o20 = _vol([-10] * 3, [10] * 3, 1.0)
    cases = {
        "radial": dict(dim=dim15, origin=o15, voxel_size=0.1, bundles=[z_fiber],
                       layers=[[(1.0, 0.004, 1.0, "r")]]),
        "parallel": dict(dim=dim15, origin=o15, voxel_size=0.1, bundles=[z_fiber],
                         layers=[[(1.0, -0.004, 1.0, "p")]]),
        "layered": dict(dim=dim15, origin=o15, voxel_size=0.1, bundles=[z_fiber],
                        layers=[[(0.3, -0.004, 1.0, "p"), (0.6, 0.0, 1.0, "b"),
                                 (1.0, 0.004, 1.0, "r")]]),
        "layered_x": dict(dim=dim20, origin=o20, voxel_size=1.0,
                          bundles=[[np.array([[-100, 0, 0, 10], [100, 0, 0, 10]], float)]],
                          layers=[LY3]),
        "dimension": dict(dim=np.array([3, 5, 7]), origin=np.zeros(3), voxel_size=1.0,
                          bundles=[[np.array([[1, 3, 0, 2], [1, 3, 7, 2]], float)]],
                          layers=[[(1.0, 0.0, 0.0, "p")]]),
        "polyline": dict(dim=np.array([10, 10, 10]), origin=np.zeros(3), voxel_size=0.2,
                         bundles=[[np.array([[0, 0, 0, 1], [1, 1, 1, 1], [2, 2, 2, 1]], float)]],
                         layers=[LY3]),
    }
    # edge cases: joints, single-point fibers, an empty bundle, fibers leaving
    # the volume, a shifted origin, tapering radii, a last layer scale < 1
    # (layer quotient past the table), two overlapping bundles
    rng = np.random.default_rng(7)
    bent = np.array([[-1, 2, 2, 1.2], [2.05, 2.0, 2.0, 0.8], [2.05, 5.5, 2.5, 1.0],
                     [4.0, 7.0, 4.5, 1.0], [9, 9, 1, 0.6]], float)
    wiggle = np.c_[np.linspace(-2, 12, 15), 3 + rng.normal(0, 0.4, 15),
                   3 + rng.normal(0, 0.4, 15), rng.uniform(0.5, 1.5, 15)]
    cases["edges"] = dict(
        dim=np.array([40, 36, 28]), origin=np.array([0.5, -0.25, 0.0]), voxel_size=0.25,
        bundles=[[bent, np.array([[3, 3, 3, 1]], float), wiggle],
                 [],
                 [np.array([[20, -5, 20, 1], [20, -4, 30, 1]], float),
                  np.c_[np.linspace(0, 10, 6), np.full(6, 4.0), np.linspace(0, 6, 6),
                        np.full(6, 0.9)]]],
        layers=[[(0.5, -0.002, 3.0, "p"), (0.6, 0.004, 2.0, "r")],
                [(1.0, 0.0, 1.0, "b")],
                LY3])
    return cases


def load_cube():
    """Fibers of the reference's golden regression (tests/cube.dat), stored in
    the fixture so the GPU machine does not need the reference tree."""
    path = os.path.join(GOLDEN, "cube_fibers.npz")
    z = np.load(path)
    return [[z[k] for k in sorted(z.files, key=lambda s: int(s[1:]))]]


def cube_case():
    dim, o = _vol([-60] * 3, [60] * 3, 5.0)
    return dict(dim=dim, origin=o, voxel_size=5.0, bundles=load_cube(), layers=[LY3])


def synth_case(w):
    return dict(dim=w.dim, origin=w.origin, voxel_size=w.voxel_size,
                bundles=w.bundles, layers=w.layers)


def crossing_small():
    return synth.crossing(seed=21, n_per_bundle=60, dim=(96, 80, 40), n_points=12)


# simulation scenarios: (generation case, setup kwargs, tilts)
def sim_cases():
    s = {}
    for interp in ("NN", "Lerp", "Slerp"):
        for untilt in (False, True):
            s[f"layered_x-{interp}-{'untilt' if untilt else 'tilt'}"] = (
                "layered_x",
                dict(light_intensity=26000.0, voxel_size=1.0, wavelength=525.0,
                     interpolate=interp, untilt_sensor_view=untilt,
                     filter_rotations=ROT6),
                [(0.0, 0.0), (np.deg2rad(8), np.deg2rad(42))])
    s["cube-Slerp"] = (
        "cube",
        dict(light_intensity=26000.0, voxel_size=5.0, wavelength=525.0,
             interpolate="Slerp", filter_rotations=ROT6),
        [tuple(t) for t in np.deg2rad([(0, 0), (5.5, 0), (5.5, 90), (5.5, 180), (5.5, 270)])])
    s["edges-Lerp-flip"] = (
        "edges",
        dict(light_intensity=1000.0, voxel_size=0.25, wavelength=600.0,
             interpolate="Lerp", flip_z=True, step_size=0.7,
             filter_rotations=np.deg2rad([0, 45, 90, 135])),
        [(0.0, 0.0), (np.deg2rad(12), np.deg2rad(200))])
    s["edges-Slerp-tilted-view"] = (
        "edges",
        dict(light_intensity=1000.0, voxel_size=0.25, wavelength=600.0,
             interpolate="Slerp", untilt_sensor_view=False, tissue_refrection=1.3,
             filter_rotations=np.deg2rad([0, 45, 90, 135])),
        [(np.deg2rad(7), np.deg2rad(30)), (np.deg2rad(5.5), np.deg2rad(270))])
    return s


def rofl_voxel():
    """tests/analysis/rofl_test.py:17-45: one voxel, axis at 45° inclination,
    dn = -0.001, 60 µm voxel, step 1/cos(theta) per tilt."""
    tissue = np.ones((1, 1, 1), np.int32)
    axis = np.zeros((1, 1, 1, 3), np.float32)
    axis[:] = [np.cos(np.deg2rad(45)), 0, np.sin(np.deg2rad(45))]
    props = np.array([[0, 0], [-0.001, 0]], float)
    tilts = np.deg2rad([(0, 0), (5.5, 0), (5.5, 90), (5.5, 180), (5.5, 270)])
    setups = [dict(light_intensity=26000.0, voxel_size=60.0, wavelength=525.0,
                   interpolate="Slerp", untilt_sensor_view=False,
                   step_size=1.0 / np.cos(t), filter_rotations=ROT6) for t, _ in tilts]
    return tissue, axis, props, tilts, setups
