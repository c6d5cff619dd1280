"""Seeded synthetic tissue for the benchmark and parity workloads.

No public dataset is involved: every workload is generated here from a fixed
numpy ``default_rng`` seed with the shapes, sizes and value distributions of
the forward-model workloads:

* ``parallel_x``   — 128x128x60 voxels at 0.2 µm, 40 straight fibers along x
                     (20 points, two N(0, 2°) direction jitters, radius
                     U(0.8, 1.2) µm), layers (0.75, 0, 10, 'b'), (1.0, 0.004, 10, 'r').
* ``crossing``     — 512x512x120 at 0.2 µm, two bundles of 1000 fibers along x
                     and y (50 points, same jitter), radii lognormal(ln 1, 0.2),
                     same two layers.
* ``watson``       — 1024x1024x240 at 0.1 µm, 20000 fibers x 50 points along
                     Watson(kappa=5) axes about a random axis, radii
                     lognormal(ln 0.8, 0.25), three layers.
* ``wide_strip``   — 5504x16384x16 at 1 µm (1.44e9 voxels, past the 32-bit
                     index range of the march), two bundles of 5 wavy fibers
                     along y confined to the last 32 x-columns (radius
                     U(1.5, 2.5) µm), layers (0.333, -0.004, 10, 'p'),
                     (0.666, 0, 5, 'b'), (1.0, 0.004, 1, 'r'); tilts (0, 0)
                     and 10° at phi = 90°.
* ``tiles``        — 256 independent tiles, xy side U{64..512}, z U{30..120} at
                     0.2 µm, 50-2000 fibers with uniform directions, per-tile
                     dn U[-0.004, 0.004] and mu U[0, 20].
Tilts: (0, 0) and 5.5° at phi = 0, 90, 180, 270°.  Polarizer angles 0..160°
in 20° steps, wavelength 525 nm, light intensity 26000.
"""

import numpy as np

TILTS_5 = np.deg2rad([(0, 0), (5.5, 0), (5.5, 90), (5.5, 180), (5.5, 270)])
ROT_9 = np.deg2rad(np.arange(0, 180, 20))
OPTICS = dict(light_intensity=26000.0, wavelength=525.0, step_size=1.0,
              tissue_refrection=1.0, untilt_sensor_view=True, flip_z=False)


class Workload:
    """A voxel volume plus fiber bundles and layers."""

    def __init__(self, name, dim, voxel_size, bundles, layers, tilts=None,
                 origin=(0.0, 0.0, 0.0), interpolate="Slerp"):
        self.name = name
        self.dim = np.asarray(dim, np.int64)
        self.voxel_size = float(voxel_size)
        self.origin = np.asarray(origin, float)
        self.bundles = bundles
        self.layers = layers
        self.tilts = TILTS_5[:1] if tilts is None else np.asarray(tilts)
        self.interpolate = interpolate
        self.rotations = ROT_9

    @property
    def n_voxels(self):
        return int(np.prod(self.dim))

    @property
    def n_fibers(self):
        return sum(len(b) for b in self.bundles)

    def setup_kwargs(self):
        return dict(OPTICS, voxel_size=self.voxel_size,
                    interpolate=self.interpolate, filter_rotations=self.rotations)

    def describe(self):
        X, Y, Z = (int(v) for v in self.dim)
        return {"workload": self.name, "volume": [X, Y, Z],
                "voxel_size_um": self.voxel_size, "fibers": self.n_fibers,
                "tilts": int(len(self.tilts)), "rho": int(len(self.rotations)),
                "interpolate": self.interpolate}


def _jitter_dir(rng, axis):
    a1, a2 = np.deg2rad(rng.normal(0.0, 2.0, 2))
    if axis == 0:
        d = np.array([np.cos(a1) * np.cos(a2), np.sin(a2), np.sin(a1)])
    else:
        d = np.array([np.sin(a2), np.cos(a1) * np.cos(a2), np.sin(a1)])
    return d / np.linalg.norm(d)


def _line(center, d, t0, t1, n, r):
    t = np.linspace(t0, t1, n)
    pts = center[None, :] + t[:, None] * d[None, :]
    return np.ascontiguousarray(np.c_[pts, np.full(n, r)])


def _crossing_span(center, d, lo, hi, margin):
    """Parameter range where center + t*d lies inside [lo, hi] (slab method),
    widened by ``margin`` on both ends."""
    tmin, tmax = -np.inf, np.inf
    for i in range(3):
        if abs(d[i]) < 1e-12:
            continue
        a, b = (lo[i] - center[i]) / d[i], (hi[i] - center[i]) / d[i]
        tmin, tmax = max(tmin, min(a, b)), min(tmax, max(a, b))
    if not np.isfinite(tmin):
        tmin, tmax = -np.linalg.norm(hi - lo), np.linalg.norm(hi - lo)
    return tmin - margin, tmax + margin


def parallel_x(seed=1):
    rng = np.random.default_rng(seed)
    dim, vs = (128, 128, 60), 0.2
    size = np.array(dim) * vs
    fibers = []
    for _ in range(40):
        c = np.array([0.0, rng.uniform(0, size[1]), rng.uniform(0, size[2])])
        d = _jitter_dir(rng, 0)
        r = rng.uniform(0.8, 1.2)
        fibers.append(_line(c, d, -r, size[0] + r, 20, r))
    layers = [[(0.75, 0.0, 10.0, "b"), (1.0, 0.004, 10.0, "r")]]
    return Workload("parallel_x 128x128x60", dim, vs, [fibers], layers)


def crossing(seed=2, n_per_bundle=1000, dim=(512, 512, 120), n_points=50):
    rng = np.random.default_rng(seed)
    vs = 0.2
    size = np.array(dim) * vs
    bundles = []
    for axis in (0, 1):
        fibers = []
        for _ in range(n_per_bundle):
            c = rng.uniform(0, 1, 3) * size
            c[axis] = 0.0
            d = _jitter_dir(rng, axis)
            r = float(rng.lognormal(np.log(1.0), 0.2))
            fibers.append(_line(c, d, -r, size[axis] + r, n_points, r))
        bundles.append(fibers)
    lys = [(0.75, 0.0, 10.0, "b"), (1.0, 0.004, 10.0, "r")]
    X, Y, Z = dim
    return Workload(f"crossing {X}x{Y}x{Z}", dim, vs, bundles, [lys, lys], tilts=TILTS_5)


def watson_axes(rng, kappa, mu, n, grid=4097):
    """Watson(kappa) axial samples about unit axis ``mu``: t = mu.x by inverse
    transform sampling of the density exp(kappa t^2) on [-1, 1], azimuth
    uniform."""
    t = np.linspace(-1.0, 1.0, grid)
    pdf = np.exp(kappa * (t * t - 1.0))
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(t))])
    cdf /= cdf[-1]
    ts = np.interp(rng.uniform(0, 1, n), cdf, t)
    ph = rng.uniform(0, 2 * np.pi, n)
    a = np.array([1.0, 0, 0]) if abs(mu[0]) < 0.9 else np.array([0, 1.0, 0])
    e1 = np.cross(mu, a)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(mu, e1)
    s = np.sqrt(np.maximum(0.0, 1 - ts * ts))
    return (ts[:, None] * mu[None] + (s * np.cos(ph))[:, None] * e1[None]
            + (s * np.sin(ph))[:, None] * e2[None])


def watson(seed=3, n_fibers=20000, dim=(1024, 1024, 240), n_points=50):
    rng = np.random.default_rng(seed)
    vs = 0.1
    size = np.array(dim) * vs
    mu = rng.normal(size=3)
    mu /= np.linalg.norm(mu)
    dirs = watson_axes(rng, 5.0, mu, n_fibers)
    fibers = []
    lo, hi = np.zeros(3), size
    for i in range(n_fibers):
        c = rng.uniform(0, 1, 3) * size
        r = float(rng.lognormal(np.log(0.8), 0.25))
        t0, t1 = _crossing_span(c, dirs[i], lo, hi, r)
        fibers.append(_line(c, dirs[i], t0, t1, n_points, r))
    lys = [(0.6, 0.0, 5.0, "b"), (0.8, -0.002, 8.0, "p"), (1.0, 0.004, 10.0, "r")]
    X, Y, Z = dim
    return Workload(f"watson {X}x{Y}x{Z}", dim, vs, [fibers], [lys])


WIDE_DIM = (5504, 16384, 16)
WIDE_STRIP = 32  # the fibers lie in x >= WIDE_DIM[0] - WIDE_STRIP


def wide_strip(seed=41):
    """A volume whose vector field is indexed past 2^32 (3 X Y Z > 2^32),
    with all tissue in its last ``WIDE_STRIP`` x-columns, where the linear
    index is largest."""
    X, Y, Z = WIDE_DIM
    x0 = X - WIDE_STRIP
    rng = np.random.default_rng(seed)
    ys = np.arange(-24.0, Y + 24.0, 48.0)
    bundles = []
    for _ in range(2):
        fibers = []
        for _ in range(5):
            a, b = rng.uniform(0, 2 * np.pi, 2)
            x = x0 + 16.0 + 5.0 * np.sin(ys / 310.0 + a) + rng.uniform(-0.5, 0.5, ys.size)
            z = 8.0 + 3.0 * np.sin(ys / 530.0 + b) + rng.uniform(-0.5, 0.5, ys.size)
            r = np.full(ys.size, rng.uniform(1.5, 2.5))
            fibers.append(np.stack([x, ys, z, r], axis=1))
        bundles.append(fibers)
    lys = [(0.333, -0.004, 10.0, "p"), (0.666, 0.0, 5.0, "b"), (1.0, 0.004, 1.0, "r")]
    return Workload(f"wide strip {X}x{Y}x{Z}", WIDE_DIM, 1.0, bundles, [lys, lys],
                    tilts=np.deg2rad([(0, 0), (10, 90)]))


def _tile_draws(rng):
    X, Y = (int(v) for v in rng.integers(64, 513, 2))
    Z = int(rng.integers(30, 121))
    nf = int(rng.integers(50, 2001))
    dn = float(rng.uniform(-0.004, 0.004))
    mu = float(rng.uniform(0.0, 20.0))
    return (X, Y, Z), nf, dn, mu


def tile_params(i, seed_base=1000):
    """(dim, fibers, dn, mu) of tile ``i`` of the uneven-tile mixture without
    generating its fibers."""
    return _tile_draws(np.random.default_rng(seed_base + i))


def tile(i, seed_base=1000, n_fibers=None, segment_um=2.0):
    """Tile ``i`` of the uneven-tile mixture."""
    rng = np.random.default_rng(seed_base + i)
    (X, Y, Z), nf, dn, mu = _tile_draws(rng)
    vs = 0.2
    size = np.array([X, Y, Z]) * vs
    nf = nf if n_fibers is None else int(n_fibers)
    v = rng.normal(size=(nf, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    fibers = []
    for k in range(nf):
        c = rng.uniform(0, 1, 3) * size
        r = float(rng.lognormal(np.log(1.0), 0.2))
        t0, t1 = _crossing_span(c, v[k], np.zeros(3), size, r)
        n = max(2, int(np.ceil((t1 - t0) / segment_um)) + 1)
        fibers.append(_line(c, v[k], t0, t1, n, r))
    lys = [(0.75, 0.0, mu, "b"), (1.0, dn, mu, "r")]
    return Workload(f"tile{i} {X}x{Y}x{Z}", (X, Y, Z), vs, [fibers], [lys],
                    tilts=TILTS_5)


def tiles(n=256, seed_base=1000):
    return [tile(i, seed_base) for i in range(n)]
