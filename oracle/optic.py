"""Optic-stage oracle — TEST INFRASTRUCTURE ONLY.

numpy restatement of fastpli's optic stage (src/fastpli/simulation/optic.py)
and epa (src/fastpli/analysis/epa.py), used by tests/ as the checker of the
device kernels in fastpli_gb300/csrc/optic.cu.  The product never imports it.

* ``gaussian_filter``: scipy.ndimage.gaussian_filter(image, sd) as optic.py:
  36-55 calls it (defaults: mode 'reflect', truncate 4.0) — the separable
  1-D correlation along axis 0, then axis 1, in scipy's summation order for a
  symmetric kernel (centre tap, then (left + right) * w from the outermost
  tap inward).  Pinned against scipy itself (tests/test_optic.py).
* ``resample``: optic.py:85-120 — every pixel i, j goes to
  (floor((i + .5) s), floor((j + .5) s)), summed in input order, divided by
  the count.  Pinned against the reference's own function run without numba
  (tests/golden/make_optic_golden.py).
* ``epa``: epa.py:9-45 in float64.
"""

import numpy as np

TRUNCATE = 4.0


def gaussian_weights(sd, truncate=TRUNCATE):
    """scipy.ndimage._gaussian_kernel1d(sd, 0, int(truncate * sd + 0.5))."""
    radius = int(truncate * float(sd) + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (float(sd) * float(sd)) * x ** 2)
    return phi / phi.sum(), radius


def _reflect(idx, n):
    p = 2 * n
    m = np.mod(idx, p)
    return np.where(m < n, m, p - 1 - m)


def correlate_axis(a, w, radius, axis):
    a = np.moveaxis(np.asarray(a, np.float64), axis, 0)
    n = a.shape[0]
    c = np.arange(n)
    acc = a * w[radius]
    for j in range(radius, 0, -1):
        left = a[_reflect(c - j, n)]
        right = a[_reflect(c + j, n)]
        acc = acc + (left + right) * w[radius + j]
    return np.moveaxis(acc, 0, axis)


def gaussian_filter(image, sd):
    """2-D (axes 0 and 1) Gaussian filter of an [X, Y] or [X, Y, R] array."""
    if sd == 0:
        return np.asarray(image, np.float64)
    w, radius = gaussian_weights(sd)
    out = correlate_axis(image, w, radius, 0)
    return correlate_axis(out, w, radius, 1)


def resample(image, scale):
    """optic.resample of an [X, Y] or [X, Y, R] array (R resampled alike)."""
    a = np.asarray(image, np.float64)
    flat = a.ndim == 2
    if flat:
        a = a[:, :, None]
    sx = int(round(a.shape[0] * scale))
    sy = int(round(a.shape[1] * scale))
    data = np.zeros((sx, sy, a.shape[2]))
    count = np.zeros((sx, sy), np.int64)
    jj = np.floor((np.arange(a.shape[1]) + 0.5) * scale).astype(np.int64)
    jkeep = jj < sy
    for i in range(a.shape[0]):
        ii = int(np.floor((i + 0.5) * scale))
        if ii >= sx:
            continue
        # np.add.at adds in index order: j ascending within row i, as the
        # reference's loop does
        np.add.at(data[ii], jj[jkeep], a[i, jkeep])
        np.add.at(count[ii], jj[jkeep], 1)
    with np.errstate(invalid="ignore", divide="ignore"):
        out = data / count[:, :, None]
    return out[:, :, 0] if flat else out


def filter_resample(image, sigma, scale):
    """optic.filter_resample (optic.py:169-187)."""
    return resample(gaussian_filter(image, sigma / scale), scale)


def epa(data):
    """epa.epa (epa.py:9-45) for float64 data [..., n]."""
    data = np.asarray(data, np.float64)
    n = data.shape[-1]
    rho_2 = 2 * np.linspace(0, np.pi, n, False)
    a0 = np.sum(data, -1) / n
    a1 = 2 * np.sum(data * np.sin(rho_2), -1) / n
    b1 = 2 * np.sum(data * np.cos(rho_2), -1) / n
    t = 2 * a0
    d = 0.5 * np.arctan2(-b1, a1) + np.pi
    a0 = np.where(a0 < np.finfo(np.float64).eps * 100, 1.0, a0)
    r = np.sqrt(a1 * a1 + b1 * b1) / a0
    return t, d % np.pi, r
