"""Analysis of simulated image series on the GPU.

* ``epa(data)`` — transmittance, direction, retardation of an image stack
  [..., n_rho] (src/fastpli/analysis/epa.py:9-45): first Fourier harmonic over
  polarizer angles equidistant in [0, pi), computed in FP64 by the library's
  ``epa_stack`` kernel.  numpy in -> numpy out (dtype of the input, as the
  reference returns), CUDA tensor in -> CUDA tensors out.  The ray march also
  fuses this epilogue (``_Simulator.run_simulation_device(..., epa=True)``).
* ``rofl(data, ...)`` — ROFL tilt analysis of one pixel's 5-tilt series
  (src/fastpli/analysis/rofl.py:16-63), and ``rofl_device`` for whole maps
  [5, X, Y, n_rho] (one thread per pixel in ``rofl.cu``, MINPACK's
  Levenberg-Marquardt as the reference's scipy.optimize.leastsq runs it).
* ``fom_hsv_black(direction, inclination, mask)`` — the colour map of ROFL
  results the pipelines return (images.py:22-56,156-186; numpy on the host).

epa and ROFL have no CPU path: they run in the native library.
"""

import numpy as np

from . import _native as N


def _torch():
    import torch
    return torch


def epa(data):
    from . import optic
    if hasattr(data, "is_cuda"):
        torch = _torch()
        out_dtype = torch.float32 if data.element_size() <= 4 else torch.float64
        t, d, r = optic.epa_device(data.to(torch.float64))
        return t.to(out_dtype), d.to(out_dtype), r.to(out_dtype)
    data = np.asarray(data)
    out_dtype = np.float32 if data.itemsize <= 4 else np.float64
    torch = _torch()
    dev = torch.from_numpy(np.ascontiguousarray(data, np.float64)).cuda()
    return tuple(x.cpu().numpy().astype(out_dtype, copy=False) for x in optic.epa_device(dev))


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def rofl_device(data, tilt_angle=np.deg2rad(5.5), gain=3, dir_offset=0, grad_mode=False,
                mask=None, stream=None):
    """ROFL of every pixel of a float64 CUDA tensor [5, X, Y, n_rho] (tilts
    (0,0), (tau,0), (tau,90), (tau,180), (tau,270) degrees).  Returns a
    [X, Y, 8] tensor: direction, inclination, t_rel, their standard
    deviations, chi^2, model evaluations; NaN where ``mask`` (bool [X, Y])
    is False."""
    torch = _torch()
    if not hasattr(data, "is_cuda") or not data.is_cuda:
        raise TypeError("data must be a CUDA tensor")
    if data.dim() != 4:
        raise TypeError("data: [tilts, x, y, stack]")
    if data.shape[0] != 5:
        raise ValueError("data need 1 + 4 measurements")
    if data.shape[-1] <= 3:
        raise ValueError("data needs at least 3 equidistant rotations")
    if gain <= 1:
        raise ValueError("rofl gain <= 1")
    d = data.to(torch.float64).contiguous()
    X, Y, R = int(d.shape[1]), int(d.shape[2]), int(d.shape[3])
    out = torch.empty((X, Y, 8), dtype=torch.float64, device=d.device)
    m = None
    if mask is not None:
        m = torch.as_tensor(np.asarray(mask, bool) if not hasattr(mask, "is_cuda") else mask,
                            device=d.device).to(torch.uint8).contiguous()
        if tuple(m.shape) != (X, Y):
            raise ValueError("mask must have shape (X, Y)")
    bad = np.zeros(1, np.int64)
    N.check(N.load().fpgb_rofl_device(N.ptr(d), X * Y, R, float(tilt_angle), float(gain),
                                      float(dir_offset), int(bool(grad_mode)), N.ptr(m),
                                      N.ptr(out), N.ptr(bad), _stream(stream)))
    if bad[0]:
        import warnings
        warnings.warn(f"rofl: {int(bad[0])} pixels stopped at the evaluation limit")
    return out


def rofl(data, tilt_angle=np.deg2rad(5.5), gain=3, dir_offset=0, grad_mode=False):
    """rofl.rofl for one pixel: data [5, n_rho] -> (direction, inclination,
    t_rel, dir_dev, incl_dev, trel_dev, chi^2, evaluations)."""
    data = np.asarray(data)
    if data.ndim != 2:
        raise TypeError("data: np.array([tilts,stack])")
    torch = _torch()
    dev = torch.from_numpy(np.ascontiguousarray(data, np.float64)).cuda()[:, None, None, :]
    out = rofl_device(dev, tilt_angle, gain, dir_offset, grad_mode)
    return tuple(float(v) for v in out[0, 0].cpu().numpy())


def fom_hsv_black(direction, inclination, mask=None):
    """Fiber orientation map in the hsv_black colour space
    (src/fastpli/analysis/images.py:22-56,156-186): hue 360 |direction| / pi,
    value 1 - 2 |inclination| / pi, full saturation, as uint8 RGB
    [X, Y, 3]; pixels outside ``mask`` black.  Host arrays (radians)."""
    direction = np.asarray(direction, np.float64)
    inclination = np.asarray(inclination, np.float64)
    if mask is None:
        mask = np.ones(direction.shape, bool)
    mask = np.asarray(mask, bool)
    h = (360.0 * np.abs(direction) / np.pi + 360) % 360
    v = 1.0 - (2 * np.abs(inclination) / np.pi)
    hi = np.floor(h / 60)
    f = h / 60.0 - hi
    p = np.zeros_like(v)  # v (1 - s), s = 1
    q = v * (1 - f)
    t = v * (1 - (1 - f))
    # sector -> (r, g, b); sector 0 and any other value: (v, t, p)
    r = np.select([hi == 1, hi == 2, hi == 3, hi == 4, hi == 5], [q, p, p, t, v], v)
    g = np.select([hi == 1, hi == 2, hi == 3, hi == 4, hi == 5], [v, v, q, p, p], t)
    b = np.select([hi == 1, hi == 2, hi == 3, hi == 4, hi == 5], [p, t, v, v, q], p)
    rgb = np.stack([r * 255, g * 255, b * 255], -1).astype(np.int64)
    out = np.zeros(direction.shape + (3,), np.uint8)
    out[mask] = rgb[mask].astype(np.uint8)
    return out
