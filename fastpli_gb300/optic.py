"""Optic stage after the ray march, on the GPU.

Mirrors ``fastpli.simulation.optic`` (src/fastpli/simulation/optic.py) as
``Simpli.apply_optic_resample`` / ``apply_optic`` use it
(src/fastpli/simulation/__simpli.py:462-552):

* ``filter_resample(image, sigma, scale)`` — optic.py:169-187: Gaussian blur
  of width ``sigma / scale`` with ``scipy.ndimage.gaussian_filter`` semantics
  (mode 'reflect', truncate 4.0; ``sigma == 0`` skips it), then the
  block-average ``resample`` of optic.py:85-120.  Accepts one image [X, Y] or
  a stack [X, Y, n_rho] (every angle at once, in the march's layout).
* ``add_noise(image, model, mask)`` — optic.py:8-33, unchanged semantics: the
  model is called on the image, masked / non-finite pixels keep their value.
* ``NegativeBinomialNoise(gain)`` — the noise model of the reference's
  pipelines (``lambda x: np.random.negative_binomial(x / (gain - 1),
  1 / gain)``) sampled on the device; usable as ``Simpli.noise_model``.
* ``*_device`` variants take and return torch CUDA tensors and stay on the
  stream: the march's image stack goes through resample, noise and epa
  without leaving HBM.

All of it runs in the native library (``optic.cu``); there is no CPU path.
"""

import numpy as np

from . import _native as N

TRUNCATE = 4.0  # scipy.ndimage.gaussian_filter default used by optic.filter


def resample_size(shape, scale):
    """(int(round(X * scale)), int(round(Y * scale))) as optic.py:100-101."""
    out = np.zeros(2, np.int64)
    N.check(N.load().fpgb_optic_resample_size(int(shape[0]), int(shape[1]), float(scale),
                                             N.ptr(out)))
    return int(out[0]), int(out[1])


def _as_stack(image):
    a = np.ascontiguousarray(np.asarray(image, dtype=np.float64))
    if a.ndim == 2:
        return a[:, :, None], True
    if a.ndim != 3:
        raise TypeError("image must be [X, Y] or [X, Y, n_rho]")
    return a, False


def filter_resample(image, sigma, scale):
    """optic.filter_resample on the GPU (host arrays in and out, float64)."""
    a, flat = _as_stack(image)
    X, Y, R = a.shape
    sx, sy = resample_size((X, Y), scale)
    out = np.empty((sx, sy, R), np.float64)
    N.check(N.load().fpgb_optic_filter_resample(N.ptr(a), X, Y, R, float(sigma), float(scale),
                                               N.ptr(out)))
    return out[:, :, 0] if flat else out


def _torch():
    import torch
    return torch


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def filter_resample_device(images, sigma, scale, out=None, stream=None):
    """Device version: ``images`` a float64 CUDA tensor [X, Y] or
    [X, Y, n_rho]; returns [SX, SY(, n_rho)] (``out`` if given)."""
    torch = _torch()
    if images.dtype != torch.float64 or not images.is_cuda:
        raise TypeError("images must be a float64 CUDA tensor")
    flat = images.dim() == 2
    a = images.contiguous()
    X, Y = int(a.shape[0]), int(a.shape[1])
    R = 1 if flat else int(a.shape[2])
    sx, sy = resample_size((X, Y), scale)
    shape = (sx, sy) if flat else (sx, sy, R)
    if out is None:
        out = torch.empty(shape, dtype=torch.float64, device=a.device)
    elif tuple(out.shape) != shape or out.dtype != torch.float64 or not out.is_contiguous():
        raise ValueError(f"out must be a contiguous float64 tensor of shape {shape}")
    N.check(N.load().fpgb_optic_filter_resample_device(
        N.ptr(a), X, Y, R, float(sigma), float(scale), N.ptr(out), _stream(stream)))
    return out


class NegativeBinomialNoise:
    """``x -> negative_binomial(x / (gain - 1), 1 / gain)`` per pixel (mean x,
    variance gain * x), drawn on the GPU from a counter-based generator.

    ``seed=None`` draws a fresh 64-bit seed from ``np.random`` on every call,
    so ``np.random.seed(...)`` makes a pipeline reproducible as it does for
    the reference's numpy-based model.  Pixels <= 0 raise ValueError, as
    numpy's negative_binomial does for n <= 0.
    """

    def __init__(self, gain=3.0, seed=None):
        gain = float(gain)
        if not gain > 1.0 or not np.isfinite(gain):
            raise ValueError("gain must be a finite number > 1")
        self.gain = gain
        self.seed = seed
        self._calls = 0

    def _seed(self):
        if self.seed is None:
            return int(np.random.randint(0, 2**63 - 1, dtype=np.int64))
        self._calls += 1
        # distinct streams for successive calls with a fixed seed
        return (int(self.seed) * 0x9E3779B97F4A7C15 + self._calls) % 2**64

    def device(self, images, out=None, offset=0, stream=None):
        torch = _torch()
        if images.dtype != torch.float64 or not images.is_cuda:
            raise TypeError("images must be a float64 CUDA tensor")
        a = images.contiguous()
        if out is None:
            out = torch.empty_like(a)
        bad = np.zeros(1, np.int64)
        N.check(N.load().fpgb_optic_noise_device(
            N.ptr(a), a.numel(), self.gain, self._seed(), int(offset), N.ptr(out), N.ptr(bad),
            _stream(stream)))
        if bad[0]:
            raise ValueError(f"negative binomial noise: {int(bad[0])} pixels with n <= 0 "
                             "(intensity <= 0 or not finite)")
        return out

    def __call__(self, image):
        torch = _torch()
        a = np.ascontiguousarray(np.asarray(image, dtype=np.float64))
        t = torch.from_numpy(a).cuda()
        return self.device(t).cpu().numpy().reshape(a.shape)


def add_noise(image, model, mask=None):
    """optic.add_noise (optic.py:8-33): ``model(image)``, with pixels outside
    ``mask`` or non-finite keeping their value."""
    image = np.asarray(image)
    noisy = np.array(model(image), copy=True)
    if mask is not None:
        keep = np.logical_not(np.logical_and(np.isfinite(image), mask))
        noisy[keep] = image[keep]
    return noisy


def epa_device(images, stream=None):
    """epa (src/fastpli/analysis/epa.py:9-45) of a float64 CUDA tensor
    [..., n_rho] in FP64: (transmittance, direction, retardation)."""
    torch = _torch()
    if images.dtype != torch.float64 or not images.is_cuda:
        raise TypeError("images must be a float64 CUDA tensor")
    a = images.contiguous()
    R = int(a.shape[-1])
    n_pix = a.numel() // R
    t, d, r = (torch.empty(a.shape[:-1], dtype=torch.float64, device=a.device)
               for _ in range(3))
    N.check(N.load().fpgb_epa_device(N.ptr(a), n_pix, R, N.ptr(t), N.ptr(d), N.ptr(r),
                                     _stream(stream)))
    return t, d, r
