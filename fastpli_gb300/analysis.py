"""epa modalities (transmittance, direction, retardation).

Same arithmetic as fastpli.analysis.epa.epa (src/fastpli/analysis/epa.py:9-45):
first Fourier harmonic over polarizer angles assumed equidistant in [0, pi).
Accepts numpy arrays (host) or torch tensors (computed where they live).  The
device ray march also fuses this epilogue
(``_Simulator.run_simulation_device(..., epa=True)``).
"""

import numpy as np


def epa(data):
    if hasattr(data, "is_cuda"):
        return _epa_torch(data)
    data = np.asarray(data)
    dtype = np.float32 if data.itemsize <= 4 else np.float64
    data = data.astype(dtype)
    n = data.shape[-1]
    rho_2 = 2 * np.linspace(0, np.pi, n, False, dtype=dtype)
    a0 = np.sum(data, -1) / n
    a1 = 2 * np.sum(data * np.sin(rho_2), -1) / n
    b1 = 2 * np.sum(data * np.cos(rho_2), -1) / n
    t = 2 * a0
    d = 0.5 * np.arctan2(-b1, a1) + np.pi
    a0[a0 < np.finfo(dtype).eps * 100] = 1
    r = np.sqrt(a1 * a1 + b1 * b1) / a0
    d = d % np.pi
    return t, d, r


def _epa_torch(data):
    import torch
    dtype = torch.float32 if data.element_size() <= 4 else torch.float64
    data = data.to(dtype)
    n = data.shape[-1]
    rho_2 = 2 * torch.arange(n, dtype=dtype, device=data.device) * (np.pi / n)
    a0 = data.sum(-1) / n
    a1 = 2 * (data * torch.sin(rho_2)).sum(-1) / n
    b1 = 2 * (data * torch.cos(rho_2)).sum(-1) / n
    t = 2 * a0
    d = torch.remainder(0.5 * torch.atan2(-b1, a1) + np.pi, np.pi)
    a0 = torch.where(a0 < torch.finfo(dtype).eps * 100, torch.ones_like(a0), a0)
    r = torch.sqrt(a1 * a1 + b1 * b1) / a0
    return t, d, r
