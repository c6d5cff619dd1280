"""Parity bars against the FP64 reference / oracle, and the session-wide
record of measured max errors that tests/conftest.py prints at the end of
every pytest run (and writes as JSON to $FPGB_PARITY_REPORT when set).

Bars:
  * labels and vectors: bit-exact (mismatch counts must be 0);
  * images: relative error <= 1e-4 per pixel (FP32 march vs FP64 reference);
  * epa transmittance / retardation <= 1e-3 relative, direction <= 1e-3 rad
    (mod pi) where the pixel has retardation > 1e-2.
"""

import numpy as np

IMG_RTOL = 1e-4
EPA_TOL = 1e-3
REPORT = {}


def record(key, **vals):
    REPORT[key] = {k: (float(v) if isinstance(v, (float, np.floating)) else v)
                   for k, v in vals.items()}


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def image_errors(got, ref):
    """max relative error per pixel, and the max error relative to the
    pixel's mean over the polarizer angles (no near-zero denominators)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    if got.size == 0:
        return {"max_rel": 0.0, "max_rel_to_pixel_mean": 0.0}
    mean = np.maximum(np.abs(ref.mean(-1, keepdims=True)), 1e-300)
    return {"max_rel": rel(got, ref),
            "max_rel_to_pixel_mean": float(np.max(np.abs(got - ref) / mean))}


def epa_errors(got, ref):
    """got / ref: (transmittance, direction, retardation) maps."""
    gt, gd, gr = (np.asarray(x, np.float64) for x in got)
    et, ed, er = (np.asarray(x, np.float64) for x in ref)
    trel = rel(gt, et)
    rrel = float(np.max(np.abs(gr - er) / np.maximum(np.abs(er), 1e-3))) if er.size else 0.0
    # direction is only defined where the pixel has retardation: on uniform
    # (background) pixels a1 = b1 = 0 up to rounding and atan2 returns noise
    defined = er > 1e-2
    dd = np.abs(gd - ed)[defined]
    derr = float(np.max(np.minimum(dd, np.pi - dd))) if dd.size else 0.0
    return {"t_rel": trel, "r_rel": rrel, "d_abs": derr}


def summary_lines():
    if not REPORT:
        return []
    out = ["parity against the FP64 reference / oracle (max errors; bars: labels and "
           "vectors 0 mismatches, images 1e-4 rel, epa 1e-3):"]
    for k in sorted(REPORT):
        vals = ", ".join(f"{n}={v:.3g}" if isinstance(v, float) else f"{n}={v}"
                         for n, v in REPORT[k].items())
        out.append(f"  {k}: {vals}")
    return out
