"""ROFL oracle — TEST INFRASTRUCTURE ONLY.

numpy restatement of fastpli's ROFL tilt analysis
(src/fastpli/analysis/rofl.py:16-63, _ROFL_with_jacobi.py:47-522) for one
pixel, used by tests/ as the checker of the device fit (rofl.cu).  The local
fit calls scipy.optimize.leastsq (MINPACK lmdif / lmder) exactly as the
reference does; everything around it (centering and weights, tilt rotation
matrices, tilted fiber parameters, model, brute-force start grid, angle
symmetrisation, covariance) is restated here.  Pinned against the
reference's own code by tests/golden/make_rofl_golden.py.
"""

import numpy as np
from scipy import optimize


def _mod(a, b):
    return np.remainder(a, b)


def symmetrize(direction, inclination):
    """_ROFL_with_jacobi.py:64-74."""
    inclination = ((_mod(inclination + np.pi / 2.0, np.pi)) - np.pi / 2.0) * \
        np.sign(-(_mod(np.floor(direction / np.pi), 2)) + 0.5)
    return _mod(direction, np.pi), inclination


def rotation_matrix(psi, tau):
    """Rotation into tilt direction psi by tau (_ROFL_with_jacobi.py:77-96)."""
    c, s, ct, st = np.cos(psi), np.sin(psi), np.cos(tau), np.sin(tau)
    return np.array([[ct * c ** 2 + s ** 2, (ct - 1) * s * c, c * st],
                     [(ct - 1) * s * c, ct * s ** 2 + c ** 2, s * st],
                     [-c * st, -s * st, ct]])


def tilt_matrices(n_tilts, tau):
    psi = np.linspace(0, 2 * np.pi, n_tilts + 1)[:-1]
    return np.array([rotation_matrix(p, tau) for p in psi])


def tilted_params(phi, alpha, t_rel, mats, tau):
    """Direction, inclination, t_rel seen in every tilt (:150-183)."""
    v = np.array([np.cos(alpha) * np.cos(phi), np.cos(alpha) * np.sin(phi), np.sin(alpha)])
    n = mats.shape[0]
    ph = np.empty(n + 1)
    al = np.empty(n + 1)
    ph[0], al[0] = phi, alpha
    for t in range(n):
        w = mats[t] @ v
        ph[t + 1] = np.arctan(w[1] / float(w[0]))
        al[t + 1] = np.arcsin(w[2])
    tr = np.full(n + 1, t_rel / np.cos(tau))
    tr[0] = t_rel
    return ph, al, tr


def model(phi_a, alpha_a, trel_a, n_rot, dir_offset):
    """Intensity model of every tilt (:186-212), flattened."""
    phi_a, alpha_a = symmetrize(phi_a, alpha_a)
    trel_a = np.abs(trel_a)
    rho = np.linspace(0, np.pi, n_rot + 1)[:-1] + dir_offset
    out = np.empty((len(phi_a), n_rot))
    for j in range(len(phi_a)):
        out[j] = np.sin(np.pi / 2 * trel_a[j] * np.cos(alpha_a[j]) ** 2) * \
            np.sin(2 * (rho - phi_a[j]))
    return out.ravel()


def jacobi(phi_a, alpha_a, trel_a, n_rot, dir_offset):
    """Derivatives of the model with respect to each tilt's own angles
    (:215-258), stacked as the reference does."""
    phi_a, alpha_a = symmetrize(phi_a, alpha_a)
    trel_a = np.abs(trel_a)
    rho = np.linspace(0, np.pi, n_rot + 1)[:-1] + dir_offset
    n = len(phi_a)
    J = np.empty((3, n, n_rot))
    for j in range(n):
        ca, sa = np.cos(alpha_a[j]), np.sin(alpha_a[j])
        arg = np.pi / 2 * trel_a[j] * ca ** 2
        s2 = np.sin(2 * (rho - phi_a[j]))
        J[0, j] = -2 * np.cos(2 * (rho - phi_a[j])) * np.sin(arg)
        J[1, j] = -np.pi * trel_a[j] * ca * sa * np.cos(arg) * s2
        J[2, j] = np.pi / 2 * ca ** 2 * s2 * np.cos(arg)
    return J.reshape(3, -1)


def centered(stack, gain):
    """Centered intensities and weights (:47-61)."""
    n_rot = stack.shape[1]
    trans = np.mean(stack, 1)[:, None]
    c = stack / trans - 1.0
    sigma = np.sqrt(gain * (stack / trans ** 2 + stack ** 2 / (trans ** 3 * n_rot)))
    return c, 1.0 / sigma


def invert3(m):
    """The reference's analytic 3x3 inverse (:14-44), including its
    determinant expression (whose fourth term is m[2,0]*m[1,2] without a
    third factor): the covariance follows the reference, not textbook algebra."""
    det = (m[0, 0] * m[1, 1] * m[2, 2] + m[1, 0] * m[2, 1] * m[0, 2] + m[2, 0] * m[1, 2]
           - m[0, 0] * m[2, 1] * m[1, 2] - m[2, 0] * m[1, 1] * m[0, 2]
           - m[1, 0] * m[0, 1] * m[2, 2])
    inv = np.empty((3, 3))
    inv[0, 0] = m[1, 1] * m[2, 2] - m[1, 2] * m[2, 1]
    inv[0, 1] = m[0, 2] * m[2, 1] - m[0, 1] * m[2, 2]
    inv[0, 2] = m[0, 1] * m[1, 2] - m[0, 2] * m[1, 1]
    inv[1, 0] = m[1, 2] * m[2, 0] - m[1, 0] * m[2, 2]
    inv[1, 1] = m[0, 0] * m[2, 2] - m[0, 2] * m[2, 0]
    inv[1, 2] = m[0, 2] * m[1, 0] - m[0, 0] * m[1, 2]
    inv[2, 0] = m[1, 0] * m[2, 1] - m[1, 1] * m[2, 0]
    inv[2, 1] = m[0, 1] * m[2, 0] - m[0, 0] * m[2, 1]
    inv[2, 2] = m[0, 0] * m[1, 1] - m[0, 1] * m[1, 0]
    return inv / det


def direction(stack0):
    """epa.direction (epa.py:48-77) of the untilted measurement."""
    n = stack0.shape[-1]
    rho_2 = 2 * np.linspace(0, np.pi, n, False)
    a1 = 2 * np.sum(stack0 * np.sin(rho_2), -1) / n
    b1 = 2 * np.sum(stack0 * np.cos(rho_2), -1) / n
    return _mod(0.5 * np.arctan2(-b1, a1) + np.pi, np.pi)


def grid_start(phi, n_incl, n_trel, n_rot, mats, dir_offset, tau, meas, w):
    """Brute-force start point (:261-328)."""
    incl = np.linspace(-np.pi / 2, np.pi / 2, n_incl + 2)[1:-1]
    trel = np.linspace(0, 0.9, n_trel + 2)[1:-1]
    best, arg = None, None
    costs = []
    for a in incl:
        for t in trel:
            m = model(*tilted_params(phi, a, t, mats, tau), n_rot, dir_offset)
            costs.append(np.sum(np.square(w * (m - meas))))
    k = int(np.argmin(costs))
    return phi, incl[k // n_trel], trel[k % n_trel]


def rofl(data, tilt_angle=np.deg2rad(5.5), gain=3, dir_offset=0, grad_mode=False):
    """rofl.rofl for one pixel: data [5, n_rot] -> (direction, inclination,
    t_rel, dir_dev, incl_dev, trel_dev, chi2, n_fev)."""
    data = np.asarray(data, np.float64)
    if data.ndim != 2 or data.shape[0] != 5 or data.shape[1] <= 3 or gain <= 1:
        raise ValueError("data [5, n_rot > 3] and gain > 1 required")
    tau = tilt_angle
    phi0 = direction(data[0]) + dir_offset
    c, w = centered(data, gain)
    n_tilt, n_rot = c.shape
    mats = tilt_matrices(n_tilt - 1, tau)
    meas, w = c.ravel(), w.ravel()

    def resid(p):
        return w * (model(*tilted_params(p[0], p[1], p[2], mats, tau), n_rot, dir_offset) - meas)

    def djac(p):
        J = jacobi(*tilted_params(p[0], p[1], p[2], mats, tau), n_rot, dir_offset)
        return J * w

    start = grid_start(phi0, 6, 6, n_rot, mats, dir_offset, tau, meas, w)
    if grad_mode:
        x, _, info, _, _ = optimize.leastsq(resid, start, full_output=1, maxfev=150, Dfun=djac,
                                            col_deriv=1)
    else:
        x, _, info, _, _ = optimize.leastsq(resid, start, full_output=1, maxfev=150)
    chi2 = np.sum(np.square(info["fvec"]))
    d, a = symmetrize(x[0], x[1])
    t = np.abs(x[2])
    sigma_sq = chi2 / float(len(meas) - 3)
    J = jacobi(*tilted_params(d, a, t, mats, tau), n_rot, dir_offset) * w
    cov = invert3(J @ J.T) * sigma_sq
    dev = np.diag(np.abs(cov) ** 0.5)
    return d, a, t, dev[0], dev[1], dev[2], chi2, info["nfev"]


def fit_residual(data, params, tilt_angle=np.deg2rad(5.5), gain=3, dir_offset=0):
    """chi^2 of given (direction, inclination, t_rel) on data [5, n_rot]."""
    c, w = centered(np.asarray(data, np.float64), gain)
    mats = tilt_matrices(4, tilt_angle)
    m = model(*tilted_params(params[0], params[1], params[2], mats, tilt_angle), c.shape[1],
              dir_offset)
    return float(np.sum(np.square(w.ravel() * (m - c.ravel()))))
