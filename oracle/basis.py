"""Radial basis, cutoff functions and real spherical harmonics (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

All functions are vectorised over an array of neighbor vectors.
"""
import math

import numpy as np

PI = 3.14159265358979323846


# --------------------------------------------------------------------------
# Cutoff functions: value and d/dr.  src/flare_pp/cutoffs.cpp:44-56 (quadratic),
# :58-73 (cosine), :75-85 (hard).  Outside r > rcut both are zero.
# --------------------------------------------------------------------------
def quadratic_cutoff(r, rcut):
    r = np.asarray(r, dtype=np.float64)
    rdiff = r - rcut
    val = rdiff * rdiff
    der = 2 * rdiff
    out = r > rcut
    return np.where(out, 0.0, val), np.where(out, 0.0, der)


def cos_cutoff(r, rcut):
    r = np.asarray(r, dtype=np.float64)
    val = 0.5 * (np.cos(PI * r / rcut) + 1)
    der = -PI * np.sin(PI * r / rcut) / (2 * rcut)
    out = r > rcut
    return np.where(out, 0.0, val), np.where(out, 0.0, der)


def hard_cutoff(r, rcut):
    r = np.asarray(r, dtype=np.float64)
    out = r > rcut
    return np.where(out, 0.0, 1.0), np.zeros_like(r)


CUTOFFS = {"quadratic": quadratic_cutoff, "cosine": cos_cutoff,
           "hard": hard_cutoff}


# --------------------------------------------------------------------------
# Chebyshev radial basis on x = (r - r1)/(r2 - r1) with the first-kind
# recurrence T_n = 2 x T_{n-1} - T_{n-2}; zero outside [r1, r2].
# src/flare_pp/radial.cpp:138-169.
# --------------------------------------------------------------------------
def chebyshev(r, N, r1, r2):
    r = np.asarray(r, dtype=np.float64)
    c = 1 / (r2 - r1)
    x = (r - r1) * c
    vals = np.zeros(r.shape + (N,))
    ders = np.zeros(r.shape + (N,))
    for n in range(N):
        if n == 0:
            vals[..., 0] = 1
            ders[..., 0] = 0
        elif n == 1:
            vals[..., 1] = x
            ders[..., 1] = c
        else:
            vals[..., n] = 2 * x * vals[..., n - 1] - vals[..., n - 2]
            ders[..., n] = (2 * vals[..., n - 1] * c + 2 * x * ders[..., n - 1]
                            - ders[..., n - 2])
    outside = (r < r1) | (r > r2)
    vals[outside] = 0
    ders[outside] = 0
    return vals, ders


def calculate_radial(x, y, z, r, rcut, N, r1, cutoff_function="quadratic"):
    """Basis x cutoff and its Cartesian gradient.

    Follows src/flare_pp/radial.cpp:344-379 with the chebyshev basis whose
    upper endpoint is reset to the pair cutoff (src/flare_pp/descriptors/
    b2.cpp:352).  Returns g, gx, gy, gz each of shape (n, N).
    """
    fc, dfc = CUTOFFS[cutoff_function](r, rcut)
    b, db = chebyshev(r, N, r1, rcut)
    xr, yr, zr = x / r, y / r, z / r
    fc = fc[..., None]
    dfc = dfc[..., None]
    g = b * fc
    gx = db * xr[..., None] * fc + b * xr[..., None] * dfc
    gy = db * yr[..., None] * fc + b * yr[..., None] * dfc
    gz = db * zr[..., None] * fc + b * zr[..., None] * dfc
    return g, gx, gy, gz


# --------------------------------------------------------------------------
# Real spherical harmonics with Cartesian gradients.
#
# The reference (src/flare_pp/y_grad.cpp:667-2754) spells out closed forms up
# to l = 10 for the orthonormal real harmonics without Condon-Shortley phase,
# ordered l*l + (m + l) with m = -l..l (sin-type for m < 0, cos-type for
# m > 0).  This restatement derives the same functions from the solid-harmonic
# recurrence instead:
#
#   r^l Y_lm = N_lm * Q_l^|m|(z, rho) * T_m(x, y) * (sqrt(2) if m != 0)
#   T_m = Re (x + i y)^m (m >= 0),  Im (x + i y)^|m| (m < 0)
#   Q_m^m = (2m-1)!!,  Q_{m+1}^m = (2m+1) z Q_m^m,
#   Q_l^m = ((2l-1) z Q_{l-1}^m - (l+m-1) rho Q_{l-2}^m) / (l-m),  rho = r^2
#   N_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!)
#
# Gradients follow by differentiating the recurrences, evaluated on the unit
# vector, and grad Y(r) = (grad R(u) - l Y(u) u) / |r|.
# --------------------------------------------------------------------------
def _norm_lm(l, m):
    return math.sqrt((2 * l + 1) / (4 * PI) * math.factorial(l - m)
                     / math.factorial(l + m))


def real_sph_harm(x, y, z, lmax):
    """Return Y, Yx, Yy, Yz of shape (n, (lmax+1)^2)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    r = np.sqrt(x * x + y * y + z * z)
    ux, uy, uz = x / r, y / r, z / r
    H = (lmax + 1) ** 2
    shp = x.shape + (H,)
    Y = np.zeros(shp)
    Yx = np.zeros(shp)
    Yy = np.zeros(shp)
    Yz = np.zeros(shp)

    # (x + i y)^m on the unit vector.
    A = [np.ones_like(ux)]
    B = [np.zeros_like(ux)]
    for m in range(1, lmax + 1):
        A.append(ux * A[m - 1] - uy * B[m - 1])
        B.append(uy * A[m - 1] + ux * B[m - 1])

    for m in range(0, lmax + 1):
        # Q, dQ/dz (rho fixed), dQ/drho for l = m..lmax (rho = 1 on u).
        dfact = 1.0
        for k in range(1, 2 * m, 2):
            dfact *= k
        Q = {m: np.full_like(ux, dfact)}
        Qz = {m: np.zeros_like(ux)}
        Qr = {m: np.zeros_like(ux)}
        if m + 1 <= lmax:
            Q[m + 1] = (2 * m + 1) * uz * Q[m]
            Qz[m + 1] = (2 * m + 1) * Q[m]
            Qr[m + 1] = np.zeros_like(ux)
        for l in range(m + 2, lmax + 1):
            a = 2 * l - 1
            b = l + m - 1
            d = l - m
            Q[l] = (a * uz * Q[l - 1] - b * Q[l - 2]) / d
            Qz[l] = (a * (Q[l - 1] + uz * Qz[l - 1]) - b * Qz[l - 2]) / d
            Qr[l] = (a * uz * Qr[l - 1] - b * (Q[l - 2] + Qr[l - 2])) / d

        for l in range(m, lmax + 1):
            nrm = _norm_lm(l, m) * (math.sqrt(2.0) if m > 0 else 1.0)
            # (sign, T, dT/dx, dT/dy) for the cos-type (+m) and sin-type (-m).
            if m == 0:
                terms = [(0, A[0], np.zeros_like(ux), np.zeros_like(ux))]
            else:
                terms = [
                    (m, A[m], m * A[m - 1], -m * B[m - 1]),
                    (-m, B[m], m * B[m - 1], m * A[m - 1]),
                ]
            for mm, T, Tx, Ty in terms:
                idx = l * l + mm + l
                R = nrm * Q[l] * T
                Rx = nrm * (Qr[l] * 2 * ux * T + Q[l] * Tx)
                Ry = nrm * (Qr[l] * 2 * uy * T + Q[l] * Ty)
                Rz = nrm * (Qz[l] + Qr[l] * 2 * uz) * T
                Y[..., idx] = R
                Yx[..., idx] = (Rx - l * R * ux) / r
                Yy[..., idx] = (Ry - l * R * uy) / r
                Yz[..., idx] = (Rz - l * R * uz) / r
    return Y, Yx, Yy, Yz
