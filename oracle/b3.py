"""B3 bispectrum descriptor (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates src/flare_pp/descriptors/b3.cpp:29-382:
  * complex single-bond coefficients c[i, (s_j N + n) H + lm] = sum_j g_n(r_ij)
    Y_l^m(r_ij) over neighbors with r <= rcut, rcut = radial_hyps[1] for every
    species pair (b3.cpp:258-270), with the complex harmonics of
    src/flare_pp/y_grad.cpp:24 (orthonormal, Condon-Shortley phase, index
    l*l + l + m);
  * B3[i, q] = Re sum_{m1+m2+m3=0} W(l1 l2 l3; m1 m2 m3) c[n1,l1m1] c[n2,l2m2]
    c[n3,l3m3], with q running n1 <= n2 <= n3, then l1, l2, l3 with
    |l1-l2| <= l3 <= l1+l2 (b3.cpp:181-233);
  * norms and stored derivatives (b3.cpp:206-240).
W is the Wigner 3j symbol, computed here from Racah's formula in exact
rational arithmetic (src/flare_pp/descriptors/wigner3j.cpp holds the same
numbers as a table; at lmax = 4 that table has 57 entries that are 0, which
reference_w3j reproduces).
"""
import math
from fractions import Fraction

import numpy as np

from .basis import calculate_radial, real_sph_harm


def wigner3j(l1, l2, l3, m1, m2, m3):
    """Wigner 3j symbol (l1 l2 l3; m1 m2 m3) by Racah's formula."""
    if m1 + m2 + m3 != 0:
        return 0.0
    if l3 < abs(l1 - l2) or l3 > l1 + l2:
        return 0.0
    if abs(m1) > l1 or abs(m2) > l2 or abs(m3) > l3:
        return 0.0
    f = math.factorial
    tri = Fraction(f(l1 + l2 - l3) * f(l1 - l2 + l3) * f(-l1 + l2 + l3),
                   f(l1 + l2 + l3 + 1))
    pre = tri * (f(l1 + m1) * f(l1 - m1) * f(l2 + m2) * f(l2 - m2) * f(l3 + m3)
                 * f(l3 - m3))
    kmin = max(0, l2 - l3 - m1, l1 - l3 + m2)
    kmax = min(l1 + l2 - l3, l1 - m1, l2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        s += Fraction((-1) ** k, f(k) * f(l3 - l2 + k + m1) * f(l3 - l1 + k - m2)
                      * f(l1 + l2 - l3 - k) * f(l1 - k - m1) * f(l2 - k + m2))
    sign = -1 if (l1 - l2 - m3) % 2 else 1
    # sqrt(pre) * s, with the square root taken once in floating point
    val = math.sqrt(pre.numerator) / math.sqrt(pre.denominator) * float(s)
    return sign * val


def _rational_quirk(l1, l2, l3, m1, m2, m3):
    """True where the reference's lmax = 4 table holds 0 instead of the
    symbol: its generated source writes the 57 symbols whose exact value is a
    non-integer rational (+-1/3, +-1/6) as C++ integer divisions such as
    `1 / 3`, which evaluate to 0 (wigner3j.cpp:590-1986, e.g. line 607)."""
    w = abs(wigner3j(l1, l2, l3, m1, m2, m3))
    if w == 0.0 or w >= 1.0:
        return False
    inv2 = 1.0 / (w * w)
    k = round(math.sqrt(inv2))
    return k > 1 and abs(inv2 - k * k) < 1e-9 * inv2


def reference_w3j(l1, l2, l3, m1, m2, m3, lmax):
    """The coefficient compute_B3 uses for this lmax (the symbol, or 0 at the
    entries of the lmax = 4 table described in _rational_quirk)."""
    if lmax == 4 and _rational_quirk(l1, l2, l3, m1, m2, m3):
        return 0.0
    return wigner3j(l1, l2, l3, m1, m2, m3)


def w3j_table(lmax):
    """The flat (lmax+1)^6 table in the layout compute_B3 indexes
    (b3.cpp:187-199): ((lmax+1)^4 l1^2 + (lmax+1)^2 l2^2 (2l1+1)
    + l3^2 (2l2+1)(2l1+1) + m1 (2l3+1)(2l2+1) + m2 (2l3+1) + m3), with m_k
    counted from -l_k."""
    L = lmax + 1
    out = np.zeros(L ** 6)
    for l1 in range(L):
        for l2 in range(L):
            for l3 in range(L):
                if abs(l1 - l2) > l3 or l3 > l1 + l2:
                    continue
                base = (L ** 4 * l1 * l1 + L ** 2 * l2 * l2 * (2 * l1 + 1)
                        + l3 * l3 * (2 * l2 + 1) * (2 * l1 + 1))
                for a in range(2 * l1 + 1):
                    for b in range(2 * l2 + 1):
                        for c in range(2 * l3 + 1):
                            idx = base + a * (2 * l3 + 1) * (2 * l2 + 1) + b * (2 * l3 + 1) + c
                            out[idx] = reference_w3j(l1, l2, l3, a - l1, b - l2,
                                                     c - l3, lmax)
    return out


def triangles(lmax):
    """(l1, l2, l3) in the reference's loop order (b3.cpp:181-186)."""
    out = []
    for l1 in range(lmax + 1):
        for l2 in range(lmax + 1):
            for l3 in range(lmax + 1):
                if abs(l1 - l2) > l3 or l3 > l1 + l2:
                    continue
                out.append((l1, l2, l3))
    return out


def n_ls(lmax):
    return len(triangles(lmax))


def n_descriptors(n_species, N, lmax):
    n_rad = n_species * N
    return n_rad * (n_rad + 1) * (n_rad + 2) // 6 * n_ls(lmax)


def radial_triples(n_rad):
    return [(a, b, c) for a in range(n_rad) for b in range(a, n_rad)
            for c in range(b, n_rad)]


def terms(lmax):
    """Per triangle: arrays (i1, i2, i3, W) of harmonic indices with
    m1 + m2 + m3 = 0 (the reference's selection, b3.cpp:193)."""
    out = []
    for (l1, l2, l3) in triangles(lmax):
        rows = []
        for m1 in range(-l1, l1 + 1):
            for m2 in range(-l2, l2 + 1):
                m3 = -m1 - m2
                if abs(m3) > l3:
                    continue
                rows.append((l1 * l1 + l1 + m1, l2 * l2 + l2 + m2,
                             l3 * l3 + l3 + m3,
                             reference_w3j(l1, l2, l3, m1, m2, m3, lmax)))
        arr = np.array(rows, dtype=np.float64).reshape(-1, 4)
        out.append((arr[:, 0].astype(np.int64), arr[:, 1].astype(np.int64),
                    arr[:, 2].astype(np.int64), arr[:, 3]))
    return out


def complex_sph_harm(x, y, z, lmax):
    """Complex harmonics and Cartesian gradients (y_grad.cpp:24 convention),
    obtained from the real ones: for m > 0 with R = Y_{l,m}, S = Y_{l,-m}
    (real), Y_l^m = (-1)^m (R + i S)/sqrt 2, Y_l^-m = (R - i S)/sqrt 2."""
    Y, Yx, Yy, Yz = real_sph_harm(x, y, z, lmax)
    outs = []
    for R in (Y, Yx, Yy, Yz):
        C = R.astype(np.complex128)
        for l in range(1, lmax + 1):
            for m in range(1, l + 1):
                p, q = l * l + l + m, l * l + l - m
                a, b = R[..., p], R[..., q]
                C[..., p] = (-1) ** m * (a + 1j * b) / math.sqrt(2.0)
                C[..., q] = (a - 1j * b) / math.sqrt(2.0)
        outs.append(C)
    return tuple(outs)


def complex_single_bond(structure, n_species, N, lmax, r1, rcut,
                        cutoff_function="quadratic", store_dervs=True):
    """b3.cpp:243-381.  c has shape (noa, n_species*N*H) complex; dc
    (3*n_kept_pairs, sb) complex with row 3*pair + comp."""
    noa = structure.noa
    H = (lmax + 1) ** 2
    sb = n_species * N * H
    nsp = structure.neighbor_species
    rel = structure.relative_positions
    cnt = structure.neighbor_count
    owner = np.repeat(np.arange(noa), cnt)
    keep = rel[:, 0] <= rcut
    ucount = np.bincount(owner[keep], minlength=noa).astype(np.int64)
    ucum = np.concatenate([[0], np.cumsum(ucount)]).astype(np.int64)
    rk = rel[keep]
    r, x, y, z = rk[:, 0], rk[:, 1], rk[:, 2], rk[:, 3]
    g, gx, gy, gz = calculate_radial(x, y, z, r, np.full(len(r), rcut), N, r1,
                                     cutoff_function)
    Y, Yx, Yy, Yz = complex_sph_harm(x, y, z, lmax)
    s_j = nsp[keep]
    own = owner[keep]
    npairs = len(r)
    c = np.zeros((noa, n_species, N, H), dtype=np.complex128)
    np.add.at(c, (own, s_j), g[:, :, None] * Y[:, None, :])
    c = c.reshape(noa, sb)
    dc = None
    if store_dervs:
        dc = np.zeros((npairs, 3, n_species, N, H), dtype=np.complex128)
        pidx = np.arange(npairs)
        for k, (gk, Yk) in enumerate(((gx, Yx), (gy, Yy), (gz, Yz))):
            dc[pidx, k, s_j] = gk[:, :, None] * Y[:, None, :] + g[:, :, None] * Yk[:, None, :]
        dc = dc.reshape(3 * npairs, sb)
    return dict(c=c, dc=dc, neighbor_coordinates=rk[:, 1:].copy(),
                unique_neighbor_count=ucount, cumulative_neighbor_count=ucum,
                neighbor_indices=structure.structure_indices[keep], keep=keep)


def compute_b3(c, n_species, N, lmax, dc=None, ucum=None):
    """B3 values, norms and optionally stored derivatives (b3.cpp:134-240)."""
    noa = c.shape[0]
    n_rad = n_species * N
    H = (lmax + 1) ** 2
    cc = c.reshape(noa, n_rad, H)
    tri = np.array(radial_triples(n_rad))
    tl = terms(lmax)
    nls = len(tl)
    p = np.zeros((noa, len(tri), nls))
    for t, (i1, i2, i3, W) in enumerate(tl):
        # sum over terms of W c1 c2 c3 for every radial triple
        a1 = cc[:, tri[:, 0]][:, :, i1]          # (noa, ntri, nterm)
        a2 = cc[:, tri[:, 1]][:, :, i2]
        a3 = cc[:, tri[:, 2]][:, :, i3]
        p[:, :, t] = np.real(np.einsum("atk,k->at", a1 * a2 * a3, W))
    p = p.reshape(noa, -1)
    norms = np.sqrt(np.einsum("ad,ad->a", p, p))
    out = dict(p=p, norms=norms)
    if dc is not None:
        nrow = dc.shape[0]
        owner3 = np.repeat(np.repeat(np.arange(noa), np.diff(ucum)), 3)
        dcc = dc.reshape(nrow, n_rad, H)
        crow = cc[owner3]
        dp = np.zeros((nrow, len(tri), nls))
        for t, (i1, i2, i3, W) in enumerate(tl):
            c1 = crow[:, tri[:, 0]][:, :, i1]
            c2 = crow[:, tri[:, 1]][:, :, i2]
            c3 = crow[:, tri[:, 2]][:, :, i3]
            d1 = dcc[:, tri[:, 0]][:, :, i1]
            d2 = dcc[:, tri[:, 1]][:, :, i2]
            d3 = dcc[:, tri[:, 2]][:, :, i3]
            v = d1 * c2 * c3 + c1 * d2 * c3 + c1 * c2 * d3
            dp[:, :, t] = np.real(np.einsum("rtk,k->rt", v, W))
        dp = dp.reshape(nrow, -1)
        out["dp"] = dp
        out["force_dots"] = np.einsum("rd,rd->r", dp, out["p"][owner3])
    return out


def b3_adjoint(c, w, n_species, N, lmax):
    """u = dE/dc (holomorphic derivative) for dE/dp = w:
    dE = Re sum u dc.  Returns complex (noa, sb)."""
    noa = c.shape[0]
    n_rad = n_species * N
    H = (lmax + 1) ** 2
    cc = c.reshape(noa, n_rad, H)
    tri = np.array(radial_triples(n_rad))
    tl = terms(lmax)
    nls = len(tl)
    ww = w.reshape(noa, len(tri), nls)
    u = np.zeros((noa, n_rad, H), dtype=np.complex128)
    for t, (i1, i2, i3, W) in enumerate(tl):
        wt = ww[:, :, t]                                 # (noa, ntri)
        c1 = cc[:, tri[:, 0]][:, :, i1]
        c2 = cc[:, tri[:, 1]][:, :, i2]
        c3 = cc[:, tri[:, 2]][:, :, i3]
        f = wt[:, :, None] * W[None, None, :]
        for (pos, val, ik) in ((0, f * c2 * c3, i1), (1, f * c1 * c3, i2),
                               (2, f * c1 * c2, i3)):
            nidx = tri[:, pos]
            for k in range(len(ik)):
                np.add.at(u, (slice(None), nidx, ik[k]), val[:, :, k])
    return u.reshape(noa, -1)


def real_adjoint(u, n_species, N, lmax):
    """dE/dc_real for the real single bond c_real of the same pairs, from the
    complex-basis adjoint u (c_complex is a fixed linear map of c_real)."""
    noa = u.shape[0]
    H = (lmax + 1) ** 2
    uu = u.reshape(noa, -1, H)
    out = np.real(uu).copy()
    s2 = math.sqrt(2.0)
    for l in range(1, lmax + 1):
        for m in range(1, l + 1):
            p, q = l * l + l + m, l * l + l - m
            sg = (-1) ** m
            up, um = uu[..., p], uu[..., q]
            out[..., p] = (sg * up.real + um.real) / s2
            out[..., q] = (um.imag - sg * up.imag) / s2
    return out.reshape(noa, -1)


def pair_forces(structure, u, n_species, N, lmax, r1, rcut, cutoff_function):
    """f_ij = Re sum u_i . d c_i / d r_ij over the structure's neighbors with
    the complex derivatives of b3.cpp:332-371 (zero beyond rcut)."""
    owner = np.repeat(np.arange(structure.noa), structure.neighbor_count)
    nsp = structure.neighbor_species
    rel = structure.relative_positions
    r, x, y, z = rel[:, 0], rel[:, 1], rel[:, 2], rel[:, 3]
    keep = r <= rcut
    H = (lmax + 1) ** 2
    g, gx, gy, gz = calculate_radial(x, y, z, r, np.full(len(r), rcut), N, r1,
                                     cutoff_function)
    Y, Yx, Yy, Yz = complex_sph_harm(x, y, z, lmax)
    uu = u.reshape(structure.noa, n_species, N, H)[owner, nsp]
    f = np.zeros((len(r), 3))
    for comp, (gd, Yd) in enumerate(((gx, Yx), (gy, Yy), (gz, Yz))):
        dbond = gd[:, :, None] * Y[:, None, :] + g[:, :, None] * Yd[:, None, :]
        f[:, comp] = np.real(np.einsum("pnh,pnh->p", uu, dbond))
    f[~keep] = 0
    return f


class B3:
    """B3 descriptor calculator (b3.h:11-33, b3.cpp:12-27)."""

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings):
        if radial_basis != "chebyshev":
            raise ValueError("oracle supports the chebyshev basis only")
        if descriptor_settings[2] > 4:
            raise ValueError("B3 is defined for lmax <= 4 (b3.cpp:150-160)")
        self.radial_basis = radial_basis
        self.cutoff_function = cutoff_function
        self.radial_hyps = list(radial_hyps)
        self.cutoff_hyps = list(cutoff_hyps)
        self.descriptor_settings = list(descriptor_settings)
        ns = descriptor_settings[0]
        self.cutoffs = np.full((ns, ns), float(radial_hyps[1]))
        self.store_dervs = True

    def compute_struc(self, structure):
        """b3.cpp:29-132."""
        from .b2 import assemble_values
        ns, N, lmax = self.descriptor_settings
        sbd = complex_single_bond(structure, ns, N, lmax, self.radial_hyps[0],
                                  self.radial_hyps[1], self.cutoff_function,
                                  store_dervs=self.store_dervs)
        b3 = compute_b3(sbd["c"], ns, N, lmax,
                        sbd["dc"] if self.store_dervs else None,
                        sbd["cumulative_neighbor_count"])
        dv = assemble_values(structure, ns, b3["p"], b3["norms"], b3.get("dp"),
                             b3.get("force_dots"), sbd, self.store_dervs)
        dv._c = sbd["c"]
        dv._p = b3["p"]
        dv._norms = b3["norms"]
        dv._sbd = sbd
        return dv
