"""Energy / force / stress through the descriptor adjoint (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Two consumers of the same chain rule:

* the mapped-beta pair style, restated from lammps_plugins/pair_flare.cpp:68-184
  and lammps_plugins/lammps_descriptor.cpp:209-304 (E_i = p^T beta p / |p|^2,
  w = dE/dp, u = dE/dc, f_ij = u . dc/dr_ij);
* the kernel form of SparseGP::predict_mean (sparse_gp.cpp:612-628 over
  normalized_dot_product.cpp:115-210), evaluated without storing
  descriptor_force_dervs: dE/dp_i = sum_k sigma^2 alpha_k power z^(power-1)
  (dhat_k - z phat_i) / |p_i|, then the same u and f_ij.

Both are checked in tests against the stored-derivative oracle.
"""
import numpy as np

from . import b3 as b3mod
from .b2 import single_bond_multiple_cutoffs, compute_b2
from .basis import calculate_radial, real_sph_harm

EMPTY_THRESH = 1e-8


def b2_adjoint(c, w, n_species, N, lmax):
    """u[n1, lm] = 2 sum_n2 w[(n1,n2),l] c[n2,lm] * (1 if n1 == n2 else 1/2).

    lammps_descriptor.cpp:272-303.  c: (noa, n_rad*H); w: (noa, n_d)."""
    noa = c.shape[0]
    n_rad = n_species * N
    H = (lmax + 1) ** 2
    cc = c.reshape(noa, n_rad, H)
    iu = np.triu_indices(n_rad)
    ww = w.reshape(noa, len(iu[0]), lmax + 1)
    u = np.zeros_like(cc)
    for l in range(lmax + 1):
        W = np.zeros((noa, n_rad, n_rad))
        W[:, iu[0], iu[1]] = ww[:, :, l]
        # symmetric with the diagonal counted twice in the product rule
        Wsym = W + np.transpose(W, (0, 2, 1))
        sl = slice(l * l, (l + 1) * (l + 1))
        u[:, :, sl] = np.einsum("ank,akm->anm", Wsym, cc[:, :, sl])
    return u.reshape(noa, n_rad * H)


def pair_forces(structure, u, n_species, N, lmax, r1, cutoffs, cutoff_function,
                strict=False):
    """Per structure-neighbor f_ij = dE/dr_ij = u_i . d c_i / d r_ij.

    Pairs outside the descriptor cutoff get zero.  ``strict`` selects the
    pair style's filter rsq < rc^2 (pair_flare.cpp:150) instead of B2's
    r <= rc (b2.cpp:277)."""
    sp = structure.species
    owner = np.repeat(np.arange(structure.noa), structure.neighbor_count)
    nsp = structure.neighbor_species
    rel = structure.relative_positions
    rc = np.asarray(cutoffs)[sp[owner], nsp]
    r, x, y, z = rel[:, 0], rel[:, 1], rel[:, 2], rel[:, 3]
    if strict:
        keep = (x * x + y * y + z * z) < rc * rc
    else:
        keep = r <= rc
    H = (lmax + 1) ** 2
    g, gx, gy, gz = calculate_radial(x, y, z, r, rc, N, r1, cutoff_function)
    Y, Yx, Yy, Yz = real_sph_harm(x, y, z, lmax)
    uu = u.reshape(structure.noa, n_species, N, H)[owner, nsp]   # (P, N, H)
    f = np.zeros((len(r), 3))
    for comp, (gd, Yd) in enumerate(((gx, Yx), (gy, Yy), (gz, Yz))):
        dbond = gd[:, :, None] * Y[:, None, :] + g[:, :, None] * Yd[:, None, :]
        f[:, comp] = np.einsum("pnh,pnh->p", uu, dbond)
    f[~keep] = 0
    return f


def gather_forces(structure, f):
    """F_i = sum_j f_ij (central), F_j -= f_ij (neighbor)."""
    owner = np.repeat(np.arange(structure.noa), structure.neighbor_count)
    F = np.zeros((structure.noa, 3))
    np.add.at(F, owner, f)
    np.add.at(F, structure.structure_indices, -f)
    return F


def flare_stress(structure, f):
    """-(1/V) sum f_a r_b in the order xx, xy, xz, yy, yz, zz
    (normalized_dot_product.cpp:197-202)."""
    r = structure.relative_positions[:, 1:]
    S = -(f.T @ r) / structure.volume
    return np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])


def lammps_virial(structure, f):
    """sum over pairs of del (x) f with del = x_i - x_j = -r_ij, in LAMMPS
    order xx, yy, zz, xy, xz, yz (ev_tally_xyz, pair_flare.cpp:169)."""
    d = -structure.relative_positions[:, 1:]
    V = d.T @ f
    return np.array([V[0, 0], V[1, 1], V[2, 2], V[0, 1], V[0, 2], V[1, 2]])


def descriptors(structure, settings):
    """c (noa, sb), p (noa, n_d), |p| for a B2 or B3 setting dict (B3 when
    settings["kind"] == "B3"; its c is complex)."""
    ns, N, lmax = settings["n_species"], settings["N"], settings["lmax"]
    if settings.get("kind", "B2") == "B3":
        sbd = b3mod.complex_single_bond(structure, ns, N, lmax, settings["r1"],
                                        settings["rcut"], settings["cutoff_function"],
                                        store_dervs=False)
        out = b3mod.compute_b3(sbd["c"], ns, N, lmax)
        return sbd["c"], out["p"], out["norms"]
    sbd = single_bond_multiple_cutoffs(structure, ns, N, lmax, settings["r1"],
                                       settings["cutoffs"],
                                       settings["cutoff_function"],
                                       store_dervs=False)
    b2 = compute_b2(sbd["c"], ns, N, lmax)
    return sbd["c"], b2["p"], b2["norms"]


def descriptor_pair_forces(structure, settings, c, w, strict=False):
    """f_ij from dE/dp = w through the descriptor's adjoint (B2 or B3)."""
    ns, N, lmax = settings["n_species"], settings["N"], settings["lmax"]
    if settings.get("kind", "B2") == "B3":
        u = b3mod.b3_adjoint(c, w, ns, N, lmax)
        return b3mod.pair_forces(structure, u, ns, N, lmax, settings["r1"],
                                 settings["rcut"], settings["cutoff_function"])
    u = b2_adjoint(c, w, ns, N, lmax)
    return pair_forces(structure, u, ns, N, lmax, settings["r1"],
                       settings["cutoffs"], settings["cutoff_function"],
                       strict=strict)


def beta_form(structure, settings, beta_matrices, power=2):
    """Mapped-beta pair style on a periodic structure.

    Per atom (pair_flare.cpp:95-180): E_i from compute_energy_and_u
    (lammps_descriptor.cpp:250-270), skipped when |p|^2 < 1e-8 (:135).
    Returns dict(energy, atom_energies, forces, virial, stress)."""
    ns, N, lmax = settings["n_species"], settings["N"], settings["lmax"]
    c, p, norms = descriptors(structure, settings)
    noa = structure.noa
    nsq = norms * norms
    E = np.zeros(noa)
    w = np.zeros_like(p)
    for s in range(ns):
        idx = np.nonzero((structure.species == s) & (nsq >= EMPTY_THRESH))[0]
        if len(idx) == 0:
            continue
        B = beta_matrices[s]
        P = p[idx]
        q = nsq[idx]
        if power == 2:
            bp = P @ B.T
            e = np.einsum("ad,ad->a", P, bp) / q
            w[idx] = 2 * (bp - e[:, None] * P) / q[:, None]
        else:
            bv = np.asarray(B).reshape(-1)
            nrm = np.sqrt(q)
            e = (P @ bv) / nrm
            w[idx] = bv[None, :] / nrm[:, None] - e[:, None] * P / q[:, None]
        E[idx] = e
    f = descriptor_pair_forces(structure, settings, c, w, strict=True)
    F = gather_forces(structure, f)
    return dict(energy=E.sum(), atom_energies=E, forces=F,
                virial=lammps_virial(structure, f),
                stress=flare_stress(structure, f), pair_f=f)


def kernel_form(structure, settings, sparse_descriptors, alpha, sigma, power):
    """SparseGP::predict_mean for one NormalizedDotProduct kernel without
    stored derivatives.  Returns dict(energy, atom_energies, forces, stress,
    mean_efs)."""
    ns, N, lmax = settings["n_species"], settings["N"], settings["lmax"]
    c, p, norms = descriptors(structure, settings)
    noa = structure.noa
    sig2 = sigma * sigma
    E = np.zeros(noa)
    w = np.zeros_like(p)
    sd = sparse_descriptors
    for s in range(ns):
        D = sd.descriptors[s]
        nD = sd.descriptor_norms[s]
        off = sd.cumulative_type_count[s]
        a = alpha[off:off + len(nD)]
        okd = nD >= EMPTY_THRESH
        idx = np.nonzero((structure.species == s) & (norms >= EMPTY_THRESH))[0]
        if len(idx) == 0 or not np.any(okd):
            continue
        Dh = D[okd] / nD[okd, None]
        a = a[okd]
        Ph = p[idx] / norms[idx, None]
        z = Ph @ Dh.T                                   # (n_s, S)
        E[idx] = sig2 * (z ** power) @ a
        C = sig2 * power * (z ** (power - 1)) * a[None, :]
        G = C @ Dh                                      # (n_s, n_d)
        zc = np.einsum("ik,ik->i", C, z)
        w[idx] = (G - zc[:, None] * Ph) / norms[idx, None]
    f = descriptor_pair_forces(structure, settings, c, w)
    F = gather_forces(structure, f)
    S = flare_stress(structure, f)
    mean = np.concatenate([[E.sum()], F.reshape(-1), S])
    return dict(energy=E.sum(), atom_energies=E, forces=F, stress=S,
                mean_efs=mean, pair_f=f, w=w, c=c, p=p, norms=norms)


def unpack_beta(packed, n_d, power=2):
    """Potential-file beta -> dense matrices (pair_flare.cpp:363-395):
    off-diagonal entries of the packed upper triangle are halved."""
    packed = np.atleast_2d(packed)
    out = []
    for row in packed:
        if power == 1:
            out.append(row.copy())
            continue
        B = np.zeros((n_d, n_d))
        iu = np.triu_indices(n_d)
        B[iu] = row
        off = iu[0] != iu[1]
        B[iu[0][off], iu[1][off]] = row[off] / 2
        B[iu[1][off], iu[0][off]] = row[off] / 2
        out.append(B)
    return out


def varmap_coefficients(sparse_descriptors, Kuu_inverse, sigma, power, alpha_ind=0):
    """NormalizedDotProduct::compute_varmap_coefficients
    (normalized_dot_product.cpp:761-850): per species s the n_d x n_d map
    sum_ij -sigma^4 Kuu^-1_ij dhat_i dhat_j^T, plus sigma^2 on the diagonal
    while visiting the pair (0, 0); empty environments are skipped.  Returns
    (n_species, n_d^2) row-major, or None for power != 1 (the reference
    prints a message and returns an empty matrix)."""
    if power != 1:
        return None
    sd = sparse_descriptors
    nd = sd.n_descriptors
    sig2 = sigma * sigma
    out = np.zeros((sd.n_types, nd * nd))
    diag = np.arange(nd) * (nd + 1)
    for s in range(sd.n_types):
        n_t = sd.n_clusters_by_type[s]
        K_ind = alpha_ind + sd.cumulative_type_count[s]
        for i in range(n_t):
            pi = sd.descriptors[s][i]
            ni = sd.descriptor_norms[s][i]
            if ni < EMPTY_THRESH:
                continue
            for j in range(n_t):
                pj = sd.descriptors[s][j]
                nj = sd.descriptor_norms[s][j]
                if nj < EMPTY_THRESH:
                    continue
                kn = Kuu_inverse[K_ind + i, K_ind + j] / ni / nj
                out[s] += (sig2 * sig2 * np.outer(pi, pj) * (-kn)).ravel()
                if i == 0 and j == 0:
                    out[s][diag] += sig2
    return out


def std_atom(structure, settings, sigma, power=None, L_inv=None, sparse_normed=None,
             varmap=None):
    """ComputeFlareStdAtom::compute_peratom (compute_flare_std_atom.cpp:98-207)
    on a periodic structure, per atom in structure order.

    Map form (varmap: (n_species, n_d, n_d)): var = p.(M p) / |p|^2 / sigma^2
    (compute_energy_and_u with power 2).  L_inv form: k over all sparse
    clusters, (dhat . phat)^power in the block of the atom's species and 0
    elsewhere, var = 1 - sigma^2 |L_inv k|^2.  std = sqrt(var), -sqrt(-var)
    for var < 0, 0 for |p|^2 < 1e-8."""
    _, p, norms = descriptors(structure, settings)
    sig2 = sigma * sigma
    out = np.zeros(structure.noa)
    for i in range(structure.noa):
        nsq = float(p[i] @ p[i])
        if nsq < EMPTY_THRESH:
            continue
        s = int(structure.species[i])
        if varmap is not None:
            B = np.asarray(varmap[s]).reshape(p.shape[1], p.shape[1])
            var = float(p[i] @ (B @ p[i])) / nsq / sig2
        else:
            ph = p[i] / nsq ** 0.5
            kv = np.zeros(L_inv.shape[0])
            cum = 0
            for t, D in enumerate(sparse_normed):
                if t == s:
                    kv[cum:cum + len(D)] = (D @ ph) ** power
                cum += len(D)
            v = L_inv @ kv
            var = 1.0 - sig2 * float(v @ v)
        out[i] = var ** 0.5 if var >= 0.0 else -abs(var) ** 0.5
    return out
