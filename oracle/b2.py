"""B2 power-spectrum descriptor and DescriptorValues (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates src/flare_pp/descriptors/b2.cpp:76-399 and the data container of
src/flare_pp/descriptors/descriptor.h:31-90.
"""
import numpy as np

from .basis import calculate_radial, real_sph_harm


def n_descriptors(n_species, N, lmax):
    n_rad = n_species * N
    return n_rad * (n_rad + 1) // 2 * (lmax + 1)


def b2_index(n_rad, lmax):
    """(n1, n2, l) for every descriptor column, in the reference's order.

    The counter runs n1, n2 >= n1, l (b2.cpp:209-231).
    """
    out = []
    for n1 in range(n_rad):
        for n2 in range(n1, n_rad):
            for l in range(lmax + 1):
                out.append((n1, n2, l))
    return np.array(out, dtype=np.int64)


class DescriptorValues:
    """Per-species descriptor blocks of one structure (descriptor.h:31-57)."""

    def __init__(self):
        self.n_descriptors = 0
        self.n_types = 0
        self.n_atoms = 0
        self.volume = 0.0
        self.descriptors = []
        self.descriptor_force_dervs = []
        self.neighbor_coordinates = []
        self.descriptor_norms = []
        self.descriptor_force_dots = []
        self.cutoff_values = []
        self.cutoff_dervs = []
        self.neighbor_counts = []
        self.cumulative_neighbor_counts = []
        self.atom_indices = []
        self.neighbor_indices = []
        self.n_clusters = 0
        self.n_clusters_by_type = []
        self.cumulative_type_count = [0]
        self.n_neighbors_by_type = []


class ClusterDescriptor:
    """Sparse-set rows grouped by type (descriptor.h:61-90, descriptor.cpp)."""

    def __init__(self, structure=None, clusters=None):
        self.descriptors = []
        self.descriptor_norms = []
        self.cutoff_values = []
        self.n_clusters_by_type = []
        self.cumulative_type_count = []
        self.n_descriptors = 0
        self.n_types = 0
        self.n_clusters = 0
        if structure is not None:
            if clusters is None:
                self.add_all_clusters(structure)
            else:
                self.add_clusters_by_type(structure, clusters)

    def initialize_cluster(self, n_types, n_descriptors):
        """descriptor.cpp:68-85."""
        if self.n_clusters != 0:
            return
        self.n_types = n_types
        self.n_descriptors = n_descriptors
        self.descriptors = [np.zeros((0, n_descriptors)) for _ in range(n_types)]
        self.descriptor_norms = [np.zeros(0) for _ in range(n_types)]
        self.cutoff_values = [np.zeros(0) for _ in range(n_types)]
        self.n_clusters_by_type = [0] * n_types
        self.cumulative_type_count = [0] * n_types

    def add_clusters_by_type(self, dv, clusters):
        """descriptor.cpp:104-140."""
        self.initialize_cluster(dv.n_types, dv.n_descriptors)
        for s in range(self.n_types):
            idx = np.asarray(clusters[s], dtype=np.int64)
            self.descriptors[s] = np.vstack(
                [self.descriptors[s], dv.descriptors[s][idx]])
            self.descriptor_norms[s] = np.concatenate(
                [self.descriptor_norms[s], dv.descriptor_norms[s][idx]])
            self.cutoff_values[s] = np.concatenate(
                [self.cutoff_values[s], dv.cutoff_values[s][idx]])
        for s in range(self.n_types):
            self.n_clusters_by_type[s] += len(clusters[s])
            self.n_clusters += len(clusters[s])
            if s > 0:
                self.cumulative_type_count[s] = (
                    self.cumulative_type_count[s - 1]
                    + self.n_clusters_by_type[s - 1])

    def add_clusters(self, dv, clusters):
        """Clusters given as structure-wide cluster indices (:87-102)."""
        by_type = [[] for _ in range(dv.n_types)]
        for c in clusters:
            for t in range(dv.n_types):
                if dv.cumulative_type_count[t] <= c < dv.cumulative_type_count[t + 1]:
                    by_type[t].append(c - dv.cumulative_type_count[t])
                    break
        self.add_clusters_by_type(dv, by_type)

    def add_all_clusters(self, dv):
        self.add_clusters_by_type(
            dv, [list(range(dv.n_clusters_by_type[s])) for s in range(dv.n_types)])


def single_bond_multiple_cutoffs(structure, n_species, N, lmax, r1, cutoffs,
                                 cutoff_function="quadratic", store_dervs=True):
    """Single-bond coefficients c and their per-neighbor derivatives.

    src/flare_pp/descriptors/b2.cpp:244-399.  A structure neighbor enters when
    r <= cutoffs[s_i, s_j] (b2.cpp:277); the radial endpoint is reset to that
    pair cutoff (b2.cpp:352).  c has shape (noa, n_species*N*H) with column
    (s*N + n)*H + lm; dc has shape (3*n_pairs, sb) with row 3*pair + comp.
    """
    noa = structure.noa
    H = (lmax + 1) ** 2
    sb = n_species * N * H
    sp = structure.species
    nsp = structure.neighbor_species
    rel = structure.relative_positions
    cnt = structure.neighbor_count
    cum = structure.cumulative_neighbor_count
    owner = np.repeat(np.arange(noa), cnt)
    rc = np.asarray(cutoffs)[sp[owner], nsp] if len(owner) else np.zeros(0)
    keep = rel[:, 0] <= rc
    ucount = np.bincount(owner[keep], minlength=noa).astype(np.int64)
    ucum = np.concatenate([[0], np.cumsum(ucount)]).astype(np.int64)
    nbr_idx = structure.structure_indices[keep]
    rk = rel[keep]
    r, x, y, z = rk[:, 0], rk[:, 1], rk[:, 2], rk[:, 3]
    g, gx, gy, gz = calculate_radial(x, y, z, r, rc[keep], N, r1,
                                     cutoff_function)
    Y, Yx, Yy, Yz = real_sph_harm(x, y, z, lmax)
    s_j = nsp[keep]
    own = owner[keep]
    npairs = len(r)
    # bond[p, n, lm] = g[p, n] * Y[p, lm]
    bond = g[:, :, None] * Y[:, None, :]
    c = np.zeros((noa, n_species, N, H))
    np.add.at(c, (own, s_j), bond)
    c = c.reshape(noa, sb)
    dc = None
    if store_dervs:
        dc = np.zeros((npairs, 3, n_species, N, H))
        pidx = np.arange(npairs)
        dc[pidx, 0, s_j] = gx[:, :, None] * Y[:, None, :] + g[:, :, None] * Yx[:, None, :]
        dc[pidx, 1, s_j] = gy[:, :, None] * Y[:, None, :] + g[:, :, None] * Yy[:, None, :]
        dc[pidx, 2, s_j] = gz[:, :, None] * Y[:, None, :] + g[:, :, None] * Yz[:, None, :]
        dc = dc.reshape(3 * npairs, sb)
    return dict(c=c, dc=dc, neighbor_coordinates=rk[:, 1:].copy(),
                unique_neighbor_count=ucount, cumulative_neighbor_count=ucum,
                neighbor_indices=nbr_idx, keep=keep)


def compute_b2(c, n_species, N, lmax, dc=None, ucum=None):
    """B2 values, norms and (optionally) stored force derivatives.

    src/flare_pp/descriptors/b2.cpp:181-242.
    """
    noa = c.shape[0]
    n_rad = n_species * N
    H = (lmax + 1) ** 2
    cc = c.reshape(noa, n_rad, H)
    iu = np.triu_indices(n_rad)
    cols = []
    for l in range(lmax + 1):
        blk = cc[:, :, l * l:(l + 1) * (l + 1)]
        P = np.einsum("anm,akm->ank", blk, blk)
        cols.append(P[:, iu[0], iu[1]])
    # column order: pair-major then l
    p = np.stack(cols, axis=2).reshape(noa, -1)
    norms = np.sqrt(np.einsum("ad,ad->a", p, p))
    out = dict(p=p, norms=norms)
    if dc is not None:
        npairs = dc.shape[0] // 3
        owner = np.repeat(np.arange(noa), np.diff(ucum))
        dcc = dc.reshape(3 * npairs, n_rad, H)
        crow = np.repeat(cc[owner], 3, axis=0)
        dcols = []
        for l in range(lmax + 1):
            sl = slice(l * l, (l + 1) * (l + 1))
            M = (np.einsum("rnm,rkm->rnk", crow[:, :, sl], dcc[:, :, sl])
                 + np.einsum("rnm,rkm->rnk", dcc[:, :, sl], crow[:, :, sl]))
            dcols.append(M[:, iu[0], iu[1]])
        dp = np.stack(dcols, axis=2).reshape(3 * npairs, -1)
        prow = np.repeat(p[owner], 3, axis=0)
        out["dp"] = dp
        out["force_dots"] = np.einsum("rd,rd->r", dp, prow)
    return out


def assemble_values(structure, ns, p, norms, dp, force_dots, sbd, store_dervs):
    """Regroup per-atom descriptors and per-pair derivative rows by central
    species into DescriptorValues (b2.cpp:103-178, b3.cpp:56-131)."""
    ucount = sbd["unique_neighbor_count"]
    ucum = sbd["cumulative_neighbor_count"]
    dv = DescriptorValues()
    noa = structure.noa
    n_d = p.shape[1]
    dv.n_descriptors = n_d
    dv.n_types = ns
    dv.n_atoms = noa
    dv.volume = structure.volume
    sp = structure.species
    dv.cumulative_type_count = [0]
    for s in range(ns):
        atoms = np.nonzero(sp == s)[0]
        n_s = len(atoms)
        nn = ucount[atoms]
        dv.n_clusters_by_type.append(n_s)
        dv.cumulative_type_count.append(dv.cumulative_type_count[s] + n_s)
        dv.n_clusters += n_s
        dv.n_neighbors_by_type.append(int(nn.sum()))
        dv.descriptors.append(p[atoms].copy())
        dv.descriptor_norms.append(norms[atoms].copy())
        dv.cutoff_values.append(np.ones(n_s))
        dv.cutoff_dervs.append(np.zeros(3 * int(nn.sum())))
        dv.neighbor_counts.append(nn.copy())
        dv.cumulative_neighbor_counts.append(
            np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.int64)
            if n_s else np.zeros(0, np.int64))
        dv.atom_indices.append(atoms.copy())
        pair_rows = (np.concatenate([np.arange(ucum[a], ucum[a + 1])
                                     for a in atoms])
                     if n_s else np.zeros(0, np.int64)).astype(np.int64)
        dv.neighbor_indices.append(sbd["neighbor_indices"][pair_rows])
        dv.neighbor_coordinates.append(sbd["neighbor_coordinates"][pair_rows])
        if store_dervs:
            frows = (3 * pair_rows[:, None] + np.arange(3)[None]).ravel()
            dv.descriptor_force_dervs.append(dp[frows])
            dv.descriptor_force_dots.append(force_dots[frows])
        else:
            dv.descriptor_force_dervs.append(None)
            dv.descriptor_force_dots.append(None)
    return dv


class B2:
    """B2 descriptor calculator (b2.h:12-53, b2.cpp:13-50)."""

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings, cutoffs=None):
        if radial_basis != "chebyshev":
            raise ValueError("oracle supports the chebyshev basis only")
        self.radial_basis = radial_basis
        self.cutoff_function = cutoff_function
        self.radial_hyps = list(radial_hyps)
        self.cutoff_hyps = list(cutoff_hyps)
        self.descriptor_settings = list(descriptor_settings)
        ns = descriptor_settings[0]
        if cutoffs is None:
            cutoffs = np.full((ns, ns), float(radial_hyps[1]))
        self.cutoffs = np.asarray(cutoffs, dtype=np.float64)
        self.store_dervs = True

    def compute_struc(self, structure):
        """src/flare_pp/descriptors/b2.cpp:76-179."""
        ns, N, lmax = self.descriptor_settings
        sbd = single_bond_multiple_cutoffs(
            structure, ns, N, lmax, self.radial_hyps[0], self.cutoffs,
            self.cutoff_function, store_dervs=self.store_dervs)
        ucount = sbd["unique_neighbor_count"]
        ucum = sbd["cumulative_neighbor_count"]
        b2 = compute_b2(sbd["c"], ns, N, lmax,
                        sbd["dc"] if self.store_dervs else None, ucum)
        dv = assemble_values(structure, ns, b2["p"], b2["norms"],
                             b2.get("dp"), b2.get("force_dots"), sbd,
                             self.store_dervs)
        # extra, for the adjoint oracle: per-atom single-bond coefficients
        dv._c = sbd["c"]
        dv._p = b2["p"]
        dv._norms = b2["norms"]
        dv._sbd = sbd
        return dv
