"""NormalizedDotProduct kernel (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates src/flare_pp/kernels/normalized_dot_product.cpp.  k(d, p) =
sigma^2 (d.p / |d||p|)^power, block-diagonal in the central species.
"""
import numpy as np
import scipy.sparse as sps

EMPTY_THRESH = 1e-8


def _force_scatter(dv, s):
    """Sparse maps from force rows (3*pair+comp) of species block s to the
    force columns 1+3*atom+comp (+1 central, -1 neighbor) and to the six
    stress columns (coefficient -coord/V), following
    normalized_dot_product.cpp:180-203."""
    n_atoms = dv.n_atoms
    n_out = 1 + 3 * n_atoms + 6
    nn = dv.neighbor_counts[s]
    npairs = int(np.sum(nn))
    atom_of_pair = np.repeat(dv.atom_indices[s], nn)
    nbr = dv.neighbor_indices[s]
    rows, cols, vals = [], [], []
    vol_inv = 1.0 / dv.volume
    coords = dv.neighbor_coordinates[s]
    stress_col = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4,
                  (2, 2): 5}
    for comp in range(3):
        fr = 3 * np.arange(npairs) + comp
        rows += [fr, fr]
        cols += [1 + 3 * nbr + comp, 1 + 3 * atom_of_pair + comp]
        vals += [-np.ones(npairs), np.ones(npairs)]
        for comp2 in range(comp, 3):
            rows.append(fr)
            cols.append(np.full(npairs, 1 + 3 * n_atoms + stress_col[(comp, comp2)]))
            vals.append(-coords[:, comp2] * vol_inv)
    if npairs == 0:
        return sps.csr_matrix((0, n_out))
    return sps.csr_matrix((np.concatenate(vals),
                           (np.concatenate(rows), np.concatenate(cols))),
                          shape=(3 * npairs, n_out))


class NormalizedDotProduct:
    def __init__(self, sigma, power):
        self.sigma = float(sigma)
        self.sig2 = self.sigma * self.sigma
        self.power = float(power)
        self.kernel_hyperparameters = np.array([self.sigma])

    # ------------------------------------------------------------------
    def envs_envs(self, envs1, envs2, hyps=None):
        """normalized_dot_product.cpp:27-87."""
        sig_sq = (hyps[0] if hyps is not None else self.sigma) ** 2
        K = np.zeros((envs1.n_clusters, envs2.n_clusters))
        for s in range(envs1.n_types):
            d1, d2 = envs1.descriptors[s], envs2.descriptors[s]
            n1, n2 = envs1.descriptor_norms[s], envs2.descriptor_norms[s]
            if len(n1) == 0 or len(n2) == 0:
                continue
            dot = d1 @ d2.T
            ok = (n1 >= EMPTY_THRESH)[:, None] & (n2 >= EMPTY_THRESH)[None, :]
            with np.errstate(divide="ignore", invalid="ignore"):
                nd = dot / np.outer(n1, n2)
                val = np.where(ok, sig_sq * nd ** self.power, 0.0)
            c1, c2 = envs1.cumulative_type_count[s], envs2.cumulative_type_count[s]
            K[c1:c1 + len(n1), c2:c2 + len(n2)] += val
        return K

    # ------------------------------------------------------------------
    def envs_struc(self, envs, struc, hyps=None):
        """Stored-derivative form, normalized_dot_product.cpp:115-210.

        Returns the (n_sparse, 1 + 3*n_atoms + 6) matrix of energy, force and
        stress kernels."""
        sig_sq = (hyps[0] if hyps is not None else self.sigma) ** 2
        n_out = 1 + 3 * struc.n_atoms + 6
        K = np.zeros((envs.n_clusters, n_out))
        pw = self.power
        for s in range(envs.n_types):
            D = envs.descriptors[s]
            nD = envs.descriptor_norms[s]
            P = struc.descriptors[s]
            nP = struc.descriptor_norms[s]
            c_sparse = envs.cumulative_type_count[s]
            if len(nD) == 0 or len(nP) == 0:
                continue
            dot = D @ P.T                                   # (S, n_s)
            F = struc.descriptor_force_dervs[s]
            fd = D @ F.T                                    # (S, 3 n_pairs)
            sfd = struc.descriptor_force_dots[s]
            ok_i = nD >= EMPTY_THRESH
            ok_j = nP >= EMPTY_THRESH
            with np.errstate(divide="ignore", invalid="ignore"):
                nij = np.outer(nD, nP)
                nd = dot / nij
                ok = ok_i[:, None] & ok_j[None, :]
                en = np.where(ok, sig_sq * nd ** pw, 0.0)
                dval = np.where(ok, pw * nd ** (pw - 1), 0.0)
            K[c_sparse:c_sparse + len(nD), 0] += en.sum(1)
            nn = struc.neighbor_counts[s]
            jrow = np.repeat(np.arange(len(nP)), 3 * nn)   # atom of each force row
            with np.errstate(divide="ignore", invalid="ignore"):
                f1 = fd / nij[:, jrow]
                f2 = dot[:, jrow] * sfd[None, :] / (nij[:, jrow] * (nP[jrow] ** 2)[None, :])
                fkv = np.where(ok[:, jrow], sig_sq * dval[:, jrow] * (f1 - f2), 0.0)
            M = _force_scatter(struc, s)
            K[c_sparse:c_sparse + len(nD)] += (M.T @ fkv.T).T
        return K

    # ------------------------------------------------------------------
    def struc_struc(self, struc1, struc2, hyps=None):
        """normalized_dot_product.cpp:212-444 (full E/F/S covariance)."""
        sig_sq = (hyps[0] if hyps is not None else self.sigma) ** 2
        pw = self.power
        n1o = 1 + 3 * struc1.n_atoms + 6
        n2o = 1 + 3 * struc2.n_atoms + 6
        K = np.zeros((n1o, n2o))
        for s in range(struc1.n_types):
            P1, P2 = struc1.descriptors[s], struc2.descriptors[s]
            a1, a2 = struc1.descriptor_norms[s], struc2.descriptor_norms[s]
            if len(a1) == 0 or len(a2) == 0:
                continue
            F1, F2 = struc1.descriptor_force_dervs[s], struc2.descriptor_force_dervs[s]
            sfd1, sfd2 = struc1.descriptor_force_dots[s], struc2.descriptor_force_dots[s]
            dot = P1 @ P2.T
            fd1 = F1 @ P2.T            # (3np1, n2)
            fd2 = F2 @ P1.T            # (3np2, n1)
            ff = F1 @ F2.T             # (3np1, 3np2)
            ok = (a1 >= EMPTY_THRESH)[:, None] & (a2 >= EMPTY_THRESH)[None, :]
            if pw < 2 and np.any(ok & (np.abs(dot / np.outer(a1, a2)) < EMPTY_THRESH)):
                raise ValueError("Dot product of descriptors is 0, and the "
                                 "negative power function in force-force "
                                 "kernel diverges.")
            with np.errstate(divide="ignore", invalid="ignore"):
                nd = dot / np.outer(a1, a2)
                c1 = np.where(ok, (pw - 1) * pw * nd ** (pw - 2), 0.0)
                c2 = np.where(ok, pw * nd ** (pw - 1), 0.0)
                e = np.where(ok, nd ** pw, 0.0)
            K[0, 0] += sig_sq * e.sum()
            nn1, nn2 = struc1.neighbor_counts[s], struc2.neighbor_counts[s]
            r1 = np.repeat(np.arange(len(a1)), 3 * nn1)   # atom of force row
            r2 = np.repeat(np.arange(len(a2)), 3 * nn2)
            M1 = _force_scatter(struc1, s)                 # (3np1, n1o)
            M2 = _force_scatter(struc2, s)
            # energy / force-stress of struc2: sum over i of d k(i, j)/d r
            with np.errstate(divide="ignore", invalid="ignore"):
                # v2[i, r2] = d(norm_dot)/d r for rows of struc2
                v2 = (fd2.T / np.outer(a1, a2)[:, r2]
                      - nd[:, r2] * sfd2[None, :] / (a2[r2] ** 2)[None, :])
                v1 = (fd1 / np.outer(a1, a2)[r1, :]
                      - nd[r1, :] * sfd1[:, None] / (a1[r1] ** 2)[:, None])
            v2 = np.where(ok[:, r2], v2, 0.0)
            v1 = np.where(ok[r1, :], v1, 0.0)
            ef = (sig_sq * c2[:, r2] * v2).sum(0)          # (3np2,)
            K[0, :] += M2.T @ ef
            fe = (sig_sq * c2[r1, :] * v1).sum(1)          # (3np1,)
            K[:, 0] += M1.T @ fe
            # force/force: for each (i, j) pair of atoms, rows of i x rows of j
            # kern = sig2 (c1 v1 v2 + c2 (ff/nij - (sfd1 fd2)/(a1^3 a2)
            #        - (sfd2 fd1)/(a1 a2^3) + sfd1 sfd2 nd/(a1^2 a2^2)))
            # (explicit blockwise loop; small structures only)
            with np.errstate(divide="ignore", invalid="ignore"):
                nij = np.outer(a1, a2)
            A = np.zeros((len(r1), len(r2)))
            for i in range(len(a1)):
                ri = np.nonzero(r1 == i)[0]
                if len(ri) == 0 or a1[i] < EMPTY_THRESH:
                    continue
                for j in range(len(a2)):
                    rj = np.nonzero(r2 == j)[0]
                    if len(rj) == 0 or not ok[i, j]:
                        continue
                    vv1 = fd1[ri, j] / nij[i, j] - nd[i, j] * sfd1[ri] / a1[i] ** 2
                    vv2 = fd2[rj, i] / nij[i, j] - nd[i, j] * sfd2[rj] / a2[j] ** 2
                    v3 = ff[np.ix_(ri, rj)] / nij[i, j]
                    v4 = np.outer(sfd1[ri], fd2[rj, i]) / (a1[i] ** 3 * a2[j])
                    v5 = np.outer(fd1[ri, j], sfd2[rj]) / (a1[i] * a2[j] ** 3)
                    v6 = np.outer(sfd1[ri], sfd2[rj]) * nd[i, j] / (a1[i] ** 2 * a2[j] ** 2)
                    A[np.ix_(ri, rj)] += sig_sq * (c1[i, j] * np.outer(vv1, vv2)
                                                   + c2[i, j] * (v3 - v4 - v5 + v6))
            K += M1.T @ (M2.T @ A.T).T
        return K

    # ------------------------------------------------------------------
    def self_kernel_struc(self, struc, hyps=None):
        """Diagonal of struc_struc(struc, struc), :446-578."""
        return np.diag(self.struc_struc(struc, struc, hyps)).copy()

    # ------------------------------------------------------------------
    def compute_map_coeff_pow2(self, sparse_descriptors, alpha):
        """beta_s = sigma^2 sum_k alpha_k dhat_k dhat_k^T as packed upper
        triangles with doubled off-diagonals, :697-759.  Returns
        (n_species, n_d (n_d + 1) / 2)."""
        envs = sparse_descriptors
        n_d = envs.n_descriptors
        out = np.zeros((envs.n_types, n_d * (n_d + 1) // 2))
        iu = np.triu_indices(n_d)
        for s in range(envs.n_types):
            D = envs.descriptors[s]
            nD = envs.descriptor_norms[s]
            c = envs.cumulative_type_count[s]
            ok = nD >= EMPTY_THRESH
            Dh = D[ok] / nD[ok, None]
            a = alpha[c:c + len(nD)][ok]
            B = self.sig2 * (Dh.T * a) @ Dh
            packed = B[iu]
            packed = np.where(iu[0] != iu[1], 2 * packed, packed)
            out[s] = packed
        return out

    def compute_map_coeff_pow1(self, sparse_descriptors, alpha):
        """beta_s = sigma^2 sum_k alpha_k dhat_k, :645-695."""
        envs = sparse_descriptors
        out = np.zeros((envs.n_types, envs.n_descriptors))
        for s in range(envs.n_types):
            D = envs.descriptors[s]
            nD = envs.descriptor_norms[s]
            c = envs.cumulative_type_count[s]
            ok = nD >= EMPTY_THRESH
            out[s] = self.sig2 * (alpha[c:c + len(nD)][ok] @ (D[ok] / nD[ok, None]))
        return out
