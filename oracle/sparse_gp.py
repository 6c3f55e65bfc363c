"""Sparse GP training solve and prediction (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates SparseGP from src/flare_pp/bffs/sparse_gp.cpp.  The reference grows
Kuu and Kuf block by block as structures and environments are added
(update_Kuu / update_Kuf / stack_*, :333-574); the finished matrices are
Kuu = envs_envs(sparse, sparse) and Kuf = envs_struc(sparse, structure)
columns, with rows ordered by type and, within a type, in insertion order.
This oracle forms those finished matrices directly.
"""
import numpy as np
import scipy.linalg as sla

from .b2 import ClusterDescriptor


class SparseGP:
    def __init__(self, kernels, energy_noise, force_noise, stress_noise):
        self.kernels = list(kernels)
        self.energy_noise = energy_noise
        self.force_noise = force_noise
        self.stress_noise = stress_noise
        self.Kuu_jitter = 1e-8
        self.sparse_descriptors = [None] * len(self.kernels)
        self.sparse_indices = [[] for _ in self.kernels]
        self.training_structures = []
        self.training_atom_indices = []
        self.y = np.zeros(0)
        self.noise_vector = np.zeros(0)
        self.label_kind = np.zeros(0, dtype=np.int32)   # 0 energy, 1 force, 2 stress

    # ------------------------------------------------------------------
    def _init_sparse(self, structure):
        for i, _ in enumerate(self.kernels):
            if self.sparse_descriptors[i] is None:
                dv = structure.descriptors[i]
                cd = ClusterDescriptor()
                cd.initialize_cluster(dv.n_types, dv.n_descriptors)
                self.sparse_descriptors[i] = cd

    def add_specific_environments(self, structure, atoms):
        """sparse_gp.cpp:135-183: clusters whose central atom is listed,
        kept in the structure's per-type order."""
        self._init_sparse(structure)
        atoms = list(atoms)
        for i, _ in enumerate(self.kernels):
            dv = structure.descriptors[i]
            self.sparse_indices[i].append(atoms)
            by_type = []
            for t in range(dv.n_types):
                ai = dv.atom_indices[t]
                by_type.append([k for k in range(len(ai))
                                for a in atoms if ai[k] == a])
            self.sparse_descriptors[i].add_clusters_by_type(dv, by_type)

    def add_all_environments(self, structure):
        """sparse_gp.cpp:305-331."""
        self._init_sparse(structure)
        for i, _ in enumerate(self.kernels):
            self.sparse_descriptors[i].add_all_clusters(structure.descriptors[i])
            self.sparse_indices[i].append(list(range(structure.noa)))

    def add_training_structure(self, structure, atom_indices=(-1,)):
        """sparse_gp.cpp:464-552: labels [energy, forces of the listed atoms,
        stress] with noise 1/sigma^2 per label type."""
        self._init_sparse(structure)
        if atom_indices[0] == -1:
            atoms = list(range(structure.noa))
            n_force = len(structure.forces)
        else:
            atoms = list(atom_indices)
            n_force = 3 * len(atoms)
        n_energy = len(structure.energy)
        n_stress = len(structure.stresses)
        y = [np.asarray(structure.energy, dtype=np.float64)]
        if n_force:
            f = np.asarray(structure.forces, dtype=np.float64)
            y.append(np.concatenate([f[3 * a:3 * a + 3] for a in atoms]))
        y.append(np.asarray(structure.stresses, dtype=np.float64))
        self.y = np.concatenate([self.y] + y)
        self.noise_vector = np.concatenate([
            self.noise_vector,
            np.full(n_energy, 1 / self.energy_noise ** 2),
            np.full(n_force, 1 / self.force_noise ** 2),
            np.full(n_stress, 1 / self.stress_noise ** 2)])
        self.label_kind = np.concatenate([
            self.label_kind, np.zeros(n_energy, np.int32), np.ones(n_force, np.int32),
            np.full(n_stress, 2, np.int32)])
        self.training_structures.append(structure)
        self.training_atom_indices.append(atoms)

    # ------------------------------------------------------------------
    @property
    def n_sparse(self):
        return sum(sd.n_clusters for sd in self.sparse_descriptors)

    def Kuu(self):
        blocks = [k.envs_envs(sd, sd) for k, sd in
                  zip(self.kernels, self.sparse_descriptors)]
        return sla.block_diag(*blocks)

    def Kuf_columns(self, structure, atoms=None):
        """Label columns of one training structure (energy, force, stress)."""
        kms = []
        for k, sd, i in zip(self.kernels, self.sparse_descriptors,
                            range(len(self.kernels))):
            kms.append(k.envs_struc(sd, structure.descriptors[i]))
        km = np.vstack(kms)
        cols = []
        n = structure.noa
        if len(structure.energy):
            cols.append(km[:, 0:1])
        if len(structure.forces):
            for a in (atoms if atoms is not None else range(n)):
                cols.append(km[:, 1 + 3 * a:4 + 3 * a])
        if len(structure.stresses):
            cols.append(km[:, 1 + 3 * n:7 + 3 * n])
        return np.hstack(cols) if cols else np.zeros((km.shape[0], 0))

    def Kuf(self):
        return np.hstack([self.Kuf_columns(s, a) for s, a in
                          zip(self.training_structures,
                              self.training_atom_indices)])

    def update_matrices_QR(self):
        """sparse_gp.cpp:576-610."""
        self.Kuu_mat, self.Kuf_mat = self.Kuu(), self.Kuf()
        self._solve()

    def _solve(self):
        Kuu, Kuf = self.Kuu_mat, self.Kuf_mat
        n = Kuu.shape[0]
        L = np.linalg.cholesky(Kuu + self.Kuu_jitter * np.eye(n))
        self.L_inv = sla.solve_triangular(L, np.eye(n), lower=True)
        self.Kuu_inverse = self.L_inv.T @ self.L_inv
        sq = np.sqrt(self.noise_vector)
        A = np.vstack([sq[:, None] * Kuf.T, L.T])
        b = np.concatenate([sq * self.y, np.zeros(n)])
        Q, R = np.linalg.qr(A, mode="reduced")
        self.R_inv = sla.solve_triangular(R, np.eye(n), lower=False)
        self.alpha = self.R_inv @ (Q.T @ b)
        self.Sigma = self.R_inv @ self.R_inv.T
        self.L_diag = np.diag(self.L_inv).copy()
        self.R_inv_diag = np.diag(self.R_inv).copy()

    # ---- likelihood (sparse_gp.cpp:704-992, 1105-1140) -------------------
    @property
    def hyperparameters(self):
        return np.array([k.sigma for k in self.kernels]
                        + [self.energy_noise, self.force_noise, self.stress_noise])

    def _kernel_blocks(self):
        """Row ranges of each kernel's sparse set in Kuu and Kuf."""
        out, o = [], 0
        for sd in self.sparse_descriptors:
            out.append((o, o + sd.n_clusters))
            o += sd.n_clusters
        return out

    def set_hyperparameters(self, hyps):
        """sparse_gp.cpp:1105-1140 for NormalizedDotProduct kernels: each
        kernel's Kuu block and Kuf rows rescaled by (sigma_new / sigma)^2
        (Kuu_grad / Kuf_grad [0], normalized_dot_product.cpp:581-615), the
        noise vector rebuilt, and the QR solve repeated."""
        nk = len(self.kernels)
        for k, (a, b), h in zip(self.kernels, self._kernel_blocks(), hyps[:nk]):
            scale = h * h / k.sig2
            self.Kuu_mat[a:b, a:b] *= scale
            self.Kuf_mat[a:b, :] *= scale
            k.sigma = float(h)
            k.sig2 = k.sigma * k.sigma
            k.kernel_hyperparameters = np.array([k.sigma])
        self.energy_noise, self.force_noise, self.stress_noise = (float(v) for v in hyps[nk:nk + 3])
        one = [self.label_kind == t for t in range(3)]
        self.noise_vector = (one[0] / self.energy_noise ** 2 + one[1] / self.force_noise ** 2
                             + one[2] / self.stress_noise ** 2)
        self._solve()

    def compute_likelihood(self):
        """sparse_gp.cpp:959-992: Qff + Lambda through a column-pivoted QR."""
        noise = 1 / self.noise_vector
        Kuu_inverse = self.L_inv.T @ self.L_inv
        Q = self.Kuf_mat.T @ Kuu_inverse @ self.Kuf_mat + np.diag(noise)
        _, R, _ = sla.qr(Q, pivoting=True)
        q_inv_y = np.linalg.solve(Q, self.y)
        self.complexity_penalty = -np.sum(np.log(np.abs(np.diag(R)))) / 2
        self.data_fit = -0.5 * self.y @ q_inv_y
        self.constant_term = -0.5 * len(self.y) * np.log(2 * np.pi)
        self.log_marginal_likelihood = (self.complexity_penalty + self.data_fit
                                        + self.constant_term)
        return self.log_marginal_likelihood

    def compute_likelihood_stable(self):
        """sparse_gp.cpp:704-732."""
        nv = self.noise_vector
        self.data_fit = -0.5 * self.y @ (nv * (self.y - self.Kuf_mat.T @ self.alpha))
        self.constant_term = -0.5 * len(self.y) * np.log(2 * np.pi)
        noise_det = np.sum(np.log(nv))
        kuu_inv_det = -2 * np.sum(np.log(np.abs(self.L_diag)))
        sigma_inv_det = 2 * np.sum(np.log(np.abs(self.R_inv_diag)))
        self.complexity_penalty = 0.5 * (noise_det + kuu_inv_det + sigma_inv_det)
        self.log_marginal_likelihood = (self.complexity_penalty + self.data_fit
                                        + self.constant_term)
        return self.log_marginal_likelihood

    def compute_likelihood_gradient_stable(self):
        """sparse_gp.cpp:734-862 (the form without precomputed KnK) for
        NormalizedDotProduct kernels: dKuu/dsigma = 2 Kuu / sigma and
        dKuf/dsigma = 2 Kuf / sigma (normalized_dot_product.cpp:581-615),
        each kernel's gradient masked to its own block of Kuu and rows of
        Kuf (:775-829).  Sets likelihood_gradient (sigma per kernel, sigma_e,
        sigma_f, sigma_s) and returns the log marginal likelihood."""
        Kuf, Kuu, S, a, y = self.Kuf_mat, self.Kuu_mat, self.Sigma, self.alpha, self.y
        nv = self.noise_vector
        r = y - Kuf.T @ a
        self.data_fit = -0.5 * y @ (nv * r)
        self.constant_term = -0.5 * len(y) * np.log(2 * np.pi)
        one = [(self.label_kind == t).astype(np.float64) for t in range(3)]
        noises = [self.energy_noise, self.force_noise, self.stress_noise]
        noise_det = -2 * sum(o.sum() * np.log(abs(s)) for o, s in zip(one, noises))
        kuu_inv_det = -2 * np.sum(np.log(np.abs(self.L_diag)))
        sigma_inv_det = 2 * np.sum(np.log(np.abs(self.R_inv_diag)))
        self.complexity_penalty = 0.5 * (noise_det + kuu_inv_det + sigma_inv_det)
        self.log_marginal_likelihood = (self.complexity_penalty + self.data_fit
                                        + self.constant_term)
        nk = len(self.kernels)
        grad = np.zeros(nk + 3)
        for i, (k, (a0, a1)) in enumerate(zip(self.kernels, self._kernel_blocks())):
            sig = k.sigma
            Kuu_grad = np.zeros_like(Kuu)
            Kuu_grad[a0:a1, a0:a1] = Kuu[a0:a1, a0:a1] * (2 / sig)
            Kuf_grad = np.zeros_like(Kuf)
            Kuf_grad[a0:a1] = Kuf[a0:a1] * (2 / sig)
            dKnK = Kuf_grad @ (nv[:, None] * Kuf.T)
            Pi = dKnK + dKnK.T + Kuu_grad
            Kuu_i = Kuu[a0:a1, a0:a1]
            cg = (0.5 * np.trace(np.linalg.inv(Kuu_i) @ Kuu_grad[a0:a1, a0:a1])
                  - 0.5 * np.trace(Pi @ S))
            dK_alpha = Kuf_grad.T @ a
            dg = dK_alpha @ (nv * r) - 0.5 * a @ Kuu_grad @ a
            grad[i] = cg + dg
        for t in range(3):
            KnK = Kuf @ (one[t][:, None] * Kuf.T)
            s3 = noises[t] ** 3
            cg = -one[t].sum() / noises[t] + np.trace(KnK @ S) / s3
            dg = (r @ (one[t] * r)) / s3
            grad[nk + t] = cg + dg
        self.likelihood_gradient = grad
        return self.log_marginal_likelihood

    # ------------------------------------------------------------------
    def kernel_mat(self, structure):
        return np.vstack([k.envs_struc(sd, structure.descriptors[i])
                          for i, (k, sd) in enumerate(
                              zip(self.kernels, self.sparse_descriptors))])

    def predict_mean(self, structure):
        """sparse_gp.cpp:612-628."""
        km = self.kernel_mat(structure)
        structure.mean_efs = km.T @ self.alpha

    def predict_SOR(self, structure):
        """sparse_gp.cpp:630-649."""
        km = self.kernel_mat(structure)
        structure.mean_efs = km.T @ self.alpha
        vs = km.T @ self.R_inv
        structure.variance_efs = np.einsum("ij,ij->i", vs, vs)

    def predict_DTC(self, structure):
        """sparse_gp.cpp:651-680."""
        km = self.kernel_mat(structure)
        structure.mean_efs = km.T @ self.alpha
        K_self = sum(k.self_kernel_struc(structure.descriptors[i])
                     for i, k in enumerate(self.kernels))
        Q_self = np.einsum("ij,ij->j", km, self.Kuu_inverse @ km)
        V_SOR = np.einsum("ij,ij->j", km, self.Sigma @ km)
        structure.variance_efs = K_self - Q_self + V_SOR

    def compute_cluster_uncertainties(self, structure):
        """Energy-energy variance per cluster, sparse_gp.cpp:93-133."""
        out = []
        count = 0
        for i, (k, sd) in enumerate(zip(self.kernels, self.sparse_descriptors)):
            cd = ClusterDescriptor(structure.descriptors[i])
            K_self = np.diag(k.envs_envs(cd, cd)).copy()
            sk = k.envs_envs(cd, sd)
            n = sd.n_clusters
            Linv = self.L_inv[count:count + n, count:count + n]
            count += n
            Q1 = Linv @ sk.T
            out.append(K_self - np.einsum("ij,ij->j", Q1, Q1))
        return out
