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
        Kuu = self.Kuu()
        Kuf = self.Kuf()
        self.Kuu_mat, self.Kuf_mat = Kuu, Kuf
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
