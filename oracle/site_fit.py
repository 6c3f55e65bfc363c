"""Host-side (FP64) fit of the benchmark models.  TEST INFRASTRUCTURE ONLY:
used by bench.py's reference arm, which must not touch the GPU library.

The same procedure as the library's model synthesis, restated with the
oracle: B2 descriptors of seeded training frames from the C oracle
(oracle_b2_descriptors; B3 from the numpy oracle), a sparse set of n environments per species drawn
with numpy's PCG64 from the frames' atoms, Lennard-Jones site energies as
labels, the NormalizedDotProduct kernels (normalized_dot_product.cpp:27-87:
sigma^2 (dhat_i . dhat_j)^power within a species), and the reference's QR
solve (sparse_gp.cpp:576-610: L = chol(Kuu + 1e-8 I), A = [Kuf^T / noise;
L^T], b = [y / noise; 0], alpha = R^-1 Q^T b).  Returns the mapped
coefficients beta_s = sigma^2 sum_k alpha_k dhat_k dhat_k^T
(normalized_dot_product.cpp:697-759) as dense per-species matrices.
"""
import numpy as np
import scipy.linalg as sla

from . import cfast
from .b2 import DescriptorValues, ClusterDescriptor
from .kernel import NormalizedDotProduct


def _descriptor_values(p, norms, species, n_species):
    dv = DescriptorValues()
    dv.n_types = n_species
    dv.n_descriptors = p.shape[1]
    dv.n_atoms = len(species)
    for s in range(n_species):
        idx = np.nonzero(species == s)[0]
        dv.descriptors.append(p[idx])
        dv.descriptor_norms.append(norms[idx])
        dv.cutoff_values.append(np.ones(len(idx)))
        dv.atom_indices.append(idx)
        dv.n_clusters_by_type.append(len(idx))
    dv.n_clusters = len(species)
    dv.cumulative_type_count = [0]
    for s in range(n_species):
        dv.cumulative_type_count.append(dv.cumulative_type_count[-1] + dv.n_clusters_by_type[s])
    return dv


def fit_site_energy_beta(frames, settings, site_energies, n_sparse_per_species, sigma=2.0,
                         power=2, noise=0.01, seed=0, n_threads=0):
    """frames: list of (cell, species, positions); site_energies: per frame,
    per atom labels.  Returns (beta list, alpha, sparse ClusterDescriptor)."""
    ns = settings["n_species"]
    rng = np.random.default_rng(seed)
    dvs = []
    for (cell, sp, pos) in frames:
        if settings.get("kind", "B2") == "B3":
            from .geometry import Structure
            from .predict import descriptors
            _, p, nrm = descriptors(Structure(cell, sp, pos, settings["rcut"]), settings)
        else:
            p, nrm = cfast.b2_descriptors(cell, sp, pos, settings, n_threads=n_threads)
        dvs.append(_descriptor_values(p, nrm, np.asarray(sp), ns))
    sparse = ClusterDescriptor()
    sparse.initialize_cluster(ns, dvs[0].n_descriptors)
    for s_ in range(ns):
        pool = [(f, k) for f, dv in enumerate(dvs) for k in range(dv.n_clusters_by_type[s_])]
        pick = rng.choice(len(pool), min(n_sparse_per_species, len(pool)), replace=False)
        by_frame = {}
        for q in sorted(pick):
            by_frame.setdefault(pool[q][0], []).append(pool[q][1])
        for f in sorted(by_frame):
            cl = [[] for _ in range(ns)]
            cl[s_] = by_frame[f]
            sparse.add_clusters_by_type(dvs[f], cl)
    train = ClusterDescriptor()
    for dv in dvs:
        train.add_all_clusters(dv)
    y = np.concatenate([np.concatenate([site_energies[f][dv.atom_indices[s_]]
                                        for f, dv in enumerate(dvs)]) for s_ in range(ns)])
    kern = NormalizedDotProduct(sigma, power)
    Kuu = kern.envs_envs(sparse, sparse)
    Kuf = kern.envs_envs(sparse, train)
    n = Kuu.shape[0]
    L = np.linalg.cholesky(Kuu + 1e-8 * np.eye(n))
    A = np.vstack([Kuf.T / noise, L.T])
    b = np.concatenate([y / noise, np.zeros(n)])
    Q, R = np.linalg.qr(A)
    alpha = sla.solve_triangular(R, Q.T @ b)
    from .predict import unpack_beta
    beta = unpack_beta(kern.compute_map_coeff_pow2(sparse, alpha), sparse.n_descriptors)
    return beta, alpha, sparse
