"""Python face of the library, mirroring the reference's ``_C_flare`` module
(src/ace_binding.cpp:26-221) for the prediction path.

Classes and the methods the hot path uses keep the reference's names and
argument meaning; the work runs in libflare_pp_gb300.so on the GPU.
"""
import numpy as np

from . import _lib
from ._lib import check, f64, i32, lib, ptr, FPP_PREC_FP64, FPP_PREC_MIXED

PRECISIONS = {"fp64": FPP_PREC_FP64, "mixed": FPP_PREC_MIXED}


def _stream(stream):
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


class _Handle:
    _destroy = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and self._destroy:
            try:
                getattr(lib(), self._destroy)(h)
            except Exception:
                pass
            self._h = None


# --------------------------------------------------------------------------
class Structure(_Handle):
    """Periodic structure with a GPU neighbor list.

    Structure(cell, species, positions[, cutoff, descriptor_calculators]),
    src/flare_pp/structure.h:92-97.  Neighbor attributes are copied from the
    device on first access.
    """
    _destroy = "fpp_structure_destroy"

    def __init__(self, cell, species, positions, cutoff=None,
                 descriptor_calculators=(), stream=None):
        self.cell = f64(cell).reshape(3, 3)
        self.species = [int(s) for s in np.asarray(species).reshape(-1)]
        self.positions = f64(positions).reshape(-1, 3)
        self.noa = len(self.species)
        self.energy = np.zeros(0)
        self.forces = np.zeros(0)
        self.stresses = np.zeros(0)
        self.mean_efs = np.zeros(0)
        self.variance_efs = np.zeros(0)
        self.descriptors = []
        self.descriptor_calculators = list(descriptor_calculators)
        self._h = None
        self._nb = None
        self.cutoff = None
        if cutoff is not None:
            self.cutoff = float(cutoff)
            h = _lib.ctypes.c_void_p()
            sp = i32(self.species)
            check(lib().fpp_structure_create(
                ptr(self.cell), ptr(sp), ptr(self.positions), self.noa,
                self.cutoff, _stream(stream), _lib.ctypes.byref(h)))
            self._h = h.value
            self.compute_descriptors()

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("structure has no neighbor list (no cutoff given)")
        return self._h

    def set_positions(self, positions, stream=None):
        """New positions (same cell and species); rebuilds the neighbor list."""
        if hasattr(positions, "data_ptr"):   # a CUDA tensor of float64
            check(lib().fpp_structure_set_positions(
                self.handle, positions.data_ptr(), 1, _stream(stream)))
            self.positions = None
        else:
            self.positions = f64(positions).reshape(-1, 3)
            check(lib().fpp_structure_set_positions(
                self.handle, ptr(self.positions), 0, _stream(stream)))
        self._nb = None

    def set_skin(self, skin, stream=None):
        """Keep the neighbor list between set_positions calls while no atom
        has moved more than skin / 2 (fpp_structure_set_skin); 0 restores a
        rebuild at every call."""
        check(lib().fpp_structure_set_skin(self.handle, float(skin), _stream(stream)))
        self._nb = None

    def neighbor_stats(self):
        """(builds, reuses, list cutoff) of the neighbor list since creation."""
        C = _lib.ctypes
        b, r, c = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().fpp_structure_neighbor_stats(self.handle, C.byref(b), C.byref(r),
                                                 C.byref(c)))
        return b.value, r.value, c.value

    def compute_descriptors(self):
        self.descriptors = [d.compute_struc(self)
                            for d in self.descriptor_calculators]

    # neighbor attributes (structure.h:12-49) ---------------------------
    def _neighbors(self):
        if self._nb is None:
            noa = _lib.ctypes.c_int32()
            nn = _lib.ctypes.c_int64()
            sw = _lib.ctypes.c_int32()
            vol = _lib.ctypes.c_double()
            check(lib().fpp_structure_info(self.handle, _lib.ctypes.byref(noa),
                                           _lib.ctypes.byref(nn),
                                           _lib.ctypes.byref(sw),
                                           _lib.ctypes.byref(vol)))
            n, np_ = noa.value, nn.value
            cnt = np.zeros(n, np.int32)
            cum = np.zeros(n + 1, np.int32)
            idx = np.zeros(np_, np.int32)
            nsp = np.zeros(np_, np.int32)
            rel = np.zeros((np_, 4))
            wp = np.zeros((n, 3))
            check(lib().fpp_structure_get_neighbors(
                self.handle, ptr(cnt), ptr(cum), ptr(idx), ptr(nsp), ptr(rel),
                ptr(wp)))
            self._nb = dict(neighbor_count=cnt, cumulative_neighbor_count=cum,
                            structure_indices=idx, neighbor_species=nsp,
                            relative_positions=rel, wrapped_positions=wp,
                            n_neighbors=np_, sweep=sw.value, volume=vol.value)
        return self._nb

    neighbor_count = property(lambda self: self._neighbors()["neighbor_count"])
    cumulative_neighbor_count = property(
        lambda self: self._neighbors()["cumulative_neighbor_count"])
    structure_indices = property(lambda self: self._neighbors()["structure_indices"])
    neighbor_species = property(lambda self: self._neighbors()["neighbor_species"])
    relative_positions = property(lambda self: self._neighbors()["relative_positions"])
    wrapped_positions = property(lambda self: self._neighbors()["wrapped_positions"])
    n_neighbors = property(lambda self: self._neighbors()["n_neighbors"])
    sweep = property(lambda self: self._neighbors()["sweep"])

    @property
    def volume(self):
        return abs(float(np.linalg.det(self.cell)))


# --------------------------------------------------------------------------
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
        self.structure = None


class ClusterDescriptor:
    """Sparse-set rows grouped by type (descriptor.h:61-90)."""

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
        if getattr(dv, "descriptor_calculator", None) is not None:
            self.descriptor_calculator = dv.descriptor_calculator
        for s in range(self.n_types):
            idx = np.asarray(clusters[s], dtype=np.int64)
            self.descriptors[s] = np.vstack([self.descriptors[s],
                                             dv.descriptors[s][idx]])
            self.descriptor_norms[s] = np.concatenate(
                [self.descriptor_norms[s], dv.descriptor_norms[s][idx]])
            self.cutoff_values[s] = np.concatenate(
                [self.cutoff_values[s], dv.cutoff_values[s][idx]])
        for s in range(self.n_types):
            self.n_clusters_by_type[s] += len(clusters[s])
            self.n_clusters += len(clusters[s])
            if s > 0:
                self.cumulative_type_count[s] = (
                    self.cumulative_type_count[s - 1] + self.n_clusters_by_type[s - 1])

    def add_all_clusters(self, dv):
        self.add_clusters_by_type(
            dv, [list(range(dv.n_clusters_by_type[s])) for s in range(dv.n_types)])


# --------------------------------------------------------------------------
class B2(_Handle):
    """B2 power spectrum (b2.h:34-46).  compute_struc runs on the GPU in FP64
    and, like the reference, returns the stored force derivatives."""
    _destroy = "fpp_b2_destroy"

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings, cutoffs=None):
        self.radial_basis = radial_basis
        self.cutoff_function = cutoff_function
        self.radial_hyps = list(map(float, radial_hyps))
        self.cutoff_hyps = list(map(float, cutoff_hyps))
        self.descriptor_settings = [int(v) for v in descriptor_settings]
        ns = self.descriptor_settings[0]
        if cutoffs is None:
            cutoffs = np.full((ns, ns), self.radial_hyps[1])
        self.cutoffs = f64(cutoffs).reshape(ns, ns)
        self.store_dervs = True
        rh = f64(self.radial_hyps)
        ch = f64(self.cutoff_hyps) if self.cutoff_hyps else f64([0.0])
        ds = i32(self.descriptor_settings)
        h = _lib.ctypes.c_void_p()
        check(lib().fpp_b2_create(radial_basis.encode(), cutoff_function.encode(),
                                  ptr(rh), len(rh), ptr(ch), len(self.cutoff_hyps),
                                  ptr(ds), ptr(self.cutoffs), _lib.ctypes.byref(h)))
        self._h = h.value
        n = _lib.ctypes.c_int32()
        check(lib().fpp_b2_n_descriptors(self._h, _lib.ctypes.byref(n)))
        self.n_descriptors = n.value

    def compute_struc(self, structure, stream=None):
        """B2::compute_struc (b2.cpp:76-179) -> DescriptorValues."""
        st = _stream(stream)
        noa, nd, ns = structure.noa, self.n_descriptors, self.descriptor_settings[0]
        desc = np.zeros((noa, nd))
        norms = np.zeros(noa)
        npairs = _lib.ctypes.c_int64()
        check(lib().fpp_b2_pair_count(self._h, structure.handle,
                                      _lib.ctypes.byref(npairs), st))
        np_ = npairs.value
        cnt = np.zeros(noa, np.int32)
        nidx = np.zeros(np_, np.int32)
        ncoord = np.zeros((np_, 3))
        dervs = np.zeros((3 * np_, nd)) if self.store_dervs else None
        dots = np.zeros(3 * np_) if self.store_dervs else None
        check(lib().fpp_b2_compute(self._h, structure.handle, ptr(desc), ptr(norms),
                                   ptr(cnt), ptr(nidx), ptr(ncoord), ptr(dervs),
                                   ptr(dots), st))
        cum = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
        sp = np.asarray(structure.species)
        dv = DescriptorValues()
        dv.n_descriptors, dv.n_types, dv.n_atoms = nd, ns, noa
        dv.volume = structure.volume
        dv.cumulative_type_count = [0]
        for s in range(ns):
            atoms = np.nonzero(sp == s)[0]
            nn = cnt[atoms].astype(np.int64)
            dv.n_clusters_by_type.append(len(atoms))
            dv.cumulative_type_count.append(dv.cumulative_type_count[s] + len(atoms))
            dv.n_clusters += len(atoms)
            dv.n_neighbors_by_type.append(int(nn.sum()))
            dv.descriptors.append(desc[atoms])
            dv.descriptor_norms.append(norms[atoms])
            dv.cutoff_values.append(np.ones(len(atoms)))
            dv.cutoff_dervs.append(np.zeros(3 * int(nn.sum())))
            dv.neighbor_counts.append(nn)
            dv.cumulative_neighbor_counts.append(
                np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.int64)
                if len(atoms) else np.zeros(0, np.int64))
            dv.atom_indices.append(atoms)
            rows = (np.concatenate([np.arange(cum[a], cum[a + 1]) for a in atoms])
                    if len(atoms) else np.zeros(0, np.int64)).astype(np.int64)
            dv.neighbor_indices.append(nidx[rows].astype(np.int64))
            dv.neighbor_coordinates.append(ncoord[rows])
            if self.store_dervs:
                frows = (3 * rows[:, None] + np.arange(3)[None]).ravel()
                dv.descriptor_force_dervs.append(dervs[frows])
                dv.descriptor_force_dots.append(dots[frows])
            else:
                dv.descriptor_force_dervs.append(None)
                dv.descriptor_force_dots.append(None)
        dv.structure = structure
        dv.descriptor_calculator = self
        return dv


# --------------------------------------------------------------------------
class B3(B2):
    """B3 bispectrum (b3.h:29-33): one cutoff, radial_hyps[1], for every
    species pair; lmax <= 4.  Same calls as B2 (compute_struc returns the
    stored force derivatives of b3.cpp:206-240; models built on it predict
    through the B3 adjoint)."""

    def __init__(self, radial_basis, cutoff_function, radial_hyps, cutoff_hyps,
                 descriptor_settings):
        self.radial_basis = radial_basis
        self.cutoff_function = cutoff_function
        self.radial_hyps = list(map(float, radial_hyps))
        self.cutoff_hyps = list(map(float, cutoff_hyps))
        self.descriptor_settings = [int(v) for v in descriptor_settings]
        ns = self.descriptor_settings[0]
        self.cutoffs = np.full((ns, ns), self.radial_hyps[1])
        self.store_dervs = True
        rh = f64(self.radial_hyps)
        ch = f64(self.cutoff_hyps) if self.cutoff_hyps else f64([0.0])
        ds = i32(self.descriptor_settings)
        h = _lib.ctypes.c_void_p()
        check(lib().fpp_b3_create(radial_basis.encode(), cutoff_function.encode(),
                                  ptr(rh), len(rh), ptr(ch), len(self.cutoff_hyps),
                                  ptr(ds), _lib.ctypes.byref(h)))
        self._h = h.value
        n = _lib.ctypes.c_int32()
        check(lib().fpp_b2_n_descriptors(self._h, _lib.ctypes.byref(n)))
        self.n_descriptors = n.value


class NormalizedDotProduct:
    """k = sigma^2 (d.p / |d||p|)^power (normalized_dot_product.h:11-73)."""

    def __init__(self, sigma, power):
        self.sigma = float(sigma)
        self.power = float(power)
        self.kernel_hyperparameters = np.array([self.sigma])

    def _model(self, b2, envs, alpha=None):
        return _Model(b2, self.sigma, self.power, envs, alpha)

    def envs_struc(self, envs, struc, hyps=None, stream=None):
        """envs_struc (normalized_dot_product.cpp:115-210), FP64 on the GPU;
        ``struc`` is the DescriptorValues of a Structure built here."""
        sigma = self.sigma if hyps is None else float(hyps[0])
        m = _Model(struc.descriptor_calculator, sigma, self.power, envs)
        n_out = 1 + 3 * struc.n_atoms + 6
        K = np.zeros((envs.n_clusters, n_out))
        check(lib().fpp_envs_struc(m.handle, struc.structure.handle, ptr(K),
                                   _stream(stream)))
        return K

    def struc_struc(self, struc1, struc2, hyps=None, stream=None):
        """struc_struc (normalized_dot_product.cpp:212-444), FP64 on the GPU:
        the (1+3N1+6) x (1+3N2+6) energy/force/stress covariance of two
        structures' DescriptorValues."""
        sigma = self.sigma if hyps is None else float(hyps[0])
        d = struc1.descriptor_calculator
        K = np.zeros((1 + 3 * struc1.n_atoms + 6, 1 + 3 * struc2.n_atoms + 6))
        check(lib().fpp_struc_struc(d._h, sigma, self.power, struc1.structure.handle,
                                    struc2.structure.handle, ptr(K), _stream(stream)))
        return K

    def self_kernel_struc(self, struc, hyps=None, stream=None):
        """self_kernel_struc (normalized_dot_product.cpp:446-578): the
        diagonal of struc_struc(struc, struc)."""
        sigma = self.sigma if hyps is None else float(hyps[0])
        d = struc.descriptor_calculator
        v = np.zeros(1 + 3 * struc.n_atoms + 6)
        check(lib().fpp_self_kernel_struc(d._h, sigma, self.power,
                                          struc.structure.handle, ptr(v), _stream(stream)))
        return v

    def envs_envs(self, envs1, envs2, hyps=None, stream=None):
        """envs_envs (normalized_dot_product.cpp:27-87), FP64 on the GPU."""
        sigma = self.sigma if hyps is None else float(hyps[0])
        b2 = _descriptor_of(envs1) or _descriptor_of(envs2)
        m1 = _Model(b2, sigma, self.power, envs1)
        m2 = _Model(b2, sigma, self.power, envs2)
        K = np.zeros((envs1.n_clusters, envs2.n_clusters))
        check(lib().fpp_envs_envs(m1.handle, m2.handle, ptr(K), _stream(stream)))
        return K


def _descriptor_of(envs):
    return getattr(envs, "descriptor_calculator", None)


class _Model(_Handle):
    """Device model: sparse set + weights (+ R_inv, mapped beta)."""
    _destroy = "fpp_model_destroy"

    def __init__(self, b2, sigma, power, envs, alpha=None, R_inv=None):
        h = _lib.ctypes.c_void_p()
        check(lib().fpp_model_create(b2._h, float(sigma), float(power),
                                     _lib.ctypes.byref(h)))
        self._h = h.value
        self.b2 = b2
        self.n_species = b2.descriptor_settings[0]
        self.n_descriptors = b2.n_descriptors
        n_tot = envs.n_clusters
        alpha = np.zeros(n_tot) if alpha is None else f64(alpha)
        for s in range(envs.n_types):
            D = f64(envs.descriptors[s])
            nrm = f64(envs.descriptor_norms[s])
            off = envs.cumulative_type_count[s]
            a = f64(alpha[off:off + len(nrm)])
            check(lib().fpp_model_set_sparse(self._h, s, len(nrm), ptr(D), ptr(nrm),
                                             ptr(a)))
        if R_inv is not None:
            R = f64(R_inv)
            check(lib().fpp_model_set_R_inv(self._h, R.shape[0], ptr(R)))
        self.beta_power = 0

    @property
    def handle(self):
        return self._h

    def compute_beta(self, power, stream=None):
        """compute_map_coeff_pow1/2 -> packed beta, (n_species, beta_size)."""
        nd, ns = self.n_descriptors, self.n_species
        size = nd if power == 1 else nd * (nd + 1) // 2
        out = np.zeros((ns, size))
        check(lib().fpp_model_compute_beta(self._h, ptr(out), _stream(stream)))
        return out

    def set_beta(self, power, beta_packed):
        b = f64(beta_packed)
        check(lib().fpp_model_set_beta(self._h, int(power), ptr(b)))

    def set_L_inv(self, L_inv):
        L = f64(L_inv)
        check(lib().fpp_model_set_L_inv(self._h, L.shape[0], ptr(L)))

    def compute_varmap(self, stream=None):
        """compute_varmap_coefficients -> (n_species, n_d^2)."""
        nd, ns = self.n_descriptors, self.n_species
        out = np.zeros((ns, nd * nd))
        check(lib().fpp_model_compute_varmap(self._h, ptr(out), _stream(stream)))
        return out

    def set_varmap(self, varmap):
        v = f64(varmap)
        check(lib().fpp_model_set_varmap(self._h, ptr(v)))


# --------------------------------------------------------------------------
def update_matrices_QR(Kuu, Kuf, y, noise_vector, jitter=1e-8, stream=None):
    """The QR solve of SparseGP::update_matrices_QR (sparse_gp.cpp:576-610),
    FP64 on the GPU.  Returns alpha, R_inv, L_inv."""
    Kuu = f64(Kuu)
    Kuf = f64(Kuf)
    n = Kuu.shape[0]
    m = Kuf.shape[1] if Kuf.ndim == 2 else 0
    y = f64(y)
    nv = f64(noise_vector)
    alpha = np.zeros(n)
    R_inv = np.zeros((n, n))
    L_inv = np.zeros((n, n))
    check(lib().fpp_update_matrices_QR(n, m, ptr(Kuu), ptr(Kuf), ptr(y), ptr(nv),
                                       float(jitter), ptr(alpha), ptr(R_inv),
                                       ptr(L_inv), _stream(stream)))
    return alpha, R_inv, L_inv


class SparseGP:
    """SparseGP (sparse_gp.h:12-112): NormalizedDotProduct kernels, kernel i
    over the structures' descriptor i (B2 or B3), training solve and
    prediction on the GPU.  With several kernels (sparse_gp.h:48-49) the
    sparse sets are per kernel, Kuu is block diagonal over the kernels and
    Kuf stacks their rows (sparse_gp.cpp:392-462, 576-610); predictions sum
    the kernels' contributions (sparse_gp.cpp:612-702)."""

    def __init__(self, kernels, energy_noise, force_noise, stress_noise):
        self.kernels = list(kernels)
        if not self.kernels:
            raise ValueError("SparseGP needs at least one kernel")
        self.energy_noise = energy_noise
        self.force_noise = force_noise
        self.stress_noise = stress_noise
        self.Kuu_jitter = 1e-8
        self.sparse_descriptors = []
        self.sparse_indices = [[] for _ in self.kernels]
        self.training_structures = []
        self.training_atom_indices = []
        self.y = np.zeros(0)
        self.noise_vector = np.zeros(0)
        self.label_kind = np.zeros(0, dtype=np.int32)  # 0 energy, 1 force, 2 stress
        self.alpha = None
        self.R_inv = None
        self.L_inv = None
        self.Sigma = None
        self.Kuu_inverse = None
        self.b2s = []
        self._models = []
        self._mapped = False

    # the first kernel's descriptor and device model (the one-kernel names)
    b2 = property(lambda self: self.b2s[0] if self.b2s else None,
                  lambda self, v: self._set_b2(v))
    _model = property(lambda self: self._models[0] if self._models else None)

    def _set_b2(self, v):
        self.b2s = [] if v is None else [v] + self.b2s[1:]

    # ---- training (sparse_gp.cpp:135-610) -------------------------------
    def _sparse(self, structure, i=0):
        """sparse_gp.cpp:135-183 initialize_sparse_descriptors: one
        ClusterDescriptor per kernel, over the structure's descriptor i."""
        if len(structure.descriptors) < len(self.kernels):
            raise ValueError("the structure has fewer descriptors than the model has kernels")
        if not self.sparse_descriptors:
            for dv in structure.descriptors[:len(self.kernels)]:
                cd = ClusterDescriptor()
                cd.initialize_cluster(dv.n_types, dv.n_descriptors)
                cd.descriptor_calculator = dv.descriptor_calculator
                self.sparse_descriptors.append(cd)
        return self.sparse_descriptors[i]

    def add_specific_environments(self, structure, atoms):
        """sparse_gp.cpp:135-183: the atoms' environments join every kernel's
        sparse set."""
        atoms = list(atoms)
        for i in range(len(self.kernels)):
            sd = self._sparse(structure, i)
            dv = structure.descriptors[i]
            self.sparse_indices[i].append(atoms)
            by_type = [[k for k in range(len(dv.atom_indices[t])) for a in atoms
                        if dv.atom_indices[t][k] == a] for t in range(dv.n_types)]
            sd.add_clusters_by_type(dv, by_type)

    def add_all_environments(self, structure):
        """sparse_gp.cpp:305-331."""
        for i in range(len(self.kernels)):
            self._sparse(structure, i).add_all_clusters(structure.descriptors[i])
            self.sparse_indices[i].append(list(range(structure.noa)))

    def add_training_structure(self, structure, atom_indices=(-1,)):
        """sparse_gp.cpp:464-552 (labels energy, forces, stress)."""
        self._sparse(structure)
        if atom_indices[0] == -1:
            atoms = list(range(structure.noa))
            n_force = len(structure.forces)
        else:
            atoms = list(atom_indices)
            n_force = 3 * len(atoms)
        n_e, n_s = len(structure.energy), len(structure.stresses)
        parts = [f64(structure.energy)]
        if n_force:
            f = f64(structure.forces).reshape(-1)
            parts.append(np.concatenate([f[3 * a:3 * a + 3] for a in atoms]))
        parts.append(f64(structure.stresses))
        self.y = np.concatenate([self.y] + parts)
        self.noise_vector = np.concatenate([
            self.noise_vector, np.full(n_e, 1 / self.energy_noise ** 2),
            np.full(n_force, 1 / self.force_noise ** 2),
            np.full(n_s, 1 / self.stress_noise ** 2)])
        self.label_kind = np.concatenate([
            self.label_kind, np.zeros(n_e, np.int32), np.ones(n_force, np.int32),
            np.full(n_s, 2, np.int32)])
        self.training_structures.append(structure)
        self.training_atom_indices.append(atoms)

    def _kuf_columns(self, structure, atoms, i=0):
        k = self.kernels[i]
        K = k.envs_struc(self.sparse_descriptors[i], structure.descriptors[i])
        n = structure.noa
        cols = []
        if len(structure.energy):
            cols.append(K[:, 0:1])
        if len(structure.forces):
            for a in atoms:
                cols.append(K[:, 1 + 3 * a:4 + 3 * a])
        if len(structure.stresses):
            cols.append(K[:, 1 + 3 * n:7 + 3 * n])
        return np.hstack(cols) if cols else np.zeros((K.shape[0], 0))

    def _kuf_batched(self, sd, k, stream=None):
        """Kuf of all training structures in one device-resident pass
        (fpp_kuf_batched; sparse_gp.cpp:392-462, 565-574)."""
        strucs = self.training_structures
        mask, offs, atoms, n_lab = [], [0], [], 0
        for s, a in zip(strucs, self.training_atom_indices):
            m = (1 if len(s.energy) else 0) | (2 if len(s.forces) else 0) | \
                (4 if len(s.stresses) else 0)
            mask.append(m)
            if m & 2:
                atoms.extend(a)
                n_lab += 3 * len(a)
            offs.append(len(atoms))
            n_lab += (1 if m & 1 else 0) + (6 if m & 4 else 0)
        model = _Model(sd.descriptor_calculator, k.sigma, k.power, sd)
        if not hasattr(self, "_kuf_models"):
            self._kuf_models = []
        self._kuf_models.append(model)
        Kuf = np.zeros((sd.n_clusters, n_lab))
        hs = (_lib.ctypes.c_void_p * max(1, len(strucs)))(*[s.handle for s in strucs])
        mask_a, offs_a = i32(mask), i32(offs)
        atoms_a = i32(atoms if atoms else [0])
        check(lib().fpp_kuf_batched(model.handle, hs, len(strucs), ptr(mask_a), ptr(offs_a),
                                    ptr(atoms_a), ptr(Kuf), n_lab, _stream(stream)))
        return Kuf

    def _block_sizes(self):
        return [sd.n_clusters for sd in self.sparse_descriptors]

    def kuf_tiles(self, kernel_index=0):
        """(sparse environments per pass, threads per block) of the batched
        Kuf launch of the last update_matrices_QR (the autotuned shape)."""
        return self.kuf_launch(kernel_index)[:2]

    def kuf_launch(self, kernel_index=0):
        """(sparse environments per pass, threads per block, kernel ms, work
        items) of the batched Kuf launch of the last update_matrices_QR: the
        autotuned tile shape, the CUDA-event time of the Kuf kernel alone and
        its (structure, atom) work items."""
        C = _lib.ctypes
        ks, th, ms, n = C.c_int32(), C.c_int32(), C.c_float(), C.c_int64()
        check(lib().fpp_model_kuf_tiles(self._kuf_models[kernel_index].handle, C.byref(ks),
                                        C.byref(th), C.byref(ms), C.byref(n)))
        return ks.value, th.value, ms.value, n.value

    def update_matrices_QR(self):
        """sparse_gp.cpp:576-610: Kuu (block diagonal over the kernels), Kuf
        (the kernels' rows stacked, sparse_gp.cpp:565-574) and the QR solve,
        on the GPU."""
        self._kuf_models = []
        self.Kuu_kernels = [k.envs_envs(sd, sd)
                            for k, sd in zip(self.kernels, self.sparse_descriptors)]
        self.Kuf_kernels = [self._kuf_batched(sd, k)
                            for k, sd in zip(self.kernels, self.sparse_descriptors)]
        self._stack_kernels()
        self._solve()

    def _stack_kernels(self):
        n = sum(self._block_sizes())
        self.Kuu = np.zeros((n, n))
        c = 0
        for K in self.Kuu_kernels:
            m = K.shape[0]
            self.Kuu[c:c + m, c:c + m] = K
            c += m
        self.Kuf = np.vstack(self.Kuf_kernels)

    def _solve(self):
        self.alpha, self.R_inv, self.L_inv = update_matrices_QR(
            self.Kuu, self.Kuf, self.y, self.noise_vector, self.Kuu_jitter)
        self.Sigma = self.R_inv @ self.R_inv.T
        self.Kuu_inverse = self.L_inv.T @ self.L_inv
        self.L_diag = np.diag(self.L_inv).copy()
        self.R_inv_diag = np.diag(self.R_inv).copy()
        self._make_models()

    def _make_models(self):
        """One device model per kernel with its slice of alpha (and, for one
        kernel, R_inv for the SOR variance on the device)."""
        self.b2s = [sd.descriptor_calculator for sd in self.sparse_descriptors]
        self._models = []
        c = 0
        one = len(self.kernels) == 1
        for k, sd, b2 in zip(self.kernels, self.sparse_descriptors, self.b2s):
            m = sd.n_clusters
            self._models.append(_Model(b2, k.sigma, k.power, sd, self.alpha[c:c + m],
                                       self.R_inv if one else None))
            c += m
        self._mapped = False

    # ---- hyperparameters and likelihood (sparse_gp.cpp:704-922, 1105-1140)
    def set_hyperparameters(self, hyps):
        """sparse_gp.cpp:1105-1140: Kuu and Kuf rescaled to the new sigma
        (normalized_dot_product.cpp:581-615), the noise vector rebuilt from the
        new noises, and the QR solve repeated on the GPU."""
        hyps = f64(hyps)
        nk = len(self.kernels)
        if len(hyps) != nk + 3:
            raise ValueError(f"expected {nk + 3} hyperparameters")
        if not hasattr(self, "Kuu_kernels"):
            self.Kuu_kernels, self.Kuf_kernels = [self.Kuu], [self.Kuf]
        for i, k in enumerate(self.kernels):
            scale = hyps[i] * hyps[i] / (k.sigma * k.sigma)
            self.Kuu_kernels[i] = self.Kuu_kernels[i] * scale
            self.Kuf_kernels[i] = self.Kuf_kernels[i] * scale
            k.sigma = float(hyps[i])
            k.kernel_hyperparameters = np.array([k.sigma])
        self._stack_kernels()
        self.energy_noise, self.force_noise, self.stress_noise = (float(v) for v in hyps[nk:])
        inv_var = np.array([1 / self.energy_noise ** 2, 1 / self.force_noise ** 2,
                            1 / self.stress_noise ** 2])
        self.noise_vector = inv_var[self.label_kind]
        self._solve()

    def _likelihood(self, want_gradient, KnK=None, stream=None):
        n, m = self.Kuf.shape
        nk = len(self.kernels)
        out = np.zeros(4 + nk + 3)
        Kuf, Kuu, y = f64(self.Kuf), f64(self.Kuu), f64(self.y)
        kinds = i32(self.label_kind)
        a, S = f64(self.alpha), f64(self.Sigma)
        Ld, Rd = f64(self.L_diag), f64(self.R_inv_diag)
        hyps = f64(self.hyperparameters)
        offs = i32(np.concatenate([[0], np.cumsum(self._block_sizes())]))
        check(lib().fpp_likelihood_gradient_stable_kernels(
            n, m, ptr(Kuf), ptr(Kuu), ptr(y), ptr(kinds), ptr(a), ptr(S), ptr(Ld), ptr(Rd),
            nk, ptr(offs), ptr(hyps), 1 if want_gradient else 0, ptr(out), ptr(KnK),
            _stream(stream)))
        (self.log_marginal_likelihood, self.data_fit, self.complexity_penalty,
         self.constant_term) = out[:4]
        if want_gradient:
            self.likelihood_gradient = out[4:].copy()
        return self.log_marginal_likelihood

    def compute_likelihood_stable(self, stream=None):
        """sparse_gp.cpp:704-732, on the GPU."""
        return self._likelihood(False, stream=stream)

    def compute_likelihood_gradient_stable(self, precomputed_KnK=False, stream=None):
        """sparse_gp.cpp:734-862, on the GPU: returns the log marginal
        likelihood and sets likelihood_gradient (each kernel's sigma, then
        sigma_e, sigma_f, sigma_s).  The traces it needs come from one GEMM per call, so the
        precomputed and direct forms of the reference give the same numbers."""
        return self._likelihood(True, stream=stream)

    def compute_KnK(self, precomputed=False, stream=None):
        """sparse_gp.cpp:888-922: KnK_e, KnK_f, KnK_s = Kuf one_x Kuf^T."""
        n = self.Kuf.shape[0]
        KnK = np.zeros((3, n, n))
        self._likelihood(False, KnK=KnK, stream=stream)
        self.KnK_e, self.KnK_f, self.KnK_s = KnK
        return KnK

    def precompute_KnK(self, stream=None):
        """sparse_gp.cpp:864-886: Kuf one_x Kuf^T / sigma^4 for later
        hyperparameter changes."""
        if len(self.kernels) > 1:
            raise NotImplementedError("precompute_KnK takes one kernel")
        sig4 = self.kernels[0].sigma ** 4
        KnK = self.compute_KnK(stream=stream)
        self.Kuf_e_noise_Kfu = [KnK[0] / sig4]
        self.Kuf_f_noise_Kfu = [KnK[1] / sig4]
        self.Kuf_s_noise_Kfu = [KnK[2] / sig4]

    # ---- the reference's JSON state (sparse_gp.h:101-111, sparse_gp.cpp:1406-1417)
    def to_json(self, file_name):
        """Write the model in the layout of SparseGP::to_json (nlohmann JSON of
        the NLOHMANN_DEFINE_TYPE_INTRUSIVE fields; Eigen matrices as lists of
        rows, vectors as lists).  The descriptor settings travel in
        training_structures[0].descriptor_calculators, as in the reference."""
        import json

        def mat(a):
            return None if a is None else np.asarray(a, dtype=np.float64).tolist()

        def desc_json(b2):
            return {"radial_basis": b2.radial_basis, "cutoff_function": b2.cutoff_function,
                    "radial_hyps": list(b2.radial_hyps), "cutoff_hyps": list(b2.cutoff_hyps),
                    "descriptor_settings": list(b2.descriptor_settings),
                    "cutoffs": mat(b2.cutoffs),
                    "descriptor_name": "B3" if isinstance(b2, B3) else "B2"}

        def cd_json(sd):
            return {"descriptors": [mat(d) for d in sd.descriptors],
                    "descriptor_norms": [mat(n) for n in sd.descriptor_norms],
                    "cutoff_values": [mat(c) for c in sd.cutoff_values],
                    "n_clusters_by_type": [int(v) for v in sd.n_clusters_by_type],
                    "cumulative_type_count": [int(v) for v in sd.cumulative_type_count],
                    "n_descriptors": int(sd.n_descriptors), "n_types": int(sd.n_types),
                    "n_clusters": int(sd.n_clusters)}

        b2s = self.b2s or [sd.descriptor_calculator for sd in self.sparse_descriptors]
        n_sparse = sum(sd.n_clusters for sd in self.sparse_descriptors)
        j = {"hyperparameters": [float(h) for h in self.hyperparameters],
             "kernels": [{"kernel_name": "NormalizedDotProduct", "sigma": k.sigma,
                          "sig2": k.sigma * k.sigma, "power": k.power,
                          "kernel_hyperparameters": [k.sigma]} for k in self.kernels],
             "n_kernels": len(self.kernels), "Kuu_jitter": self.Kuu_jitter,
             "Kuu": mat(getattr(self, "Kuu", None)), "Kuf": mat(getattr(self, "Kuf", None)),
             "Sigma": mat(self.Sigma), "Kuu_inverse": mat(self.Kuu_inverse),
             "R_inv": mat(self.R_inv), "L_inv": mat(self.L_inv), "alpha": mat(self.alpha),
             "sparse_descriptors": [cd_json(sd) for sd in self.sparse_descriptors],
             "noise_vector": mat(self.noise_vector),
             "y": mat(self.y), "n_sparse": int(n_sparse),
             "energy_noise": self.energy_noise, "force_noise": self.force_noise,
             "stress_noise": self.stress_noise,
             "training_structures": [{"descriptor_calculators": [desc_json(b)
                                                                  for b in b2s]}]}
        with open(file_name, "w") as f:
            json.dump(j, f)

    @staticmethod
    def from_json(file_name):
        """SparseGP::from_json: a model saved by the reference (or by to_json),
        loaded for GPU prediction (NormalizedDotProduct kernels over B2 or
        B3 descriptors)."""
        import json
        with open(file_name) as f:
            j = json.load(f)

        def arr(v, shape2=False):
            if v is None:
                return np.zeros((0, 0)) if shape2 else np.zeros(0)
            return np.asarray(v, dtype=np.float64)

        kernels, b2s, cds = [], [], []
        djs = j["training_structures"][0]["descriptor_calculators"]
        for i, kj in enumerate(j["kernels"]):
            if kj.get("kernel_name") != "NormalizedDotProduct":
                raise ValueError(f"unsupported kernel {kj.get('kernel_name')}")
            kernels.append(NormalizedDotProduct(kj["sigma"], kj["power"]))
            dj = djs[i]
            if dj.get("descriptor_name", "B2") == "B3":
                b2 = B3(dj["radial_basis"], dj["cutoff_function"], dj["radial_hyps"],
                        dj["cutoff_hyps"], dj["descriptor_settings"])
            else:
                b2 = B2(dj["radial_basis"], dj["cutoff_function"], dj["radial_hyps"],
                        dj["cutoff_hyps"], dj["descriptor_settings"],
                        None if dj.get("cutoffs") is None else np.asarray(dj["cutoffs"]))
            b2s.append(b2)
            sj = j["sparse_descriptors"][i]
            cd = ClusterDescriptor()
            nt, nd = int(sj["n_types"]), int(sj["n_descriptors"])
            cd.initialize_cluster(nt, nd)
            cd.descriptors = [arr(d, True).reshape(-1, nd) for d in sj["descriptors"]]
            cd.descriptor_norms = [arr(v) for v in sj["descriptor_norms"]]
            cd.cutoff_values = [arr(v) for v in sj["cutoff_values"]]
            cd.n_clusters_by_type = [int(v) for v in sj["n_clusters_by_type"]]
            cd.cumulative_type_count = [int(v) for v in sj["cumulative_type_count"]]
            cd.n_clusters = int(sj["n_clusters"])
            cd.descriptor_calculator = b2
            cds.append(cd)
        gp = SparseGP(kernels, j.get("energy_noise", 1.0), j.get("force_noise", 1.0),
                      j.get("stress_noise", 1.0))
        gp.Kuu_jitter = j.get("Kuu_jitter", gp.Kuu_jitter)
        R_inv = arr(j.get("R_inv"), True)
        L_inv = arr(j.get("L_inv"), True)
        one = len(kernels) == 1
        gp.set_model(b2s[0] if one else b2s, cds[0] if one else cds, arr(j["alpha"]),
                     R_inv if R_inv.size else None, L_inv if L_inv.size else None)
        for key in ("Sigma", "Kuu_inverse"):
            v = arr(j.get(key), True)
            setattr(gp, key, v if v.size else None)
        gp.y = arr(j.get("y"))
        gp.noise_vector = arr(j.get("noise_vector"))
        return gp

    def set_model(self, b2, sparse_descriptors, alpha, R_inv=None, L_inv=None):
        """Load a trained model: the sparse ClusterDescriptor(s), alpha and
        optionally R_inv and L_inv (the outputs of update_matrices_QR).  With
        several kernels, b2 and sparse_descriptors are lists (one per kernel,
        in kernel order) and alpha, R_inv, L_inv cover the stacked sets."""
        multi = isinstance(sparse_descriptors, (list, tuple))
        sds = list(sparse_descriptors) if multi else [sparse_descriptors]
        b2s = list(b2) if multi else [b2]
        if len(sds) != len(self.kernels) or len(b2s) != len(self.kernels):
            raise ValueError("one descriptor and sparse set per kernel")
        for cd, d in zip(sds, b2s):
            cd.descriptor_calculator = d
        self.sparse_descriptors = sds
        self.alpha = f64(alpha)
        self.R_inv = None if R_inv is None else f64(R_inv)
        self.L_inv = None if L_inv is None else f64(L_inv)
        self._make_models()

    def _ensure_mapped(self, stream=None):
        if not self._mapped:
            self.mapping_coefficients_kernels = [
                m.compute_beta(k.power, stream) for m, k in zip(self._models, self.kernels)]
            self.mapping_coefficients = self.mapping_coefficients_kernels[0]
            self._mapped = True

    def _descriptors_of(self, structure):
        if len(structure.descriptors) < len(self.kernels):
            if not structure.descriptor_calculators:
                structure.descriptor_calculators = list(self.b2s)
            structure.compute_descriptors()
        return structure.descriptors

    def _kernel_mat(self, structure, stream=None):
        """The stacked envs_struc blocks of the kernels (sparse_gp.cpp:617-626)."""
        dvs = self._descriptors_of(structure)
        return np.vstack([k.envs_struc(sd, dvs[i], stream=stream) for i, (k, sd) in
                          enumerate(zip(self.kernels, self.sparse_descriptors))])

    def predict_mean(self, structure, stream=None):
        """sparse_gp.cpp:612-628 -> structure.mean_efs (the kernels' sum)."""
        total = np.zeros(1 + 3 * structure.noa + 6)
        out = np.zeros_like(total)
        for m in self._models:
            check(lib().fpp_predict(m.handle, structure.handle, ptr(out), None,
                                    _stream(stream)))
            total += out
        structure.mean_efs = total

    def predict_SOR(self, structure, stream=None):
        """sparse_gp.cpp:630-649 -> structure.mean_efs, structure.variance_efs."""
        if self.R_inv is None:
            raise ValueError("predict_SOR needs R_inv")
        if len(self.kernels) > 1:
            K = self._kernel_mat(structure, stream)
            structure.mean_efs = K.T @ self.alpha
            v = K.T @ self.R_inv
            structure.variance_efs = np.einsum("ij,ij->i", v, v)
            return
        out = np.zeros(1 + 3 * structure.noa + 6)
        var = np.zeros_like(out)
        check(lib().fpp_predict(self._model.handle, structure.handle, ptr(out),
                                ptr(var), _stream(stream)))
        structure.mean_efs = out
        structure.variance_efs = var

    def predict_DTC(self, structure, stream=None):
        """sparse_gp.cpp:651-680 -> structure.mean_efs, structure.variance_efs:
        variance = K_self - diag(K^T Kuu^-1 K) + diag(K^T Sigma K), with K the
        environment/structure kernel and K_self the structure self kernel
        (summed over the kernels), both from the GPU (the trained model's
        Kuu^-1 and Sigma)."""
        if self.Sigma is None or self.Kuu_inverse is None:
            raise ValueError("predict_DTC needs a model trained with update_matrices_QR")
        dvs = self._descriptors_of(structure)
        K = self._kernel_mat(structure, stream)
        structure.mean_efs = K.T @ self.alpha
        k_self = sum(k.self_kernel_struc(dvs[i], stream=stream)
                     for i, k in enumerate(self.kernels))
        q_self = np.einsum("ij,ij->j", K, self.Kuu_inverse @ K)
        v_sor = np.einsum("ij,ij->j", K, self.Sigma @ K)
        structure.variance_efs = k_self - q_self + v_sor

    def compute_cluster_uncertainties(self, structure, stream=None):
        """sparse_gp.cpp:93-133: per kernel, the energy variance of every
        cluster (species by species, atoms in structure order) from that
        kernel's block of L_inv, on the GPU."""
        if self.L_inv is None:
            raise ValueError("compute_cluster_uncertainties needs L_inv")
        out = []
        for i, m in enumerate(self._models):
            L = self._L_inv_block(i)
            v = np.zeros(structure.noa)
            check(lib().fpp_local_uncertainties(m.handle, structure.handle, ptr(L),
                                                L.shape[0], ptr(v), _stream(stream)))
            out.append(v)
        return out

    def predict_energy_uncertainty(self, structure, local=True, stream=None):
        """At MD sizes: the energy and energy variance of predict_SOR
        (sparse_gp.cpp:630-649: mean_efs[0], variance_efs[0]) and, with
        local, the per-atom variances of compute_cluster_uncertainties
        (sparse_gp.cpp:93-133) in structure atom order; only the energy
        column of the kernel matrix is formed.  Returns (energy, variance,
        local variances or None).  One kernel."""
        if len(self.kernels) > 1:
            raise NotImplementedError("predict_energy_uncertainty takes one kernel")
        if self.R_inv is None or (local and self.L_inv is None):
            raise ValueError("predict_energy_uncertainty needs R_inv (and L_inv)")
        if local and not getattr(self._model, "_L_inv_set", False):
            self._model.set_L_inv(self.L_inv)
            self._model._L_inv_set = True
        e, v = np.zeros(1), np.zeros(1)
        lv = np.zeros(structure.noa) if local else None
        check(lib().fpp_predict_energy_uncertainty(self._model.handle, structure.handle,
                                                   ptr(e), ptr(v), ptr(lv), _stream(stream)))
        return e[0], v[0], lv

    def predict_local_uncertainties(self, structure, stream=None):
        """sparse_gp.cpp:682-702: mean_efs and local_uncertainties."""
        self.predict_mean(structure, stream)
        structure.local_uncertainties = self.compute_cluster_uncertainties(structure, stream)

    # ---- coefficient files (sparse_gp.cpp:1142-1404) ----------------------
    @property
    def hyperparameters(self):
        """sparse_gp.cpp:1105-1140 order: every kernel's sigma, then the
        energy, force and stress noises."""
        return np.array([k.sigma for k in self.kernels] +
                        [self.energy_noise, self.force_noise, self.stress_noise])

    def _file_header(self, kernel_index=0):
        b2 = self.b2s[kernel_index]
        ns, N, lmax = b2.descriptor_settings
        return dict(n_species=ns, n_max=N, l_max=lmax, cutoffs=b2.cutoffs,
                    cutoff_function=b2.cutoff_function, radial=b2.radial_basis)

    def write_mapping_coefficients(self, file_name, contributor, kernel_index=0,
                                   stream=None):
        """SparseGP::write_mapping_coefficients (sparse_gp.cpp:1142-1206):
        the mapped coefficients of kernel kernel_index."""
        from .potential import write_potential
        self._ensure_mapped(stream)
        write_potential(file_name, self.mapping_coefficients_kernels[kernel_index],
                        self.kernels[kernel_index].power, contributor=contributor,
                        **self._file_header(kernel_index))

    def write_varmap_coefficients(self, file_name, contributor, kernel_index=0,
                                  stream=None):
        """SparseGP::write_varmap_coefficients (sparse_gp.cpp:1208-1281):
        the variance map of a power-1 model, computed on the GPU."""
        from .potential import write_varmap
        if self.L_inv is None:
            raise ValueError("write_varmap_coefficients needs L_inv")
        m = self._models[kernel_index]
        m.set_L_inv(self._L_inv_block(kernel_index))
        self.varmap_coeffs = m.compute_varmap(stream)
        write_varmap(file_name, self.varmap_coeffs, self._kernel_hyps(kernel_index),
                     contributor=contributor, **self._file_header(kernel_index))

    def write_L_inverse(self, file_name, contributor, kernel_index=0):
        """SparseGP::write_L_inverse (sparse_gp.cpp:1283-1344)."""
        from .potential import write_L_inverse
        if self.L_inv is None:
            raise ValueError("write_L_inverse needs L_inv")
        write_L_inverse(file_name, self._L_inv_block(kernel_index),
                        self.kernels[kernel_index].power, self._kernel_hyps(kernel_index),
                        contributor=contributor, **self._file_header(kernel_index))

    def _L_inv_block(self, i):
        """The block of L_inv that belongs to kernel i (Kuu is block diagonal
        over the kernels, so L_inv is too)."""
        c = sum(self._block_sizes()[:i])
        m = self._block_sizes()[i]
        return np.ascontiguousarray(self.L_inv[c:c + m, c:c + m])

    def _kernel_hyps(self, i):
        return np.array([self.kernels[i].sigma, self.energy_noise, self.force_noise,
                         self.stress_noise])

    def write_sparse_descriptors(self, file_name, contributor, kernel_index=0):
        """SparseGP::write_sparse_descriptors (sparse_gp.cpp:1346-1404)."""
        from .potential import write_sparse_descriptors
        sd = self.sparse_descriptors[kernel_index]
        write_sparse_descriptors(file_name, sd.descriptors, sd.descriptor_norms,
                                 contributor=contributor)

    def predict_mapped(self, structure, precision="mixed", stream=None,
                       atom_energies=False):
        """Energy, forces and stress through the mapped coefficients (the pair
        style's evaluation) on the periodic structure."""
        self._ensure_mapped(stream)
        E, F, S = 0.0, np.zeros((structure.noa, 3)), np.zeros(6)
        AE = np.zeros(structure.noa) if atom_energies else None
        e = np.zeros(1)
        f = np.zeros((structure.noa, 3))
        s = np.zeros(6)
        ae = np.zeros(structure.noa) if atom_energies else None
        for m in self._models:      # the kernels' contributions add
            check(lib().fpp_predict_mapped(m.handle, structure.handle,
                                           PRECISIONS[precision], ptr(e), ptr(f), ptr(s),
                                           ptr(ae), 0, _stream(stream)))
            E, F, S = E + e[0], F + f, S + s
            if atom_energies:
                AE = AE + ae
        return (E, F, S, AE) if atom_energies else (E, F, S)

    def predict_mapped_batched(self, structures, precision="mixed", stream=None):
        """Energies (n,), forces (a list of (noa_k, 3)) and stresses (n, 6) of
        a batch of structures of any sizes in one pass of the mapped form
        (fpp_predict_mapped_batched: the structures' atoms packed into one
        launch per stage)."""
        self._ensure_mapped(stream)
        n = len(structures)
        counts = [s.noa for s in structures]
        hs = (_lib.ctypes.c_void_p * max(1, n))(*[s.handle for s in structures])
        E, F, S = np.zeros(n), np.zeros((sum(counts), 3)), np.zeros((n, 6))
        e, f, st = np.zeros(n), np.zeros((sum(counts), 3)), np.zeros((n, 6))
        for m in self._models:      # the kernels' contributions add
            check(lib().fpp_predict_mapped_batched(m.handle, hs, n, PRECISIONS[precision],
                                                   ptr(e), ptr(f), ptr(st), _stream(stream)))
            E, F, S = E + e, F + f, S + st
        offs = np.concatenate([[0], np.cumsum(counts)])
        return E, [F[offs[k]:offs[k + 1]] for k in range(n)], S

    def center_mixed_on(self, structure, stream=None):
        """Centre the mixed-precision mapped form on this structure's mean
        environment per species (lowers its energy error on structures far
        from the sparse set's mean; see fpp_model_center_on)."""
        self._ensure_mapped(stream)
        for m in self._models:
            check(lib().fpp_model_center_on(m.handle, structure.handle, _stream(stream)))


class PairFLARE:
    """Mapped-beta pair style (lammps_plugins/pair_flare.h:20-50): reads the
    potential file and computes energy, forces and virial on LAMMPS-shaped
    arrays (full neighbor list, 1-based types, ghost atoms)."""

    def __init__(self, filename=None, model=None, b2=None):
        if filename is not None:
            self.read_file(filename)
        elif model is not None:
            self.model = model
        self.precision = "fp64"

    def read_file(self, filename):
        """pair_flare.cpp:263-396."""
        from .potential import read_potential
        pot = read_potential(filename)
        self.pot = pot
        ns, N, lmax = pot["n_species"], pot["n_max"], pot["l_max"]
        cut = pot["cutoffs"].reshape(ns, ns)
        self.cutoff = float(cut.max())
        b2 = B2(pot["radial"], pot["cutoff_function"], [0.0, self.cutoff], [],
                [ns, N, lmax], cut)
        envs = ClusterDescriptor()
        envs.initialize_cluster(ns, b2.n_descriptors)
        self.b2 = b2
        self.model = _Model(b2, 1.0, pot["power"], envs)
        self.model.set_beta(pot["power"], pot["beta"])

    def set_max_memory(self, bytes_):
        """The Kokkos pair style's MAXMEM (bytes; 0 = no cap): the atoms are
        evaluated in batches that fit (pair_flare_kokkos.cpp:145-177)."""
        check(lib().fpp_model_set_max_memory(self.model.handle, float(bytes_)))

    @property
    def last_batches(self):
        n = _lib.ctypes.c_int32()
        check(lib().fpp_model_pair_batches(self.model.handle, _lib.ctypes.byref(n)))
        return n.value

    def compute(self, x, type_, ilist, numneigh, neighbors, nlocal=None,
                precision=None, eatom=False, stream=None):
        """PairFLARE::compute (pair_flare.cpp:68-184).  Returns
        (f, eng_vdwl, virial[, eatom])."""
        x = f64(x).reshape(-1, 3)
        t = i32(type_)
        il = i32(ilist)
        nn = i32(numneigh)
        nb = i32(neighbors)
        nall = len(x)
        nlocal = len(il) if nlocal is None else int(nlocal)
        f = np.zeros((nall, 3))
        e = np.zeros(1)
        v = np.zeros(6)
        ea = np.zeros(nall) if eatom else None
        prec = PRECISIONS[precision or self.precision]
        check(lib().fpp_pair_compute(self.model.handle, nlocal, nall, ptr(x), ptr(t),
                                     len(il), ptr(il), ptr(nn), ptr(nb), prec, ptr(f),
                                     ptr(e), ptr(v), ptr(ea), _stream(stream)))
        return (f, e[0], v, ea) if eatom else (f, e[0], v)


class ComputeFlareStdAtom:
    """The LAMMPS compute flare/std/atom (lammps_plugins/compute_flare_std_atom.h):
    per-atom uncertainty from a variance-map file (one file), or from an
    L_inverse file and a sparse-descriptor file (two files), evaluated on the
    GPU on LAMMPS-shaped arrays."""

    def __init__(self, *files):
        self.use_map = False
        if files:
            self.coeff(*files)

    def coeff(self, *files):
        """ComputeFlareStdAtom::coeff (compute_flare_std_atom.cpp:287-307)."""
        from .potential import read_L_inverse, read_sparse_descriptors, read_varmap
        if len(files) == 1:
            hdr = read_varmap(files[0])
            self.use_map = True
        elif len(files) == 2:
            hdr = read_L_inverse(files[0])
            self.use_map = False
        else:
            raise ValueError("Incorrect args for compute coefficients")
        ns, N, lmax = hdr["n_species"], hdr["n_max"], hdr["l_max"]
        self.hyperparameters = hdr["hyps"]
        self.cutoff_matrix = hdr["cutoffs"]
        self.cutoff = float(self.cutoff_matrix.max())
        b2 = B2(hdr["radial"], hdr["cutoff_function"], [0.0, self.cutoff], [],
                [ns, N, lmax], self.cutoff_matrix)
        self.b2 = b2
        envs = ClusterDescriptor()
        envs.initialize_cluster(ns, b2.n_descriptors)
        sigma = float(self.hyperparameters[0])
        if self.use_map:
            self.model = _Model(b2, sigma, 2, envs)
            self.model.set_varmap(hdr["varmap"].reshape(ns, -1))
            return
        self.power = hdr["power"]
        rows = read_sparse_descriptors(files[1], b2.n_descriptors, hdr["n_clusters"])
        if len(rows) != ns:
            raise ValueError("sparse descriptors hold a different species count")
        envs.n_clusters_by_type = [len(r) for r in rows]
        envs.cumulative_type_count = [int(v) for v in np.concatenate(
            [[0], np.cumsum(envs.n_clusters_by_type)[:-1]])]
        envs.n_clusters = int(sum(envs.n_clusters_by_type))
        envs.descriptors = [f64(r) for r in rows]
        # the file's rows are normalized already: unit norms (0 for the zero
        # rows of empty environments) keep them as they are
        envs.descriptor_norms = [np.where(np.abs(r).max(axis=1, initial=0.0) > 0, 1.0, 0.0)
                                 for r in rows]
        self.model = _Model(b2, sigma, self.power, envs)
        self.model.set_L_inv(hdr["L_inv"])

    def compute_peratom(self, x, type_, ilist, numneigh, neighbors, nlocal=None,
                        stream=None):
        """ComputeFlareStdAtom::compute_peratom (compute_flare_std_atom.cpp:98-207):
        stds (nall), 0 for atoms outside ilist and for empty environments."""
        x = f64(x).reshape(-1, 3)
        t = i32(type_)
        il = i32(ilist)
        nn = i32(numneigh)
        nb = i32(neighbors)
        nall = len(x)
        nlocal = len(il) if nlocal is None else int(nlocal)
        out = np.zeros(nall)
        check(lib().fpp_std_atom_compute(self.model.handle, nlocal, nall, ptr(x), ptr(t),
                                         len(il), ptr(il), ptr(nn), ptr(nb),
                                         1 if self.use_map else 0, ptr(out),
                                         _stream(stream)))
        return out
