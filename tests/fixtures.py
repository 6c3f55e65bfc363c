"""Shared seeded workloads and oracle-trained models for the tests."""
import numpy as np

from oracle.b2 import B2 as OB2, ClusterDescriptor as OCD
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from oracle.sparse_gp import SparseGP as OSGP
from oracle import predict as opred
from flare_pp_gb300 import synth


def settings(n_species, N, lmax, rc, cutoffs=None, cutoff_function="quadratic"):
    cut = np.full((n_species, n_species), rc) if cutoffs is None else np.asarray(cutoffs)
    return dict(n_species=n_species, N=N, lmax=lmax, r1=0.0, cutoffs=cut,
                cutoff_function=cutoff_function)


def settings_b3(n_species, N, lmax, rc, cutoff_function="quadratic"):
    return dict(kind="B3", n_species=n_species, N=N, lmax=lmax, r1=0.0, rcut=rc,
                cutoffs=np.full((n_species, n_species), rc),
                cutoff_function=cutoff_function)


def config1_model(n_frames=5, n_sparse=50, power=2):
    """FCC Al 108 atoms, 5 LJ-labelled frames, 50 sparse environments:
    trained with the oracle's SparseGP (E, F, S labels, QR solve)."""
    rc = 5.0
    b2 = OB2("chebyshev", "quadratic", [0, rc], [], [1, 8, 3])
    kern = ONDP(2.0, power)
    gp = OSGP([kern], 0.001, 0.05, 0.006)
    rng = np.random.default_rng(101)
    frames = []
    for k in range(n_frames):
        cell, sp, pos = synth.fcc_al_108(101, k)
        s = OStructure(cell, sp, pos, rc, [b2])
        e, f, st, _ = synth.lennard_jones(cell, pos)
        s.energy = np.array([e])
        s.forces = f.reshape(-1)
        s.stresses = st
        gp.add_training_structure(s)
        frames.append(s)
    allc = [(k, a) for k in range(n_frames) for a in range(108)]
    pick = rng.choice(len(allc), n_sparse, replace=False)
    for k in range(n_frames):
        atoms = sorted(allc[p][1] for p in pick if allc[p][0] == k)
        gp.add_specific_environments(frames[k], atoms)
    gp.update_matrices_QR()
    return dict(b2=b2, kernel=kern, gp=gp, frames=frames, rc=rc,
                settings=settings(1, 8, 3, rc))


def site_energy_model(b2, frames, n_sparse_per_species, sigma=2.0, power=2,
                      noise=0.01, seed=0):
    """Sparse set drawn from the frames' atoms; weights fitted (the
    reference's QR solve) to Lennard-Jones site energies."""
    rng = np.random.default_rng(seed)
    ns = b2.descriptor_settings[0]
    kern = ONDP(sigma, power)
    dvs, ys = [], []
    for (cell, sp, pos) in frames:
        s = OStructure(cell, sp, pos, b2.cutoffs.max(), [])
        b2.store_dervs = False
        dv = b2.compute_struc(s)
        dvs.append(dv)
        _, _, _, site = synth.lennard_jones(cell, pos)
        ys.append(site)
    sparse = OCD()
    sparse.initialize_cluster(ns, dvs[0].n_descriptors)
    for s_ in range(ns):
        pool = [(f, k) for f, dv in enumerate(dvs) for k in range(dv.n_clusters_by_type[s_])]
        pick = rng.choice(len(pool), min(n_sparse_per_species, len(pool)), replace=False)
        by_frame = {}
        for p in sorted(pick):
            by_frame.setdefault(pool[p][0], []).append(pool[p][1])
        for f, ks in by_frame.items():
            cl = [[] for _ in range(ns)]
            cl[s_] = ks
            sparse.add_clusters_by_type(dvs[f], cl)
    train = OCD()
    for dv in dvs:
        train.add_all_clusters(dv)
    y = np.concatenate([np.concatenate([ys[f][dv.atom_indices[s_]] for f, dv in enumerate(dvs)])
                        for s_ in range(ns)])
    Kuu = kern.envs_envs(sparse, sparse)
    Kuf = kern.envs_envs(sparse, train)
    n = Kuu.shape[0]
    L = np.linalg.cholesky(Kuu + 1e-8 * np.eye(n))
    A = np.vstack([Kuf.T / noise, L.T])
    b = np.concatenate([y / noise, np.zeros(n)])
    Q, R = np.linalg.qr(A)
    import scipy.linalg as sla
    R_inv = sla.solve_triangular(R, np.eye(n))
    alpha = R_inv @ (Q.T @ b)
    return dict(kernel=kern, sparse=sparse, alpha=alpha, R_inv=R_inv, sigma=sigma,
                power=power)


def to_gpu_model(b2_settings_list, oracle_sparse, alpha, sigma, power, R_inv=None,
                 cutoffs=None, kind="B2"):
    """A GPU SparseGP loaded with the same sparse set and weights."""
    import flare_pp_gb300 as fg
    ns, N, lmax, rc = b2_settings_list
    if kind == "B3":
        b2 = fg.B3("chebyshev", "quadratic", [0.0, rc], [], [ns, N, lmax])
    else:
        b2 = fg.B2("chebyshev", "quadratic", [0.0, rc], [], [ns, N, lmax], cutoffs)
    cd = fg.ClusterDescriptor()
    cd.initialize_cluster(ns, oracle_sparse.n_descriptors)
    cd.descriptors = [np.array(d) for d in oracle_sparse.descriptors]
    cd.descriptor_norms = [np.array(n) for n in oracle_sparse.descriptor_norms]
    cd.cutoff_values = [np.array(c) for c in oracle_sparse.cutoff_values]
    cd.n_clusters_by_type = list(oracle_sparse.n_clusters_by_type)
    cd.cumulative_type_count = list(oracle_sparse.cumulative_type_count)
    cd.n_clusters = oracle_sparse.n_clusters
    gp = fg.SparseGP([fg.NormalizedDotProduct(sigma, power)], 0.001, 0.05, 0.006)
    gp.set_model(b2, cd, alpha, R_inv)
    return gp, b2


def lammps_arrays(cell, sp, pos, rc):
    """Full neighbor list with ghost atoms from the periodic structure."""
    o = OStructure(cell, sp, pos, rc)
    wp = o.wrapped_positions
    noa = o.noa
    x = [wp[i] for i in range(noa)]
    types = [int(s) + 1 for s in sp]
    owner = list(range(noa))
    ghost_of = {}
    numneigh, nbrs = [], []
    off = o.cumulative_neighbor_count
    for i in range(noa):
        numneigh.append(int(off[i + 1] - off[i]))
        for p in range(off[i], off[i + 1]):
            j = int(o.structure_indices[p])
            img = wp[i] + o.relative_positions[p, 1:]
            key = (j, tuple(np.round(img - wp[j], 6)))
            if np.allclose(img, wp[j]):
                nbrs.append(j)
                continue
            if key not in ghost_of:
                ghost_of[key] = len(x)
                x.append(img)
                types.append(int(sp[j]) + 1)
                owner.append(j)
            nbrs.append(ghost_of[key])
    return (np.array(x), np.array(types), np.arange(noa), np.array(numneigh),
            np.array(nbrs), np.array(owner))


def seeded_beta(seed, n_species, n_d, power=2):
    """Mapped coefficients for pinning the pair-style math: per species a
    dense symmetric n_d x n_d matrix (power 2) or an n_d vector (power 1) of
    seeded normal entries scaled by 1/n_d."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_species):
        if power == 1:
            out.append(rng.normal(size=n_d) / n_d)
        else:
            a = rng.normal(size=(n_d, n_d)) / n_d
            out.append(0.5 * (a + a.T))
    return out


# Pair-style cases pinned to the reference's own lammps_descriptor.cpp
# (tests/golden/make_golden.py records them): name -> (structure builder
# arguments, n_species, N, lmax, cutoff matrix, power, beta seed).
BETA_CASES = {
    "fcc108_n8l3": (("fcc", 101, 5), 1, 8, 3, [[5.0]], 2, 7001),
    "fcc108_n8l3_p1": (("fcc", 101, 5), 1, 8, 3, [[5.0]], 1, 7002),
    "bcc250_n10l4_mixed_cut": (("bcc", (5, 5, 5), 202), 2, 10, 4,
                               [[5.5, 5.0], [5.0, 5.2]], 2, 7003),
    "bcc432_n12l4": (("bcc", (6, 6, 6), 303), 2, 12, 4, [[5.5, 5.5], [5.5, 5.5]], 2, 7004),
}


def beta_case(name):
    """(cell, species, positions, settings, beta list, power) of a pinned
    pair-style case."""
    geo, ns, N, lmax, cut, power, seed = BETA_CASES[name]
    if geo[0] == "fcc":
        cell, sp, pos = synth.fcc_al_108(geo[1], geo[2])
    else:
        cell, sp, pos = synth.bcc_alloy(geo[1], geo[2])
    cut = np.asarray(cut, dtype=float)
    st = settings(ns, N, lmax, float(cut.max()), cutoffs=cut)
    from oracle.b2 import n_descriptors
    beta = seeded_beta(seed, ns, n_descriptors(ns, N, lmax), power)
    return cell, np.asarray(sp), np.asarray(pos), st, beta, power


# Structure / B2 / kernel cases pinned to the reference's own structure.cpp,
# b2.cpp and normalized_dot_product.cpp (tests/golden/make_golden.py records
# them): name -> (cell, species, positions, cutoff, B2 settings
# (n_species, N, lmax), cutoff matrix).
def struc_cases():
    rng = np.random.default_rng(31)
    out = {}
    cell, sp, pos = synth.fcc_al_108(101, 5)
    out["fcc108"] = (cell, np.asarray(sp), pos, 5.0, (1, 8, 3), [[5.0]])
    tri = np.array([[5.0, 0.3, 0.1], [-0.4, 4.6, 0.2], [0.3, 0.5, 4.9]])
    out["triclinic_sweep2"] = (tri, rng.integers(0, 2, 9), rng.uniform(-3, 8, size=(9, 3)),
                               6.5, (2, 4, 2), [[6.5, 5.9], [5.9, 6.2]])
    out["single_atom"] = (np.eye(3) * 3.1, np.array([0]), np.array([[0.2, 0.3, 0.4]]), 5.0,
                          (1, 3, 2), [[5.0]])
    # a sheared cell whose determinant is exactly 420 in floating point (the
    # kernels' stress columns divide by the volume; see the neighbor-list test)
    cell = np.array([[8.0, 0.5, 0.0], [0.0, 7.0, 0.25], [0.0, 0.0, 7.5]])
    out["two_species_20"] = (cell, rng.integers(0, 2, size=20), rng.uniform(0, 7, size=(20, 3)),
                             4.2, (2, 5, 3), [[4.2, 3.6], [3.6, 4.0]])
    cell, sp, pos = synth.bcc_alloy((3, 3, 3), 7)
    out["bcc54"] = (cell, np.asarray(sp), pos, 4.2, (2, 5, 3), [[4.2, 3.6], [3.6, 4.0]])
    return out


def b3_cases():
    """B3 cases pinned to the reference's b3.cpp: (cell, species, positions,
    cutoff, (n_species, N, lmax)); B3 uses one cutoff for every species pair
    (b3.cpp:258)."""
    base = struc_cases()
    out = {}
    cell, sp, pos, _, _, _ = base["fcc108"]
    out["fcc108_n4l3"] = (cell, sp, pos, 5.0, (1, 4, 3))
    cell, sp, pos, _, _, _ = base["two_species_20"]
    out["two_species_20_n3l2"] = (cell, sp, pos, 4.2, (2, 3, 2))
    cell, sp, pos, _, _, _ = base["triclinic_sweep2"]
    out["triclinic_n2l3"] = (cell, sp, pos, 6.0, (2, 2, 3))
    cell, sp, pos, _, _, _ = base["bcc54"]
    out["bcc54_n2l4"] = (cell, sp, pos, 4.2, (2, 2, 4))
    return out


# B3 kernel cases: a sparse set from two B3 structures, and the two structures
B3_KERNEL_SPARSE = [("two_species_20_n3l2", [[0, 2], [1, 3, 5]]),
                    ("two_species_20_n3l2", [[4], [7]])]
B3_KERNEL_STRUCS = ("two_species_20_n3l2", "two_species_20_n3l2")


def sgp_scenario(two_kernels=False, power=2.0):
    """The sparse-GP case pinned to the reference's sparse_gp.cpp: three
    16-atom BCC alloy frames (a = 3.6 A, rattled 0.2 A, Lennard-Jones E/F/S
    labels; frame 1 trains on the forces of atoms 0, 3, 5), 5 sparse
    environments per frame, noises (1, 2, 3), a held-out frame; one B2 kernel
    (sigma 2, power 2) or B2 + B3 (sigma 2 and 1.5).  Returns the frames as
    (cell, species, positions, energy, forces, stress), the training atom
    lists, the sparse atoms per frame, the held-out frame, rc and the
    descriptor / kernel settings."""
    rc = 4.0
    frames = []
    for k in range(3):
        cell, sp, pos = synth.bcc_alloy((2, 2, 2), 808 + k, sigma=0.2, a=3.6)
        e, f, st, _ = synth.lennard_jones(cell, pos)
        frames.append((cell, sp, pos, np.array([e]), f.reshape(-1), st))
    train_atoms = [None, [0, 3, 5], None]
    sparse_atoms = [[(3 * k + 5 * j) % 16 for j in range(5)] for k in range(3)]
    test = synth.bcc_alloy((2, 2, 2), 900, sigma=0.2, a=3.6)
    descs = [("B2", (2, 4, 2))] + ([("B3", (2, 2, 2))] if two_kernels else [])
    hyps = [(2.0, power)] + ([(1.5, power)] if two_kernels else [])
    return dict(rc=rc, frames=frames, train_atoms=train_atoms, sparse_atoms=sparse_atoms,
                test=test, descs=descs, hyps=hyps, noises=(1.0, 2.0, 3.0))


# Sparse sets of the kernel cases: (structure case, clusters per species).
KERNEL_SPARSE = [("two_species_20", [[0, 2, 4], [1, 3]]), ("bcc54", [[1, 5], [0, 2, 7]])]
KERNEL_STRUCS = ("two_species_20", "bcc54")
KERNEL_HYPS = [(1.7, 1.0), (1.7, 2.0)]


def build_pair_harness(out_dir):
    """Compile tests/cpp/pair_harness.cpp with the C++ pair-style core
    (flare_pp_gb300/lammps/pair_flare_gb300.cpp), linked against
    libflare_pp_gb300.so.  Returns the executable's path."""
    import os
    import subprocess
    from flare_pp_gb300 import build
    lib = build.build()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(lib)
    exe = os.path.join(str(out_dir), "pair_harness")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                    "-I", os.path.join(root, "include"),
                    "-I", os.path.join(root, "flare_pp_gb300", "lammps"),
                    os.path.join(root, "tests", "cpp", "pair_harness.cpp"),
                    os.path.join(root, "flare_pp_gb300", "lammps", "pair_flare_gb300.cpp"),
                    "-L", libdir, "-lflare_pp_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True)
    return exe


def write_case(fn, x, types, ilist, numneigh, nbrs):
    """A LAMMPS-shaped case file for the pair harness (local atoms first,
    numneigh and the neighbor lists in ilist order = atom order)."""
    nlocal = len(numneigh)
    with open(fn, "w") as f:
        f.write(f"{nlocal} {len(x) - nlocal} {len(ilist)}\n")
        for r in x:
            f.write(f"{r[0]:.17g} {r[1]:.17g} {r[2]:.17g}\n")
        f.write(" ".join(str(int(t)) for t in types) + "\n")
        f.write(" ".join(str(int(i)) for i in ilist) + "\n")
        f.write(" ".join(str(int(n)) for n in numneigh) + "\n")
        f.write(" ".join(str(int(j)) for j in nbrs) + "\n")


def read_harness_output(fn, nall):
    with open(fn) as f:
        e = float(f.readline().split()[0])
        vir = np.array([float(v) for v in f.readline().split()])
        rows = np.array([[float(v) for v in f.readline().split()] for _ in range(nall)])
    return e, vir, rows[:, :3], rows[:, 3]


def std_atom_model(power, sigma=1.5, seed=606, n_per_species=10):
    """Two-species sparse set (10 environments per species of a 54-atom BCC
    alloy frame, per-pair cutoffs) and the inverse Cholesky factor of its
    Kuu + 1e-8 I: the coefficients of the compute flare/std/atom."""
    import scipy.linalg as sla
    rc = 4.5
    cut = np.array([[4.5, 4.0], [4.0, 4.2]])
    b2 = OB2("chebyshev", "quadratic", [0, rc], [], [2, 4, 2], cut)
    cell, sp, pos = synth.bcc_alloy((3, 3, 3), seed)
    frame = OStructure(cell, sp, pos, rc, [b2])
    dv = frame.descriptors[0]
    rng = np.random.default_rng(seed)
    clusters = [sorted(int(v) for v in rng.choice(dv.n_clusters_by_type[s],
                                                   n_per_species, replace=False))
                for s in range(2)]
    sd = OCD(dv, clusters)
    Kuu = ONDP(sigma, power).envs_envs(sd, sd)
    n = Kuu.shape[0]
    L = np.linalg.cholesky(Kuu + 1e-8 * np.eye(n))
    L_inv = sla.solve_triangular(L, np.eye(n), lower=True)
    sparse_normed = [sd.descriptors[s] / sd.descriptor_norms[s][:, None] for s in range(2)]
    return dict(b2=b2, sd=sd, L_inv=L_inv, Kuu_inverse=L_inv.T @ L_inv, sigma=sigma,
                power=power, cutoffs=cut, rc=rc, sparse_normed=sparse_normed,
                settings=settings(2, 4, 2, rc, cut))


def likelihood_model(seed=808, sigma=2.0, noises=(1.0, 2.0, 3.0), power=2,
                     second_kernel=None):
    """Two-species model for the likelihood tests: three 16-atom BCC alloy
    frames (a = 3.6 A) rattled by 0.2 A (E, F, S labels from Lennard-Jones;
    the second frame labels the forces of three atoms only) and 5 sparse
    environments per frame, so that Kuu is well conditioned.  second_kernel
    = (sigma, [N, lmax]) adds a second NormalizedDotProduct kernel over a
    second B2 descriptor."""
    rc = 4.0
    b2 = OB2("chebyshev", "quadratic", [0, rc], [], [2, 4, 2])
    kernels, descs = [ONDP(sigma, power)], [b2]
    if second_kernel is not None:
        kernels.append(ONDP(second_kernel[0], power))
        descs.append(OB2("chebyshev", "quadratic", [0, rc], [], [2] + list(second_kernel[1])))
    gp = OSGP(kernels, *noises)
    frames = []
    for k in range(3):
        cell, sp, pos = synth.bcc_alloy((2, 2, 2), seed + k, sigma=0.2, a=3.6)
        s = OStructure(cell, sp, pos, rc, descs)
        e, f, st, _ = synth.lennard_jones(cell, pos)
        s.energy = np.array([e])
        s.forces = f.reshape(-1)
        s.stresses = st
        gp.add_training_structure(s, [0, 3, 5] if k == 1 else (-1,))
        frames.append(s)
    for k in range(3):
        gp.add_specific_environments(frames[k], [(3 * k + 5 * j) % 16 for j in range(5)])
    gp.update_matrices_QR()
    return dict(b2=b2, gp=gp, frames=frames, rc=rc)
