"""Seeded synthetic structures and a Lennard-Jones labeller.

No public dataset is involved on this path: the workloads are lattices with
seeded Gaussian rattles (numpy PCG64 generators), and training labels come from
a Lennard-Jones surrogate evaluated here in FP64 on the host.

Workloads (name, lattice, sizes):

* ``fcc_al_108``   FCC a=4.05 A, 3x3x3 cells, rattle 0.05 A, 1 species, rc 5.0,
                   chebyshev N=8, lmax=3, 50 sparse environments, seed 101.
* ``bcc_alloy_2000`` BCC a=3.0 A, 10x10x10 cells, 50/50 species, rattle 0.08 A,
                   rc 5.5, N=10, lmax=4, 400 sparse, seed 202.
* ``bcc_alloy_32k`` BCC a=3.0 A, 32x32x16 cells (32768 atoms), 50/50 species,
                   rattle 0.08 A, rc 5.5, N=12, lmax=4, 2000 sparse per species,
                   seed 303.
* ``fcc_batch_256`` 256 FCC two-species cells with 32..512 atoms, strain +-3 %,
                   rattle 0.1 A, rc 5.0, N=8, lmax=3, 1000 sparse, seed 404.
* ``b3_fcc_1m``    FCC a=4.05 A, 64^3 cells (1,048,576 atoms), rattle 0.05 A,
                   B3 N=6, lmax=3, 500 sparse, seed 505.
"""
import numpy as np

FCC_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
BCC_BASIS = np.array([[0, 0, 0], [.5, .5, .5]])


def lattice(basis, a, reps):
    n1, n2, n3 = reps
    g = np.stack(np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3),
                             indexing="ij"), -1).reshape(-1, 3)
    pos = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    cell = np.diag([n1 * a, n2 * a, n3 * a]).astype(np.float64)
    return cell, pos.astype(np.float64)


def rattled(basis, a, reps, sigma, rng, n_species=1, strain=0.0):
    cell, pos = lattice(basis, a, reps)
    if strain:
        eps = rng.uniform(-strain, strain, size=(3, 3))
        eps = 0.5 * (eps + eps.T)
        F = np.eye(3) + eps
        cell = cell @ F
        pos = pos @ F
    pos = pos + rng.normal(scale=sigma, size=pos.shape)
    if n_species == 1:
        species = np.zeros(len(pos), dtype=np.int32)
    else:
        species = rng.integers(0, n_species, size=len(pos)).astype(np.int32)
    return cell, species, pos


def fcc_al_108(seed=101, frame=0):
    rng = np.random.default_rng(seed + frame)
    return rattled(FCC_BASIS, 4.05, (3, 3, 3), 0.05, rng)


def bcc_alloy(reps, seed, sigma=0.08, a=3.0):
    rng = np.random.default_rng(seed)
    return rattled(BCC_BASIS, a, reps, sigma, rng, n_species=2)


def fcc_batch(n_structures=256, seed=404, lo=32, hi=512):
    """Uneven FCC two-species cells: draw a target atom count in [lo, hi],
    pick the n1*n2*n3*4 supercell nearest to it, strain by U(+-3 %) and
    rattle by 0.1 A.  Returns a list of (cell, species, positions)."""
    rng = np.random.default_rng(seed)
    shapes = []
    for n1 in range(1, 9):
        for n2 in range(n1, 9):
            for n3 in range(n2, 9):
                shapes.append((n1 * n2 * n3 * 4, (n1, n2, n3)))
    out = []
    for _ in range(n_structures):
        target = rng.integers(lo, hi + 1)
        best = min(shapes, key=lambda s: (abs(s[0] - target), s[1]))
        out.append(rattled(FCC_BASIS, 4.05, best[1], 0.1, rng, n_species=2,
                           strain=0.03))
    return out


# --------------------------------------------------------------------------
# Lennard-Jones surrogate labels (epsilon 0.4 eV, sigma 2.6 A, cutoff 3 sigma,
# energy shifted to zero at the cutoff).  Stress uses the flare convention
# -(1/V) sum over directed pairs of (dE/dr_ij)_a (r_ij)_b, order
# xx, xy, xz, yy, yz, zz.
# --------------------------------------------------------------------------
def lennard_jones(cell, positions, eps=0.4, sig=2.6, rc=None):
    rc = 3 * sig if rc is None else rc
    cell = np.asarray(cell, dtype=np.float64)
    pos = np.asarray(positions, dtype=np.float64)
    n = len(pos)
    inv = np.linalg.inv(cell)
    frac = pos @ inv
    heights = [abs(np.linalg.det(cell)) / np.linalg.norm(np.cross(cell[(k + 1) % 3], cell[(k + 2) % 3]))
               for k in range(3)]
    reach = [int(np.ceil(rc / h)) for h in heights]
    shifts = np.stack(np.meshgrid(*[np.arange(-r, r + 1) for r in reach],
                                  indexing="ij"), -1).reshape(-1, 3)
    e0 = 4 * eps * ((sig / rc) ** 12 - (sig / rc) ** 6)
    site = np.zeros(n)
    F = np.zeros((n, 3))
    S = np.zeros((3, 3))
    for i in range(n):
        d = frac - frac[i]
        d -= np.round(d)
        vec = (d[:, None, :] + shifts[None, :, :]) @ cell       # (n, ns, 3)
        r2 = np.einsum("jsk,jsk->js", vec, vec)
        m = (r2 < rc * rc) & (r2 > 1e-12)
        rv = vec[m]
        r = np.sqrt(r2[m])
        sr6 = (sig / r) ** 6
        phi = 4 * eps * (sr6 * sr6 - sr6) - e0
        dphi = 4 * eps * (-12 * sr6 * sr6 + 6 * sr6) / r
        site[i] = 0.5 * phi.sum()
        # dE/dr_ij for the directed pair, counting half of each bond
        g = (0.5 * dphi / r)[:, None] * rv
        jj = np.nonzero(m)[0]
        F[i] += g.sum(0)
        np.add.at(F, jj, -g)
        S -= g.T @ rv
    vol = abs(np.linalg.det(cell))
    S /= vol
    stress = np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]])
    return site.sum(), F, stress, site


# --------------------------------------------------------------------------
# Model synthesis for the benchmarks: a sparse GP over B2 whose sparse set is
# drawn from seeded frames and whose weights are the reference's QR solve
# (sparse_gp.cpp:576-610: LLT(Kuu + 1e-8 I), A = [Kuf^T / noise; L^T],
# alpha = R^-1 Q^T b) fitted to Lennard-Jones site energies, so that the
# weights carry the cancellations of a real fit.  Descriptors, kernel
# matrices and the QR solve all run in the GPU library in FP64.
# --------------------------------------------------------------------------
def fit_site_energy_model(b2, frames, n_sparse_per_species, sigma=2.0, power=2,
                          noise=0.01, seed=0, device="cuda"):
    from .api import ClusterDescriptor, NormalizedDotProduct, Structure, update_matrices_QR
    rng = np.random.default_rng(seed)
    ns = b2.descriptor_settings[0]
    rc = float(np.max(b2.cutoffs))
    store = b2.store_dervs
    b2.store_dervs = False
    dvs, ys = [], []
    try:
        for (cell, sp, pos) in frames:
            s = Structure(cell, sp, pos, rc, [b2])
            dvs.append(s.descriptors[0])
            ys.append(lennard_jones(cell, pos)[3])
    finally:
        b2.store_dervs = store
    sparse = ClusterDescriptor()
    sparse.initialize_cluster(ns, dvs[0].n_descriptors)
    for s_ in range(ns):
        pool = [(f, k) for f, dv in enumerate(dvs) for k in range(dv.n_clusters_by_type[s_])]
        pick = rng.choice(len(pool), min(n_sparse_per_species, len(pool)), replace=False)
        by_frame = {}
        for p in sorted(pick):
            by_frame.setdefault(pool[p][0], []).append(pool[p][1])
        for f in sorted(by_frame):
            cl = [[] for _ in range(ns)]
            cl[s_] = by_frame[f]
            sparse.add_clusters_by_type(dvs[f], cl)
    train = ClusterDescriptor()
    for dv in dvs:
        train.add_all_clusters(dv)
    y = np.concatenate([np.concatenate([ys[f][dv.atom_indices[s_]] for f, dv in enumerate(dvs)])
                        for s_ in range(ns)])
    kern = NormalizedDotProduct(sigma, power)
    Kuu = kern.envs_envs(sparse, sparse)
    Kuf = kern.envs_envs(sparse, train)
    alpha, R_inv, L_inv = update_matrices_QR(Kuu, Kuf, y, np.full(len(y), 1 / noise ** 2))
    return dict(sparse=sparse, alpha=alpha, R_inv=R_inv, L_inv=L_inv, sigma=sigma,
                power=power, n_train=train.n_clusters)


def bcc_alloy_32k_recipe(seed=303, n_sparse=2000, reps=(32, 32, 16)):
    """The 32,768-atom two-species BCC workload (32x32x16 cells, a=3.0 A,
    rattle 0.08 A, rc 5.5 A, chebyshev N=12, lmax=4, quadratic cutoff) and
    the recipe of its model: n_sparse environments per species drawn from
    four 16x8x8-cell frames of the same alloy (seeds seed+1..seed+4), weights
    fitted to Lennard-Jones site energies (sigma 2, power 2).  numpy only.
    reps sets the evaluated frame's cells (the same model for any size)."""
    frames = [bcc_alloy((16, 8, 8), seed + k) for k in range(1, 5)]
    cell, sp, pos = bcc_alloy(tuple(reps), seed)
    return dict(kind="B2", descriptor=("chebyshev", "quadratic", [0.0, 5.5], [], [2, 12, 4]),
                frames=frames, n_sparse=n_sparse, seed=seed, sigma=2.0, power=2,
                cell=cell, species=sp, positions=pos)


def bcc_alloy_16k_recipe(seed=303, n_sparse=2000):
    """The 32k workload's model on a 16,384-atom frame (32x16x16 cells): the
    small case for hardware-counter captures of the same kernels."""
    return bcc_alloy_32k_recipe(seed, n_sparse, reps=(32, 16, 16))


def fcc_al(reps, seed, rattle=0.05, a=4.05):
    """FCC aluminium supercell of reps conventional cells, rattled."""
    rng = np.random.default_rng(seed)
    return rattled(FCC_BASIS, a, reps, rattle, rng)


def fcc_al_b3_1m_recipe(seed=505, n_sparse=500, reps=(64, 64, 64)):
    """The B3 workload: FCC Al, a = 4.05 A, 64^3 conventional cells
    (1,048,576 atoms), rattle 0.05 A, rc 5.0 A, chebyshev N=6, lmax=3,
    quadratic cutoff, with n_sparse environments drawn from four 6x6x6-cell
    frames (seeds seed+1..seed+4) and weights fitted to Lennard-Jones site
    energies.  numpy only."""
    frames = [fcc_al((6, 6, 6), seed + k) for k in range(1, 5)]
    cell, sp, pos = fcc_al(reps, seed)
    return dict(kind="B3", descriptor=("chebyshev", "quadratic", [0.0, 5.0], [], [1, 6, 3]),
                frames=frames, n_sparse=n_sparse, seed=seed, sigma=2.0, power=2,
                cell=cell, species=sp, positions=pos)


def model_from_recipe(r, device="cuda"):
    """The GPU model of a workload recipe (descriptors, kernels and the QR
    solve in the library, FP64)."""
    from .api import B2, B3, NormalizedDotProduct, SparseGP
    desc = (B3 if r["kind"] == "B3" else B2)(*r["descriptor"])
    fit = fit_site_energy_model(desc, r["frames"], r["n_sparse"], sigma=r["sigma"],
                                power=r["power"], seed=r["seed"], device=device)
    gp = SparseGP([NormalizedDotProduct(r["sigma"], r["power"])], 0.001, 0.05, 0.006)
    gp.set_model(desc, fit["sparse"], fit["alpha"], fit["R_inv"], fit["L_inv"])
    return dict(b2=desc, gp=gp, cell=r["cell"], species=r["species"],
                positions=r["positions"], fit=fit)


def bcc_alloy_32k_model(seed=303, n_sparse=2000, device="cuda"):
    """bcc_alloy_32k_recipe with its model built in the library."""
    return model_from_recipe(bcc_alloy_32k_recipe(seed, n_sparse), device)


def fcc_al_b3_1m_model(seed=505, n_sparse=500, reps=(64, 64, 64), device="cuda"):
    """fcc_al_b3_1m_recipe with its model built in the library."""
    return model_from_recipe(fcc_al_b3_1m_recipe(seed, n_sparse, reps), device)
