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
