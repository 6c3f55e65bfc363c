"""Periodic structure and neighbor list (FP64 numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates ``Structure`` from src/flare_pp/structure.cpp.  Every floating-point
operation is spelled out elementwise (no BLAS, no fused multiply-add) so that
the GPU neighbor builder, which uses the same operation order, reproduces the
distances bit for bit.
"""
import math

import numpy as np


def inv3(m):
    """Inverse of a 3x3 matrix by cofactors, fixed operation order.

    The GPU library computes the same cofactor expansion on the host with
    contraction disabled, so both sides get identical bits.
    """
    a = [[float(m[i][j]) for j in range(3)] for i in range(3)]
    c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1]
    c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2]
    c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0]
    det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02
    inv = np.empty((3, 3))
    inv[0, 0] = c00 / det
    inv[1, 0] = c01 / det
    inv[2, 0] = c02 / det
    inv[0, 1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det
    inv[1, 1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det
    inv[2, 1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det
    inv[0, 2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det
    inv[1, 2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det
    inv[2, 2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det
    return inv, det


def matmul3(p, m):
    """(n,3) x (3,3) with the sum order ((a0 b0 + a1 b1) + a2 b2)."""
    p = np.asarray(p, dtype=np.float64)
    out = np.empty_like(p)
    for j in range(3):
        out[:, j] = (p[:, 0] * m[0, j] + p[:, 1] * m[1, j]) + p[:, 2] * m[2, j]
    return out


def cell_matrices(cell):
    """cell_transpose, its inverse, cell_dot, its inverse, volume.

    src/flare_pp/structure.cpp:15-22.
    """
    cell = np.asarray(cell, dtype=np.float64)
    ct = cell.T.copy()
    ct_inv, _ = inv3(ct)
    cdot = np.empty((3, 3))
    for i in range(3):
        for j in range(3):
            cdot[i, j] = (cell[i, 0] * ct[0, j] + cell[i, 1] * ct[1, j]) + \
                cell[i, 2] * ct[2, j]
    cdot_inv, _ = inv3(cdot)
    _, det = inv3(cell)
    return ct, ct_inv, cdot, cdot_inv, abs(det)


def wrap_positions(cell, positions):
    """src/flare_pp/structure.cpp:120-133."""
    ct, ct_inv, cdot, cdot_inv, _ = cell_matrices(cell)
    rel = matmul3(matmul3(positions, ct), cdot_inv)
    rel_wrapped = rel - np.floor(rel)
    return matmul3(matmul3(rel_wrapped, cdot), ct_inv)


def single_sweep_cutoff(cell):
    """src/flare_pp/structure.cpp:135-165."""
    v = np.asarray(cell, dtype=np.float64)

    def dot(a, b):
        return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]

    a_b, a_c, b_c = dot(v[0], v[1]), dot(v[0], v[2]), dot(v[1], v[2])
    a = math.sqrt(dot(v[0], v[0]))
    b = math.sqrt(dot(v[1], v[1]))
    c = math.sqrt(dot(v[2], v[2]))

    def h(x, cosv):
        t = cosv
        return x * math.sqrt(1 - t * t)

    cands = [h(a, a_b / (a * b)), h(b, a_b / (a * b)), h(a, a_c / (a * c)),
             h(c, a_c / (a * c)), h(b, b_c / (b * c)), h(c, b_c / (b * c))]
    return min(cands)


class Structure:
    """Periodic cell with an O(N^2 (2s+1)^3) neighbor scan.

    src/flare_pp/structure.cpp:27-118.  Neighbors of atom i are ordered by
    j ascending, then s1, s2, s3 ascending in [-sweep, sweep]; a pair enters
    when dist < cutoff and dist != 0 (structure.cpp:77).
    """

    def __init__(self, cell, species, positions, cutoff=None,
                 descriptor_calculators=()):
        self.cell = np.asarray(cell, dtype=np.float64)
        self.species = np.asarray(species, dtype=np.int64)
        self.positions = np.asarray(positions, dtype=np.float64)
        self.noa = len(self.species)
        (self.cell_transpose, self.cell_transpose_inverse, self.cell_dot,
         self.cell_dot_inverse, self.volume) = cell_matrices(self.cell)
        self.single_sweep_cutoff = single_sweep_cutoff(self.cell)
        self.wrapped_positions = wrap_positions(self.cell, self.positions)
        self.energy = np.zeros(0)
        self.forces = np.zeros(0)
        self.stresses = np.zeros(0)
        self.descriptors = []
        if cutoff is not None:
            self.cutoff = float(cutoff)
            self.sweep = int(math.ceil(self.cutoff / self.single_sweep_cutoff))
            self.descriptor_calculators = list(descriptor_calculators)
            self.compute_neighbors()
            self.compute_descriptors()

    def compute_descriptors(self):
        self.descriptors = [d.compute_struc(self)
                            for d in self.descriptor_calculators]

    def compute_neighbors(self):
        noa, sweep, cell = self.noa, self.sweep, self.cell
        rng = np.arange(-sweep, sweep + 1)
        s1, s2, s3 = np.meshgrid(rng, rng, rng, indexing="ij")
        shifts = np.stack([s1.ravel(), s2.ravel(), s3.ravel()], 1).astype(
            np.float64)
        # shift vectors computed per term so the additions keep the
        # reference's left-to-right order: ((diff + s1 c0) + s2 c1) + s3 c2
        t1 = shifts[:, 0:1] * cell[0][None, :]
        t2 = shifts[:, 1:2] * cell[1][None, :]
        t3 = shifts[:, 2:3] * cell[2][None, :]
        wp = self.wrapped_positions
        counts = np.zeros(noa, dtype=np.int64)
        all_idx, all_rel = [], []
        for i in range(noa):
            diff = wp - wp[i]                                  # (noa, 3)
            im = ((diff[:, None, :] + t1[None]) + t2[None]) + t3[None]
            dist = np.sqrt((im[..., 0] * im[..., 0] + im[..., 1] * im[..., 1])
                           + im[..., 2] * im[..., 2])
            mask = (dist < self.cutoff) & (dist != 0)
            jj, ss = np.nonzero(mask)                          # j asc, s asc
            counts[i] = len(jj)
            all_idx.append(jj)
            rel = np.empty((len(jj), 4))
            rel[:, 0] = dist[jj, ss]
            rel[:, 1:] = im[jj, ss]
            all_rel.append(rel)
        self.neighbor_count = counts
        self.cumulative_neighbor_count = np.concatenate(
            [[0], np.cumsum(counts)]).astype(np.int64)
        self.n_neighbors = int(self.cumulative_neighbor_count[-1])
        self.structure_indices = (np.concatenate(all_idx).astype(np.int64)
                                  if noa else np.zeros(0, np.int64))
        self.relative_positions = (np.concatenate(all_rel) if noa
                                   else np.zeros((0, 4)))
        self.neighbor_species = self.species[self.structure_indices]
