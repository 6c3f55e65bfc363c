"""Mapped-beta potential files.

Writer: the layout of SparseGP::write_mapping_coefficients
(src/flare_pp/bffs/sparse_gp.cpp:1142-1206) with B2::write_to_file
(src/flare_pp/descriptors/b2.cpp:52-74).  Reader: PairFLARE::read_file
(lammps_plugins/pair_flare.cpp:263-396).

    DATE: ... CONTRIBUTOR: ...
    <power>
    chebyshev
    <n_species> <n_max> <l_max> <beta_size>
    <cutoff function>
    <n_species^2 cutoffs>
    <beta of species 0, five per line> then each further species on a new line

The reader also takes the older layout that files written before the power
line and the per-species-pair cutoffs existed use (the reference's own
lammps_plugins/test_compute/Si.txt and beta.txt): no power line (power 2),
and one cutoff on its own line for every species pair.
"""
import time

import numpy as np


def write_potential(filename, beta, power, n_species, n_max, l_max, cutoffs,
                    cutoff_function="quadratic", radial="chebyshev",
                    contributor="flare_pp_gb300"):
    beta = np.atleast_2d(np.asarray(beta, dtype=np.float64))
    with open(filename, "w") as f:
        f.write(f"DATE: {time.ctime()} CONTRIBUTOR: {contributor}\n")
        f.write(f"{int(power)}\n")
        f.write(f"{radial}\n")
        f.write(f"{n_species} {n_max} {l_max} {beta.shape[1]}\n")
        f.write(f"{cutoff_function}\n")
        f.write(" ".join(f"{c:.2f}" for c in np.asarray(cutoffs).ravel()) + " \n")
        count = 0
        for i, row in enumerate(beta):
            if count != 0:
                f.write("\n")
            for v in row:
                f.write("  " if v > 0 else " ")
                f.write(f"{v:.16e}")
                count += 1
                if count == 5:
                    count = 0
                    f.write("\n")


def read_potential(filename):
    with open(filename) as f:
        lines = f.read().splitlines()
    try:
        power = int(lines[1].split()[0])
        legacy = False
    except ValueError:      # older layout: no power line, one cutoff
        power = 2
        legacy = True
        lines = lines[:1] + ["2"] + lines[1:]
    radial = lines[2].split()[0]
    ns, n_max, l_max, beta_size = (int(v) for v in lines[3].split()[:4])
    cutoff_function = lines[4].split()[0]
    vals = []
    rest = lines[5:]
    k = 0
    n_cut = 1 if legacy else ns * ns
    while len(vals) < n_cut:
        vals += [float(v) for v in rest[k].split()]
        k += 1
    cutoffs = np.full(ns * ns, vals[0]) if legacy else np.array(vals[:ns * ns])
    nums = []
    for line in rest[k:]:
        nums += [float(v) for v in line.split()]
    n_rad = ns * n_max
    n_d = n_rad * (n_rad + 1) // 2 * (l_max + 1)
    check = n_d if power == 1 else n_d * (n_d + 1) // 2
    if power not in (1, 2):
        raise ValueError("Power should be 1 or 2.")
    if check != beta_size:
        raise ValueError("Beta size doesn't match the number of descriptors.")
    if len(nums) < beta_size * ns:
        raise ValueError("potential file holds too few beta values")
    beta = np.array(nums[:beta_size * ns]).reshape(ns, beta_size)
    return dict(power=power, radial=radial, n_species=ns, n_max=n_max,
                l_max=l_max, beta_size=beta_size, cutoff_function=cutoff_function,
                cutoffs=cutoffs, beta=beta, legacy=legacy)


# ---------------------------------------------------------------------------
# Coefficient files of the LAMMPS compute flare/std/atom.
# ---------------------------------------------------------------------------
def _descriptor_header(f, radial, n_species, n_max, l_max, size, cutoff_function,
                       cutoffs):
    """B2::write_to_file (src/flare_pp/descriptors/b2.cpp:52-74)."""
    f.write(f"{radial}\n")
    f.write(f"{n_species} {n_max} {l_max} {size}\n")
    f.write(f"{cutoff_function}\n")
    f.write("".join(f"{c:.2f} " for c in np.asarray(cutoffs, dtype=np.float64).ravel())
            + "\n")


def _hyps_lines(f, hyps):
    hyps = np.asarray(hyps, dtype=np.float64).ravel()
    f.write(f"{len(hyps)}\n")
    f.write("".join(f"{h:.16e} " for h in hyps) + "\n")


def _read_descriptor_header(lines, k):
    radial = lines[k].split()[0]
    ns, n_max, l_max, size = (int(v) for v in lines[k + 1].split()[:4])
    cutoff_function = lines[k + 2].split()[0]
    k += 3
    vals = []
    while len(vals) < ns * ns:
        vals += [float(v) for v in lines[k].split()]
        k += 1
    cutoffs = np.array(vals[:ns * ns]).reshape(ns, ns)
    return dict(radial=radial, n_species=ns, n_max=n_max, l_max=l_max, size=size,
                cutoff_function=cutoff_function, cutoffs=cutoffs), k


def _grab(lines, k, n):
    """ComputeFlareStdAtom::grab (compute_flare_std_atom.cpp:652-664): whole
    lines until n numbers have been read."""
    out = []
    while len(out) < n:
        if k >= len(lines):
            raise ValueError("coefficient file ends early")
        out += [float(v) for v in lines[k].split()]
        k += 1
    return np.array(out[:n]), k


def _n_descriptors(ns, n_max, l_max):
    n_rad = ns * n_max
    return n_rad * (n_rad + 1) // 2 * (l_max + 1)


def write_varmap(filename, varmap, hyps, n_species, n_max, l_max, cutoffs,
                 cutoff_function="quadratic", radial="chebyshev",
                 contributor="flare_pp_gb300"):
    """SparseGP::write_varmap_coefficients (sparse_gp.cpp:1208-1281): one row
    of n_d^2 values per species, five per line."""
    varmap = np.atleast_2d(np.asarray(varmap, dtype=np.float64))
    with open(filename, "w") as f:
        f.write(f"DATE: {time.ctime()} CONTRIBUTOR: {contributor}\n")
        _hyps_lines(f, hyps)
        _descriptor_header(f, radial, n_species, n_max, l_max, varmap.shape[1],
                           cutoff_function, cutoffs)
        count = 0
        for row in varmap:
            if count != 0:
                f.write("\n")
                count = 0
            for v in row:
                f.write("  " if v > 0 else " ")
                f.write(f"{v:.16e}")
                count += 1
                if count == 5:
                    count = 0
                    f.write("\n")


def read_varmap(filename):
    """ComputeFlareStdAtom::read_file (compute_flare_std_atom.cpp:345-454)."""
    with open(filename) as f:
        lines = f.read().splitlines()
    n_hyps = int(lines[1].split()[0])
    hyps = np.array([float(v) for v in lines[2].split()[:n_hyps]])
    hdr, k = _read_descriptor_header(lines, 3)
    nd = _n_descriptors(hdr["n_species"], hdr["n_max"], hdr["l_max"])
    if nd * nd != hdr["size"]:
        raise ValueError("Beta size doesn't match the number of descriptors.")
    vals, _ = _grab(lines, k, hdr["size"] * hdr["n_species"])
    hdr.update(hyps=hyps, n_descriptors=nd,
               varmap=vals.reshape(hdr["n_species"], nd, nd))
    return hdr


def write_L_inverse(filename, L_inv, power, hyps, n_species, n_max, l_max, cutoffs,
                    cutoff_function="quadratic", radial="chebyshev",
                    contributor="flare_pp_gb300", n_kernels=1):
    """SparseGP::write_L_inverse (sparse_gp.cpp:1283-1344): the lower
    triangle of L_inv row by row, five numbers per line."""
    L = np.asarray(L_inv, dtype=np.float64)
    with open(filename, "w") as f:
        f.write(f"L_inverse_block file DATE: {time.ctime()} CONTRIBUTOR: {contributor}\n")
        f.write(f"{int(power)}\n")
        _hyps_lines(f, hyps)
        _descriptor_header(f, radial, n_species, n_max, l_max, n_kernels,
                           cutoff_function, cutoffs)
        n = L.shape[0]
        f.write(f"{n}\n")
        count = 1
        for j in range(n):
            for k in range(j + 1):
                f.write(f"{L[j, k]:.16e} ")
                if count % 5 == 0:
                    f.write("\n")
                count += 1
        if count % 5 != 0:
            f.write("\n")


def read_L_inverse(filename):
    """ComputeFlareStdAtom::read_L_inverse (compute_flare_std_atom.cpp:456-568):
    returns the header and the dense n x n lower-triangular L_inv."""
    with open(filename) as f:
        lines = f.read().splitlines()
    power = int(lines[1].split()[0])
    n_hyps = int(lines[2].split()[0])
    hyps = np.array([float(v) for v in lines[3].split()[:n_hyps]])
    hdr, k = _read_descriptor_header(lines, 4)
    n = int(lines[k].split()[0])
    vals, _ = _grab(lines, k + 1, n * (n + 1) // 2)
    L = np.zeros((n, n))
    L[np.tril_indices(n)] = vals
    hdr.update(power=power, hyps=hyps, n_kernels=hdr["size"], n_clusters=n, L_inv=L,
               n_descriptors=_n_descriptors(hdr["n_species"], hdr["n_max"],
                                            hdr["l_max"]))
    return hdr


def write_sparse_descriptors(filename, descriptors, norms,
                             contributor="flare_pp_gb300"):
    """SparseGP::write_sparse_descriptors (sparse_gp.cpp:1346-1404) for one
    kernel: per species its count, then the normalized rows (zeros for an
    empty environment, |p| < 1e-8)."""
    with open(filename, "w") as f:
        f.write(f"sparse_descriptors file DATE: {time.ctime()} CONTRIBUTOR: {contributor}\n")
        f.write("1\n")
        n_types = len(descriptors)
        n_clusters = sum(len(n) for n in norms)
        f.write(f"0 {n_clusters} {n_types}\n")
        count = 1
        for D, nrm in zip(descriptors, norms):
            D = np.atleast_2d(np.asarray(D, dtype=np.float64))
            nrm = np.asarray(nrm, dtype=np.float64)
            f.write(f"{len(nrm)}\n")
            for j in range(len(nrm)):
                for k in range(D.shape[1] if len(nrm) else 0):
                    v = 0.0 if nrm[j] < 1e-8 else D[j, k] / nrm[j]
                    f.write(f"{v:.16e} ")
                    if count % 5 == 0:
                        f.write("\n")
                    count += 1
            if count % 5 != 1:
                f.write("\n")


def read_sparse_descriptors(filename, n_descriptors, n_clusters=None):
    """ComputeFlareStdAtom::read_sparse_descriptors
    (compute_flare_std_atom.cpp:570-650): per species the normalized rows."""
    with open(filename) as f:
        lines = f.read().splitlines()
    n_kern = int(lines[1].split()[0])
    if n_kern != 1:
        raise ValueError("n_kernals in sparse_descriptors and L_inv not match")
    _, n_clst, n_types = (int(v) for v in lines[2].split()[:3])
    if n_clusters is not None and n_clst != n_clusters:
        raise ValueError("n_clusters in sparse_descriptors and L_inv not match")
    k = 3
    out = []
    for _ in range(n_types):
        while not lines[k].split():  # the line break after a species with no rows
            k += 1
        m = int(lines[k].split()[0])
        vals, k = _grab(lines, k + 1, m * n_descriptors)
        out.append(vals.reshape(m, n_descriptors))
    return out
