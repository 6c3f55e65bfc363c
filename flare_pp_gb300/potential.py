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
    power = int(lines[1].split()[0])
    radial = lines[2].split()[0]
    ns, n_max, l_max, beta_size = (int(v) for v in lines[3].split()[:4])
    cutoff_function = lines[4].split()[0]
    vals = []
    rest = lines[5:]
    k = 0
    while len(vals) < ns * ns:
        vals += [float(v) for v in rest[k].split()]
        k += 1
    cutoffs = np.array(vals[:ns * ns])
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
                cutoffs=cutoffs, beta=beta)
