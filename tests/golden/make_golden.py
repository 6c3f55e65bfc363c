"""Record golden vectors from the reference's own L0 math.

Builds oracle/_ref/libflare_ref.so from the reference sources
(oracle/ref/build_ref.sh: radial.cpp, cutoffs.cpp, y_grad.cpp and
descriptors/wigner3j.cpp compiled where they lie) and evaluates:
  * get_Y (y_grad.cpp:667) up to l = 10 at seeded random vectors,
  * get_complex_Y (y_grad.cpp:24) up to l = 6,
  * calculate_radial (radial.cpp:344) with the chebyshev basis and the
    quadratic and cosine cutoffs (cutoffs.cpp:44-73), N = 12,
  * compute_coeffs (descriptors/wigner3j.cpp:5), the Wigner 3j tables of
    B3, for lmax = 0..4 (nonzero entries as index/value pairs).
Writes tests/golden/l0_golden.npz.

Then the pair style's per-atom math: lammps_plugins/lammps_descriptor.cpp
(single_bond_multiple_cutoffs, B2_descriptor, compute_energy_and_u),
compiled unmodified against a small Eigen stand-in, driven by the per-atom
loop of pair_flare.cpp:95-180 (ref_pair_flare in oracle/ref/ref_shim.cpp)
over LAMMPS-shaped arrays with ghost atoms, on the seeded cases of
tests/fixtures.BETA_CASES: per-atom energies, forces folded onto the owning
atoms, the virial, and the single-bond values, B2 values, u and E_i of the
first listed atoms.  Writes tests/golden/beta_form_golden.npz.

Run from the repository root:
    python tests/golden/make_golden.py [/path/to/reference]
(default: $FLARE_PP_REFERENCE, else /root/reference)
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
N_REC = 6


def beta_form_golden(lib):
    from tests import fixtures
    from oracle.b2 import n_descriptors
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    lib.ref_pair_flare.restype = ctypes.c_int
    out = {}
    for name in fixtures.BETA_CASES:
        cell, sp, pos, st, beta, power = fixtures.beta_case(name)
        ns, N, lmax = st["n_species"], st["N"], st["lmax"]
        cut = np.ascontiguousarray(st["cutoffs"], dtype=np.float64)
        x, types, ilist, numneigh, nbrs, owner = fixtures.lammps_arrays(
            cell, sp, pos, float(cut.max()))
        nall, noa = len(x), len(sp)
        x = np.ascontiguousarray(x, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        ilist = np.ascontiguousarray(ilist, dtype=np.int32)
        numneigh = np.ascontiguousarray(numneigh, dtype=np.int32)
        off = np.zeros(noa + 1, dtype=np.int32)
        off[1:] = np.cumsum(numneigh)
        nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        B = np.ascontiguousarray(np.stack(beta), dtype=np.float64)
        n_rad = ns * N
        nb, nd = n_rad * (lmax + 1) ** 2, n_descriptors(ns, N, lmax)
        f = np.zeros((nall, 3))
        eat = np.zeros(nall)
        vir = np.zeros(6)
        rsb, rb2, ru, re = (np.zeros((N_REC, nb)), np.zeros((N_REC, nd)),
                            np.zeros((N_REC, nb)), np.zeros(N_REC))
        rc = lib.ref_pair_flare(
            nall, x.ctypes.data_as(D), types.ctypes.data_as(I), noa, ilist.ctypes.data_as(I),
            numneigh.ctypes.data_as(I), off.ctypes.data_as(I), nbrs.ctypes.data_as(I),
            ns, N, lmax, ctypes.c_double(st["r1"]), cut.ctypes.data_as(D),
            st["cutoff_function"].encode(), power, B.ctypes.data_as(D), f.ctypes.data_as(D),
            eat.ctypes.data_as(D), vir.ctypes.data_as(D), N_REC, rsb.ctypes.data_as(D),
            rb2.ctypes.data_as(D), ru.ctypes.data_as(D), re.ctypes.data_as(D))
        assert rc == 0, name
        F = np.zeros((noa, 3))
        np.add.at(F, owner, f)
        out[f"{name}/atom_energies"] = eat[:noa]
        out[f"{name}/forces"] = F
        out[f"{name}/virial"] = vir
        out[f"{name}/rec_single_bond"] = rsb
        out[f"{name}/rec_b2"] = rb2
        out[f"{name}/rec_u"] = ru
        out[f"{name}/rec_energy"] = re
        print(f"{name}: {noa} atoms, {nall - noa} ghosts, E = {eat[:noa].sum():.12g}")
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "beta_form_golden.npz"), **out)
    print("wrote tests/golden/beta_form_golden.npz")


def _proj(m, seed=4242):
    """A seeded random projection of a wide matrix (a check of every entry
    without storing them all)."""
    r = np.random.default_rng(seed).normal(size=(m.shape[1], 4))
    return m @ r


def struc_kernel_golden(lib):
    from tests import fixtures
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    lib.ref_b2_new.restype = vp
    lib.ref_b2_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, D, ctypes.c_char_p]
    lib.ref_structure_new.restype = vp
    lib.ref_structure_new.argtypes = [D, I, D, ctypes.c_int, ctypes.c_double, vp]
    for fn in ("ref_structure_dbl", "ref_structure_int"):
        getattr(lib, fn).argtypes = [vp, ctypes.c_char_p, ctypes.c_void_p]
    for fn in ("ref_dv_dbl", "ref_dv_int"):
        getattr(lib, fn).argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    lib.ref_cluster_new.restype = vp
    lib.ref_cluster_add.argtypes = [vp, vp, I, I]
    lib.ref_kernel.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, vp, vp,
                               ctypes.c_void_p, I, I]
    lib.ref_structure_free.argtypes = [vp]
    lib.ref_b2_free.argtypes = [vp]
    lib.ref_cluster_free.argtypes = [vp]

    def dbl(fn, h, field, *extra):
        n = fn(h, field.encode(), *extra, None)
        assert n >= 0, field
        out = np.zeros(n)
        fn(h, field.encode(), *extra, out.ctypes.data)
        return out

    def ints(fn, h, field, *extra):
        n = fn(h, field.encode(), *extra, None)
        assert n >= 0, field
        out = np.zeros(n, dtype=np.int32)
        fn(h, field.encode(), *extra, out.ctypes.data)
        return out

    out = {}
    handles = {}
    cases = fixtures.struc_cases()
    for name, (cell, sp, pos, rc, (ns, N, lmax), cut) in cases.items():
        cut = np.ascontiguousarray(cut, dtype=np.float64)
        b2 = lib.ref_b2_new(ns, N, lmax, 0.0, float(rc), cut.ctypes.data_as(D), b"quadratic")
        c = np.ascontiguousarray(cell, dtype=np.float64)
        spi = np.ascontiguousarray(sp, dtype=np.int32)
        p = np.ascontiguousarray(pos, dtype=np.float64)
        h = lib.ref_structure_new(c.ctypes.data_as(D), spi.ctypes.data_as(I),
                                  p.ctypes.data_as(D), len(sp), float(rc), b2)
        handles[name] = (h, b2)
        k = f"struc/{name}/"
        for f in ("neighbor_count", "cumulative_neighbor_count", "structure_indices",
                  "neighbor_species"):
            out[k + f] = ints(lib.ref_structure_int, h, f)
        out[k + "relative_positions"] = dbl(lib.ref_structure_dbl, h,
                                            "relative_positions").reshape(-1, 4)
        out[k + "wrapped_positions"] = dbl(lib.ref_structure_dbl, h,
                                           "wrapped_positions").reshape(-1, 3)
        for f in ("volume", "sweep"):
            out[k + f] = dbl(lib.ref_structure_dbl, h, f)
        nd = int(ints(lib.ref_dv_int, h, "n_descriptors", 0)[0])
        for s_ in range(ns):
            kd = f"dv/{name}/{s_}/"
            out[kd + "descriptors"] = dbl(lib.ref_dv_dbl, h, "descriptors", s_).reshape(-1, nd)
            fd = dbl(lib.ref_dv_dbl, h, "descriptor_force_dervs", s_).reshape(-1, nd)
            out[kd + "force_dervs_rows"] = fd[:48]
            out[kd + "force_dervs_proj"] = _proj(fd) if len(fd) else np.zeros((0, 4))
            out[kd + "neighbor_coordinates"] = dbl(lib.ref_dv_dbl, h, "neighbor_coordinates",
                                                   s_).reshape(-1, 3)
            for f in ("descriptor_norms", "descriptor_force_dots", "cutoff_values"):
                out[kd + f] = dbl(lib.ref_dv_dbl, h, f, s_)
            for f in ("neighbor_counts", "cumulative_neighbor_counts", "atom_indices",
                      "neighbor_indices"):
                out[kd + f] = ints(lib.ref_dv_int, h, f, s_)
    # kernels on a sparse set drawn from two structures
    ns, nd = 2, int(ints(lib.ref_dv_int, handles["bcc54"][0], "n_descriptors", 0)[0])
    cd = lib.ref_cluster_new(ns, nd)
    for name, cl in fixtures.KERNEL_SPARSE:
        counts = np.array([len(x) for x in cl], dtype=np.int32)
        flat = np.array([a for x in cl for a in x], dtype=np.int32)
        assert lib.ref_cluster_add(cd, handles[name][0], counts.ctypes.data_as(I),
                                   flat.ctypes.data_as(I)) == 0
    a_, b_ = (handles[n][0] for n in fixtures.KERNEL_STRUCS)
    for sig, pw in fixtures.KERNEL_HYPS:
        for what, x, y in (("envs_envs", cd, cd), ("envs_struc", cd, b_),
                           ("struc_struc", a_, b_), ("self_kernel_struc", b_, None)):
            r, cc = ctypes.c_int(), ctypes.c_int()
            n = lib.ref_kernel(what.encode(), sig, pw, x, y, None, ctypes.byref(r),
                               ctypes.byref(cc))
            if n == -2:      # the reference throws (power < 2, zero dot product)
                out[f"kernel/{what}/{sig}/{pw}/throws"] = np.array(1)
                continue
            m = np.zeros(n)
            lib.ref_kernel(what.encode(), sig, pw, x, y, m.ctypes.data, ctypes.byref(r),
                           ctypes.byref(cc))
            out[f"kernel/{what}/{sig}/{pw}"] = m.reshape(r.value, cc.value)
    lib.ref_cluster_free(cd)
    for h, b2 in handles.values():
        lib.ref_structure_free(h)
        lib.ref_b2_free(b2)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "struc_kernel_golden.npz"), **out)
    print("wrote tests/golden/struc_kernel_golden.npz")


def b3_golden(lib):
    """DescriptorValues of the reference's B3 (descriptors/b3.cpp) on the
    tests.fixtures.b3_cases structures, and the NormalizedDotProduct kernels
    on B3 descriptors, into tests/golden/b3_golden.npz."""
    from tests import fixtures
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    lib.ref_b3_new.restype = vp
    lib.ref_b3_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, ctypes.c_char_p]
    lib.ref_b3_free.argtypes = [vp]
    lib.ref_structure_new.restype = vp
    lib.ref_structure_new.argtypes = [D, I, D, ctypes.c_int, ctypes.c_double, vp]
    lib.ref_structure_free.argtypes = [vp]
    for fn in ("ref_dv_dbl", "ref_dv_int"):
        getattr(lib, fn).argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    lib.ref_cluster_new.restype = vp
    lib.ref_cluster_add.argtypes = [vp, vp, I, I]
    lib.ref_cluster_free.argtypes = [vp]
    lib.ref_kernel.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, vp, vp,
                               ctypes.c_void_p, I, I]

    def dbl(h, field, s_):
        n = lib.ref_dv_dbl(h, field.encode(), s_, None)
        assert n >= 0, field
        out = np.zeros(n)
        lib.ref_dv_dbl(h, field.encode(), s_, out.ctypes.data)
        return out

    def ints(h, field, s_):
        n = lib.ref_dv_int(h, field.encode(), s_, None)
        assert n >= 0, field
        out = np.zeros(n, dtype=np.int32)
        lib.ref_dv_int(h, field.encode(), s_, out.ctypes.data)
        return out

    out, handles = {}, {}
    for name, (cell, sp, pos, rc, (ns, N, lmax)) in fixtures.b3_cases().items():
        b3 = lib.ref_b3_new(ns, N, lmax, 0.0, float(rc), b"quadratic")
        c = np.ascontiguousarray(cell, dtype=np.float64)
        spi = np.ascontiguousarray(sp, dtype=np.int32)
        p = np.ascontiguousarray(pos, dtype=np.float64)
        h = lib.ref_structure_new(c.ctypes.data_as(D), spi.ctypes.data_as(I),
                                  p.ctypes.data_as(D), len(sp), float(rc), b3)
        handles[name] = (h, b3)
        nd = int(ints(h, "n_descriptors", 0)[0])
        for s_ in range(ns):
            kd = f"dv/{name}/{s_}/"
            out[kd + "descriptors"] = dbl(h, "descriptors", s_).reshape(-1, nd)
            fd = dbl(h, "descriptor_force_dervs", s_).reshape(-1, nd)
            out[kd + "force_dervs_rows"] = fd[:48]
            out[kd + "force_dervs_proj"] = _proj(fd) if len(fd) else np.zeros((0, 4))
            for f in ("descriptor_norms", "descriptor_force_dots", "cutoff_values"):
                out[kd + f] = dbl(h, f, s_)
            for f in ("neighbor_counts", "cumulative_neighbor_counts", "atom_indices",
                      "neighbor_indices"):
                out[kd + f] = ints(h, f, s_)
    name0 = fixtures.B3_KERNEL_SPARSE[0][0]
    nd = int(ints(handles[name0][0], "n_descriptors", 0)[0])
    cd = lib.ref_cluster_new(2, nd)
    for name, cl in fixtures.B3_KERNEL_SPARSE:
        counts = np.array([len(x) for x in cl], dtype=np.int32)
        flat = np.array([a for x in cl for a in x], dtype=np.int32)
        assert lib.ref_cluster_add(cd, handles[name][0], counts.ctypes.data_as(I),
                                   flat.ctypes.data_as(I)) == 0
    a_, b_ = (handles[n][0] for n in fixtures.B3_KERNEL_STRUCS)
    for sig, pw in fixtures.KERNEL_HYPS:
        for what, x, y in (("envs_envs", cd, cd), ("envs_struc", cd, b_),
                           ("struc_struc", a_, b_), ("self_kernel_struc", b_, None)):
            r, cc = ctypes.c_int(), ctypes.c_int()
            n = lib.ref_kernel(what.encode(), sig, pw, x, y, None, ctypes.byref(r),
                               ctypes.byref(cc))
            if n == -2:
                out[f"kernel/{what}/{sig}/{pw}/throws"] = np.array(1)
                continue
            m = np.zeros(n)
            lib.ref_kernel(what.encode(), sig, pw, x, y, m.ctypes.data, ctypes.byref(r),
                           ctypes.byref(cc))
            out[f"kernel/{what}/{sig}/{pw}"] = m.reshape(r.value, cc.value)
    lib.ref_cluster_free(cd)
    for h, b3 in handles.values():
        lib.ref_structure_free(h)
        lib.ref_b3_free(b3)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "b3_golden.npz"), **out)
    print("wrote tests/golden/b3_golden.npz")


def sgp_golden(lib):
    """The reference's SparseGP (bffs/sparse_gp.cpp) on tests.fixtures.
    sgp_scenario, one kernel and two (B2 + B3): Kuu, Kuf, y, noise vector,
    alpha, R_inv, L_inv, the stable likelihood and its gradient, the same after
    set_hyperparameters, predict_mean / SOR / DTC and the cluster
    uncertainties of the held-out frame, into tests/golden/sgp_golden.npz."""
    from tests import fixtures
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    lib.ref_b2_new.restype = vp
    lib.ref_b2_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, D, ctypes.c_char_p]
    lib.ref_b3_new.restype = vp
    lib.ref_b3_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, ctypes.c_char_p]
    lib.ref_b2_free.argtypes = [vp]
    lib.ref_b3_free.argtypes = [vp]
    lib.ref_sgp_structure_new.restype = vp
    lib.ref_sgp_structure_new.argtypes = [D, I, D, ctypes.c_int, ctypes.c_double,
                                          ctypes.POINTER(vp), ctypes.c_int]
    lib.ref_sgp_structure_free.argtypes = [vp]
    lib.ref_sgp_structure_set_labels.argtypes = [vp, D, ctypes.c_int, D, ctypes.c_int, D,
                                                 ctypes.c_int]
    lib.ref_sgp_structure_get.argtypes = [vp, ctypes.c_char_p, ctypes.c_void_p]
    lib.ref_sgp_new.restype = vp
    lib.ref_sgp_new.argtypes = [ctypes.c_int, D, D, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double]
    lib.ref_sgp_free.argtypes = [vp]
    lib.ref_sgp_add_training_structure.argtypes = [vp, vp, I, ctypes.c_int]
    lib.ref_sgp_add_specific_environments.argtypes = [vp, vp, I, ctypes.c_int]
    lib.ref_sgp_update_matrices_QR.argtypes = [vp]
    lib.ref_sgp_set_hyperparameters.argtypes = [vp, D, ctypes.c_int]
    lib.ref_sgp_compute_likelihood_stable.argtypes = [vp]
    lib.ref_sgp_compute_likelihood_gradient_stable.argtypes = [vp]
    lib.ref_sgp_compute_likelihood_gradient_stable.restype = ctypes.c_double
    lib.ref_sgp_predict.argtypes = [vp, ctypes.c_char_p, vp]
    lib.ref_sgp_cluster_uncertainties.argtypes = [vp, vp, ctypes.c_int, ctypes.c_void_p]
    lib.ref_sgp_get.argtypes = [vp, ctypes.c_char_p, ctypes.c_void_p, I, I]
    for fn in ("ref_sgp_mapping_coefficients", "ref_sgp_varmap_coefficients"):
        getattr(lib, fn).argtypes = [vp, ctypes.c_int, ctypes.c_void_p, I, I]

    def coeffs(fn, gp, ki):
        r, c = ctypes.c_int(), ctypes.c_int()
        n = fn(gp, ki, None, ctypes.byref(r), ctypes.byref(c))
        assert n >= 0
        out = np.zeros(n)
        fn(gp, ki, out.ctypes.data, None, None)
        return out.reshape(r.value, c.value)

    def arr(x, t=np.float64):
        return np.ascontiguousarray(x, dtype=t)

    def get(h, f):
        r, c = ctypes.c_int(), ctypes.c_int()
        n = lib.ref_sgp_get(h, f.encode(), None, ctypes.byref(r), ctypes.byref(c))
        assert n >= 0, f
        out = np.zeros(n)
        lib.ref_sgp_get(h, f.encode(), out.ctypes.data, None, None)
        return out.reshape(r.value, c.value)

    def sget(s, f):
        n = lib.ref_sgp_structure_get(s, f.encode(), None)
        out = np.zeros(n)
        lib.ref_sgp_structure_get(s, f.encode(), out.ctypes.data)
        return out

    out = {}
    for tag, two, power in (("one", False, 2.0), ("two", True, 2.0), ("pow1", False, 1.0)):
        sc = fixtures.sgp_scenario(two, power)
        rc = sc["rc"]
        descs = []
        for kind, (ns, N, lmax) in sc["descs"]:
            if kind == "B2":
                cut = arr(np.full((ns, ns), rc))
                descs.append(lib.ref_b2_new(ns, N, lmax, 0.0, rc, cut.ctypes.data_as(D),
                                            b"quadratic"))
            else:
                descs.append(lib.ref_b3_new(ns, N, lmax, 0.0, rc, b"quadratic"))
        dv = (vp * len(descs))(*descs)

        def structure(cell, sp, pos):
            c, s_, p = arr(cell), arr(sp, np.int32), arr(pos)
            return lib.ref_sgp_structure_new(c.ctypes.data_as(D), s_.ctypes.data_as(I),
                                             p.ctypes.data_as(D), len(sp), rc, dv, len(descs))
        sig = arr([h[0] for h in sc["hyps"]])
        pw = arr([h[1] for h in sc["hyps"]])
        gp = lib.ref_sgp_new(len(descs), sig.ctypes.data_as(D), pw.ctypes.data_as(D),
                             *sc["noises"])
        strucs = []
        for (cell, sp, pos, e, f, st), atoms in zip(sc["frames"], sc["train_atoms"]):
            s = structure(cell, sp, pos)
            e, f, st = arr(e), arr(f), arr(st)
            lib.ref_sgp_structure_set_labels(s, e.ctypes.data_as(D), len(e),
                                             f.ctypes.data_as(D), len(f),
                                             st.ctypes.data_as(D), len(st))
            a = arr(atoms if atoms is not None else [0], np.int32)
            lib.ref_sgp_add_training_structure(gp, s, a.ctypes.data_as(I),
                                               -1 if atoms is None else len(atoms))
            strucs.append(s)
        for s, atoms in zip(strucs, sc["sparse_atoms"]):
            a = arr(atoms, np.int32)
            lib.ref_sgp_add_specific_environments(gp, s, a.ctypes.data_as(I), len(atoms))
        lib.ref_sgp_update_matrices_QR(gp)
        k = f"{tag}/"
        for f in ("Kuu", "Kuf", "y", "noise_vector", "alpha", "R_inv", "L_inv",
                  "hyperparameters"):
            out[k + f] = get(gp, f)
        lib.ref_sgp_compute_likelihood_stable(gp)
        for f in ("log_marginal_likelihood", "data_fit", "complexity_penalty"):
            out[k + "stable/" + f] = get(gp, f)
        out[k + "grad/value"] = np.array(lib.ref_sgp_compute_likelihood_gradient_stable(gp))
        out[k + "grad/likelihood_gradient"] = get(gp, "likelihood_gradient")
        test = structure(*sc["test"])
        for what in ("mean", "SOR", "DTC"):
            assert lib.ref_sgp_predict(gp, what.encode(), test) == 0
            out[k + f"predict/{what}/mean_efs"] = sget(test, "mean_efs")
            if what != "mean":
                out[k + f"predict/{what}/variance_efs"] = sget(test, "variance_efs")
        for ki in range(len(descs)):
            n = lib.ref_sgp_cluster_uncertainties(gp, test, ki, None)
            u = np.zeros(n)
            lib.ref_sgp_cluster_uncertainties(gp, test, ki, u.ctypes.data)
            out[k + f"cluster_uncertainties/{ki}"] = u
            out[k + f"mapping/{ki}"] = coeffs(lib.ref_sgp_mapping_coefficients, gp, ki)
            if power == 1.0:
                out[k + f"varmap/{ki}"] = coeffs(lib.ref_sgp_varmap_coefficients, gp, ki)
        # new hyperparameters: each kernel's sigma and the noises changed
        h2 = arr([s_ * 1.25 for s_ in sig] + [1.3, 1.7, 2.6])
        lib.ref_sgp_set_hyperparameters(gp, h2.ctypes.data_as(D), len(h2))
        out[k + "set_hyps/hyps"] = h2
        out[k + "set_hyps/alpha"] = get(gp, "alpha")
        out[k + "set_hyps/grad/value"] = np.array(
            lib.ref_sgp_compute_likelihood_gradient_stable(gp))
        out[k + "set_hyps/grad/likelihood_gradient"] = get(gp, "likelihood_gradient")
        lib.ref_sgp_structure_free(test)
        for s in strucs:
            lib.ref_sgp_structure_free(s)
        lib.ref_sgp_free(gp)
        for (kind, _), d in zip(sc["descs"], descs):
            (lib.ref_b2_free if kind == "B2" else lib.ref_b3_free)(d)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "sgp_golden.npz"), **out)
    print("wrote tests/golden/sgp_golden.npz")


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("FLARE_PP_REFERENCE", "/root/reference")
    subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh"), ref_root],
                   check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libflare_ref.so"))
    D = ctypes.POINTER(ctypes.c_double)
    cd = ctypes.c_double
    rng = np.random.default_rng(20261203)
    out = {}
    # real harmonics
    lmax = 10
    H = (lmax + 1) ** 2
    vecs = rng.normal(size=(64, 3)) * rng.uniform(0.3, 6.0, size=(64, 1))
    vecs[0] = [0.0, 0.0, 1.7]        # on the z axis
    vecs[1] = [2.16, 7.12, -3.14]    # the vector of ctests/test_y_grad.cpp
    Ys = np.zeros((4, len(vecs), H))
    for i, v in enumerate(vecs):
        bufs = [np.zeros(H) for _ in range(4)]
        lib.ref_get_Y(cd(v[0]), cd(v[1]), cd(v[2]), lmax,
                      *[b.ctypes.data_as(D) for b in bufs])
        for k in range(4):
            Ys[k, i] = bufs[k]
    out["Y_vecs"] = vecs
    out["Y"], out["Yx"], out["Yy"], out["Yz"] = Ys
    # complex harmonics (re, im interleaved)
    lc = 6
    Hc = (lc + 1) ** 2
    Yc = np.zeros((4, len(vecs), 2 * Hc))
    for i, v in enumerate(vecs):
        bufs = [np.zeros(2 * Hc) for _ in range(4)]
        lib.ref_get_complex_Y(cd(v[0]), cd(v[1]), cd(v[2]), lc,
                              *[b.ctypes.data_as(D) for b in bufs])
        for k in range(4):
            Yc[k, i] = bufs[k]
    out["Yc"], out["Ycx"], out["Ycy"], out["Ycz"] = Yc
    # radial basis x cutoff
    N, rc, r1 = 12, 5.5, 0.0
    dirs = rng.normal(size=(64, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rs = np.concatenate([rng.uniform(0.5, rc, 60), [rc, rc - 1e-9, 1e-3, rc + 0.1]])
    pts = dirs * rs[:, None]
    out["rad_pts"] = pts
    for cut in ("quadratic", "cosine"):
        G = np.zeros((4, len(pts), N))
        for i, p in enumerate(pts):
            bufs = [np.zeros(N) for _ in range(4)]
            r = float(np.linalg.norm(p))
            rcv = lib.ref_calculate_radial(b"chebyshev", cut.encode(), cd(p[0]),
                                           cd(p[1]), cd(p[2]), cd(r), cd(rc), N,
                                           cd(r1), *[b.ctypes.data_as(D) for b in bufs])
            assert rcv == 0
            for k in range(4):
                G[k, i] = bufs[k]
        out[f"g_{cut}"] = G
    out["rad_N"], out["rad_rc"], out["rad_r1"] = N, rc, r1
    # Wigner 3j tables of B3
    for lmax in range(5):
        n = (lmax + 1) ** 6
        tab = np.zeros(n)
        assert lib.ref_compute_coeffs(lmax, tab.ctypes.data_as(D), ctypes.c_long(n)) == 0
        nz = np.nonzero(tab)[0]
        out[f"w3j_{lmax}_idx"] = nz.astype(np.int32)
        out[f"w3j_{lmax}_val"] = tab[nz]
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "l0_golden.npz"), **out)
    print("wrote tests/golden/l0_golden.npz")
    beta_form_golden(lib)
    struc_kernel_golden(lib)
    b3_golden(lib)
    sgp_golden(lib)


if __name__ == "__main__":
    main(*sys.argv[1:])
