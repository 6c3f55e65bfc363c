"""GPU path against the oracle, through the C ABI (ctypes) and its Python face.

Bit-exact: neighbor lists (counts, order, FP64 geometry).
FP64 path: descriptors, stored derivatives, envs_struc, predict_mean/SOR,
mapped beta: relative 1e-9 or tighter.
Mixed path: energy within 1e-6 eV/atom and forces within 1e-4 eV/A of the
FP64 oracle (the gates of the mixed-precision form); stress reported.
"""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle import predict as opred
from oracle.b2 import B2 as OB2, ClusterDescriptor as OCD
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from tests import fixtures

pytestmark = pytest.mark.gpu

E_GATE = 1e-6   # eV / atom
F_GATE = 1e-4   # eV / A


def _cases():
    rng = np.random.default_rng(11)
    out = []
    cell, sp, pos = synth.fcc_al_108(101, 0)
    out.append(("fcc108", cell, sp, pos, 5.0))
    tri = np.array([[5.0, 0.3, 0.1], [-0.4, 4.6, 0.2], [0.3, 0.5, 4.9]])
    out.append(("triclinic_sweep2", tri, rng.integers(0, 2, 9),
                rng.uniform(-3, 8, size=(9, 3)), 6.5))
    out.append(("single_atom", np.eye(3) * 3.1, np.array([0]),
                np.array([[0.2, 0.3, 0.4]]), 5.0))
    cell, sp, pos = synth.bcc_alloy((10, 10, 10), 202)
    out.append(("bcc2000", cell, sp, pos, 5.5))
    # ~320 neighbors per atom: more than the one-pass build's 256-key slab,
    # so the list comes from the two-pass (count / fill / sort) build
    dense = np.array([[0.0, 0.0, 0.0], [1.5, 1.5, 0.0], [1.5, 0.0, 1.5], [0.0, 1.5, 1.5]])
    out.append(("dense_two_pass", np.eye(3) * 3.0, np.array([0, 1, 0, 1]),
                dense + rng.uniform(-0.05, 0.05, size=(4, 3)), 8.0))
    return out


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_neighbor_list_bit_exact(gpu_lib, case):
    name, cell, sp, pos, rc = case
    o = OStructure(cell, sp, pos, rc)
    g = fg.Structure(cell, sp, pos, rc)
    assert g.sweep == o.sweep
    np.testing.assert_array_equal(g.neighbor_count, o.neighbor_count)
    np.testing.assert_array_equal(g.cumulative_neighbor_count, o.cumulative_neighbor_count)
    np.testing.assert_array_equal(g.structure_indices, o.structure_indices)
    np.testing.assert_array_equal(g.neighbor_species, o.neighbor_species)
    np.testing.assert_array_equal(g.relative_positions, o.relative_positions)
    np.testing.assert_array_equal(g.wrapped_positions, o.wrapped_positions)


def test_empty_structure(gpu_lib):
    g = fg.Structure(np.eye(3) * 5, np.zeros(0, int), np.zeros((0, 3)), 4.0)
    assert g.n_neighbors == 0 and len(g.neighbor_count) == 0


def _two_species_case():
    rng = np.random.default_rng(5)
    cell = np.array([[7.5, 0.2, 0.0], [0.3, 7.0, 0.1], [0.0, -0.4, 7.7]])
    pos = rng.uniform(0, 7, size=(20, 3))
    sp = rng.integers(0, 2, size=20)
    cut = np.array([[4.2, 3.6], [3.6, 4.0]])
    return cell, sp, pos, cut


def test_descriptors_fp64_and_stored_derivatives(gpu_lib):
    cell, sp, pos, cut = _two_species_case()
    rc = 4.2
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 4, 3], cut)
    gb = fg.B2("chebyshev", "quadratic", [0, rc], [], [2, 4, 3], cut)
    od = OStructure(cell, sp, pos, rc, [ob]).descriptors[0]
    gd = fg.Structure(cell, sp, pos, rc, [gb]).descriptors[0]
    for s in range(2):
        np.testing.assert_array_equal(gd.atom_indices[s], od.atom_indices[s])
        np.testing.assert_array_equal(gd.neighbor_counts[s], od.neighbor_counts[s])
        np.testing.assert_array_equal(gd.neighbor_indices[s], od.neighbor_indices[s])
        np.testing.assert_array_equal(gd.neighbor_coordinates[s], od.neighbor_coordinates[s])
        sc = np.abs(od.descriptors[s]).max()
        np.testing.assert_allclose(gd.descriptors[s], od.descriptors[s], rtol=0,
                                   atol=1e-12 * sc)
        np.testing.assert_allclose(gd.descriptor_norms[s], od.descriptor_norms[s],
                                   rtol=1e-12)
        fs = np.abs(od.descriptor_force_dervs[s]).max()
        np.testing.assert_allclose(gd.descriptor_force_dervs[s],
                                   od.descriptor_force_dervs[s], rtol=0, atol=1e-11 * fs)
        ds = np.abs(od.descriptor_force_dots[s]).max()
        np.testing.assert_allclose(gd.descriptor_force_dots[s],
                                   od.descriptor_force_dots[s], rtol=0, atol=1e-11 * ds)


@pytest.mark.parametrize("power", [1, 2])
def test_envs_struc_fp64(gpu_lib, power):
    cell, sp, pos, cut = _two_species_case()
    rc = 4.2
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 4, 3], cut)
    gb = fg.B2("chebyshev", "quadratic", [0, rc], [], [2, 4, 3], cut)
    od = OStructure(cell, sp, pos, rc, [ob]).descriptors[0]
    gs = fg.Structure(cell, sp, pos, rc, [gb])
    envs = OCD(od)
    K_ref = ONDP(1.7, power).envs_struc(envs, od)
    genvs = fg.ClusterDescriptor(gs.descriptors[0])
    K = fg.NormalizedDotProduct(1.7, power).envs_struc(genvs, gs.descriptors[0])
    np.testing.assert_allclose(K, K_ref, rtol=0, atol=1e-10 * np.abs(K_ref).max())


@pytest.fixture(scope="module")
def c1():
    m = fixtures.config1_model()
    gp = m["gp"]
    ggp, gb2 = fixtures.to_gpu_model((1, 8, 3, 5.0), gp.sparse_descriptors[0], gp.alpha,
                                     2.0, 2, gp.R_inv)
    cell, sp, pos = synth.fcc_al_108(101, 5)
    os_ = OStructure(cell, sp, pos, 5.0, [m["b2"]])
    gp.predict_SOR(os_)
    gs = fg.Structure(cell, sp, pos, 5.0)
    return dict(m=m, ggp=ggp, gb2=gb2, os=os_, gs=gs, cell=cell, sp=sp, pos=pos)


def test_predict_mean_and_sor_fp64(gpu_lib, c1):
    ggp, gs, os_ = c1["ggp"], c1["gs"], c1["os"]
    ggp.predict_mean(gs)
    scale = np.abs(os_.mean_efs).max()
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-10 * scale)
    ggp.predict_SOR(gs)
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-10 * scale)
    # the energy variance is a difference of O(1e4) terms that ends at O(1e-5):
    # FP64 conditioning limits its agreement to ~1e-7 relative
    np.testing.assert_allclose(gs.variance_efs[0], os_.variance_efs[0], rtol=1e-5)
    np.testing.assert_allclose(gs.variance_efs[1:], os_.variance_efs[1:], rtol=1e-7,
                               atol=1e-9 * np.abs(os_.variance_efs).max())


def test_mapped_fp64_and_mixed_config1(gpu_lib, c1):
    m, ggp, gs, os_ = c1["m"], c1["ggp"], c1["gs"], c1["os"]
    gp = m["gp"]
    beta_ref = m["kernel"].compute_map_coeff_pow2(gp.sparse_descriptors[0], gp.alpha)
    e, f, s = ggp.predict_mapped(gs, "fp64")
    np.testing.assert_allclose(ggp.mapping_coefficients, beta_ref, rtol=0,
                               atol=1e-10 * np.abs(beta_ref).max())
    ref_e, ref_f, ref_s = os_.mean_efs[0], os_.mean_efs[1:-6], os_.mean_efs[-6:]
    assert abs(e - ref_e) < 1e-9 * abs(ref_e)
    np.testing.assert_allclose(f.ravel(), ref_f, rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, ref_s, rtol=0, atol=1e-10)
    e, f, s = ggp.predict_mapped(gs, "mixed")
    n = gs.noa
    assert abs(e - ref_e) / n < E_GATE
    assert np.abs(f.ravel() - ref_f).max() < F_GATE
    assert np.abs(s - ref_s).max() < 1e-5


@pytest.fixture(scope="module")
def c2():
    """Two-species BCC alloy at 2000 atoms, N=10, lmax=4, rc=5.5, 400 sparse
    environments fitted to Lennard-Jones site energies."""
    rc = 5.5
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 10, 4])
    frames = [synth.bcc_alloy((6, 6, 6), 202 + 10 * k) for k in range(1, 3)]
    fit = fixtures.site_energy_model(ob, frames, 200, sigma=2.0, power=2)
    ggp, gb2 = fixtures.to_gpu_model((2, 10, 4, rc), fit["sparse"], fit["alpha"], 2.0, 2)
    cell, sp, pos = synth.bcc_alloy((10, 10, 10), 202)
    os_ = OStructure(cell, sp, pos, rc)
    st = fixtures.settings(2, 10, 4, rc)
    beta = ONDP(2.0, 2).compute_map_coeff_pow2(fit["sparse"], fit["alpha"])
    B = opred.unpack_beta(beta, ob_n(ob))
    ref = opred.beta_form(os_, st, B)
    gs = fg.Structure(cell, sp, pos, rc)
    return dict(ggp=ggp, gs=gs, ref=ref, noa=len(sp))


def ob_n(ob):
    ns, N, lmax = ob.descriptor_settings
    nr = ns * N
    return nr * (nr + 1) // 2 * (lmax + 1)


def test_mapped_config2_fp64(gpu_lib, c2):
    e, f, s = c2["ggp"].predict_mapped(c2["gs"], "fp64")
    ref = c2["ref"]
    assert abs(e - ref["energy"]) < 1e-9 * abs(ref["energy"])
    np.testing.assert_allclose(f, ref["forces"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(s, ref["stress"], rtol=0, atol=1e-9)


def test_mapped_config2_mixed_gates(gpu_lib, c2):
    e, f, s, ae = c2["ggp"].predict_mapped(c2["gs"], "mixed", atom_energies=True)
    ref = c2["ref"]
    n = c2["noa"]
    err_e = abs(e - ref["energy"]) / n
    err_f = np.abs(f - ref["forces"]).max()
    print(f"mixed config2: energy err/atom {err_e:.3e}, max force err {err_f:.3e}, "
          f"max atom-energy err {np.abs(ae - ref['atom_energies']).max():.3e}, "
          f"stress err {np.abs(s - ref['stress']).max():.3e}")
    assert err_e < E_GATE
    assert err_f < F_GATE


@pytest.fixture(scope="module")
def c3s():
    """The shape of the 32k-atom workload at 2000 atoms: two-species BCC
    alloy (10 x 10 x 10 cells, a = 3.0 A, 0.08 A rattle), chebyshev N = 12,
    lmax = 4, rc = 5.5 A, 600 sparse environments per species fitted to
    Lennard-Jones site energies.  These settings run the library's compiled
    N = 12, lmax = 4, two-species kernels (the headline's).  The reference
    values come from the C oracle (oracle/c/flare_oracle.c), whose pair-style
    math is pinned to the reference's lammps_descriptor.cpp."""
    from oracle import cfast
    rc = 5.5
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 12, 4])
    ob.store_dervs = False
    frames = [synth.bcc_alloy((8, 8, 8), 303 + 10 * k) for k in range(1, 3)]
    fit = fixtures.site_energy_model(ob, frames, 600, sigma=2.0, power=2)
    ggp, gb2 = fixtures.to_gpu_model((2, 12, 4, rc), fit["sparse"], fit["alpha"], 2.0, 2)
    cell, sp, pos = synth.bcc_alloy((10, 10, 10), 303)
    st = fixtures.settings(2, 12, 4, rc)
    beta = ONDP(2.0, 2).compute_map_coeff_pow2(fit["sparse"], fit["alpha"])
    B = opred.unpack_beta(beta, ob_n(ob))
    ref = cfast.beta_form(cell, sp, pos, st, B)
    gs = fg.Structure(cell, sp, pos, rc)
    return dict(ggp=ggp, gs=gs, ref=ref, noa=len(sp), cell=cell, sp=sp, pos=pos)


def test_mapped_headline_shape_fp64_vs_oracle(gpu_lib, c3s):
    e, f, s, ae = c3s["ggp"].predict_mapped(c3s["gs"], "fp64", atom_energies=True)
    ref = c3s["ref"]
    assert abs(e - ref["energy"]) < 1e-9 * np.abs(ref["atom_energies"]).sum()
    np.testing.assert_allclose(ae, ref["atom_energies"], rtol=0,
                               atol=1e-9 * np.abs(ref["atom_energies"]).max())
    np.testing.assert_allclose(f, ref["forces"], rtol=0, atol=1e-9 * np.abs(ref["forces"]).max())
    np.testing.assert_allclose(s, ref["stress"], rtol=0, atol=1e-9 * np.abs(ref["stress"]).max())


def test_mapped_headline_shape_mixed_gates_vs_oracle(gpu_lib, c3s):
    """Mixed form (FP32 descriptors, split-fp16 tcgen05 contraction) within the
    gates against the FP64 oracle: 1e-6 eV/atom, 1e-4 eV/A."""
    e, f, s, ae = c3s["ggp"].predict_mapped(c3s["gs"], "mixed", atom_energies=True)
    ref = c3s["ref"]
    n = c3s["noa"]
    err_e = abs(e - ref["energy"]) / n
    err_f = np.abs(f - ref["forces"]).max()
    err_s = np.abs(s - ref["stress"]).max()
    print(f"mixed N=12 lmax=4 at 2000 atoms: energy err/atom {err_e:.3e}, max force err "
          f"{err_f:.3e}, stress err {err_s:.3e}")
    assert err_e < E_GATE
    assert err_f < F_GATE
    assert err_s < 1e-5


def test_pair_compute_matches_mapped(gpu_lib, c1, tmp_path):
    from flare_pp_gb300.potential import write_potential
    m, ggp = c1["m"], c1["ggp"]
    ggp.predict_mapped(c1["gs"], "fp64")
    fn = tmp_path / "Al.txt"
    write_potential(fn, ggp.mapping_coefficients, 2, 1, 8, 3, np.array([[5.0]]))
    pair = fg.PairFLARE(str(fn))
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(c1["cell"], c1["sp"], c1["pos"], 5.0)
    for prec, tol in (("fp64", 1e-9), ("mixed", F_GATE)):
        f, e, vir, ea = pair.compute(x, t, il, nn, nb, precision=prec, eatom=True)
        F = np.zeros((c1["gs"].noa, 3))
        np.add.at(F, owner, f)
        ref = c1["os"].mean_efs
        n = c1["gs"].noa
        assert abs(e - ref[0]) / n < (1e-10 if prec == "fp64" else E_GATE)
        assert np.abs(F.ravel() - ref[1:-6]).max() < tol
        assert abs(ea.sum() - e) < 1e-9 * abs(e)
        # virial (xx, yy, zz, xy, xz, yz) = V * flare stress (xx, xy, xz, yy, yz, zz)
        V = abs(np.linalg.det(c1["cell"]))
        st = ref[-6:]
        np.testing.assert_allclose(vir, V * st[[0, 3, 5, 1, 2, 4]], rtol=0,
                                   atol=(1e-8 if prec == "fp64" else 1e-3))


def test_device_errors_are_reported(gpu_lib, c1):
    from flare_pp_gb300._lib import FlareGpuError
    cell, sp, pos = c1["cell"], c1["sp"].copy(), c1["pos"]
    sp[3] = 1  # species outside the model's single species
    gs = fg.Structure(cell, sp, pos, 5.0)
    with pytest.raises(FlareGpuError):
        c1["ggp"].predict_mapped(gs, "mixed")


def test_autograd_forces_and_stress_finite_differences(gpu_lib, c2):
    """Forces from the adjoint (torch.autograd) against central differences
    (h = 1e-4 A) on 20 seeded atoms, and the virial stress against strain
    differences, in the FP64 form (the mixed form is checked against the
    FP64 oracle above)."""
    import torch
    from flare_pp_gb300.autograd import FlareEnergy, energy_forces_stress
    gp, gs = c2["ggp"], c2["gs"]
    pos0 = torch.tensor(gs.positions, dtype=torch.float64, device="cuda")
    e, F, S = energy_forces_stress(gp, gs, pos0, "fp64")
    np.testing.assert_allclose(F.cpu().numpy(), c2["ref"]["forces"], rtol=0, atol=1e-8)
    rng = np.random.default_rng(20)
    h = 1e-4
    for a in rng.choice(gs.noa, 20, replace=False):
        for comp in range(3):
            pp, pm = pos0.clone(), pos0.clone()
            pp[a, comp] += h
            pm[a, comp] -= h
            ep = FlareEnergy.apply(pp, gp, gs, "fp64").item()
            em = FlareEnergy.apply(pm, gp, gs, "fp64").item()
            fd = -(ep - em) / (2 * h)
            assert abs(fd - F[a, comp].item()) < 1e-5 + 1e-6 * abs(fd)
    # stress = -(1/V) dE/d(strain) with x -> (1 + eps) x and cell -> cell (1 + eps)
    FlareEnergy.apply(pos0, gp, gs, "fp64")
    cell0 = np.array(gs.cell)
    V = abs(np.linalg.det(cell0))
    idx = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 1): 3, (1, 2): 4, (2, 2): 5}
    for (i, j), k in idx.items():
        vals = []
        for sgn in (1, -1):
            eps = np.zeros((3, 3))
            eps[i, j] += sgn * h / 2
            eps[j, i] += sgn * h / 2
            Fm = np.eye(3) + eps
            st = fg.Structure(cell0 @ Fm, gs.species, gs.positions @ Fm, 5.5)
            vals.append(c2["ggp"].predict_mapped(st, "fp64")[0])
        fd = -(vals[0] - vals[1]) / (2 * h) / V
        assert abs(fd - S[k].item()) < 1e-6 + 1e-5 * abs(fd), (i, j, fd, S[k].item())


def test_training_solve_matches_oracle(gpu_lib):
    """SparseGP training on the GPU (B2 with stored derivatives, envs_envs,
    envs_struc columns, cuSOLVER QR) against the oracle's update_matrices_QR
    on the config-1 training set (E, F, S labels)."""
    m = fixtures.config1_model(n_frames=3, n_sparse=30)
    ogp = m["gp"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.0], [], [1, 8, 3])
    gp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 0.001, 0.05, 0.006)
    frames = []
    for k, of in enumerate(ogp.training_structures):
        s = fg.Structure(of.cell, of.species, of.positions, 5.0, [b2])
        s.energy, s.forces, s.stresses = of.energy, of.forces, of.stresses
        gp.add_training_structure(s)
        frames.append(s)
    for k, atoms in enumerate(ogp.sparse_indices[0]):
        gp.add_specific_environments(frames[k], atoms)
    gp.update_matrices_QR()
    np.testing.assert_allclose(gp.Kuu, ogp.Kuu_mat, rtol=0, atol=1e-10 * np.abs(ogp.Kuu_mat).max())
    np.testing.assert_allclose(gp.Kuf, ogp.Kuf_mat, rtol=0, atol=1e-9 * np.abs(ogp.Kuf_mat).max())
    # alpha carries the conditioning of the solve: compare predictions and
    # alpha relative to its scale
    np.testing.assert_allclose(gp.alpha, ogp.alpha, rtol=0, atol=1e-5 * np.abs(ogp.alpha).max())
    cell, sp, pos = synth.fcc_al_108(101, 5)
    os_ = OStructure(cell, sp, pos, 5.0, [m["b2"]])
    ogp.predict_SOR(os_)
    gs = fg.Structure(cell, sp, pos, 5.0)
    gp.predict_SOR(gs)
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-6)
    np.testing.assert_allclose(gs.variance_efs[1:], os_.variance_efs[1:], rtol=1e-4,
                               atol=1e-8)


def test_cpp_pair_style_core_matches_oracle(gpu_lib, c3s, tmp_path):
    """The C++ pair-style core (flare_pp_gb300/lammps/pair_flare_gb300.cpp),
    linked with -lflare_pp_gb300 and driven by a LAMMPS-shaped harness
    (double** x / f, 1-based types, full neighbor list with ghost atoms),
    against the FP64 oracle: FP64 to 1e-9, mixed within the gates."""
    from flare_pp_gb300.potential import write_potential
    exe = fixtures.build_pair_harness(tmp_path)
    ggp = c3s["ggp"]
    ggp._ensure_mapped()
    pot = tmp_path / "alloy.txt"
    write_potential(pot, ggp.mapping_coefficients, 2, 2, 12, 4, np.full((2, 2), 5.5))
    gs = c3s["gs"]
    cell, sp, pos = c3s["cell"], c3s["sp"], c3s["pos"]
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(cell, sp, pos, 5.5)
    case = tmp_path / "case.txt"
    fixtures.write_case(case, x, t, il, nn, nb)
    ref = c3s["ref"]
    V = abs(np.linalg.det(cell))
    n = gs.noa
    for prec in ("fp64", "mixed"):
        out = tmp_path / f"out_{prec}.txt"
        import subprocess
        subprocess.run([exe, str(pot), str(case), str(out), prec], check=True)
        e, vir, f, ea = fixtures.read_harness_output(out, len(x))
        F = np.zeros((n, 3))
        np.add.at(F, owner, f)
        st = ref["stress"]
        vir_ref = V * st[[0, 3, 5, 1, 2, 4]]
        if prec == "fp64":
            assert abs(e - ref["energy"]) < 1e-9 * np.abs(ref["atom_energies"]).sum()
            np.testing.assert_allclose(F, ref["forces"], rtol=0,
                                       atol=1e-9 * np.abs(ref["forces"]).max())
            np.testing.assert_allclose(vir, vir_ref, rtol=0, atol=1e-9 * np.abs(vir_ref).max())
        else:
            assert abs(e - ref["energy"]) / n < E_GATE
            assert np.abs(F - ref["forces"]).max() < F_GATE
        assert abs(ea[:n].sum() - e) < 1e-9 * max(1.0, abs(e))


def test_pair_compute_memory_batches(gpu_lib, c3s, tmp_path):
    """Under a device-memory cap (the Kokkos pair style's MAXMEM) the pair
    style evaluates the atoms in batches; the results equal the one-batch
    call (up to the order of the force scatter's additions)."""
    from flare_pp_gb300.potential import write_potential
    ggp = c3s["ggp"]
    ggp._ensure_mapped()
    pot = tmp_path / "alloy.txt"
    write_potential(pot, ggp.mapping_coefficients, 2, 2, 12, 4, np.full((2, 2), 5.5))
    pair = fg.PairFLARE(str(pot))
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(c3s["cell"], c3s["sp"], c3s["pos"], 5.5)
    beta_mem = 2 * 1500 * 1500 * 8.0
    for prec in ("fp64", "mixed"):
        pair.set_max_memory(0)
        f1, e1, v1, a1 = pair.compute(x, t, il, nn, nb, precision=prec, eatom=True)
        assert pair.last_batches == 1
        pair.set_max_memory(beta_mem + 25e6)
        f2, e2, v2, a2 = pair.compute(x, t, il, nn, nb, precision=prec, eatom=True)
        assert pair.last_batches >= 2
        assert abs(e2 - e1) <= 1e-12 * np.abs(a1).sum()
        np.testing.assert_allclose(a2, a1, rtol=0, atol=1e-12 * np.abs(a1).max())
        np.testing.assert_allclose(f2, f1, rtol=0, atol=1e-11 * np.abs(f1).max())
        np.testing.assert_allclose(v2, v1, rtol=0, atol=1e-11 * np.abs(v1).max())
    pair.set_max_memory(1.0)
    from flare_pp_gb300._lib import FlareGpuError
    with pytest.raises(FlareGpuError):
        pair.compute(x, t, il, nn, nb, precision="fp64")
