"""ctypes wrapper of the C oracle (oracle/c/flare_oracle.c).  Test
infrastructure only."""
import ctypes

import numpy as np

from .c.build import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.oracle_beta_form.restype = ctypes.c_int
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        _lib.oracle_beta_form.argtypes = [ci, vp, vp, vp, ci, ci, ci, cd, vp, vp, ci,
                                          vp, ci, ci, vp, vp, vp, vp]
        _lib.oracle_b3_beta_form.restype = ctypes.c_int
        _lib.oracle_b3_beta_form.argtypes = [ci, vp, vp, vp, ci, ci, ci, cd, cd, vp, ci,
                                             vp, ci, ci, vp, vp, vp, vp]
        _lib.oracle_b2_descriptors.restype = ctypes.c_int
        _lib.oracle_b2_descriptors.argtypes = [ci, vp, vp, vp, ci, ci, ci, cd, vp, ci, vp, vp]
        _lib.oracle_max_threads.restype = ctypes.c_int
    return _lib


def beta_form(cell, species, positions, settings, beta, power=2, atoms=None,
              n_threads=0):
    """Mapped-beta E/F/S (FP64) for B2, or B3 when settings["kind"] == "B3".
    beta: list of dense n_d x n_d (power 2) or vectors (power 1).  Returns dict(energy, forces, stress, atom_energies)."""
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    sp = np.ascontiguousarray(species, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    cut = np.ascontiguousarray(settings["cutoffs"], dtype=np.float64)
    B = np.ascontiguousarray(np.stack([np.asarray(b) for b in beta]), dtype=np.float64)
    noa = len(sp)
    F = np.zeros((noa, 3))
    S = np.zeros(6)
    ae = np.zeros(noa)
    e = ctypes.c_double()
    at = None if atoms is None else np.ascontiguousarray(atoms, dtype=np.int32)
    P = lambda a: None if a is None else a.ctypes.data
    if settings.get("kind", "B2") == "B3":
        rc = lib().oracle_b3_beta_form(
            noa, P(cell), P(sp), P(pos), settings["n_species"], settings["N"],
            settings["lmax"], ctypes.c_double(settings["r1"]),
            ctypes.c_double(settings["rcut"]), P(B), power, P(at),
            0 if at is None else len(at), n_threads, ctypes.byref(e), P(F), P(S), P(ae))
    else:
        rc = lib().oracle_beta_form(
            noa, P(cell), P(sp), P(pos), settings["n_species"], settings["N"],
            settings["lmax"], ctypes.c_double(settings["r1"]), P(cut), P(B), power,
            P(at), 0 if at is None else len(at), n_threads, ctypes.byref(e), P(F), P(S),
            P(ae))
    if rc != 0:
        raise RuntimeError(f"oracle_beta_form failed ({rc})")
    return dict(energy=e.value, forces=F, stress=S, atom_energies=ae)


def b2_descriptors(cell, species, positions, settings, n_threads=0):
    """B2 descriptors p (noa x n_d) and norms of every atom, FP64."""
    from .b2 import n_descriptors
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    sp = np.ascontiguousarray(species, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    cut = np.ascontiguousarray(settings["cutoffs"], dtype=np.float64)
    ns, N, lmax = settings["n_species"], settings["N"], settings["lmax"]
    noa = len(sp)
    p = np.zeros((noa, n_descriptors(ns, N, lmax)))
    nrm = np.zeros(noa)
    P = lambda a: a.ctypes.data
    rc = lib().oracle_b2_descriptors(noa, P(cell), P(sp), P(pos), ns, N, lmax,
                                     ctypes.c_double(settings["r1"]), P(cut), n_threads,
                                     P(p), P(nrm))
    if rc != 0:
        raise RuntimeError(f"oracle_b2_descriptors failed ({rc})")
    return p, nrm


def max_threads():
    return lib().oracle_max_threads()
