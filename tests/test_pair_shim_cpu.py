"""The C++ pair-style core (flare_pp_gb300/lammps/pair_flare_gb300.cpp)
compiles and links against libflare_pp_gb300.so from C++, and parses the
potential file's two layouts with no device calls (tests/cpp/pair_harness.cpp
--parse-only)."""
import shutil
import subprocess

import numpy as np
import pytest

from flare_pp_gb300.potential import write_potential
from tests import fixtures


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    return fixtures.build_pair_harness(tmp_path_factory.mktemp("harness"))


def _fields(out):
    w = out.split()
    return {w[i]: w[i + 1] for i in range(0, len(w), 2)}


def test_parses_current_layout(harness, tmp_path):
    fn = tmp_path / "pot.txt"
    nd = 4 * 5 // 2 * 3                       # n_rad = 4: 10 radial pairs x 3 l
    beta = np.arange(2 * nd * (nd + 1) // 2, dtype=float).reshape(2, -1) * 1e-4
    write_potential(fn, beta, 2, 2, 2, 2, np.array([[4.5, 4.0], [4.0, 4.2]]))
    r = subprocess.run([harness, "--parse-only", str(fn)], capture_output=True, text=True,
                       check=True)
    f = _fields(r.stdout)
    assert f["power"] == "2" and f["n_species"] == "2" and f["n_max"] == "2"
    assert f["l_max"] == "2" and f["legacy"] == "0" and float(f["cutoff"]) == 4.5
    assert int(f["n_beta"]) == beta.size and int(f["beta_size"]) == nd * (nd + 1) // 2


def test_parses_older_layout(harness, tmp_path):
    fn = tmp_path / "old.txt"
    with open(fn, "w") as f:
        f.write("DATE: x CONTRIBUTOR: y\nchebyshev\n2 1 1 21\ncosine\n4.50\n")
        for s in range(2):
            vals = np.arange(21) * 1e-3 + s
            for k in range(0, 21, 5):
                f.write(" ".join(f"{v:.16e}" for v in vals[k:k + 5]) + "\n")
    r = subprocess.run([harness, "--parse-only", str(fn)], capture_output=True, text=True,
                       check=True)
    f = _fields(r.stdout)
    assert f["power"] == "2" and f["legacy"] == "1" and f["cutoff_function"] == "cosine"
    assert int(f["n_beta"]) == 42 and float(f["cutoff"]) == 4.5


def test_rejects_a_mismatched_beta_size(harness, tmp_path):
    fn = tmp_path / "bad.txt"
    with open(fn, "w") as f:
        f.write("DATE: x\n2\nchebyshev\n1 2 1 7\nquadratic\n4.0\n" + "0.1 " * 7 + "\n")
    r = subprocess.run([harness, "--parse-only", str(fn)], capture_output=True, text=True)
    assert r.returncode == 1 and "Beta size" in r.stderr
