"""The C++ drop-in classes (include/pecs_dropin.hpp) driven as the reference's
SolarCellProblem drives its own (tests/dropin_check.cpp): LDG_System::LDG and
MixedPoisson::MixedFEM assemble the carrier, mass and mixed Poisson matrices
cell by cell through Assembly::AssemblyScratch / CopyData, and the results
must equal the library's own setup (CPU); Carrier::set_solver/solve and
PoissonData::set_solver/solve then solve on the GPU, checked against scipy."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CASES = [(1, 0), (2, 0), (1, 1), (2, 1)]


@pytest.fixture(scope="module")
def check_exe(pecs_lib, tmp_path_factory):
    from pecs_gb300._build import LIB
    libdir = LIB.parent
    exe = tmp_path_factory.mktemp("dropin") / "dropin_check"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "dropin_check.cpp"), "-o", str(exe), f"-L{libdir}",
                        "-lpecs_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    return exe


@pytest.mark.parametrize("degree,pairing", CASES, ids=[f"k{k}_pairing{p}" for k, p in CASES])
def test_dropin_assembly_equals_the_library_setup(check_exe, degree, pairing):
    r = subprocess.run([str(check_exe), "assemble", str(degree), str(pairing)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "assemble ok" in r.stdout


def _csr(d, stem):
    import scipy.sparse as sp
    rp = np.fromfile(d / f"{stem}_rowptr.bin", dtype=np.int32)
    ci = np.fromfile(d / f"{stem}_col.bin", dtype=np.int32)
    v = np.fromfile(d / f"{stem}_val.bin", dtype=np.float64)
    return sp.csr_matrix((v, ci, rp), shape=(len(rp) - 1, len(rp) - 1))


@pytest.mark.gpu
@pytest.mark.parametrize("degree,pairing", [(1, 0), (2, 1)], ids=["k1_pairing0", "k2_pairing1"])
def test_dropin_solvers_on_the_gpu_match_scipy(check_exe, tmp_path, degree, pairing):
    import scipy.sparse.linalg as spla
    r = subprocess.run([str(check_exe), "solve", str(degree), str(pairing), str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for stem in ("carrier", "poisson"):
        A = _csr(tmp_path, stem + "_A")
        b = np.fromfile(tmp_path / f"{stem}_b.bin")
        x = np.fromfile(tmp_path / f"{stem}_x.bin")
        ref = spla.spsolve(A.tocsc(), b)
        err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
        assert err < 1e-12, (stem, err)
