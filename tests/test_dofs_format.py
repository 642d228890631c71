"""Restart files: CarrierPair::print_dofs / read_dofs (CarrierPair.cpp:89-121)
write each carrier's solution with deal.II's Vector::block_write layout --
the size in ASCII decimal, a newline, '[', the raw doubles, ']'.  The Python
mirror and the C++ drop-in header must both write and read that layout."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from pecs_gb300.reference_api import CarrierPair, block_read, block_write

ROOT = Path(__file__).resolve().parents[1]


def test_python_block_layout_and_round_trip(tmp_path):
    v = np.array([1.0, -2.5, 3.25e-300, 7.0])
    p = tmp_path / "x.dofs"
    with open(p, "wb") as fh:
        block_write(fh, v)
    raw = p.read_bytes()
    assert raw[:3] == b"4\n[" and raw[-1:] == b"]" and len(raw) == 3 + 32 + 1
    assert np.array_equal(np.frombuffer(raw[3:-1], dtype=np.float64), v)
    with open(p, "rb") as fh:
        assert np.array_equal(block_read(fh), v)
    cp = CarrierPair()
    cp.carrier_1.name, cp.carrier_2.name = "Electrons", "Holes"
    cp.carrier_1.solution = np.arange(5.0)
    cp.carrier_2.solution = -np.arange(3.0)
    cp.print_dofs(str(tmp_path))
    back = CarrierPair()
    back.carrier_1.name, back.carrier_2.name = "Electrons", "Holes"
    back.read_dofs(str(tmp_path))
    assert np.array_equal(back.carrier_1.solution, cp.carrier_1.solution)
    assert np.array_equal(back.carrier_2.solution, cp.carrier_2.solution)


def test_cpp_dropin_reads_python_files_and_writes_the_same_bytes(tmp_path, pecs_lib):
    src = tmp_path / "dofs_rt.cpp"
    src.write_text('''
#include "pecs_dropin.hpp"
int main() {
  pecs_dropin::ChargeCarrierSpace::CarrierPair cp;
  cp.carrier_1.name = "Electrons"; cp.carrier_2.name = "Holes";
  cp.read_dofs();
  cp.carrier_1.name = "E2"; cp.carrier_2.name = "H2";
  cp.print_dofs();
  return 0;
}
''')
    exe = tmp_path / "dofs_rt"
    from pecs_gb300._build import LIB
    libdir = LIB.parent
    r = subprocess.run(["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                        f"-L{libdir}", "-lpecs_gb300", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    cp = CarrierPair()
    cp.carrier_1.name, cp.carrier_2.name = "Electrons", "Holes"
    cp.carrier_1.solution = np.linspace(-1, 1, 7)
    cp.carrier_2.solution = np.array([np.pi])
    cp.print_dofs(str(tmp_path))
    subprocess.run([str(exe)], cwd=tmp_path, check=True)
    assert (tmp_path / "E2.dofs").read_bytes() == (tmp_path / "Electrons.dofs").read_bytes()
    assert (tmp_path / "H2.dofs").read_bytes() == (tmp_path / "Holes.dofs").read_bytes()
