"""The C-ABI library loads and exports every function include/*.h declares."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b([a-z_0-9]+)\s*\(", text):
            name = m.group(1)
            if name.startswith("pecs_") and not name.endswith("_t"):
                names.add(name)
    return sorted(names)


def test_headers_declare_functions():
    names = declared_functions()
    assert "pecs_create" in names and "pecs_lu_factor" in names and "pecs_lu_host_apply" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(pecs_lib):
    missing = [n for n in declared_functions() if not hasattr(pecs_lib, n)]
    assert not missing, missing


def test_no_device_is_a_clean_error(pecs_lib):
    import pecs_gb300 as pg
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg.PecsError) as ei:
        pg.Context(pg.half_cell(n_refine=2))
    assert ei.value.code == pg._ffi.PECS_E_NODEVICE


def test_sweep_stream_rejects_points_with_other_matrices(pecs_lib):
    """Every streamed point must share the context's fixed matrices; the
    check runs before any device work (host-only context here)."""
    import pecs_gb300 as pg
    base = pg.half_cell(n_refine=2)
    ctx = pg.Context([base], host_setup_only=True)
    with pytest.raises(pg.PecsError, match="dt"):
        ctx.sweep_stream([base, base.copy(dt=2e-3)], 10, 1e-6)
    with pytest.raises(pg.PecsError, match="host_setup_only"):
        ctx.sweep_stream([base, base.copy(phi_app=0.3)], 10, 1e-6)


@pytest.mark.parametrize("full", [True, False])
def test_boundary_layout_abi_matches_python(pecs_lib, full):
    """pecs_apply_boundary_layout (for C++ callers) and
    pecs_gb300.boundary_layout set the same ids; other fields are untouched."""
    import ctypes as C

    import pecs_gb300 as pg
    base = pg.half_cell(n_refine=2) if full else pg.pn_junction()
    for insulated in (False, True):
        for schottky in (False, True):
            c = base.to_c()
            assert pecs_lib.pecs_apply_boundary_layout(C.byref(c), int(insulated), int(schottky)) == 0
            ref = pg.boundary_layout(base, insulated=insulated, schottky=schottky)
            for f in ("bc_semi", "bc_elec", "bc_poisson", "bc_poisson_elec"):
                assert tuple(getattr(c, f)) == tuple(getattr(ref, f)), (f, insulated, schottky)
            assert c.nx_semi == base.nx_semi and c.phi_app == base.phi_app
    assert pecs_lib.pecs_apply_boundary_layout(None, 0, 0) != 0


def test_headers_are_c99(pecs_lib, tmp_path):
    """include/pecs.h and pecs_debug.h compile as strict C99 and a C program
    links against the library (the ABI is plain C: no C++ types cross it)."""
    import subprocess
    from pecs_gb300._build import LIB
    src = tmp_path / "abi.c"
    src.write_text('#include <string.h>\n#include "pecs.h"\n#include "pecs_debug.h"\n'
                   "int main(void) {\n"
                   "  pecs_params p; pecs_options o;\n"
                   "  memset(&p, 0, sizeof p); p.full_system = 1;\n"
                   "  pecs_default_options(&o);\n"
                   "  if (pecs_apply_boundary_layout(&p, 1, 1) != 0) return 1;\n"
                   "  return p.bc_poisson_elec[3] == 3 && p.bc_semi[0] == 2 ? 0 : 2;\n"
                   "}\n")
    exe = tmp_path / "abi"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{LIB.parent}",
                        "-lpecs_gb300", f"-Wl,-rpath,{LIB.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0
