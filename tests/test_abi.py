"""The C ABI library: loads without a GPU, exports every declared symbol,
and its host-only mesh calls work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from picfoam_gb300 import abi, build, cases, native
from picfoam_gb300.simulation import Mesh, PicError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load()


def declared_symbols():
    """Every function declared by a header under include/."""
    syms = set()
    inc = os.path.join(ROOT, "include")
    for name in sorted(os.listdir(inc)):
        if not name.endswith(".h"):
            continue
        src = open(os.path.join(inc, name)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        syms.update(re.findall(r"\b(picgpu_[a-z0-9_]+)\s*\(", src))
    return sorted(syms)


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_sizes_match_header_layout():
    # the ctypes mirror must have the C layout (natural alignment, no packing)
    assert C.sizeof(abi.Patch) == 16
    assert C.sizeof(abi.MeshDesc) == 12 + 4 + 24 + 24 + 6 * 16 + 8 + abi.MAX_BOXES * 40
    assert C.sizeof(abi.Species) == 32
    assert C.sizeof(abi.StepStats) % 8 == 0


MIRRORS = {
    "Patch": "picgpu_patch", "Box": "picgpu_box", "MeshDesc": "picgpu_mesh_desc", "Species": "picgpu_species",
    "Mcc": "picgpu_mcc", "IonMcc": "picgpu_ion_mcc", "Coulomb": "picgpu_coulomb", "Learned": "picgpu_learned",
    "Multigrid": "picgpu_multigrid", "Config": "picgpu_config", "StepStats": "picgpu_step_stats",
    "MeshInfo": "picgpu_mesh_info", "Diagnostics": "picgpu_diagnostics",
    "Binary": "picgpu_binary", "Circuit": "picgpu_circuit", "Merging": "picgpu_merging", "Perez": "picgpu_perez", "PerezIon": "picgpu_perez_ion",
    "FreeStream": "picgpu_freestream",
    "Injection": "picgpu_injection", "Emission": "picgpu_emission", "ParticlesSoa": "picgpu_particles_soa",
}


def test_every_field_offset_matches_the_header(tmp_path):
    """A C probe compiled against include/picgpu.h prints sizeof and the
    offset of every field the ctypes mirrors declare."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines, expect = [], []
    for py, cname in MIRRORS.items():
        st = getattr(abi, py)
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(st))
        for f in st._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {f[0]}));')
            expect.append(getattr(st, f[0]).offset)
    src = tmp_path / "probe.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"picgpu.h\"\nint main(void) {\n"
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect


def test_mesh_handle_without_gpu(lib):
    case = cases.two_species_3d(n_cells=6, per_cell=3, L=0.003)
    m = Mesh(case.mesh)
    assert m.n_cells == 216 and m.n_points == 343
    tet, bary, _ = case.particles[0]
    x = m.position(tet, bary)
    t2, b2 = m.locate(x)
    np.testing.assert_array_equal(t2, tet)
    np.testing.assert_allclose(b2, bary, atol=1e-12)
    cc, vol = m.cells()
    np.testing.assert_allclose(vol, (0.003 / 6) ** 3, rtol=1e-12)
    assert np.all((cc > 0) & (cc < 0.003))


def test_invalid_mesh_rejected(lib):
    case = cases.two_species_3d(n_cells=4, per_cell=1)
    case.mesh.side[0].kind = abi.PATCH_CYCLIC  # cyclic without its pair
    with pytest.raises(PicError):
        Mesh(case.mesh)


def test_position_rejects_bad_tet(lib):
    case = cases.two_species_3d(n_cells=2, per_cell=1)
    m = Mesh(case.mesh)
    with pytest.raises(PicError):
        m.position(np.array([8 * 12]), np.zeros((1, 3)))
