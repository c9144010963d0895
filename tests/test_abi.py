"""CPU checks of the C-ABI boundary and the host-side helpers (no GPU calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    hdr = (ROOT / "include" / "asend_gpu.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(asend_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(gpu_lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(gpu_lib, s), f"{s} declared in include/asend_gpu.h but not exported"
    assert b"sm_103a" in gpu_lib.asend_version()


def test_python_binding_covers_header():
    from asend3d_gb300 import _lib

    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_null_context_is_rejected(gpu_lib):
    # every entry point guards a null context instead of crashing
    assert gpu_lib.asend_set_modulus(None, None) == -1
    assert gpu_lib.asend_n_dof(None) == -1
    assert gpu_lib.asend_kernel_launches(None) == -1
    assert gpu_lib.asend_last_error(None) == b"null context"


def test_block_mesh_layout():
    from asend3d_gb300.mesh import block_hex8, block_tet4

    m = block_hex8(3, 2, 2, 3.0, 2.0, 2.0)
    assert m.n_nodes == 4 * 3 * 3 and m.n_elems == 12
    x = m.coords[m.conn]
    # reference corner order: node 1 is +x of node 0, node 3 is +y, node 4 is +z
    assert np.allclose(x[:, 1] - x[:, 0], [1, 0, 0])
    assert np.allclose(x[:, 3] - x[:, 0], [0, 1, 0])
    assert np.allclose(x[:, 4] - x[:, 0], [0, 0, 1])
    t = block_tet4(2, 2, 2, 1.0, 1.0, 1.0)
    v = t.coords[t.conn]
    det = np.einsum("ij,ij->i", v[:, 1] - v[:, 0], np.cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]))
    assert (det > 0).all()
    assert np.isclose(det.sum() / 6.0, 1.0)


def test_lognormal_field_statistics():
    from asend3d_gb300.mesh import ar1_field

    rng = np.random.default_rng(3)
    g = ar1_field((400, 30, 30), (0.01, 0.01, 0.01), 0.05, rng)
    assert abs(g.mean()) < 0.1
    assert abs(g.std() - 1.0) < 0.1
    # lag-1 correlation along x equals exp(-h / l)
    r = np.corrcoef(g[:-1].ravel(), g[1:].ravel())[0, 1]
    assert abs(r - np.exp(-0.01 / 0.05)) < 0.02


def test_constraint_rows_semantics():
    """Constraint::build_mat (const_meth.rs:30-90) row semantics."""
    from asend3d_gb300.mesh import block_hex8
    from asend3d_gb300.solver import Problem
    from oracle.pyoracle import constraint_rows

    m = block_hex8(1, 1, 1, 1.0, 1.0, 1.0)
    p = Problem(m, np.ones(1), np.zeros(1))
    p.add_node_set("face", [0, 1, 2, 3])
    p.add_node_set("one", [5])
    p.constraints.append(([("face", 2, 1.0), ("one", 2, -1.0)], 0.0))  # tie face u_y to node 5 u_y
    ptr, dof, coef, rhs = constraint_rows(p)
    assert len(rhs) == 4
    assert list(dof[ptr[0]:ptr[1]]) == [1, 16]
    assert list(coef[ptr[3]:ptr[4]]) == [1.0, -1.0]


def test_header_is_plain_c(gpu_lib, tmp_path):
    """include/asend_gpu.h compiles as strict C99 and a C program links and
    runs against the library (no device call): the boundary is a C ABI."""
    import shutil
    import subprocess
    from pathlib import Path

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    root = Path(__file__).resolve().parents[1]
    src = tmp_path / "abi.c"
    src.write_text('#include "asend_gpu.h"\n#include <string.h>\n'
                   "int main(void) { asend_solve_opts o; asend_eigen_opts e; memset(&o, 0, sizeof o);\n"
                   "  memset(&e, 0, sizeof e); e.inner = o; return asend_version() ? 0 : 1; }\n")
    from asend3d_gb300 import build
    cuda_lib = Path(build.nvcc()).resolve().parent.parent / "lib64"
    exe = tmp_path / "abi"
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{root / 'include'}", str(src),
           f"-L{root / 'asend3d_gb300'}", "-lasend_gpu", f"-L{cuda_lib}", f"-Wl,-rpath-link,{cuda_lib}",
           f"-Wl,-rpath,{root / 'asend3d_gb300'}", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
