"""The allocation-free entry point asend_operator_energy_noalloc.

Some callers cannot let a library call cudaMalloc: applications that own all
device memory through their own pool allocator or a fixed HBM budget, and
optimisation loops that evaluate the strain energy at every line-search step.
For them the library offers y = A x and x^T A x on caller-provided device
buffers, with its reduction scratch in a fixed array compiled into the
library.  This test calls it through the C ABI twice in a row (the shared
scratch keeps the previous call's contents) and compares each result with the
regular entry point asend_apply_operator within the operator tolerance used
by the other GPU tests (1e-11 relative).  It lives in its own file so that it
is collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_operator_energy_noalloc_matches_apply(gpu_lib):
    torch = pytest.importorskip("torch")
    from asend3d_gb300 import configs
    from asend3d_gb300.solver import GpuSolver

    p = configs.block_large(nx=40, ny=8, nz=8, seed=4)
    g = GpuSolver(p)
    g.assemble(precision=64)
    rng = np.random.default_rng(42)
    for call in range(2):
        x = rng.standard_normal(g.n_dof) * (1.0 + call)
        y_ref = g.apply(x, 64)  # existing entry point (host buffers)
        e_ref = float(x @ y_ref)
        xd = torch.from_numpy(x).to("cuda")
        yd = torch.full_like(xd, float("nan"))
        ed = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
        rc = g.lib.asend_operator_energy_noalloc(g.ctx, xd.data_ptr(), yd.data_ptr(), ed.data_ptr())
        assert rc == 0, g.lib.asend_last_error(g.ctx)
        torch.cuda.synchronize()
        if call > 0:  # the first call may load the module (lazy loading); later calls take no device memory
            assert torch.cuda.mem_get_info()[0] == free0
            assert torch.cuda.memory_allocated() == alloc0
        y = yd.cpu().numpy()
        assert np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref) < 1e-11
        assert float(ed.cpu()[0]) == pytest.approx(e_ref, rel=1e-11)
    # an in-place product (x and y sharing memory) is rejected, not computed wrongly
    rc = g.lib.asend_operator_energy_noalloc(g.ctx, xd.data_ptr(), xd.data_ptr(), ed.data_ptr())
    assert rc == -1
    g.close()
