"""Allocation-free adjoint entry point (spde_adjoint_noalloc).

Some callers cannot allocate device memory while they run this code: a host
framework that owns every device byte through its own pool, or code that must
not let cudaMalloc / cudaFree synchronise the device in the middle of a stream.
spde_adjoint_noalloc gives them the log-likelihood adjoint with its work array
in a fixed static device array instead of a per-call allocation.  This file is
collected last on purpose (it checks a process-wide shared array); it must pass
both on its own in a fresh process and after every other test.
"""
import ctypes

import numpy as np
import pytest

from golden_cases import load
from gpu_cases import gpu_model, separable_gpu_model

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _symmetric_gbar(grid, rng, nslots):
    from spdepy_gb300.spdes import stencil_offsets
    offs = stencil_offsets(grid.T, nslots)
    ns = len(offs)
    n = grid.n
    r = rng.normal(size=(n, ns))
    k = np.arange(n)
    t, rem = np.divmod(k, grid.Mx * grid.Ny)
    y, x = np.divmod(rem, grid.Mx)
    g = np.zeros_like(r)
    for s, (dx, dy, dt) in enumerate(offs):
        ok = (x + dx >= 0) & (x + dx < grid.Mx) & (y + dy >= 0) & (y + dy < grid.Ny) & (t + dt >= 0) & (t + dt < grid.T)
        nb = ((t + dt) * grid.Ny + y + dy) * grid.Mx + x + dx
        g[ok, s] = r[ok, s] + r[nb[ok], ns - 1 - s]
    return torch.as_tensor(g).cuda().contiguous()


def _noalloc(plan, gbar, nt):
    from spdepy_gb300 import _native as nat
    out = torch.empty(nt, dtype=torch.float64, device="cuda")
    nat.check(nat.lib().spde_adjoint_noalloc(plan.h, gbar.data_ptr(), out.data_ptr()), plan.h, "adjoint_noalloc")
    torch.cuda.synchronize()  # the call only enqueues the work on the plan's stream
    return out.cpu().numpy()


@pytest.mark.parametrize("name", ["covadv_vardiff_bc1", "wm_ani_bc1", "separable_ani_bc1"])
def test_noalloc_matches_allocating_adjoint_twice(name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spdepy_gb300 import build
    build.build()
    g = load(name)
    # separable plans take the temporal-reduction branch of the adjoint
    mod = separable_gpu_model(g, "fp64") if name.startswith("separable_") else gpu_model(g, "fp64")
    mod._assemble(g["par"])
    plan = mod.plan
    nt = mod.layout.ncanon - 1
    rng = np.random.default_rng(5)
    for call in range(2):
        gbar = _symmetric_gbar(mod.grid, rng, plan.nslots)
        ref = plan.adjoint(gbar)
        got = _noalloc(plan, gbar, nt)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-13 * scale), (call, np.abs(got - ref).max() / scale)


def test_noalloc_rejects_grids_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import spdepy_gb300 as sp
    from spdepy_gb300 import _native as nat
    grid = sp.grid(x=np.arange(100.0), y=np.arange(100.0))   # 10,000 cells > 9,892
    mod = sp.spde_init("whittle-matern", grid, ani=True, ha=False, bc=3, precision="fp64")
    mod._assemble(mod.par)
    gbar = torch.zeros(grid.n * 25, dtype=torch.float64, device="cuda")
    out = torch.empty(8, dtype=torch.float64, device="cuda")
    rc = nat.lib().spde_adjoint_noalloc(mod.plan.h, gbar.data_ptr(), out.data_ptr())
    assert rc == 1
    assert b"too large" in nat.lib().spde_last_error(mod.plan.h)
