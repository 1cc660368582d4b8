"""The allocation-free solve (clowns_pcgpme_static_dev) against the workspace
solve (clowns_pcgpme_dev), both called through the C ABI.

Callers that cannot allocate device memory -- a host model whose device memory
belongs to another runtime or to a fixed budget -- use the allocation-free
entry point, whose scratch lives in a static device array (limit: 32768 rows).
Two calls in a row must each match the workspace solve within the tolerance of
the other solve tests (1e-10 relative L2 at ERR <= 1e-13), and the second call
must not change the device's free memory.  This file is collected last."""
import ctypes as C

import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu


def _static_solve(gpu, ds, x, eps):
    import torch
    L = gpu.lib()
    nl, na = ds.alu.shape
    info = gpu.SolveInfo()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.clowns_pcgpme_static_dev(ds.alu.data_ptr(), nl, na, ds.llu.data_ptr(), ds.de.data_ptr(), ds.mnoe,
                                    ds.b.data_ptr(), x.data_ptr(), eps, 5.0, 10000, stream, C.byref(info))
    assert rc == 0, gpu.last_error()
    return info


@pytest.mark.parametrize("idx", [1, 2])
def test_static_solve_matches_workspace_solve_twice(gpu, idx):
    import torch
    label, case = small_cases()[idx]
    dc, ds = gpu.prepare_dev(case)
    n = ds.mnoe
    assert n <= 32768
    xw = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    iw = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, xw, eps=1e-13)
    ref = xw[:n].cpu().numpy()
    free_after_first = None
    for call in range(2):
        xs = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        info = _static_solve(gpu, ds, xs, 1e-13)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free_after == free_before, "the allocation-free solve changed free device memory"
        got = xs[:n].cpu().numpy()
        assert info.ier == iw.ier == 0
        assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref), (label, call)
        assert abs(info.iter - iw.iter) <= max(5, iw.iter // 4)
        free_after_first = free_after
    assert free_after_first is not None


def test_static_solve_rejects_oversized_systems(gpu):
    """n beyond CLOWNS_STATIC_MAX_ROWS is refused before any device work."""
    L = gpu.lib()
    info = gpu.SolveInfo()
    dummy = C.c_void_p(16)          # never dereferenced: the size check comes first
    rc = L.clowns_pcgpme_static_dev(dummy, 6, 40000, dummy, dummy, 40000, dummy, dummy, 1e-10, 5.0, 100,
                                    None, C.byref(info))
    assert rc == -5                 # CLOWNS_ERR_LIMIT
    assert "32768" in gpu.last_error()
