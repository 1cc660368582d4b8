"""The allocation-free solve (clowns_pcgpme_static_dev) against the workspace
solve (clowns_pcgpme_dev) and the oracle, called through the C ABI.

Callers that cannot allocate device memory -- a host model whose device memory
belongs to another runtime or to a fixed budget -- use the allocation-free
entry point, whose scratch lives in a static device array (limit: 32768 rows).
It runs the workspace solve's kernels and summation tree, so two calls in a
row must each reproduce the workspace solve's iteration count and pressure
bit for bit, lie within 1e-10 relative L2 of the oracle's pressure (both at
ERR <= 1e-13, the tolerance of the other solve tests), and the second call
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
def test_static_solve_matches_workspace_solve_twice(gpu, ora, idx):
    import torch
    label, case = small_cases()[idx]
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    n = ds.mnoe
    assert n <= 32768
    xw = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    iw = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, xw, eps=1e-13)
    ref = xw[:n].cpu().numpy()
    oracle = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
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
        assert (info.iter, info.eps) == (iw.iter, iw.eps), (label, call)
        assert np.array_equal(got, ref), (label, call)
        assert np.linalg.norm(got - oracle.x) <= 1e-10 * np.linalg.norm(oracle.x), (label, call)
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
