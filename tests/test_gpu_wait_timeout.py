"""Failure detection on the device without a GPU fault.

The persistent and wavefront loops wait on other blocks (grid barriers,
completion counters, reduction epochs).  Every such wait is bounded: a block
that has polled `limit` times raises the abort flag and returns, every other
block leaves at its next wait, and the host turns the flag into an error.  The
test hook clowns_test_arm_wait_timeout makes the next solve's wait run out on
purpose -- a short poll limit, and one block that leaves the kernel without
arriving anywhere, so the barrier it never reaches is a flag nothing sets --
and the test checks that the kernel returns, the API reports the failure
(CLOWNS_ERR_NOCONV from the device entry point, IER 9102 from the PCGPME
drop-in), and the next solve on the same context gives the normal answer."""
import ctypes as C
import time

import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system(gpu):
    import torch
    label, case = small_cases()[1]
    dc, ds = gpu.prepare_dev(case)
    torch.cuda.synchronize()
    return ds


@pytest.mark.parametrize("loop", ["persistent", "wave"])
def test_device_wait_runs_out_and_context_recovers(gpu, system, monkeypatch, loop):
    import torch
    ds = system
    n = ds.mnoe
    L = gpu.lib()
    monkeypatch.setenv("CLOWNS_LOOP_MODE", loop)
    solver = gpu.Solver(n)
    x_ok = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    info_ok = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x_ok, eps=1e-13)      # tunes this execution
    assert info_ok.ier == 0
    assert gpu.tuned_shape([n], 0)["mode"] == loop

    # device entry point: the wait gives up, the call fails, nothing hangs
    assert L.clowns_test_arm_wait_timeout(C.c_long(10000), 0) == 0
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    t0 = time.perf_counter()
    with pytest.raises(gpu.ClownsError) as err:
        solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    assert time.perf_counter() - t0 < 60.0
    assert "(-4)" in str(err.value) and "abandoned" in str(err.value), str(err.value)

    # the context is usable: the next solve is the normal one, bit for bit
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    info = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    assert (info.ier, info.iter, info.eps) == (info_ok.ier, info_ok.iter, info_ok.eps)
    assert torch.equal(x, x_ok)

    # the host-array drop-in reports the same failure as IER 9102
    al = ds.alu.cpu().numpy().copy()
    ll = ds.llu.cpu().numpy().copy()
    d = ds.de.cpu().numpy().copy()
    b = ds.b.cpu().numpy().copy()
    assert L.clowns_test_arm_wait_timeout(C.c_long(10000), 0) == 0
    xh = np.zeros(ds.mm2)
    eps, it, ier = gpu.pcgpme(al, ll, d, b, xh, n, eps=1e-13)
    assert ier == gpu.IER_DEVICE
    xh = np.zeros(ds.mm2)
    eps, it, ier = gpu.pcgpme(al, ll, d, b, xh, n, eps=1e-13)
    assert ier == 0 and it == info_ok.iter
    assert np.array_equal(xh[:n], x_ok.cpu().numpy()[:n])


def test_arm_rejects_bad_arguments(gpu):
    L = gpu.lib()
    assert L.clowns_test_arm_wait_timeout(C.c_long(0), 0) == -2
    assert L.clowns_test_arm_wait_timeout(C.c_long(100), -1) == -2
