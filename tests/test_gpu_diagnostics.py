"""Diagnostics of the C ABI that the benchmark reports: the measured FP64 rate
(the FP64 roofline's denominator) and the count of kernels a solve launched."""
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu


def test_fp64_fma_rate_is_plausible(gpu):
    """About 6e11 fused multiply-adds per second on a GB300 (1.2 TFLOP/s); a
    rate far outside this window would mean the probe does not time its work."""
    rates = [gpu.fp64_fma_rate() for _ in range(2)]
    for r in rates:
        assert 1e11 < r < 5e12, rates
    assert abs(rates[0] - rates[1]) <= 0.1 * max(rates), rates


def test_kernel_launch_count_covers_every_iteration(gpu, monkeypatch):
    """A solve's launch count includes the kernel nodes its loop graph ran: with
    the graph of tile kernels and fused LDUSUB sweep pairs, 11 per iteration
    plus the loop guard."""
    import torch
    monkeypatch.setenv("CLOWNS_LOOP_MODE", "graph")
    monkeypatch.setenv("CLOWNS_SWEEP_FUSE", "1")
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", "0")
    label, case = small_cases()[1]
    dc, ds = gpu.prepare_dev(case)
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    info = gpu.Solver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-10)
    launches = gpu.last_kernel_launches()
    assert info.ier == 0
    assert launches >= 12 * info.iter, (launches, info.iter)
