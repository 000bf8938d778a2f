"""Host-side logic that needs no GPU: the bench's clock-sample summary and the autograd wrapper
of the adjoint (with a stand-in network that returns fixed gradients)."""

from __future__ import annotations

import numpy as np
import pytest

import bench


def _sampler_with(lines, skip):
    s = bench.ClockSampler()
    s.proc = None
    s.lines = list(lines)
    s.skip = skip
    return s


def _summary(s):
    # stop() without a process: the "unavailable" answer; summarise the lines the way stop() does
    class _Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s.proc = _Done()
    s.thread = None
    return s.stop()


def test_clock_summary_counts_the_timed_region_only():
    before = "0, 1200, 2070, 300, 0x0, Not Active, Not Active, Not Active, Not Active"
    during = ["0, 2070, 2070, 900, 0x0, Not Active, Not Active, Not Active, Not Active",
              "0, 2055, 2070, 950, 0x4, Not Active, Not Active, Not Active, Active",
              "0, 2070, 2070, 940, 0x0, Not Active, Not Active, Not Active, Not Active"]
    out = _summary(_sampler_with([before] + during, skip=1))
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_summary_keeps_the_last_sample_when_the_region_was_shorter():
    line = "0, 2070, 2070, 900, 0x0, Active, Not Active, Not Active, Not Active"
    out = _summary(_sampler_with([line], skip=1))
    assert out["samples"] == 1 and out["reasons"] == ["hw_slowdown"]


def test_clock_summary_without_nvidia_smi():
    s = bench.ClockSampler()
    s.proc = None
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]


class _StubNet:
    """Stands in for a set-up network: records what the wrapper sets and returns fixed gradients."""

    def __init__(self, n, ns):
        self.n, self.ns = n, ns
        self.k = self.r0 = self.q = None

    def setSpringParameters(self, k, r0):
        self.k, self.r0 = k.copy(), r0.copy()

    def setCharges(self, q):
        self.q = q.copy()

    def adjoint(self, nsteps, target, checkpoint=20, charges=False):
        gk = np.arange(self.ns, dtype=np.float32)
        gr = -np.arange(self.ns, dtype=np.float32)
        loss = float(np.sum(self.k) + np.sum(self.r0))
        if charges:
            return loss, gk, gr, np.full(self.n, 0.5, np.float32)
        return loss, gk, gr


def test_fit_wrapper_routes_parameters_and_gradients():
    torch = pytest.importorskip("torch")
    from biospring_gb300.fit import SpringFitLoss
    net = _StubNet(n=5, ns=4)
    k = torch.ones(4, requires_grad=True)
    r0 = torch.full((4,), 2.0, requires_grad=True)
    loss = SpringFitLoss.apply(k, r0, net, np.zeros((5, 3), np.float32), 10, 5)
    (3.0 * loss).backward()
    assert float(loss.detach()) == 12.0 and net.q is None
    np.testing.assert_array_equal(k.grad.numpy(), 3.0 * np.arange(4))
    np.testing.assert_array_equal(r0.grad.numpy(), -3.0 * np.arange(4))
    q = torch.tensor([1.0, -1.0, 0.0, 0.5, 0.0], requires_grad=True)
    k.grad = r0.grad = None
    loss = SpringFitLoss.apply(k, r0, net, np.zeros((5, 3), np.float32), 10, 5, q)
    loss.backward()
    np.testing.assert_array_equal(net.q, q.detach().numpy())
    np.testing.assert_array_equal(q.grad.numpy(), np.full(5, 0.5, np.float32))
    np.testing.assert_array_equal(k.grad.numpy(), np.arange(4))
