"""A bounded wait that runs out is a failed call, not a wrong product returned as
success (the reference's calls return false on failure, src/lib.rs:21-24).

The failure is made on the host: the test hook ntt_debug_stall_lookback makes the
next CRT launch start its tile counter at 1, so no CTA takes tile 0 and tile 1's
look-back waits for a state that nothing writes. The wait is bounded (about 70 ms),
after which the kernel flags the failure and completes; the GPU stays usable and
the next call is exact. Nothing here faults or hangs the GPU.

This file is collected after the other GPU test files, whose check that no
look-back wait ever gave up would otherwise count these deliberate ones."""
import numpy as np
import pytest

import oracle
from nttanafis_gb300.operands import operand

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1
SHAPE = (70000, 50000)  # four-step transforms, then the look-back CRT kernel


def test_stalled_lookback_fails_the_host_call(gpu):
    ws = gpu.GpuMulWorkspace()
    a, b = operand(SHAPE[0], 1), operand(SHAPE[1], 2)
    expected = oracle.mul(a, b)
    before = gpu.lookback_timeouts()
    try:
        gpu.debug_stall_lookback(1)
        dst = np.full(sum(SHAPE), MASK, dtype=np.uint64)
        assert not ws.mul(dst, a, b)
        assert "look-back" in gpu.last_error()
    finally:
        gpu.debug_stall_lookback(0)
    assert gpu.lookback_timeouts() > before
    # the context is usable and the next call exact
    dst = np.full(sum(SHAPE), MASK, dtype=np.uint64)
    assert ws.mul(dst, a, b), gpu.last_error()
    assert np.array_equal(dst, expected)
    ws.close()


def test_stalled_lookback_sets_the_workspace_status(gpu):
    import torch

    stream = torch.cuda.current_stream()
    ws = gpu.GpuMulWorkspace()
    a_h, b_h = operand(SHAPE[0], 3), operand(SHAPE[1], 4)
    a = torch.from_numpy(a_h.view(np.int64)).cuda()
    b = torch.from_numpy(b_h.view(np.int64)).cuda()
    dst = torch.empty(sum(SHAPE), dtype=torch.int64, device="cuda")
    try:
        gpu.debug_stall_lookback(1)
        assert ws.mul_device(dst, a, b, stream)  # enqueued: the failure comes later
        torch.cuda.synchronize()
    finally:
        gpu.debug_stall_lookback(0)
    assert ws.status() == gpu.STATUS_LOOKBACK
    assert ws.status() == 0
    assert ws.mul_device(dst, a, b, stream)
    torch.cuda.synchronize()
    assert ws.status() == 0
    assert np.array_equal(dst.cpu().numpy().view(np.uint64), oracle.mul(a_h, b_h))
    ws.close()
