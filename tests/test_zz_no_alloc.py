"""ntt_mul_noalloc_device: the product entry point for callers that must not
allocate device memory (a budget owned by another allocator, or a path that cannot
afford cudaMalloc's device-wide synchronisation). Its scratch is a static device
array, shared by every call.

The test calls it through the C ABI twice in a row on different operands (the
second call runs over the scratch the first one left behind) and compares each
result with the regular workspace entry point, bit for bit, since the products are
exact integers. It also checks that a shape above the stated limit is refused
without touching the destination. This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_COEFFICIENTS = 4096  # NTT_NOALLOC_MAX_COEFFICIENTS in include/ntt_gb300.h


def _device_limbs(torch, values):
    return torch.from_numpy(np.ascontiguousarray(values).view(np.int64)).cuda()


def test_noalloc_matches_workspace_on_two_calls_in_a_row(gpu):
    import torch

    from nttanafis_gb300.operands import operand

    lib = gpu.library()
    ws = gpu.GpuMulWorkspace()
    stream = torch.cuda.current_stream()
    handle = stream.cuda_stream
    for la, lb, sa, sb in [(2048, 2049, 71, 72), (1000, 37, 73, 74)]:
        a = _device_limbs(torch, operand(la, sa))
        b = _device_limbs(torch, operand(lb, sb))
        expected = torch.full((la + lb + 1,), -1, dtype=torch.int64, device="cuda")
        got = torch.full((la + lb + 1,), -1, dtype=torch.int64, device="cuda")
        assert ws.mul_device(expected, a, b, stream), gpu.last_error()
        ok = lib.ntt_mul_noalloc_device(got.data_ptr(), got.numel(), a.data_ptr(), la, b.data_ptr(), lb, handle)
        assert ok == 1, gpu.last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, expected)  # exact, including the untouched last limb
    # the same array twice squares it, like the workspace call
    a = _device_limbs(torch, operand(1500, 75))
    expected = torch.empty(3000, dtype=torch.int64, device="cuda")
    got = torch.empty(3000, dtype=torch.int64, device="cuda")
    assert ws.sqr_device(expected, a, stream)
    assert lib.ntt_mul_noalloc_device(got.data_ptr(), 3000, a.data_ptr(), 1500, a.data_ptr(), 1500, handle) == 1
    torch.cuda.synchronize()
    assert torch.equal(got, expected)
    ws.close()


def test_noalloc_refuses_shapes_above_its_limit(gpu):
    import torch

    from nttanafis_gb300.operands import operand

    lib = gpu.library()
    la, lb = MAX_COEFFICIENTS, 2  # la + lb - 1 = 4097 coefficients
    a = _device_limbs(torch, operand(la, 1))
    b = _device_limbs(torch, operand(lb, 2))
    dst = torch.full((la + lb,), 7, dtype=torch.int64, device="cuda")
    assert lib.ntt_mul_noalloc_device(dst.data_ptr(), dst.numel(), a.data_ptr(), la, b.data_ptr(), lb, 0) == 0
    assert "4096" in gpu.last_error()
    torch.cuda.synchronize()
    assert bool((dst == 7).all())
