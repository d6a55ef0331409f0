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


def test_noalloc_edge_shapes(gpu):
    # an empty operand (zeros, no kernel), the smallest transform (1 x 1 and 3 x 5),
    # and all-ones operands at the limit, whose carries cross every CRT tile; each
    # bit for bit against the workspace call, the limb past the result untouched
    import torch

    lib = gpu.library()
    ws = gpu.GpuMulWorkspace()
    stream = torch.cuda.current_stream()
    handle = stream.cuda_stream
    empty = torch.empty(0, dtype=torch.int64, device="cuda")
    b = _device_limbs(torch, np.arange(1, 8, dtype=np.uint64))
    got = torch.full((8,), -1, dtype=torch.int64, device="cuda")
    assert lib.ntt_mul_noalloc_device(got.data_ptr(), 8, empty.data_ptr(), 0, b.data_ptr(), 7, handle) == 1
    torch.cuda.synchronize()
    assert bool((got[:7] == 0).all()) and int(got[7]) == -1
    ones = np.full(2049, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64)
    from nttanafis_gb300.operands import operand

    for a_h, b_h in [(operand(1, 5), operand(1, 6)), (operand(3, 7), operand(5, 8)), (ones[:2048], ones)]:
        a, b = _device_limbs(torch, a_h), _device_limbs(torch, b_h)
        n = a_h.size + b_h.size
        expected = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
        got = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
        assert ws.mul_device(expected, a, b, stream), gpu.last_error()
        ok = lib.ntt_mul_noalloc_device(got.data_ptr(), n, a.data_ptr(), a_h.size, b.data_ptr(), b_h.size, handle)
        assert ok == 1, gpu.last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, expected), (a_h.size, b_h.size)
        assert int(got[n]) == -1
    ws.close()
