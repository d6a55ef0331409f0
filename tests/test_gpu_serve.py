"""Served form on the GPU: every request's result is the same computed alone and
in the continuous-batching mix (exact products, so 'the same' means bit-equal)."""
import pytest

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(gpu):
    import torch

    from nttanafis_gb300.serve import GpuExecutor, serve
    from nttanafis_gb300.workloads import served_stream

    ex = GpuExecutor(slots=3, pool_limbs=1 << 18)
    stream = served_stream(90, rate_hz=20000.0, seed=11, max_limbs=1 << 17)
    stats = serve(stream, ex, budget_bytes=256 << 20, slots=3, max_batch=16)
    torch.cuda.synchronize()
    assert stats["requests"] == len(stream)
    assert stats["batches"] >= 2
    assert stats["peak_budget_bytes"] <= 256 << 20 or stats["batches"] == stats["requests"]
    for p in stats["finished"]:
        assert torch.equal(p.payload.dst, ex.alone(stream[p.rid])), stream[p.rid]
    ex.close()
