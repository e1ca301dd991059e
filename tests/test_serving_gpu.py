"""Continuous batching: overlapping batches, admission by free device memory.

The reference serves one request at a time (its encoder loop,
end2end_eval/sparse_transformer_magicube/end_to_end.py:47-85); these tests
cover what makes the server here a continuous-batching one: batches run on
the device at the same time and every request's result is the same as when
it is served alone, and admission follows the free device memory, which a
test replaces by a fake (host-side injection, no real exhaustion)."""
import pytest
import torch

from magicube_gb300 import model, serving

pytestmark = pytest.mark.gpu

KW = dict(hidden=256, layers=2, sparsity=0.9, median=1024, clip=(512, 2048), seed=21)


def _encoder(cuda, attention="fused"):
    torch.manual_seed(0)
    return model.SparseEncoder(layers=2, hidden=256, heads=4, ffn=512).to(cuda).half().eval().set_attention(attention)


def _same_as_alone(enc, reqs, cuda, kw=KW):
    alone = serving.make_requests(len(reqs), rate=0.0, **kw)
    serving.serve_sequential(enc, alone, device=cuda)
    for a, m in zip(alone, reqs):
        ref, got = a.out.float().cpu(), m.out.float().cpu()
        assert torch.isfinite(ref).all()
        # the attention is exact in both; the dense fp16 layers may pick other
        # GEMM kernels for other token counts
        assert (got - ref).abs().max() <= 2e-2 * ref.abs().max(), a.rid


@pytest.mark.parametrize("attention", ["fused", "separate"])
def test_batches_overlap_and_each_result_equals_served_alone(cuda, attention):
    """Staggered arrivals with a small overlap threshold: several batches are
    in flight on their own streams at once, and each request's output equals
    its served-alone output within the stated tolerance."""
    enc = _encoder(cuda, attention)
    reqs = serving.make_requests(12, rate=20000.0, **KW)
    srv = serving.ContinuousBatchingServer(enc, hidden=256, heads=4, max_inflight=3, max_batch_tokens=2048,
                                           overlap_tokens=1, device=cuda)
    stats = srv.serve(reqs)
    assert stats["requests"] == 12 and stats["rejected"] == 0
    assert srv.peak_inflight >= 2, srv.batches
    assert sorted(r for b in srv.batches for r in b) == list(range(12))
    _same_as_alone(enc, reqs, cuda)


def _fake_free_memory(monkeypatch, srv, budget: int, per_batch: int):
    """Free device memory = budget minus `per_batch` for every batch in flight."""
    total = torch.cuda.get_device_properties(0).total_memory

    def fake(device=None):
        return max(0, budget - per_batch * len(getattr(srv, "inflight", []))), total

    monkeypatch.setattr(torch.cuda, "mem_get_info", fake)


def test_admission_holds_requests_back_while_memory_is_taken(cuda, monkeypatch):
    """Free memory for one request at a time: queued requests wait for the
    batch in flight instead of joining it or overlapping it, and all are
    served with the results they have alone."""
    enc = _encoder(cuda)
    kw = dict(KW, clip=(768, 1024))  # any two requests need more than the largest one
    reqs = serving.make_requests(6, rate=0.0, **kw)
    srv = serving.ContinuousBatchingServer(enc, hidden=256, heads=4, max_inflight=3, max_batch_tokens=1 << 20,
                                           overlap_tokens=1, hbm_reserve=0, device=cuda)
    one = max(serving.footprint_bytes([r], 256, 4, 2, 8) for r in reqs)
    two = min(serving.footprint_bytes([a, b], 256, 4, 2, 8) for a in reqs for b in reqs if a is not b)
    assert two > one
    _fake_free_memory(monkeypatch, srv, budget=(one + two) // 2, per_batch=one)
    stats = srv.serve(reqs)
    assert stats["requests"] == 6 and stats["rejected"] == 0
    assert all(len(b) == 1 for b in srv.batches)
    assert srv.peak_inflight == 1
    assert srv.held_back > 0
    _same_as_alone(enc, reqs, cuda, kw)


def test_oversize_request_is_rejected_not_launched(cuda, monkeypatch):
    """A request whose working set exceeds the free memory of an idle device
    is rejected at admission (never launched); the others are served."""
    enc = _encoder(cuda)
    reqs = serving.make_requests(4, rate=0.0, **KW)
    big = max(reqs, key=lambda r: r.seq_len)
    srv = serving.ContinuousBatchingServer(enc, hidden=256, heads=4, max_inflight=2, max_batch_tokens=1 << 20,
                                           hbm_reserve=0, device=cuda)
    fit = max(serving.footprint_bytes([r], 256, 4, 2, 8) for r in reqs if r is not big)
    assert serving.footprint_bytes([big], 256, 4, 2, 8) > fit
    _fake_free_memory(monkeypatch, srv, budget=fit, per_batch=fit)
    stats = srv.serve(reqs)
    assert srv.rejected == [big.rid] and big.error is not None and big.out is None
    assert stats["requests"] == 3 and stats["rejected"] == 1
    assert all(r.out is not None for r in reqs if r is not big)
