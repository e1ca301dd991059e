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


def _same_as_alone(enc, reqs, cuda, kw=KW, rate=0.0):
    alone = serving.make_requests(len(reqs), rate=rate, **kw)  # the same requests (same draws)
    serving.serve_sequential(enc, alone, device=cuda)
    for a, m in zip(alone, reqs):
        ref, got = a.out.float().cpu(), m.out.float().cpu()
        assert torch.isfinite(ref).all()
        # the attention is exact in both; the dense fp16 layers may pick other
        # GEMM kernels for other token counts
        assert (got - ref).abs().max() <= 2e-2 * ref.abs().max(), a.rid


class _SlowBatches(torch.nn.Module):
    """The encoder followed by a fixed spin of about a millisecond on the
    batch's stream (torch.cuda._sleep: a bounded busy loop), so a batch
    stays on the device while the host admits the next ones -- at these
    small sizes the host would otherwise launch slower than the device
    finishes."""

    def __init__(self, enc):
        super().__init__()
        self.enc, self.layers = enc, enc.layers

    def forward(self, x, masks):
        y = self.enc(x, masks)
        torch.cuda._sleep(2_000_000)
        return y


@pytest.mark.parametrize("attention", ["fused", "separate"])
def test_batches_overlap_and_each_result_equals_served_alone(cuda, attention):
    """Staggered arrivals with a small overlap threshold: several batches are
    in flight on their own streams at once, and each request's output equals
    its served-alone output within the stated tolerance."""
    enc = _encoder(cuda, attention)
    reqs = serving.make_requests(12, rate=20000.0, **KW)
    srv = serving.ContinuousBatchingServer(_SlowBatches(enc), hidden=256, heads=4, max_inflight=3,
                                           max_batch_tokens=2048, overlap_tokens=1, device=cuda)
    stats = srv.serve(reqs)
    assert stats["requests"] == 12 and stats["rejected"] == 0
    assert srv.peak_inflight >= 2, srv.batches
    assert sorted(r for b in srv.batches for r in b) == list(range(12))
    _same_as_alone(enc, reqs, cuda, rate=20000.0)


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
    one = max(srv.footprint([r]) for r in reqs)
    two = min(srv.footprint([a, b]) for a in reqs for b in reqs if a is not b)
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
    reqs = serving.make_requests(3, rate=0.0, **dict(KW, clip=(512, 1536)))
    big = serving.make_requests(1, rate=0.0, **dict(KW, clip=(2048, 2048), seed=99))[0]
    big.rid = 3
    reqs.insert(1, big)  # arrives between the others
    srv = serving.ContinuousBatchingServer(enc, hidden=256, heads=4, max_inflight=2, max_batch_tokens=1 << 20,
                                           hbm_reserve=0, device=cuda)
    fit = max(srv.footprint([r]) for r in reqs if r is not big)
    assert srv.footprint([big]) > fit
    _fake_free_memory(monkeypatch, srv, budget=fit, per_batch=fit)
    stats = srv.serve(reqs)
    assert srv.rejected == [big.rid] and big.error is not None and big.out is None
    assert stats["requests"] == 3 and stats["rejected"] == 1
    assert all(r.out is not None for r in reqs if r is not big)


@pytest.mark.parametrize("attention", ["fused", "separate"])
def test_footprint_bounds_the_measured_peak(cuda, attention):
    """The admission estimate is an upper bound of the measured peak device
    memory of a batch (torch.cuda.max_memory_allocated) and within 2x of it,
    on encoder-request lengths from 512 to 8192 tokens."""
    enc = _encoder(cuda, attention)
    srv = serving.ContinuousBatchingServer(enc, hidden=256, heads=4, device=cuda)
    for lens in ([512], [2048], [8192], [2048] * 4, [1024, 4096, 8192]):
        reqs = [serving.make_requests(1, 0.0, hidden=256, layers=2, median=L, clip=(L, L), seed=60 + i)[0]
                for i, L in enumerate(lens)]
        for r in reqs:
            serving._upload_csr(r, cuda)
        with torch.no_grad():
            for warm in (True, False):  # the first pass creates library handles outside the measurement
                torch.cuda.synchronize()
                base = torch.cuda.memory_allocated()
                torch.cuda.reset_peak_memory_stats()
                masks = serving.pack_batch_masks(reqs, 2, 8, 16, cuda)
                x = torch.cat([r.dev["x"] for r in reqs], 0)
                y = enc(x, masks)
                torch.cuda.synchronize()
                peak = torch.cuda.max_memory_allocated() - base
                del y, x, masks
        est = srv.footprint(reqs)
        assert peak <= est <= 2 * peak, (lens, peak, est)
