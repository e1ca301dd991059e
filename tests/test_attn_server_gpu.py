"""The C++ attention request server (mcAttnServer*): every request's output
equals its output served alone, bit for bit, and the batched engine's; a
burst keeps two batches on the device; admission by device memory holds a
request back while another batch runs and rejects one that cannot fit an
idle device (never launched)."""
import numpy as np
import pytest
import torch

from magicube_gb300 import _lib, batched, synth

pytestmark = pytest.mark.gpu

H = 4
SCALE_QKV = 40.0


def _requests(cuda, lens, seed=0, arrivals=None):
    masks = [synth.band_random_mask(L, 8, 64, 0.9, seed=seed + i) for i, L in enumerate(lens)]
    g = torch.Generator().manual_seed(seed)
    qkvs = [(torch.randn(3, H, L, 64, generator=g) * 0.5).half().to(cuda) for L in lens]
    outs = [torch.full((H, L, 64), float("nan"), dtype=torch.float16, device=cuda) for L in lens]
    arrivals = arrivals or [0.0] * len(lens)
    made = [batched.NativeAttentionServer.request(m, q, o, a, cuda) for m, q, o, a in zip(masks, qkvs, outs, arrivals)]
    return masks, qkvs, outs, [r for r, _ in made], [keep for _, keep in made]


def _server(**kw):
    return batched.NativeAttentionServer(heads=H, scale_qkv=SCALE_QKV, **kw)


def _alone(cuda, mask, qkv):
    out = torch.full_like(qkv[0], float("nan"))
    r, keep = batched.NativeAttentionServer.request(mask, qkv, out, 0.0, cuda)
    lat, st = _server(max_batch_tokens=1 << 20, max_inflight=1).run([r])
    assert st["served"] == 1 and lat[0] >= 0
    return out


def test_mixed_equals_alone_and_engine(cuda):
    """A burst of eight sequences of different lengths in batches of at most
    2,048 tokens, two on the device at once: each output equals the
    sequence served alone and the batched engine's single-instance run."""
    lens = [256, 512, 1024, 320, 768, 2048, 128, 512]
    masks, qkvs, outs, reqs, _keep = _requests(cuda, lens, seed=3)
    lat, st = _server(max_batch_tokens=2048, max_inflight=2).run(reqs)
    torch.cuda.synchronize()
    assert st["served"] == len(lens) and st["rejected"] == 0
    assert st["batches"] >= 3 and st["max_inflight_seen"] == 2
    assert (lat >= 0).all() and st["p99_ms"] >= st["p50_ms"] > 0
    for i, (m, q) in enumerate(zip(masks, qkvs)):
        assert not torch.isnan(outs[i]).any()
        assert torch.equal(outs[i], _alone(cuda, m, q)), i
    for i in (0, 5):
        eng = batched.NativeBatchedSparseAttention([masks[i]], H, scale_qkv=SCALE_QKV, scale_sfmx=127.0,
                                                   device=cuda, requant="rowmax")
        eng.qkv.copy_(qkvs[i])
        assert torch.equal(eng(), outs[i]), i


def test_staggered_arrivals(cuda):
    """Requests arriving one millisecond apart are served as they come, in
    small batches, each with the output it has alone."""
    lens = [512, 256, 1024, 512, 768, 256]
    masks, qkvs, outs, reqs, _keep = _requests(cuda, lens, seed=11, arrivals=[1e-3 * i for i in range(6)])
    lat, st = _server(max_batch_tokens=4096, max_inflight=2).run(reqs)
    torch.cuda.synchronize()
    assert st["served"] == 6 and st["rejected"] == 0 and (lat >= 0).all()
    assert st["makespan_s"] >= 5e-3
    for i, (m, q) in enumerate(zip(masks, qkvs)):
        assert torch.equal(outs[i], _alone(cuda, m, q)), i


def test_admission_holds_back_while_a_batch_runs(cuda):
    """With a budget that fits one batch but not two, the second request
    waits for the first batch to finish; both are served."""
    masks, qkvs, outs, reqs, _keep = _requests(cuda, [2048, 2048], seed=21)
    probe = _server(max_batch_tokens=2048, max_inflight=2)
    need, budget = probe.memory(reqs[:1])
    srv = _server(max_batch_tokens=2048, max_inflight=2, hbm_reserve_bytes=budget - int(1.1 * need))
    lat, st = srv.run(reqs)
    torch.cuda.synchronize()
    assert st["served"] == 2 and st["rejected"] == 0 and st["held_back"] >= 1
    assert st["max_inflight_seen"] == 1
    for i, (m, q) in enumerate(zip(masks, qkvs)):
        assert torch.equal(outs[i], _alone(cuda, m, q)), i


def test_admission_rejects_a_request_that_cannot_fit(cuda):
    """A budget below one request's batch: on an idle device the request is
    rejected (latency -1) and never launched (its output stays untouched)."""
    masks, qkvs, outs, reqs, _keep = _requests(cuda, [1024, 512], seed=31)
    probe = _server()
    need, budget = probe.memory(reqs[:1])
    need2, _ = probe.memory(reqs[1:])
    srv = _server(hbm_reserve_bytes=budget - min(need, need2) // 2)
    lat, st = srv.run(reqs)
    torch.cuda.synchronize()
    assert st["rejected"] == 2 and st["served"] == 0 and (lat == -1).all()
    assert all(torch.isnan(o).all() for o in outs)


def test_request_beyond_int_offsets_is_refused(cuda):
    """A request whose aligned nonzero count leaves the int range of the
    stacked CSR is refused before any batch is launched."""
    masks, qkvs, outs, reqs, _keep = _requests(cuda, [256], seed=41)
    reqs[0].nnz_vec = (1 << 31) - 64
    with pytest.raises(_lib.MagicubeError, match="int range"):
        _server(max_batch_tokens=4096, max_inflight=1).run(reqs)
