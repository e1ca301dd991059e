"""Batched uneven sparse attention and the continuous-batching server."""
import numpy as np
import pytest
import torch

from magicube_gb300 import batched, model, serving, synth

pytestmark = pytest.mark.gpu


def _instances(lens, V=8, sparsity=0.8, band=64, seed=0):
    return [synth.band_random_mask(L, V, band, sparsity, seed=seed + i) for i, L in enumerate(lens)]


@pytest.mark.parametrize("lhs_bits,rhs_bits", [(8, 8), (16, 8), (8, 4), (4, 4)])
def test_batched_matches_per_instance(cuda, lhs_bits, rhs_bits):
    """Every instance's output from the single block-diagonal launch sequence
    equals, bit for bit, its output from its own launches."""
    lens = [64, 320, 128, 512, 192]
    masks = _instances(lens)
    H, d = 3, 64
    gen = torch.Generator().manual_seed(1)
    qkvs = [(torch.randn(3, H, L, d, generator=gen) * 0.5).half().to(cuda) for L in lens]
    b = batched.BatchedSparseAttention(masks, H, d, lhs_bits, rhs_bits, scale_qkv=60.0, scale_sfmx=100.0,
                                       device=cuda, tune=True)
    b.qkv.copy_(torch.cat(qkvs, dim=2))
    b()
    p = batched.PerInstanceSparseAttention(masks, H, d, lhs_bits, rhs_bits, scale_qkv=60.0, scale_sfmx=100.0,
                                           device=cuda)
    outs = p(qkvs)
    torch.cuda.synchronize()
    for i, o in enumerate(outs):
        assert torch.equal(b.instance_output(i), o), f"instance {i}"


def test_batched_graph_replay(cuda):
    lens = [128, 256, 64]
    b = batched.BatchedSparseAttention(_instances(lens, seed=5), 2, 64, device=cuda, tune=False)
    b.qkv.copy_((torch.randn(b.qkv.shape, generator=torch.Generator().manual_seed(2)) * 0.5).half())
    eager = b().clone()
    b.capture()
    b.qkv.mul_(1.0)
    g = b.replay().clone()
    torch.cuda.synchronize()
    assert torch.equal(eager, g)
    b.qkv.mul_(-1.0)  # new inputs in the same buffer
    g2 = b.replay().clone()
    assert not torch.equal(g2, g)


def test_server_results_same_alone_and_mixed(cuda):
    """Requests served in mixed batches give the same result as served alone,
    within the tolerance of the dense fp16 layers (the integer attention is
    exact in both; cuBLAS may pick different GEMM kernels for different token
    counts): max |mixed - alone| <= 2e-2 * max |alone|."""
    torch.manual_seed(0)
    enc = model.SparseEncoder(layers=2, hidden=128, heads=2, ffn=256).to(cuda).half().eval()
    reqs = serving.make_requests(8, rate=0.0, hidden=128, layers=2, sparsity=0.9, median=256, clip=(128, 640),
                                 seed=3)
    srv = serving.ContinuousBatchingServer(enc, hidden=128, heads=2, max_inflight=2, max_batch_tokens=1024,
                                           device=cuda)
    stats = srv.serve(reqs)
    assert stats["requests"] == 8 and any(len(b) > 1 for b in srv.batches)
    mixed = [r.out.float().cpu() for r in reqs]
    alone = serving.make_requests(8, rate=0.0, hidden=128, layers=2, sparsity=0.9, median=256, clip=(128, 640),
                                  seed=3)
    serving.serve_sequential(enc, alone, device=cuda)
    for a, m in zip(alone, mixed):
        ref = a.out.float().cpu()
        assert torch.isfinite(ref).all()
        assert (m - ref).abs().max() <= 2e-2 * ref.abs().max()
