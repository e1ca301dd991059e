"""The C++ batched attention engine (mcAttnBatch*) against the Python
batched path: the same bits for every precision pair and requantization
mode, eager and replayed from the CUDA graph the library records, with the
launch configuration its own tuner picks."""
import numpy as np
import pytest
import torch

from magicube_gb300 import batched, synth

pytestmark = pytest.mark.gpu

CASES = [(8, 8, "fixed", 60.0, 100.0), (8, 8, "rowmax", 60.0, 127.0), (16, 8, "fixed", 60.0, 32767.0),
         (8, 4, "rowmax", 3.0, 127.0)]


@pytest.mark.parametrize("lb,rb,mode,sq,ss", CASES)
@pytest.mark.parametrize("V", [2, 8])
def test_engine_equals_python_batched_fused(cuda, lb, rb, mode, sq, ss, V):
    lens = [64, 512, 128, 1024, 192, 8 * V]
    masks = [synth.band_random_mask(L, V, 64, 0.8, seed=110 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(11)) * 0.5).half().to(cuda)
    ref = batched.BatchedSparseAttention(masks, H, d, lb, rb, scale_qkv=sq, scale_sfmx=ss, device=cuda, tune=False,
                                         requant=mode)
    a = ref(qkv).clone()
    eng = batched.NativeBatchedSparseAttention(masks, H, d, lb, rb, scale_qkv=sq, scale_sfmx=ss, device=cuda,
                                               requant=mode)
    np.testing.assert_array_equal(eng.token_offsets, ref.token_offsets)
    eng.qkv.copy_(qkv)
    eng.out.fill_(1000.0)
    b = eng().clone()
    torch.cuda.synchronize()
    assert eng.status() == 0
    assert torch.equal(a, b)
    cfg = eng.tune()
    assert cfg["warps"] in (4, 8) and cfg["stages"] in (2, 3) and cfg["ctas_per_sm"] in (0, 2, 4)
    eng.out.fill_(1000.0)
    eng.capture()
    eng.out.fill_(1000.0)
    c = eng.replay().clone()
    torch.cuda.synchronize()
    assert torch.equal(a, c)
    # new inputs in the same buffer: the graph reads them
    eng.qkv.mul_(-1.0)
    ref_neg = ref(eng.qkv).clone()
    c2 = eng.replay().clone()
    torch.cuda.synchronize()
    assert torch.equal(ref_neg, c2)
    for i in range(len(lens)):
        assert eng.instance_output(i).shape == (H, lens[i], d)


def test_engine_on_the_batched_attention_workload(cuda):
    """64 instances x 4 heads, lengths 512-4096, band + random V = 8 masks at
    sparsity 0.9 (the batched-attention benchmark's workload), row-max: the
    engine's graph replay equals the Python fused path bit for bit."""
    rng = np.random.default_rng(11)
    lens = (rng.integers(512, 4097, size=64) // 64 * 64).clip(512, 4096).tolist()
    masks = [synth.band_random_mask(L, 8, 256, 0.9, seed=100 + i) for i, L in enumerate(lens)]
    qkv = (torch.randn(3, 4, sum(lens), 64, generator=torch.Generator().manual_seed(12)) * 0.5).half().to(cuda)
    kw = dict(scale_qkv=40.0, scale_sfmx=127.0, device=cuda, requant="rowmax")
    ref = batched.BatchedSparseAttention(masks, 4, 64, fused=True, tune=False, **kw)
    a = ref(qkv).clone()
    eng = batched.NativeBatchedSparseAttention(masks, 4, 64, **kw)
    eng.qkv.copy_(qkv)
    eng.tune()
    eng.capture()
    b = eng.replay().clone()
    torch.cuda.synchronize()
    assert eng.status() == 0
    assert torch.equal(a, b)
