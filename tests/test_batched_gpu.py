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


@pytest.mark.parametrize("requant", ["fixed", "rowmax"])
def test_encoder_fused_attention_equals_separate(cuda, requant):
    """The encoder with the fused attention kernel gives the same bits as with
    the separate SDDMM / softmax / SpMM launches, in either requant mode."""
    torch.manual_seed(0)
    enc = model.SparseEncoder(layers=2, hidden=256, heads=4, ffn=512).to(cuda).half().eval()
    reqs = serving.make_requests(3, rate=0.0, hidden=256, layers=2, sparsity=0.9, median=256, clip=(128, 512),
                                 seed=8)
    for r in reqs:
        serving._upload(r, 16, cuda)
    masks = serving.batch_masks(reqs, 2, 8)
    assert all(m.max_row_nnz > 0 for m in masks)
    x = torch.cat([r.dev["x"] for r in reqs], dim=0)
    with torch.no_grad():
        a = enc.set_attention("separate", requant)(x, masks).clone()
        b = enc.set_attention("fused", requant)(x, masks).clone()
    torch.cuda.synchronize()
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)


@pytest.mark.parametrize("attention", ["separate", "fused"])
def test_batch_packed_masks_give_same_output(cuda, attention):
    """Masks of a whole batch packed by one device call per layer (rows sorted
    across requests) give the same encoder output, bit for bit, as the
    per-request packed masks stacked block-diagonally."""
    torch.manual_seed(0)
    enc = model.SparseEncoder(layers=2, hidden=256, heads=4, ffn=512).to(cuda).half().eval()
    enc.set_attention(attention)
    kw = dict(rate=0.0, hidden=256, layers=2, sparsity=0.9, median=256, clip=(128, 640), seed=9)
    a_reqs, b_reqs = serving.make_requests(5, **kw), serving.make_requests(5, **kw)
    for r in a_reqs:
        serving._upload(r, 16, cuda)
    for r in b_reqs:
        serving._upload_csr(r, cuda)
    ma = serving.batch_masks(a_reqs, 2, 8)
    mb = serving.pack_batch_masks(b_reqs, 2, 8, 16, cuda)
    assert [m.max_row_nnz for m in ma] == [m.max_row_nnz for m in mb]
    x = torch.cat([r.dev["x"] for r in a_reqs], dim=0)
    with torch.no_grad():
        ya = enc(x, ma).clone()
        yb = enc(x, mb).clone()
    torch.cuda.synchronize()
    assert torch.equal(ya, yb)


def test_server_fused_mixed_same_as_sequential_separate(cuda):
    """Continuous batching on the fused attention kernel against one request
    at a time on the separate launches: the same results within the fp16
    tolerance of the dense layers."""
    torch.manual_seed(0)
    enc = model.SparseEncoder(layers=2, hidden=256, heads=4, ffn=512).to(cuda).half().eval()
    kw = dict(rate=0.0, hidden=256, layers=2, sparsity=0.9, median=256, clip=(128, 640), seed=4)
    reqs = serving.make_requests(8, **kw)
    srv = serving.ContinuousBatchingServer(enc.set_attention("fused"), hidden=256, heads=4, max_inflight=2,
                                           max_batch_tokens=1024, device=cuda)
    srv.serve(reqs)
    assert any(len(b) > 1 for b in srv.batches)
    mixed = [r.out.float().cpu() for r in reqs]
    alone = serving.make_requests(8, **kw)
    serving.serve_sequential(enc.set_attention("separate"), alone, device=cuda)
    for a, m in zip(alone, mixed):
        ref = a.out.float().cpu()
        assert torch.isfinite(ref).all()
        assert (m - ref).abs().max() <= 2e-2 * ref.abs().max()


@pytest.mark.parametrize("V", [2, 4, 8])
def test_fused_fixed_equals_separate_steps(cuda, V):
    """The fused kernel with fixed requantization reproduces the separate
    SDDMM -> softmax -> SpMM launches bit for bit."""
    lens = [64, 512, 128, 1024, 192]
    masks = [synth.band_random_mask(L, V, 64, 0.8, seed=30 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(3)) * 0.5).half().to(cuda)
    sep = batched.BatchedSparseAttention(masks, H, d, scale_qkv=60.0, scale_sfmx=100.0, device=cuda, tune=False)
    fus = batched.BatchedSparseAttention(masks, H, d, scale_qkv=60.0, scale_sfmx=100.0, device=cuda, fused=True)
    a = sep(qkv).clone()
    b = fus(qkv).clone()
    torch.cuda.synchronize()
    assert int(fus.core.status.item()) == 0
    assert torch.equal(a, b)


@pytest.mark.parametrize("V", [2, 4, 8])
def test_fused_rowmax_equals_separate_and_per_instance(cuda, V):
    """Row-max requantization gives the same bits fused (one launch), as
    separate batched launches (SDDMM, row-max softmax writing per-row
    divisors, SpMM dividing by them) and as per-instance launches."""
    lens = [64, 512, 128, 1024, 192]
    masks = [synth.band_random_mask(L, V, 64, 0.8, seed=60 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(6)) * 0.5).half().to(cuda)
    kw = dict(scale_qkv=60.0, scale_sfmx=127.0, device=cuda, requant="rowmax")
    sep = batched.BatchedSparseAttention(masks, H, d, tune=False, **kw)
    fus = batched.BatchedSparseAttention(masks, H, d, fused=True, **kw)
    per = batched.PerInstanceSparseAttention(masks, H, d, **kw)
    a = sep(qkv).clone()
    b = fus(qkv).clone()
    offs = sep.token_offsets
    outs = per([qkv[:, :, int(offs[i]):int(offs[i + 1])].contiguous() for i in range(len(lens))])
    torch.cuda.synchronize()
    assert int(fus.core.status.item()) == 0
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)
    for i, o in enumerate(outs):
        assert torch.equal(fus.instance_output(i), o), f"instance {i}"


def test_fused_rowmax_error_vs_fp64(cuda):
    """Row-max requantization keeps 7 bits relative to each row's largest
    probability: the output error against the float64 unquantized attention
    is far below the fixed-scale scheme's."""
    import oracle.attention as oatt
    from magicube_gb300 import formats
    lens = [256, 512]
    masks = [synth.band_random_mask(L, 8, 128, 0.8, seed=40 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv_h = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(4)) * 0.5).half()
    sq = 127.0 / float(qkv_h.abs().max())
    fus = batched.BatchedSparseAttention(masks, H, d, scale_qkv=sq, scale_sfmx=127.0, device=cuda, fused=True,
                                         requant="rowmax")
    fus(qkv_h.to(cuda))
    torch.cuda.synchronize()
    for i, m in enumerate(masks):
        a, z = int(fus.token_offsets[i]), int(fus.token_offsets[i + 1])
        pairs, n = formats.align_row_offsets(m, 16)
        cols = formats.pad_column_indices(m, pairs, n, False)
        mk = oatt.dense_mask(pairs, cols, m.m_vec, 8, lens[i])
        q, k, v = (qkv_h[j, :, a:z].double().numpy() for j in range(3))
        ref = oatt.sparse_attention_fp64(q, k, v, mk, d ** -0.5)
        got = fus.instance_output(i).double().cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 0.05, err


def test_fused_reports_rows_longer_than_declared(cuda):
    """A max_row_nnz smaller than a row's length must not touch memory out of
    bounds: the kernel skips that row and sets the status word."""
    masks = [synth.band_random_mask(512, 8, 64, 0.8, seed=50)]
    fus = batched.BatchedSparseAttention(masks, 1, 64, scale_qkv=60.0, scale_sfmx=100.0, device=cuda, fused=True)
    fus.mask.max_row_nnz = 32  # deliberately too small
    fus.core.m.max_row_nnz = 32
    fus.core.out.fill_(7.0)
    fus((torch.randn(3, 1, 512, 64) * 0.5).half().to(cuda))
    torch.cuda.synchronize()
    assert int(fus.core.status.item()) == 1
    assert torch.all(fus.core.out == 7.0)  # every row exceeds 32 nonzero vectors: nothing written


def test_device_packed_request_masks_equal_host_packed(cuda):
    """Requests uploaded with the GPU packer (upper-bound slot arrays, no host
    round trip) give the same encoder output as the host-packed block-diagonal
    mask of the same requests."""
    torch.manual_seed(1)
    enc = model.SparseEncoder(layers=2, hidden=128, heads=2, ffn=256).to(cuda).half().eval()
    reqs = serving.make_requests(3, rate=0.0, hidden=128, layers=2, sparsity=0.9, median=256, clip=(128, 512),
                                 seed=8)
    for r in reqs:
        serving._upload(r, 16, cuda)
    dev_masks = serving.batch_masks(reqs, 2, 8)
    host_masks = [batched.to_device(batched.block_diagonal([r.masks[l] for r in reqs])[0], 16, cuda)
                  for l in range(2)]
    x = torch.cat([r.dev["x"] for r in reqs], dim=0)
    with torch.no_grad():
        a = enc(x, dev_masks)
        b = enc(x, host_masks)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


FUSED_CFGS = [{"warps": w, "stages": st, "ctas_per_sm": c} for w in (4, 8) for st in (2, 3) for c in (0, 3)]
PAIR_SCALES = {(8, 8): (60.0, 100.0), (16, 8): (60.0, 32767.0), (8, 4): (3.0, 100.0)}


@pytest.mark.parametrize("pair", [(8, 8), (16, 8), (8, 4)])
@pytest.mark.parametrize("V", [2, 4, 8])
def test_fused_fixed_every_pair_and_config_equals_separate(cuda, pair, V):
    """Every precision pair of the fused kernel, in every launch
    configuration the autotuner chooses from (warps per CTA = k-split,
    ring stages, CTAs per SM), reproduces the separate SDDMM -> softmax ->
    SpMM launches of the same pair bit for bit."""
    lb, rb = pair
    sq, ss = PAIR_SCALES[pair]
    lens = [64, 512, 128, 1024, 192]
    masks = [synth.band_random_mask(L, V, 64, 0.8, seed=70 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(7)) * 0.5).half().to(cuda)
    sep = batched.BatchedSparseAttention(masks, H, d, lb, rb, scale_qkv=sq, scale_sfmx=ss, device=cuda, tune=False)
    a = sep(qkv).clone()
    fus = batched.BatchedSparseAttention(masks, H, d, lb, rb, scale_qkv=sq, scale_sfmx=ss, device=cuda, fused=True,
                                         tune=False)
    for cfg in FUSED_CFGS:
        fus.core.fused_cfg = cfg
        fus.core.out.fill_(1000.0)
        b = fus(qkv).clone()
        torch.cuda.synchronize()
        assert int(fus.core.status.item()) == 0
        assert torch.equal(a, b), cfg


@pytest.mark.parametrize("pair", [(8, 8), (8, 4)])
@pytest.mark.parametrize("V", [2, 8])
def test_fused_rowmax_every_config_equals_separate(cuda, pair, V):
    lb, rb = pair
    lens = [64, 512, 128, 1024, 192]
    masks = [synth.band_random_mask(L, V, 64, 0.8, seed=90 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(9)) * 0.5).half().to(cuda)
    kw = dict(scale_qkv=PAIR_SCALES[pair][0], scale_sfmx=127.0, device=cuda, requant="rowmax", tune=False)
    sep = batched.BatchedSparseAttention(masks, H, d, lb, rb, **kw)
    a = sep(qkv).clone()
    fus = batched.BatchedSparseAttention(masks, H, d, lb, rb, fused=True, **kw)
    assert torch.isfinite(a).all()
    for cfg in FUSED_CFGS:
        fus.core.fused_cfg = cfg
        fus.core.out.fill_(1000.0)
        b = fus(qkv).clone()
        torch.cuda.synchronize()
        assert torch.equal(a, b), cfg


def test_fused_autotuned_configuration_is_used(cuda, tmp_path, monkeypatch):
    """With tuning on, the fused kernel's configuration comes from the
    autotuner's candidates, is cached, and the tuned launch keeps the bits."""
    from magicube_gb300 import autotune
    monkeypatch.setenv("MC_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_cache", None)
    lens = [256, 768]
    masks = [synth.band_random_mask(L, 8, 64, 0.8, seed=80 + i) for i, L in enumerate(lens)]
    qkv = (torch.randn(3, 2, sum(lens), 64, generator=torch.Generator().manual_seed(8)) * 0.5).half().to(cuda)
    sep = batched.BatchedSparseAttention(masks, 2, 64, 16, 8, scale_qkv=60.0, scale_sfmx=32767.0, device=cuda,
                                         tune=False)
    fus = batched.BatchedSparseAttention(masks, 2, 64, 16, 8, scale_qkv=60.0, scale_sfmx=32767.0, device=cuda,
                                         fused=True, tune=True)
    a = sep(qkv).clone()
    b = fus(qkv).clone()
    assert fus.core.fused_cfg in autotune.fused_attention_candidates()
    assert torch.equal(a, b)
    assert any(k.split("|")[1].startswith("attn_fused") for k in autotune._load())


def test_fused_L16R8_error_vs_fp64(cuda):
    """16-bit probabilities at the full output range: the attention error
    against the float64 unquantized attention."""
    import oracle.attention as oatt
    lens = [256, 512]
    masks = [synth.band_random_mask(L, 8, 128, 0.8, seed=40 + i) for i, L in enumerate(lens)]
    H, d = 2, 64
    qkv_h = (torch.randn(3, H, sum(lens), d, generator=torch.Generator().manual_seed(4)) * 0.5).half()
    sq = 127.0 / float(qkv_h.abs().max())
    fus = batched.BatchedSparseAttention(masks, H, d, 16, 8, scale_qkv=sq, scale_sfmx=32767.0, device=cuda,
                                         fused=True, tune=False)
    fus(qkv_h.to(cuda))
    torch.cuda.synchronize()
    for i, m in enumerate(masks):
        a, z = int(fus.token_offsets[i]), int(fus.token_offsets[i + 1])
        q, k, v = (qkv_h[j, :, a:z].double().numpy() for j in range(3))
        ref = oatt.sparse_attention_fp64_rows(q, k, v, m.row_offsets, m.col_indices, 8, d ** -0.5)
        got = fus.instance_output(i).double().cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 0.05, err
