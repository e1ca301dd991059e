"""The TMA-gather SpMM (MC_KERNEL_TMA: a producer warp gathers B rows with
tile::gather4 into an mbarrier ring, consumer warps multiply), 8-bit and 4-bit
B, against the CPU oracle, bit-exact, and against the streaming kernel."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

RAGGED = [0, 1, 3, 4, 5, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250, 2]
PAIRS8 = [(8, 8), (16, 8), (12, 8)]
PAIRS4 = [(4, 4), (8, 4), (16, 4), (12, 4)]


def _run(cuda, mask, vals, rhs, pa, pb, N, signed, variant=_lib.KERNEL_TMA, **kw):
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    return ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=signed, variant=variant, **kw)


def _vals(mask, V, pa, seed):
    return synth.random_bytes(mask.nnz_vec * V * formats.lane_bits(pa) // 8, seed)


@pytest.mark.parametrize("pa,pb", PAIRS8)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [128, 256, 384])
def test_tma_ragged(cuda, pa, pb, V, signed, N):
    """Row lengths around every group-of-4, 16-slot and 32-slot boundary,
    empty rows included; N = 384 runs three 128-column tiles."""
    if pa == 12 and signed:
        pytest.skip("12-bit lanes are unsigned")
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V)
    vals = _vals(mask, V, pa, 30 + V)
    rhs = synth.random_bytes(K * N, 31 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                           16 if pa == 12 else pa, pb, oracle.SIGNED if signed else oracle.UNSIGNED,
                           **({"preA_cut": 12} if pa == 12 else {}))
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS4)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [256, 512])
def test_tma_ragged_4bit_rhs(cuda, pa, pb, V, signed, N):
    """4-bit B (256 columns per 128-byte row box; column indices shuffled
    within groups of 8 by the packer), every A precision."""
    if pa == 12 and signed:
        pytest.skip("12-bit lanes are unsigned")
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V + 1)
    vals = _vals(mask, V, pa, 32 + V)
    rhs = synth.random_bytes(K * N // 2, 33 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                           16 if pa == 12 else pa, pb, oracle.SIGNED if signed else oracle.UNSIGNED,
                           **({"preA_cut": 12} if pa == 12 else {}))
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4)])
@pytest.mark.parametrize("N", [128, 256])
@pytest.mark.parametrize("shared_rhs", [False, True])
def test_tma_batched_many_tasks(cuda, pa, pb, N, shared_rhs):
    """Far more tasks than resident CTAs (every CTA streams many rows through
    its ring), per-entry values, B per entry or shared (rhs_stride 0)."""
    if pb == 4:
        N *= 2  # 4-bit B runs 256-column tiles
    V, K, B = 8, 512, 4
    lengths = np.random.default_rng(pa + N).integers(0, 90, size=700)
    lengths[::29] = 0
    lengths[3] = 512
    mask = synth.lengths_mask(lengths, K, V, seed=41)
    vals_all = [_vals(mask, V, pa, 50 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 60 + b) for b in range(B)]
    if shared_rhs:
        rhs_all = [rhs_all[0]] * B
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(rhs_all[0] if shared_rhs else np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size,
                   rhs_stride=0 if shared_rhs else K * N * pb // 8, variant=_lib.KERNEL_TMA)
    for b in range(B):
        ref = oracle.spmm_host(vals_all[b], rhs_all[b], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                               pa, pb, oracle.SIGNED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4), (16, 4)])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
def test_tma_extreme_values_long_rows(cuda, pa, pb, signed, fill):
    V, K, N = 8, 2048, 128 if pb == 8 else 256
    mask = synth.lengths_mask([2048, 1000, 257, 256, 255, 0, 31, 1], K, V, seed=17)
    nv, nr = mask.nnz_vec * V * pa // 8, K * N * pb // 8
    if fill == "alt":
        vals = np.tile(np.array([0x80, 0x7F], np.uint8), nv // 2 + 1)[:nv]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        vals, rhs = np.full(nv, fill, np.uint8), np.full(nr, fill, np.uint8)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4)])
@pytest.mark.parametrize("V", [2, 4, 8])
def test_tma_half_output_equals_stream(cuda, pa, pb, V):
    """Dequantised half output on the softmax value layout, bit-identical to
    the streaming kernel and to the oracle's integer result / scale."""
    K, N, scale = 512, 256, 36.0 * 32.0
    mask = synth.lengths_mask(RAGGED, K, V, seed=70 + V)
    vals = _vals(mask, V, pa, 71)
    rhs = synth.random_bytes(K * N * pb // 8, 72)
    h = formats.prepare_spmm(mask, vals, pa, pb, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    r = torch.from_numpy(rhs).to(cuda)
    outs = [ops.spmm(d, r, N, signed=True, out_half=True, scale=scale, variant=v)
            for v in (_lib.KERNEL_TMA, _lib.KERNEL_STREAM)]
    assert torch.equal(outs[0], outs[1])
    acc = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb, oracle.SIGNED)
    with np.errstate(over="ignore"):  # 16-bit A: sums beyond the half range round to inf, as on the GPU
        ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    np.testing.assert_array_equal(outs[0].cpu().numpy().view(np.uint16), ref.view(np.uint16))


def test_tma_equals_stream_headline(cuda):
    """A 1024 x 1024 V=8 sparsity-0.9 operand times 1024 x 256, 16 batch
    entries: identical int32 results from the two kernels."""
    M = K = 1024
    N, V, B = 256, 8, 16
    mask = synth.uniform_mask(M // V, K, V, 0.9, seed=7)
    vals = synth.random_bytes(mask.nnz_vec * V, 8)
    h = formats.prepare_spmm(mask, vals, 8, 8)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    d.values = d.values.repeat(B)
    rhs = torch.randint(0, 256, (B, K * N), dtype=torch.uint8, device=cuda)
    outs = [ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=h.values.size, variant=v)
            for v in (_lib.KERNEL_TMA, _lib.KERNEL_STREAM)]
    assert torch.equal(outs[0], outs[1])
    ref = oracle.spmm_host(vals, rhs[3].cpu().numpy(), mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, 8, 8,
                           oracle.SIGNED)
    np.testing.assert_array_equal(outs[0][3].cpu().numpy(), ref)


def test_tma_rejects_ineligible(cuda):
    V, K = 8, 256
    mask = synth.lengths_mask([5, 40], K, V, seed=3)
    for pa, pb, N, mma in ((8, 8, 64, _lib.MMA_INT8), (8, 4, 128, _lib.MMA_INT8), (8, 8, 128, _lib.MMA_F16),
                           (16, 16, 128, _lib.MMA_INT8), (4, 4, 384, _lib.MMA_INT8)):
        vals = _vals(mask, V, pa, 1)
        rhs = synth.random_bytes(K * N * pb // 8, 2)
        with pytest.raises(_lib.MagicubeError):
            _run(cuda, mask, vals, rhs, pa, pb, N, True, mma_kind=mma)


def test_tma_no_timeouts(cuda):
    torch.cuda.synchronize()
    assert _lib.lib().mcTensorCoreTimeouts() == 0


DP4A_PAIRS = [(8, 8), (8, 4), (4, 4)]


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("V", [2, 4])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [128, 256, 512])
def test_dp4a_spmm_ragged(cuda, pa, pb, V, signed, N):
    """The dp4a consumers of the TMA kernel (MC_MMA_DP4A, V = 2 and 4): row
    lengths around every group-of-4, 16-slot and 32-slot boundary, empty
    rows, bit-exact against the oracle."""
    if pb == 4 and N == 128:
        N = 256
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V + 7)
    vals = _vals(mask, V, pa, 40 + V)
    rhs = synth.random_bytes(K * N * pb // 8, 41 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed, variant=_lib.KERNEL_AUTO, mma_kind=_lib.MMA_DP4A)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("V", [2, 4])
@pytest.mark.parametrize("fill", [0x80, 0x7F, 0xFF])
def test_dp4a_spmm_extreme_values_long_rows(cuda, pa, pb, V, fill):
    """Extreme lanes over rows of up to K = 2048 nonzero vectors."""
    K, N = 2048, 256
    mask = synth.lengths_mask([2048, 1, 0, 999, 33, 2047, 64, 16], K, V, seed=V + pa)
    vals = np.full(mask.nnz_vec * V * pa // 8, fill, np.uint8)
    rhs = np.full(K * N * pb // 8, fill, np.uint8)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, True, variant=_lib.KERNEL_AUTO, mma_kind=_lib.MMA_DP4A)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("V", [2, 4])
def test_dp4a_spmm_batched_many_tasks_equals_int8(cuda, pa, pb, V):
    """Many tasks per CTA, per-entry values and B: dp4a and int8 MMA give the
    same integers."""
    K, N, B = 1024, 256, 3
    mask = synth.normal_mask(700, K, V, 0.9, seed=V * 3 + pa)
    h = formats.prepare_spmm(mask, _vals(mask, V, pa, 50), pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    d.values = torch.cat([d.values, torch.randint(0, 256, (2 * d.values.numel(),), dtype=torch.uint8,
                                                  device=cuda)])
    rhs = torch.randint(0, 256, (B, K * N * pb // 8), dtype=torch.uint8, device=cuda)
    kw = dict(signed=True, batch=B, values_stride=h.values.size)
    a = ops.spmm(d, rhs, N, mma_kind=_lib.MMA_DP4A, **kw)
    b = ops.spmm(d, rhs, N, mma_kind=_lib.MMA_INT8, variant=_lib.KERNEL_TMA, **kw)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    i = B - 1
    vals_i = d.values[i * h.values.size:(i + 1) * h.values.size].cpu().numpy()
    ref = oracle.spmm_device(h.row_offsets, h.col_indices, vals_i, rhs[i].cpu().numpy(), mask.m_vec, V, K, N, pa, pb,
                             oracle.SIGNED)
    np.testing.assert_array_equal(a[i].cpu().numpy(), ref)


def test_dp4a_spmm_rejects_unsupported(cuda):
    mask = synth.lengths_mask([5, 9], 64, 8, seed=1)
    with pytest.raises(_lib.MagicubeError):
        _run(cuda, mask, _vals(mask, 8, 8, 1), synth.random_bytes(64 * 128, 2), 8, 8, 128, True,
             variant=_lib.KERNEL_AUTO, mma_kind=_lib.MMA_DP4A)
    mask = synth.lengths_mask([5, 9], 64, 4, seed=1)
    with pytest.raises(_lib.MagicubeError):
        _run(cuda, mask, _vals(mask, 4, 16, 1), synth.random_bytes(64 * 128, 2), 16, 8, 128, True,
             variant=_lib.KERNEL_AUTO, mma_kind=_lib.MMA_DP4A)
