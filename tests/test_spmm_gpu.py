"""SpMM parity on the GPU: the CUDA library against the CPU oracle (bit-exact)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

PAIRS = [(4, 4), (8, 4), (16, 4), (8, 8), (16, 8)]
RAGGED = [0, 1, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250]


def _case(pa, pb, V, K, N, lengths, seed):
    mask = synth.lengths_mask(lengths, K, V, seed=seed)
    vals = synth.random_bytes(mask.nnz_vec * V * pa // 8, seed + 1)
    rhs = synth.random_bytes(K * N * pb // 8, seed + 2)
    return mask, vals, rhs


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [64, 256])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
@pytest.mark.parametrize("variant", [_lib.KERNEL_PER_ROW, _lib.KERNEL_STREAM])
def test_spmm_ragged(cuda, pa, pb, V, signed, N, mma, variant):
    K = 256
    mask, vals, rhs = _case(pa, pb, V, K, N, RAGGED, seed=pa * 100 + pb * 10 + V)
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    out = ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=signed, mma_kind=mma, variant=variant)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("V", [2, 8])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
def test_spmm_streaming_many_tasks(cuda, pa, pb, V, mma):
    """Far more (batch entry, vector-row) tasks than resident CTAs: every CTA
    streams many rows, including empty and long ones, through its pipeline."""
    K, N, B = 512, 128, 4
    lengths = np.random.default_rng(pa * 10 + pb + V).integers(0, 70, size=1024)
    lengths[::37] = 0
    lengths[5] = 512
    mask = synth.lengths_mask(lengths, K, V, seed=23)
    vals_all = [synth.random_bytes(mask.nnz_vec * V * pa // 8, 50 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 60 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    out = ops.spmm(d, torch.from_numpy(np.concatenate(rhs_all)).to(cuda), N, signed=True, batch=B,
                   values_stride=packed[0].values.size, mma_kind=mma, variant=_lib.KERNEL_STREAM)
    for b in range(B):
        ref = oracle.spmm_host(vals_all[b], rhs_all[b], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                               pa, pb, oracle.SIGNED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
def test_spmm_extreme_values_long_rows(cuda, pa, pb, signed, fill, mma):
    """All lanes at an extreme of their range, rows up to 2048 nonzeros: the
    largest partial sums either tensor path can see (f16 path: f32 partial
    sums near 2^24 before each flush into int32)."""
    V, K, N = 8, 2048, 64
    mask = synth.lengths_mask([2048, 1000, 257, 256, 255, 0, 31, 1], K, V, seed=17)
    nv, nr = mask.nnz_vec * V * pa // 8, K * N * pb // 8
    if fill == "alt":
        vals = np.tile(np.array([0x80, 0x7F], np.uint8), nv // 2 + 1)[:nv]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        vals, rhs = np.full(nv, fill, np.uint8), np.full(nr, fill, np.uint8)
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    out = ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=signed, mma_kind=mma)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
def test_spmm_batched_strided(cuda, pa, pb):
    V, K, N, B = 8, 512, 128, 3
    mask = synth.normal_mask(32, K, V, 0.9, seed=7)
    h = None
    outs = []
    vals_all = [synth.random_bytes(mask.nnz_vec * V * pa // 8, 10 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 20 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    h = packed[0]
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    vstride = h.values.size
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=vstride)
    for b in range(B):
        ref = oracle.spmm_host(vals_all[b], rhs_all[b], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                               pa, pb, oracle.SIGNED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", [(4, 4), (8, 4), (8, 8), (16, 8)])
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("variant", [_lib.KERNEL_PER_ROW, _lib.KERNEL_STREAM])
def test_spmm_half_output(cuda, pa, pb, V, variant):
    """Dequantised half output on the softmax value layout (the extension's bspmm)."""
    K, N, scale = 256, 64, 36.0 * 32.0
    mask, vals, rhs = _case(pa, pb, V, K, N, RAGGED, seed=5)
    h = formats.prepare_spmm(mask, vals, pa, pb, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    out = ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=True, out_half=True, scale=scale, variant=variant)
    acc = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb, oracle.SIGNED)
    with np.errstate(over="ignore"):  # 16-bit A: sums beyond the half range round to inf, as on the GPU
        ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16), ref.view(np.uint16))


@pytest.mark.parametrize("name,pa,pb", [("4b", 4, 4), ("8b4b", 8, 4), ("16b4b", 16, 4), ("8b", 8, 8),
                                        ("16b8b", 16, 8)])
def test_reference_entry_points(cuda, name, pa, pb):
    """mcWmmaSpmm_<P>: reference argument list, unsigned lanes, default stream."""
    V, K, N = 4, 256, 128
    mask, vals, rhs = _case(pa, pb, V, K, N, RAGGED, seed=11)
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    rhs_t = torch.from_numpy(rhs).to(cuda)
    out = torch.full((mask.rows, N), -7, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    fn = getattr(_lib.lib(), f"mcWmmaSpmm_{name}")
    _lib.check(fn(mask.m_vec, V, N, K, d.row_indices.data_ptr(), d.row_offsets.data_ptr(), d.col_indices.data_ptr(),
                  d.values.data_ptr(), rhs_t.data_ptr(), out.data_ptr()), name)
    torch.cuda.synchronize()
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_spmm_rejects_bad_arguments(cuda):
    d = _lib.McSpmmDesc(m_vec=4, vec_length=3, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1)
    rc = _lib.lib().mcSpmm(ctypes.byref(d), None)
    assert rc == 1 and b"vec_length" in _lib.lib().mcGetLastErrorString()
    d.vec_length, d.n = 8, 100
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 1
