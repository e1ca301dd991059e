"""SpMM with 12-bit values (the reference's wmmaSpmm_12b4b / _12b8b: 16-bit
lanes, top 4 bits cleared by the packer, unsigned lanes) and with 16-bit x
16-bit operands (wmmaSpmm_16b: 16-bit B split into byte planes), bit-exact
against the CPU oracle."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

RAGGED = [0, 1, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250]


def _run(cuda, mask, vals, rhs, pa, pb, N, signed, **kw):
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    return ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=signed, **kw)


@pytest.mark.parametrize("pb", [4, 8])
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("N", [64, 256])
@pytest.mark.parametrize("variant", [_lib.KERNEL_PER_ROW, _lib.KERNEL_AUTO])
def test_spmm_12bit_values(cuda, pb, V, N, variant):
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=12 * pb + V)
    vals = synth.random_bytes(mask.nnz_vec * V * 2, 40 + V)  # 16-bit lanes, top bits set at random
    rhs = synth.random_bytes(K * N * pb // 8, 41 + V)
    out = _run(cuda, mask, vals, rhs, 12, pb, N, False, variant=variant)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, 16, pb,
                           oracle.UNSIGNED, preA_cut=12)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_spmm_12bit_rejects_signed(cuda):
    mask = synth.lengths_mask([5, 9], 64, 8, seed=1)
    vals = synth.random_bytes(mask.nnz_vec * 8 * 2, 2)
    rhs = synth.random_bytes(64 * 64, 3)
    with pytest.raises(_lib.MagicubeError):
        _run(cuda, mask, vals, rhs, 12, 8, 64, True)


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [64, 128, 320])
def test_spmm_16x16_ragged(cuda, V, signed, N):
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=160 + V)
    vals = synth.random_bytes(mask.nnz_vec * V * 2, 50 + V)
    rhs = synth.random_bytes(K * N * 2, 51 + V)
    out = _run(cuda, mask, vals, rhs, 16, 16, N, signed)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, 16, 16,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
def test_spmm_16x16_extreme_values_long_rows(cuda, signed, fill):
    """Every lane at an extreme of the 16-bit range, rows up to 2048 nonzeros:
    products up to 2^32 wrap modulo 2^32 exactly as the oracle does."""
    V, K, N = 8, 2048, 64
    mask = synth.lengths_mask([2048, 1000, 257, 256, 255, 0, 31, 1], K, V, seed=17)
    nv, nr = mask.nnz_vec * V * 2, K * N * 2
    if fill == "alt":
        vals = np.tile(np.array([0x00, 0x80, 0xFF, 0x7F], np.uint8), nv // 4 + 1)[:nv]
        rhs = np.tile(np.array([0xFF, 0x7F, 0x00, 0x80], np.uint8), nr // 4 + 1)[:nr]
    else:
        vals, rhs = np.full(nv, fill, np.uint8), np.full(nr, fill, np.uint8)
    out = _run(cuda, mask, vals, rhs, 16, 16, N, signed)
    ref = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, 16, 16,
                           oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_spmm_16x16_batched_strided_and_f16_request(cuda):
    """Batch entries at byte strides; asking for the f16 path gives the same
    integers (16-bit B always runs on the int8 path)."""
    V, K, N, B = 8, 512, 128, 3
    mask = synth.normal_mask(32, K, V, 0.9, seed=7)
    vals_all = [synth.random_bytes(mask.nnz_vec * V * 2, 10 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * 2, 20 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, 16, 16) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size, mma_kind=_lib.MMA_F16)
    for b in range(B):
        ref = oracle.spmm_host(vals_all[b], rhs_all[b], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                               16, 16, oracle.SIGNED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


def test_spmm_16x16_stream_variant_is_rejected(cuda):
    mask = synth.lengths_mask([5, 9], 64, 8, seed=1)
    vals = synth.random_bytes(mask.nnz_vec * 8 * 2, 2)
    rhs = synth.random_bytes(64 * 64 * 2, 3)
    with pytest.raises(_lib.MagicubeError):
        _run(cuda, mask, vals, rhs, 16, 16, 64, True, variant=_lib.KERNEL_STREAM)
