"""The n == 64 SpMM (the attention's P x V: 8-bit softmax-layout values,
gathered 64-byte rows, half output; k split over four warps) against the CPU
oracle and the per-row kernel, bit for bit."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

# empty rows, rows shorter than one 32-slot step, rows of exactly 1-8 steps per
# warp, and long rows whose steps all four warps share
LENGTHS = [0, 1, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250, 511, 640, 129, 97]


def _case(V, K, lengths, seed, B=1):
    mask = synth.lengths_mask(lengths, K, V, seed=seed)
    vals = [synth.random_bytes(mask.nnz_vec * V, seed + 1 + b) for b in range(B)]
    rhs = [synth.random_bytes(K * 64, seed + 11 + b) for b in range(B)]
    return mask, vals, rhs


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("variant", [_lib.KERNEL_AUTO, _lib.KERNEL_STREAM])
def test_n64_matches_oracle(cuda, V, variant):
    K, scale = 1024, 36.0 * 32.0
    mask, vals, rhs = _case(V, K, LENGTHS, seed=70 + V)
    h = formats.prepare_spmm(mask, vals[0], 8, 8, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    out = ops.spmm(d, torch.from_numpy(rhs[0]).to(cuda), 64, signed=True, out_half=True, scale=scale,
                   variant=variant)
    acc = oracle.spmm_host(vals[0], rhs[0], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, 64, 8, 8,
                           oracle.SIGNED)
    ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16), ref.view(np.uint16))


@pytest.mark.parametrize("V", [2, 8])
def test_n64_batched_equals_per_row_kernel(cuda, V):
    """Several batch entries with their own values and B, many rows per CTA:
    the same bits as the per-row kernel."""
    K, B, scale = 2048, 3, 127.0 * 44.0
    lengths = np.random.default_rng(V).integers(0, 400, size=600)
    lengths[::17] = 0
    lengths[4] = 2048
    mask, vals, rhs = _case(V, K, lengths, seed=90 + V, B=B)
    h = formats.prepare_spmm(mask, vals[0], 8, 8, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    per = h.values.size
    d.values = torch.cat([torch.from_numpy(formats.prepare_spmm(mask, v, 8, 8, layout=formats.VALUES_SOFTMAX).values)
                          for v in vals]).to(cuda)
    rhs_t = torch.from_numpy(np.concatenate(rhs)).to(cuda)
    args = dict(signed=True, out_half=True, scale=scale, batch=B, values_stride=per)
    a = ops.spmm(d, rhs_t, 64, variant=_lib.KERNEL_AUTO, **args)
    b = ops.spmm(d, rhs_t, 64, variant=_lib.KERNEL_PER_ROW, **args)
    np.testing.assert_array_equal(a.cpu().numpy().view(np.uint16), b.cpu().numpy().view(np.uint16))
    acc = oracle.spmm_host(vals[2], rhs[2], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, 64, 8, 8,
                           oracle.SIGNED)
    ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    np.testing.assert_array_equal(a[2].cpu().numpy().view(np.uint16), ref.view(np.uint16))


@pytest.mark.parametrize("fill", [0x80, 0x7F, "alt"])
def test_n64_extreme_values(cuda, fill):
    """The largest products over long rows stay exact (int32 sums)."""
    V, K, scale = 8, 4096, 1.0
    mask = synth.lengths_mask([4096, 1, 4000, 33, 0, 512], K, V, seed=7)
    nv = mask.nnz_vec * V
    if fill == "alt":
        vals = np.tile(np.array([0x80, 0x7F], np.uint8), nv // 2 + 1)[:nv]
        rhs = np.tile(np.array([0x7F, 0x80, 0x80, 0x7F], np.uint8), K * 16 + 1)[:K * 64]
    else:
        vals, rhs = np.full(nv, fill, np.uint8), np.full(K * 64, fill, np.uint8)
    h = formats.prepare_spmm(mask, vals, 8, 8, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    a = ops.spmm(d, torch.from_numpy(rhs).to(cuda), 64, signed=True, out_half=True, scale=scale)
    b = ops.spmm(d, torch.from_numpy(rhs).to(cuda), 64, signed=True, out_half=True, scale=scale,
                 variant=_lib.KERNEL_PER_ROW)
    np.testing.assert_array_equal(a.cpu().numpy().view(np.uint16), b.cpu().numpy().view(np.uint16))


def test_n64_row_divisors(cuda):
    """Per-row divisors (the row-max requantization's) as the per-row kernel."""
    V, K = 8, 1024
    mask, vals, rhs = _case(V, K, LENGTHS, seed=31)
    h = formats.prepare_spmm(mask, vals[0], 8, 8, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    rt = torch.from_numpy(rhs[0]).to(cuda)
    M = mask.m_vec * V
    div = torch.from_numpy(np.random.default_rng(3).uniform(50.0, 5000.0, size=M).astype(np.float32)).to(cuda)
    outs = []
    for variant in (_lib.KERNEL_AUTO, _lib.KERNEL_PER_ROW):
        out = torch.zeros((M, 64), dtype=torch.float16, device=cuda)
        desc = _lib.McSpmmDesc(
            m_vec=mask.m_vec, vec_length=V, n=64, k=K, lhs_bits=8, rhs_bits=8, is_signed=1, out_half=1, scale=1.0,
            batch=1, row_indices=d.row_indices.data_ptr(), row_offsets=d.row_offsets.data_ptr(),
            column_indices=d.col_indices.data_ptr(), values=d.values.data_ptr(), rhs=rt.data_ptr(),
            out=out.data_ptr(), kernel_variant=variant, value_layout=_lib.VALUES_SOFTMAX,
            row_div=div.data_ptr(), row_div_stride=0)
        _lib.check(_lib.lib().mcSpmm(ctypes.byref(desc), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "mcSpmm")
        outs.append(out.cpu().numpy().view(np.uint16))
    np.testing.assert_array_equal(outs[0], outs[1])
    acc = oracle.spmm_host(vals[0], rhs[0], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, 64, 8, 8,
                           oracle.SIGNED).reshape(M, 64)
    ref = (acc.astype(np.float32) / div.cpu().numpy()[:, None]).astype(np.float16)
    np.testing.assert_array_equal(outs[0], ref.view(np.uint16))
