"""Parity at the benchmark configurations' own shapes, on the default paths.

SDDMM: A, B 4096 x 64, mask 4096 x 4096 with V = 8 vectors at sparsity 0.9
(uniform placement, seed 42 -- the headline workload), signed lanes, int32
output, in L8-R8, L4-R4 and L16-R8, through `ops.sddmm` with the automatic
kernel and the default tensor path (the exact f16 path for L16-R8 at k = 64).
A batched launch of four instances is compared with the oracle's restatement
of Host_sddmm_integers (SDDMM/SDDMM/sddmm_benchmark.cpp:24-60) instance by
instance, bit for bit.

SpMM: A 1024 x 1024 at V = 8, sparsity 0.9, B 1024 x 256, in every precision
pair, through `ops.spmm` on the default path; a batched launch of four
instances is compared with the oracle's restatement of compute_ref_integers
(SpMM/SpMM/spmm_benchmark.cpp:69-120)."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import formats, ops, synth

pytestmark = pytest.mark.gpu

SEQ, D, V, SPARSITY = 4096, 64, 8, 0.9


@pytest.fixture(scope="module")
def headline_mask():
    mask = synth.uniform_mask(SEQ // V, SEQ, V, SPARSITY, seed=42)
    return mask, formats.prepare_sddmm(mask, alignment=8)


@pytest.mark.parametrize("pa,pb", [(8, 8), (4, 4), (16, 8)])
def test_sddmm_headline_shape_default_path(cuda, headline_mask, pa, pb):
    mask, hm = headline_mask
    B = 4
    rng = np.random.default_rng(43 + pa)
    lhs = rng.integers(0, 256, size=(B, SEQ * D * pa // 8), dtype=np.uint8)
    rhs = rng.integers(0, 256, size=(B, SEQ * D * pb // 8), dtype=np.uint8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), D, pa, pb, signed=True,
                    batch=B).cpu().numpy()
    pairs, n = oracle.align_pairs(mask.row_offsets, 8)
    assert n == hm.aligned_nnz
    cols = oracle.pad_columns(mask.row_offsets, mask.col_indices, pairs, n)
    for i in range(B):
        ref = oracle.sddmm_host(lhs[i], rhs[i], pairs, cols, mask.m_vec, V, D, SEQ, pa, pb, oracle.SIGNED)
        np.testing.assert_array_equal(out[i], ref, err_msg=f"instance {i}")


@pytest.mark.parametrize("pa,pb", [(8, 8), (4, 4), (16, 8)])
def test_sddmm_headline_shape_extreme_values(cuda, headline_mask, pa, pb):
    """All lanes at the most negative value: the largest partial sums the
    f16 path's flush interval sees at this shape."""
    mask, hm = headline_mask
    lhs = np.full(SEQ * D * pa // 8, 0x88 if pa == 4 else 0x80, np.uint8)
    rhs = np.full(SEQ * D * pb // 8, 0x88 if pb == 4 else 0x80, np.uint8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), D, pa, pb,
                    signed=True).cpu().numpy()
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, D, SEQ, pa, pb, oracle.SIGNED)
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (8, 4), (4, 4), (16, 4)])
def test_spmm_cfg1_shape_default_path(cuda, pa, pb):
    M = K = 1024
    N, B = 256, 4
    mask = synth.uniform_mask(M // V, K, V, SPARSITY, seed=7)
    rng = np.random.default_rng(8 + pa + pb)
    vals = rng.integers(0, 256, size=mask.nnz_vec * V * pa // 8, dtype=np.uint8)
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    rhs = rng.integers(0, 256, size=(B, K * N * pb // 8), dtype=np.uint8)
    out = ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=True, batch=B, values_stride=0).cpu().numpy()
    for i in range(B):
        ref = oracle.spmm_host(vals, rhs[i], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                               oracle.SIGNED)
        np.testing.assert_array_equal(out[i], ref, err_msg=f"instance {i}")
