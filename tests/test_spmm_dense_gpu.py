"""The dense-tile SpMM (MC_KERNEL_DENSE_TILE: each 256-row block of A expanded
into f16 tiles in shared memory and multiplied whole on the tcgen05 tensor
cores) against the CPU oracle bit for bit: every V, signed and unsigned
lanes, ragged and empty rows, k across accumulation segments, batches with
their own or shared operands, extreme values at the exactness bound."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

DENSE = _lib.KERNEL_DENSE_TILE
RAGGED = [0, 1, 3, 4, 5, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250, 2]


def _ref(mask, vals, rhs, V, K, N, signed):
    return oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, 8, 8,
                            oracle.SIGNED if signed else oracle.UNSIGNED)


SLOT = formats.VALUES_SLOT_MAJOR


def _dev(cuda, mask, vals, layout=formats.VALUES_PACKED):
    return ops.DeviceSpmmLhs.from_host(formats.prepare_spmm(mask, vals, 8, 8, layout=layout), cuda)


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [128, 384])
@pytest.mark.parametrize("layout", [formats.VALUES_PACKED, formats.VALUES_SLOT_MAJOR])
def test_dense_ragged(cuda, V, signed, N, layout):
    """Row lengths around every chunk boundary, empty rows, a row count that
    leaves the last 256-row block partly empty; packed and slot-major values."""
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=V + 11)
    vals = synth.random_bytes(mask.nnz_vec * V, 40 + V)
    rhs = synth.random_bytes(K * N, 41 + V)
    out = ops.spmm(_dev(cuda, mask, vals, layout), torch.from_numpy(rhs).to(cuda), N, signed=signed, variant=DENSE,
                   value_layout=layout)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, signed))


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("K", [40, 64, 100, 257, 1024, 1100, 2500])
@pytest.mark.parametrize("layout", [formats.VALUES_PACKED, formats.VALUES_SLOT_MAJOR])
def test_dense_k_segments(cuda, signed, K, layout):
    """k not a multiple of 64 (the last chunk's B rows reach past the matrix
    or into the next batch entry), k across accumulation segments (1024
    columns signed, 256 unsigned), two batch entries with their own A values
    and B."""
    V, B, N = 8, 2, 256
    lengths = np.random.default_rng(K).integers(0, K + 1, size=70)
    lengths[0], lengths[1] = K, 0
    mask = synth.lengths_mask(lengths, K, V, seed=K + 1)
    vals = [synth.random_bytes(mask.nnz_vec * V, 50 + b) for b in range(B)]
    rhs = [synth.random_bytes(K * N, 60 + b) for b in range(B)]
    h = [formats.prepare_spmm(mask, v, 8, 8, layout=layout) for v in vals]
    d = ops.DeviceSpmmLhs.from_host(h[0], cuda)
    vstride = h[0].values.size
    d.values = torch.from_numpy(np.concatenate([x.values for x in h])).to(cuda)
    out = ops.spmm(d, torch.from_numpy(np.concatenate(rhs)).to(cuda), N, signed=signed, batch=B,
                   values_stride=vstride, variant=DENSE, value_layout=layout)
    for b in range(B):
        np.testing.assert_array_equal(out[b].cpu().numpy(), _ref(mask, vals[b], rhs[b], V, K, N, signed))


@pytest.mark.parametrize("signed", [False, True])
def test_dense_extreme_values_at_the_bound(cuda, signed):
    """Every value at the largest product magnitude (-128 x -128 signed, 255 x
    255 unsigned) over full rows: each segment's f32 sum reaches its bound
    (2^24 signed, 256 x 255^2 unsigned) and stays exact."""
    V, K, N = 8, 2048, 128
    mask = synth.lengths_mask([K, K, 5, K - 1], K, V, seed=3)
    byte = 0x80 if signed else 0xFF
    vals = np.full(mask.nnz_vec * V, byte, np.uint8)
    rhs = np.full(K * N, byte, np.uint8)
    out = ops.spmm(_dev(cuda, mask, vals), torch.from_numpy(rhs).to(cuda), N, signed=signed, variant=DENSE)
    ref = _ref(mask, vals, rhs, V, K, N, signed)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_dense_shared_rhs_and_values(cuda):
    """Zero strides share A's values and B across three batch entries."""
    V, K, N, B = 4, 512, 256, 3
    mask = synth.uniform_mask(K // V * 4, K, V, 0.8, seed=5)
    vals = synth.random_bytes(mask.nnz_vec * V, 70)
    rhs = synth.random_bytes(K * N, 71)
    out = ops.spmm(_dev(cuda, mask, vals), torch.from_numpy(rhs).to(cuda), N, signed=True, batch=B,
                   values_stride=0, rhs_stride=0, variant=DENSE)
    ref = _ref(mask, vals, rhs, V, K, N, True)
    for b in range(B):
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("V", [2, 4, 8])
def test_dense_matches_default_kernel_at_headline_shape(cuda, V):
    """1024 x 1024 x 256 at sparsity 0.9, 16 batch entries with their own
    values and B: the dense-tile kernel equals the default kernel on every
    entry and the oracle on two of them."""
    K, N, B = 1024, 256, 16
    mask = synth.uniform_mask(1024 // V, K, V, 0.9, seed=42)
    plain = [synth.random_bytes(mask.nnz_vec * V, 100 + b) for b in range(B)]
    h = [formats.prepare_spmm(mask, v, 8, 8) for v in plain]
    d = ops.DeviceSpmmLhs.from_host(h[0], cuda)
    d.values = torch.from_numpy(np.concatenate([x.values for x in h])).to(cuda)
    rhs = synth.random_bytes(K * N * B, 3)
    rt = torch.from_numpy(rhs).to(cuda)
    kw = dict(signed=True, batch=B, values_stride=h[0].values.size)
    dense = ops.spmm(d, rt, N, variant=DENSE, **kw)
    other = ops.spmm(d, rt, N, variant=_lib.KERNEL_AUTO, **kw)
    torch.testing.assert_close(dense, other, rtol=0, atol=0)
    for b in (0, B - 1):
        np.testing.assert_array_equal(dense[b].cpu().numpy(),
                                      _ref(mask, plain[b], rhs[b * K * N:(b + 1) * K * N], V, K, N, True))


def test_chunk_starts_reject_unsorted_columns(cuda):
    """A vector-row whose columns are not strictly increasing is reported by
    the chunk table and the dense-tile kernel is not used."""
    V, K = 8, 256
    mask = synth.lengths_mask([5, 9], K, V, seed=1)
    cols = mask.col_indices.copy()
    cols[0], cols[1] = cols[1], cols[0]
    bad = formats.VectorSparse(mask.m_vec, mask.vec_length, mask.ncols, mask.row_offsets, cols)
    vals = synth.random_bytes(bad.nnz_vec * V, 1)
    d = _dev(cuda, bad, vals)
    with pytest.raises(_lib.MagicubeError):
        d.chunk_starts()


def test_chunk_starts_table(cuda):
    """The table against a host computation: first slot per 64-column chunk."""
    V, K = 4, 700
    mask = synth.lengths_mask([0, 1, 63, 64, 65, 300, 700, 12], K, V, seed=9)
    d = _dev(cuda, mask, synth.random_bytes(mask.nnz_vec * V, 2))
    got = d.chunk_starts().cpu().numpy()
    h = formats.prepare_spmm(mask, synth.random_bytes(mask.nnz_vec * V, 2), 8, 8)
    nchunks = (K + 63) // 64
    for r in range(mask.m_vec):
        start = h.row_offsets[2 * r]
        cols = mask.col_indices[mask.row_offsets[r]:mask.row_offsets[r + 1]]
        want = [start + int(np.searchsorted(cols, 64 * c)) for c in range(nchunks + 1)]
        assert got[r].tolist() == want


def test_chunk_table_cache_follows_the_mask(cuda):
    """The chunk table is cached, and rebuilt when the mask's columns are
    modified in place or replaced."""
    V, K = 8, 256
    mask = synth.lengths_mask([5, 9, 40], K, V, seed=2)
    d = _dev(cuda, mask, synth.random_bytes(mask.nnz_vec * V, 3))
    t1 = d.chunk_starts()
    assert d.chunk_starts() is t1
    first = d.col_indices[:2].clone()
    d.col_indices[:2] = first.flip(0)  # the first row's columns out of order
    with pytest.raises(_lib.MagicubeError):
        d.chunk_starts()
    d.col_indices = d.col_indices.clone()
    d.col_indices[:2] = first
    assert torch.equal(d.chunk_starts(), t1)
