"""Host-side logic of the batched attention and the server (CPU only)."""
import numpy as np
import torch

import oracle.attention as oatt
from magicube_gb300 import batched, formats, serving, synth


def test_block_diagonal_mask():
    masks = [synth.band_random_mask(L, 8, 32, 0.7, seed=i) for i, L in enumerate([64, 128, 32])]
    mega, tok = batched.block_diagonal(masks)
    assert list(tok) == [0, 64, 192, 224]
    assert mega.m_vec == sum(m.m_vec for m in masks) and mega.ncols == 224
    dense = np.zeros((224, 224), bool)
    for m, t0 in zip(masks, tok[:-1]):
        pairs, n = formats.align_row_offsets(m, 8)
        cols = formats.pad_column_indices(m, pairs, n, False)
        dense[t0:t0 + m.ncols, t0:t0 + m.ncols] = oatt.dense_mask(pairs, cols, m.m_vec, 8, m.ncols)
    pairs, n = formats.align_row_offsets(mega, 8)
    cols = formats.pad_column_indices(mega, pairs, n, False)
    np.testing.assert_array_equal(oatt.dense_mask(pairs, cols, mega.m_vec, 8, 224), dense)


def test_batch_masks_on_device_arrays_match_block_diagonal():
    reqs = serving.make_requests(4, rate=0.0, hidden=32, layers=2, sparsity=0.9, median=128, clip=(64, 256), seed=1)
    for r in reqs:
        serving._upload(r, 16, "cpu")
    got = serving.batch_masks(reqs, 2, 8)
    for layer in range(2):
        mega, _ = batched.block_diagonal([r.masks[layer] for r in reqs])
        pairs, n = formats.align_row_offsets(mega, 16)
        cols = formats.pad_column_indices(mega, pairs, n, False)
        assert got[layer].aligned_nnz == n and got[layer].m_vec == mega.m_vec
        np.testing.assert_array_equal(got[layer].row_offsets.numpy(), pairs)
        np.testing.assert_array_equal(got[layer].col_indices.numpy(), cols)
        assert sorted(got[layer].row_indices.tolist()) == list(range(mega.m_vec))


def test_request_generator_shapes():
    reqs = serving.make_requests(20, rate=100.0, hidden=16, layers=2, median=2048, clip=(256, 8192), seed=2)
    lens = [r.seq_len for r in reqs]
    assert all(256 <= L <= 8192 and L % 64 == 0 for L in lens)
    arr = [r.arrival for r in reqs]
    assert arr == sorted(arr) and arr[0] == 0.0
    assert all(len(r.masks) == 2 and r.masks[0].m_vec == r.seq_len // 8 for r in reqs)


def test_footprint_grows_with_batch():
    reqs = serving.make_requests(3, rate=0.0, hidden=64, layers=2, median=512, clip=(256, 1024), seed=4)
    f1 = serving.footprint_bytes(reqs[:1], 64, 4, 2, 8)
    f3 = serving.footprint_bytes(reqs, 64, 4, 2, 8)
    assert 0 < f1 < f3


def test_rowwise_fp64_attention_equals_dense_fp64():
    """The vector-row-wise float64 attention oracle (gathered K and V rows)
    equals the dense-mask form, including a row without nonzeros."""
    import oracle
    from oracle import attention as oa
    m = synth.band_random_mask(256, 8, 64, 0.8, seed=3)
    ro = m.row_offsets.copy()
    ro[5:] -= ro[5] - ro[4]  # vector-row 4 left empty
    cols = np.concatenate([m.col_indices[:ro[4]], m.col_indices[m.row_offsets[5]:]])
    rng = np.random.default_rng(0)
    q, k, v = (rng.standard_normal((2, 256, 64)) for _ in range(3))
    pairs, n = oracle.align_pairs(ro, 16)
    mk = oa.dense_mask(pairs, oracle.pad_columns(ro, cols, pairs, n), m.m_vec, 8, 256)
    a = oa.sparse_attention_fp64(q, k, v, mk, 0.125)
    b = oa.sparse_attention_fp64_rows(q, k, v, ro, cols, 8, 0.125)
    np.testing.assert_allclose(b, a, rtol=0, atol=1e-12)
    assert not b[:, 32:40].any()
