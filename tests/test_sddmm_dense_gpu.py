"""The dense-tile tcgen05 SDDMM (MC_KERNEL_DENSE_TILE) against the CPU oracle:
bit-exact on ragged rows, partial tiles, batches, extreme values and half
output; its tile bitmap against a host restatement; an unsorted mask is
refused."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

DENSE = _lib.KERNEL_DENSE_TILE
RAGGED = [0, 1, 7, 8, 9, 15, 16, 17, 33, 64, 100, 5, 250, 0, 31, 40, 256, 200, 3, 128]


def _case(V, N, lengths, seed, K=64):
    mask = synth.lengths_mask(lengths, N, V, seed=seed)
    lhs = synth.random_bytes(mask.rows * K, seed + 1)
    rhs = synth.random_bytes(N * K, seed + 2)
    return mask, lhs, rhs


def _timeouts():
    return _lib.lib().mcTensorCoreTimeouts()


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("vecmajor", [False, True])
@pytest.mark.parametrize("N", [256, 200, 1000])
def test_dense_tile_ragged(cuda, V, signed, vecmajor, N):
    """Rows of every length class (empty, shorter than a word, whole column
    blocks, the full width), n not a multiple of 128, m_vec * V not a
    multiple of 256."""
    lengths = [min(n, N) for n in RAGGED] + [N]
    mask, lhs, rhs = _case(V, N, lengths, seed=V + N + int(signed))
    hm = formats.prepare_sddmm(mask, alignment=16 if vecmajor else 8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    t0 = _timeouts()
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), 64, 8, 8, signed=signed,
                    vecmajor=vecmajor, variant=DENSE)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, 64, N, 8, 8,
                            oracle.SIGNED if signed else oracle.UNSIGNED, alignment=8,
                            layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    assert _timeouts() == t0


@pytest.mark.parametrize("V", [2, 8])
@pytest.mark.parametrize("vecmajor", [False, True])
def test_dense_tile_batched_many_items(cuda, V, vecmajor):
    """More work items than SMs (each CTA loops over items with its two A
    buffers and its B ring), several batch entries with their own operands."""
    N, B = 1024, 3
    lengths = np.random.default_rng(V).integers(0, 200, size=700)
    lengths[::31] = 0
    lengths[5] = N
    mask = synth.lengths_mask(lengths, N, V, seed=37)
    hm = formats.prepare_sddmm(mask, alignment=16 if vecmajor else 8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs_all = [synth.random_bytes(mask.rows * 64, 60 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(N * 64, 65 + b) for b in range(B)]
    out = ops.sddmm(dm, torch.from_numpy(np.concatenate(lhs_all)).to(cuda),
                    torch.from_numpy(np.concatenate(rhs_all)).to(cuda), 64, 8, 8, signed=True, batch=B,
                    vecmajor=vecmajor, variant=DENSE)
    for b in range(B):
        ref = oracle.sddmm_host(lhs_all[b], rhs_all[b], hm.row_offsets, hm.col_indices, mask.m_vec, V, 64, N, 8, 8,
                                oracle.SIGNED, layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
def test_dense_tile_extreme_values(cuda, signed, fill):
    """The largest products: 64 x 128^2 (signed) and 64 x 255^2 (unsigned)
    stay exact in the f32 accumulator."""
    V, N = 8, 384
    mask = synth.lengths_mask([384, 3, 17, 0, 64, 8, 100, 1, 200], N, V, seed=19)
    nl, nr = mask.rows * 64, N * 64
    if fill == "alt":
        lhs = np.tile(np.array([0x80, 0x7F], np.uint8), nl // 2 + 1)[:nl]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        lhs, rhs = np.full(nl, fill, np.uint8), np.full(nr, fill, np.uint8)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), 64, 8, 8, signed=signed,
                    variant=DENSE)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, 64, N, 8, 8,
                            oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("V", [2, 4, 8])
def test_dense_tile_half_equals_int8_path(cuda, V):
    """Half scores (the attention's SDDMM output) equal the int8 MMA path's
    bit for bit, padding slots included."""
    N, scale = 512, 36.0 * 36.0
    mask, lhs, rhs = _case(V, N, [min(n, N) for n in RAGGED], seed=43 + V)
    hm = formats.prepare_sddmm(mask, alignment=16)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    args = (dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), 64, 8, 8)
    a = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, variant=DENSE,
                  out=torch.full((hm.aligned_nnz * V,), 7.0, dtype=torch.float16, device=cuda))
    b = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, mma_kind=_lib.MMA_INT8,
                  out=torch.full((hm.aligned_nnz * V,), 7.0, dtype=torch.float16, device=cuda))
    np.testing.assert_array_equal(a.cpu().numpy().view(np.uint16), b.cpu().numpy().view(np.uint16))


def test_tile_mask_matches_host(cuda):
    """mcSddmmTileMask: bits of the stored columns, prefix = stored columns
    below each word."""
    V, N = 4, 300
    mask, _, _ = _case(V, N, [0, 1, 31, 32, 33, 64, 200, 300, 7], seed=5)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    bitmap, prefix = dm.tile_mask()
    words = _lib.lib().mcSddmmTileMaskWords(N)
    assert words == 12 and bitmap.shape == (mask.m_vec, words)
    bm, pf = bitmap.cpu().numpy().view(np.uint32), prefix.cpu().numpy()
    for r in range(mask.m_vec):
        s, e = hm.row_offsets[2 * r], hm.row_offsets[2 * r + 1]
        cols = hm.col_indices[s:e]
        for w in range(words):
            sel = cols[(cols >= 32 * w) & (cols < 32 * w + 32)]
            assert bm[r, w] == sum(1 << int(c - 32 * w) for c in sel)
            assert pf[r, w] == int((cols < 32 * w).sum())


def test_tile_mask_refuses_unsorted(cuda):
    V, N = 8, 256
    mask, lhs, rhs = _case(V, N, [16, 16], seed=3)
    hm = formats.prepare_sddmm(mask)
    cols = hm.col_indices.copy()
    s = hm.row_offsets[0]
    cols[s], cols[s + 1] = cols[s + 1], cols[s]  # swap two columns of row 0
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    dm.col_indices = torch.from_numpy(cols).to(cuda)
    with pytest.raises(_lib.MagicubeError, match="strictly increasing"):
        dm.tile_mask()


def test_tile_mask_cache_follows_the_mask(cuda):
    """The bitmap is cached, and rebuilt when the mask's columns are modified
    in place (here: two columns swapped, then swapped back)."""
    V, N = 8, 256
    mask, _, _ = _case(V, N, [16, 40], seed=6)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    t1 = dm.tile_mask()
    assert dm.tile_mask() is t1
    s = int(hm.row_offsets[0])
    first = dm.col_indices[s:s + 2].clone()
    dm.col_indices[s:s + 2] = first.flip(0)
    with pytest.raises(_lib.MagicubeError, match="strictly increasing"):
        dm.tile_mask()
    dm.col_indices[s:s + 2] = first
    b2, p2 = dm.tile_mask()
    assert torch.equal(b2, t1[0]) and torch.equal(p2, t1[1])


def test_dense_tile_rejects(cuda):
    V, N = 8, 256
    mask, lhs, rhs = _case(V, N, [16, 16], seed=3)
    dm = ops.DeviceSddmmMask.from_host(formats.prepare_sddmm(mask), cuda)
    with pytest.raises(_lib.MagicubeError, match="L8-R8 with k == 64"):
        ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), 64, 4, 4, variant=DENSE)
    import ctypes
    d = _lib.McSddmmDesc(m_vec=mask.m_vec, vec_length=V, n=N, k=64, lhs_bits=8, rhs_bits=8, is_signed=1, scale=1.0,
                         batch=1, row_indices=dm.row_indices.data_ptr(), row_offsets=dm.row_offsets.data_ptr(),
                         column_indices=dm.col_indices.data_ptr(), lhs=dm.row_offsets.data_ptr(),
                         rhs=dm.row_offsets.data_ptr(), out=dm.row_offsets.data_ptr(), kernel_variant=DENSE)
    assert _lib.lib().mcSddmm(ctypes.byref(d), None) != 0  # no tile bitmap
    assert "tile bitmap" in _lib.lib().mcGetLastErrorString().decode()
