"""Host-side format code: .smtx round trip and packer edge cases.  CPU only."""
import numpy as np
import pytest

import oracle
from magicube_gb300 import formats, smtx, synth


def test_smtx_round_trip(tmp_path):
    m = synth.normal_mask(33, 500, 4, 0.7, seed=3)
    smtx.write(tmp_path / "m.smtx", m)
    r = smtx.read(tmp_path / "m.smtx", 4)
    assert (r.m_vec, r.ncols) == (33, 500)
    np.testing.assert_array_equal(r.row_offsets, m.row_offsets)
    np.testing.assert_array_equal(r.col_indices, m.col_indices)


def test_smtx_rejects_malformed(tmp_path):
    p = tmp_path / "bad.smtx"
    p.write_text("2, 10, 3\n0 2 1\n1 2 3\n")
    with pytest.raises(ValueError):
        smtx.read(p, 2)
    p.write_text("1, 4, 2\n0 2\n1 9\n")
    with pytest.raises(ValueError):
        smtx.read(p, 2)
    p.write_text("-1, 4, 0\n0\n\n")
    with pytest.raises(ValueError, match="header out of range"):
        smtx.read(p, 2)


@pytest.mark.parametrize("alignment", [8, 16, 32])
def test_alignment_edges(alignment):
    m = synth.lengths_mask([0, 1, alignment - 1, alignment, alignment + 1, 0], 256, 8, seed=1)
    pairs, n = formats.align_row_offsets(m, alignment)
    assert n % alignment == 0
    assert np.all(pairs[0::2] % alignment == 0)
    np.testing.assert_array_equal(pairs[1::2] - pairs[0::2], m.row_lengths())


@pytest.mark.parametrize("pa,pb", [(4, 4), (8, 4), (16, 4), (8, 8), (16, 8)])
@pytest.mark.parametrize("V", [2, 4, 8])
def test_pack_then_decode_equals_oracle(pa, pb, V):
    """Packer + the oracle's device-layout decoder == oracle on the original layout."""
    K, N = 128, 64
    m = synth.lengths_mask([0, 1, 31, 32, 33, 100, 7], K, V, seed=pa + pb + V)
    vals = synth.random_bytes(m.nnz_vec * V * pa // 8, 1)
    rhs = synth.random_bytes(K * N * pb // 8, 2)
    for layout in (formats.VALUES_PACKED, formats.VALUES_SOFTMAX):
        h = formats.prepare_spmm(m, vals, pa, pb, layout=layout)
        for mode in (oracle.UNSIGNED, oracle.SIGNED):
            a = oracle.spmm_host(vals, rhs, m.row_offsets, m.col_indices, m.m_vec, V, K, N, pa, pb, mode)
            b = oracle.spmm_device(h.row_offsets, h.col_indices, h.values, rhs, m.m_vec, V, K, N, pa, pb, mode,
                                   layout)
            np.testing.assert_array_equal(a, b)


def test_empty_matrix_packs():
    m = synth.lengths_mask([0, 0, 0], 64, 4, seed=1)
    h = formats.prepare_spmm(m, np.zeros(0, np.uint8), 8, 8)
    assert h.aligned_nnz == 0 and h.values.size == 0


@pytest.mark.parametrize("pa,pb", [(12, 4), (12, 8), (16, 16)])
@pytest.mark.parametrize("V", [2, 4, 8])
def test_pack_then_decode_wide_pairs(pa, pb, V):
    """12-bit values (16-bit lanes, top 4 bits dropped by the packer) and
    16 x 16: packer + the oracle's device-layout decoder == oracle on the
    original layout."""
    K, N = 128, 64
    m = synth.lengths_mask([0, 1, 31, 32, 33, 100, 7], K, V, seed=pa + pb + V)
    vals = synth.random_bytes(m.nnz_vec * V * 2, 1)
    rhs = synth.random_bytes(K * N * pb // 8, 2)
    h = formats.prepare_spmm(m, vals, pa, pb)
    modes = (oracle.UNSIGNED,) if pa == 12 else (oracle.UNSIGNED, oracle.SIGNED)
    for mode in modes:
        a = oracle.spmm_host(vals, rhs, m.row_offsets, m.col_indices, m.m_vec, V, K, N, 16, pb, mode, preA_cut=pa)
        b = oracle.spmm_device(h.row_offsets, h.col_indices, h.values, rhs, m.m_vec, V, K, N, 16, pb, mode)
        np.testing.assert_array_equal(a, b)


def test_slot_major_layout_on_the_host():
    """The slot-major layout is the plain values of each slot side by side at
    the slot's aligned position, zeros in the padding slots."""
    V, K = 4, 256
    mask = synth.lengths_mask([3, 0, 17, 5], K, V, seed=2)
    vals = synth.random_bytes(mask.nnz_vec * V, 3)
    h = formats.prepare_spmm(mask, vals, 8, 8, layout=formats.VALUES_SLOT_MAJOR)
    got = h.values.reshape(-1, V)
    for r in range(mask.m_vec):
        start, n = h.row_offsets[2 * r], mask.row_offsets[r + 1] - mask.row_offsets[r]
        want = vals.reshape(-1, V)[mask.row_offsets[r]:mask.row_offsets[r + 1]]
        np.testing.assert_array_equal(got[start:start + n], want)
        end = h.aligned_nnz if r == mask.m_vec - 1 else h.row_offsets[2 * r + 2]
        assert not got[start + n:end].any()


def test_slot_major_host_packer_refusals():
    """The host packer writes slot-major values for L8-R8 only, and refuses an
    aligned count that the rows' slots overrun."""
    import ctypes
    from magicube_gb300 import _lib
    lib = _lib.lib()
    ro = np.array([0, 3], np.int32)
    pairs = np.array([0, 3], np.int32)
    vals = np.arange(3 * 8, dtype=np.uint8)
    out = np.zeros(16 * 8, np.uint8)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = lib.mcPackSpmmValuesEx(1, 8, 8, 4, p(ro), p(pairs), 16, p(vals), p(out), _lib.VALUES_SLOT_MAJOR)
    assert rc == 1 and b"invalid arguments" in lib.mcGetLastErrorString()
    rc = lib.mcPackSpmmValuesEx(1, 8, 8, 8, p(ro), p(pairs), 2, p(vals), p(out), _lib.VALUES_SLOT_MAJOR)
    assert rc == 1 and b"aligned_nnz too small" in lib.mcGetLastErrorString()
    rc = lib.mcPackSpmmValuesEx(1, 8, 8, 8, p(ro), p(pairs), 16, p(vals), p(out), _lib.VALUES_SLOT_MAJOR)
    assert rc == 0
    np.testing.assert_array_equal(out[:24], vals)
    assert not out[24:].any()


def test_host_packer_refuses_bad_offsets_without_writing_out_of_bounds():
    """Negative aligned starts, missing arrays and sizes beyond the int range
    are refused before any write."""
    import ctypes
    from magicube_gb300 import _lib
    lib = _lib.lib()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    ro = np.array([0, 3], np.int32)
    cols = np.array([1, 5, 9], np.int32)
    bad_pairs = np.array([-16, -13], np.int32)
    out_cols = np.zeros(16, np.int32)
    assert lib.mcPadColumnIndices(1, p(ro), p(cols), p(bad_pairs), 16, 0, p(out_cols)) == 1
    assert b"negative aligned start" in lib.mcGetLastErrorString()
    pairs = np.array([0, 3], np.int32)
    assert lib.mcPadColumnIndices(1, p(ro), None, p(pairs), 16, 0, p(out_cols)) == 1
    assert b"null col_indices" in lib.mcGetLastErrorString()
    vals = np.zeros(3 * 8, np.uint8)
    out = np.zeros(16 * 8, np.uint8)
    for layout in (_lib.VALUES_PACKED, _lib.VALUES_SLOT_MAJOR):
        assert lib.mcPackSpmmValuesEx(1, 8, 8, 8, p(ro), p(bad_pairs), 16, p(vals), p(out), layout) == 1
        assert b"negative aligned start" in lib.mcGetLastErrorString()
        assert lib.mcPackSpmmValuesEx(1, 8, 8, 8, p(ro), p(pairs), 16, None, p(out), layout) == 1
        assert b"null values" in lib.mcGetLastErrorString()
    huge = np.array([0, 2_147_483_641], np.int32)  # rounds up past the int range
    apairs = np.zeros(4, np.int32)
    assert lib.mcAlignRowOffsets(1, p(huge), 16, p(apairs)) == -1
    assert b"overflows int" in lib.mcGetLastErrorString()
    spread = np.array([-2_000_000_000, 2_000_000_000], np.int32)  # a length beyond the int range
    assert lib.mcAlignRowOffsets(1, p(spread), 16, p(apairs)) == -1
    assert b"overflows int" in lib.mcGetLastErrorString()
