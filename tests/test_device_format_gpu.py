"""The GPU packer (mcDevice*) against the host packer and the reference's own
packed arrays: byte-identical aligned pairs, padded columns and values."""
import numpy as np
import pytest
import torch

import oracle
from golden_util import load, names, unpack_spmm_values
from magicube_gb300 import device_format as dfm
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

PAIRS = [(4, 4), (8, 4), (16, 4), (8, 8), (16, 8), (12, 4), (12, 8), (16, 16)]


def _dev(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _stable_order(row_offsets):
    return np.argsort(-np.diff(row_offsets), kind="stable").astype(np.int32)


def _check_spmm(m, vals, pa, pb, layout, dev, sync=True):
    h = formats.prepare_spmm(m, vals, pa, pb, layout=layout)
    d = dfm.prepare_spmm(_dev(m.row_offsets, dev), _dev(m.col_indices, dev), _dev(vals, dev), m.vec_length,
                         m.ncols, pa, pb, layout=layout, sync=sync)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.row_offsets.cpu().numpy(), h.row_offsets)
    n = h.aligned_nnz
    np.testing.assert_array_equal(d.col_indices.cpu().numpy()[:n], h.col_indices)
    nb = n * m.vec_length * formats.lane_bits(pa) // 8
    np.testing.assert_array_equal(d.values.cpu().numpy()[:nb], h.values)
    np.testing.assert_array_equal(d.row_indices.cpu().numpy(), _stable_order(m.row_offsets))
    return h, d


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("layout", [formats.VALUES_PACKED, formats.VALUES_SOFTMAX])
def test_device_packer_equals_host_packer(cuda, pa, pb, V, layout):
    if pa == 12 and layout == formats.VALUES_SOFTMAX:
        pytest.skip("12-bit values have the packed layout only")
    m = synth.lengths_mask([0, 1, 15, 16, 17, 31, 32, 33, 100, 0, 7, 64], 256, V, seed=pa * 7 + pb + V)
    vals = synth.random_bytes(m.nnz_vec * V * formats.lane_bits(pa) // 8, V + pa)
    _check_spmm(m, vals, pa, pb, layout, cuda)


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("offset", [0, 1])
def test_device_slot_major_equals_host(cuda, V, offset):
    """Slot-major 8-bit values ([aligned slot][V] bytes, zero padding) from the
    GPU packer equal the host packer's, from an aligned and an odd source
    address; the separate values entry point writes the same bytes."""
    m = synth.lengths_mask([0, 1, 15, 16, 17, 31, 32, 33, 100, 0, 7, 64, 250], 256, V, seed=V + 3)
    vals = synth.random_bytes(m.nnz_vec * V, V + 21)
    buf = torch.zeros(vals.size + offset, dtype=torch.uint8, device=cuda)
    buf[offset:] = _dev(vals, cuda)
    h = formats.prepare_spmm(m, vals, 8, 8, layout=formats.VALUES_SLOT_MAJOR)
    d = dfm.prepare_spmm(_dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), buf[offset:], V, m.ncols, 8, 8,
                         layout=formats.VALUES_SLOT_MAJOR)
    np.testing.assert_array_equal(d.row_offsets.cpu().numpy(), h.row_offsets)
    np.testing.assert_array_equal(d.col_indices.cpu().numpy(), h.col_indices)
    np.testing.assert_array_equal(d.values.cpu().numpy(), h.values)
    n = torch.tensor([h.aligned_nnz], dtype=torch.int32, device=cuda)
    sep = dfm.pack_spmm_values(_dev(m.row_offsets, cuda), d.row_offsets, n, buf[offset:], V, 8, 8, h.aligned_nnz,
                               layout=formats.VALUES_SLOT_MAJOR)
    np.testing.assert_array_equal(sep.cpu().numpy(), h.values)


def test_device_slot_major_feeds_dense_tile_spmm(cuda):
    """A slot-major operand packed on the GPU gives the dense-tile SpMM the
    oracle's result bit for bit, named or picked by MC_KERNEL_AUTO."""
    V, K, N = 8, 512, 256
    m = synth.uniform_mask(96, K, V, 0.8, seed=17)
    vals = synth.random_bytes(m.nnz_vec * V, 18)
    rhs = synth.random_bytes(K * N, 19)
    d = dfm.prepare_spmm(_dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), _dev(vals, cuda), V, m.ncols, 8, 8,
                         layout=formats.VALUES_SLOT_MAJOR)
    out = ops.spmm(d, _dev(rhs, cuda), N, signed=True, variant=_lib.KERNEL_DENSE_TILE,
                   value_layout=formats.VALUES_SLOT_MAJOR)
    ref = oracle.spmm_host(vals, rhs, m.row_offsets, m.col_indices, m.m_vec, V, K, N, 8, 8, oracle.SIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    auto = ops.spmm(d, _dev(rhs, cuda), N, signed=True, value_layout=formats.VALUES_SLOT_MAJOR)
    assert torch.equal(auto, out)


@pytest.mark.parametrize("name", names("ref_spmm_"))
def test_device_packer_reproduces_reference_packer(cuda, name):
    """Plain CSR + original values from the reference's own run -> the exact
    device arrays the reference's packer produced."""
    d = load(name)
    V, pa, pb = int(d["V"]), int(d["preA"]), int(d["preB"])
    ro, ci = d["csr_row_offsets"], d["csr_col_indices"]
    orig = unpack_spmm_values(d["values"], d["row_offsets"], ro, V, pa, pb)
    dv = dfm.prepare_spmm(_dev(ro, cuda), _dev(ci, cuda), _dev(orig, cuda), V, int(d["K"]), pa, pb)
    np.testing.assert_array_equal(dv.row_offsets.cpu().numpy(), d["row_offsets"])
    np.testing.assert_array_equal(dv.col_indices.cpu().numpy(), d["col_indices"])
    np.testing.assert_array_equal(dv.values.cpu().numpy(), d["values"])
    # The reference orders equal-length rows by std::sort (unspecified); the
    # lengths along both orders agree.
    lens = np.diff(ro)
    np.testing.assert_array_equal(lens[dv.row_indices.cpu().numpy()], lens[d["row_indices"]])


@pytest.mark.parametrize("name", names("ref_sddmm_"))
def test_device_sddmm_mask_reproduces_reference(cuda, name):
    d = load(name)
    ro, ci = d["csr_row_offsets"], d["csr_col_indices"]
    dm = dfm.prepare_sddmm(_dev(ro, cuda), _dev(ci, cuda), int(d["V"]), int(d["N"]))
    np.testing.assert_array_equal(dm.row_offsets.cpu().numpy(), d["row_offsets"])
    np.testing.assert_array_equal(dm.col_indices.cpu().numpy(), d["col_indices"])


@pytest.mark.parametrize("alignment", [8, 16, 32])
def test_device_sddmm_mask_equals_host(cuda, alignment):
    m = synth.normal_mask(300, 1000, 8, 0.9, seed=alignment)
    h = formats.prepare_sddmm(m, alignment)
    dm = dfm.prepare_sddmm(_dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), 8, m.ncols, alignment=alignment)
    assert dm.aligned_nnz == h.aligned_nnz
    np.testing.assert_array_equal(dm.row_offsets.cpu().numpy(), h.row_offsets)
    np.testing.assert_array_equal(dm.col_indices.cpu().numpy(), h.col_indices)


@pytest.mark.parametrize("m_vec", [1, 1023, 1024, 1025, 2048, 4095, 4096, 4097, 9000, 16383, 16384, 16385, 20011])
def test_multi_tile_scan(cuda, m_vec):
    """Row counts on and across the 1,024-row scan tiles of the align step."""
    m = synth.normal_mask(m_vec, 512, 4, 0.95, seed=m_vec)
    vals = synth.random_bytes(m.nnz_vec * 4, 5)
    _check_spmm(m, vals, 8, 8, formats.VALUES_PACKED, cuda)


def test_empty_and_zero_rows(cuda):
    m = synth.lengths_mask([0, 0, 0], 64, 4, seed=1)
    h, d = _check_spmm(m, np.zeros(0, np.uint8), 8, 8, formats.VALUES_PACKED, cuda)
    assert h.aligned_nnz == 0
    pairs, n = dfm.align_row_offsets(torch.zeros(1, dtype=torch.int32, device=cuda), 16)
    assert pairs.numel() == 0 and int(n.item()) == 0


def test_unsynchronised_upper_bound_operand_computes_same_spmm(cuda):
    """sync=False: buffers sized by the upper bound, no host round trip; the
    SpMM result equals the one on the host-packed operand."""
    m = synth.normal_mask(64, 256, 8, 0.8, seed=9)
    vals = synth.random_bytes(m.nnz_vec * 8, 3)
    h, d = _check_spmm(m, vals, 8, 8, formats.VALUES_PACKED, cuda, sync=False)
    rhs = torch.randint(0, 256, (256 * 128,), dtype=torch.uint8, device=cuda)
    a = ops.spmm(ops.DeviceSpmmLhs.from_host(h, cuda), rhs, 128)
    b = ops.spmm(d, rhs, 128)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_non_monotone_offsets_are_reported(cuda):
    ro = torch.tensor([0, 5, 3, 9], dtype=torch.int32, device=cuda)
    ci = torch.arange(9, dtype=torch.int32, device=cuda)
    pairs, n = dfm.align_row_offsets(ro, 16)
    assert int(n.item()) == -1
    with pytest.raises(dfm.PackError):
        dfm.prepare_spmm(ro, ci, torch.zeros(9 * 8, dtype=torch.uint8, device=cuda), 8, 16, 8, 8)


def test_capacity_too_small_is_reported(cuda):
    m = synth.lengths_mask([20, 20], 64, 8, seed=2)
    ro, ci = _dev(m.row_offsets, cuda), _dev(m.col_indices, cuda)
    pairs, n = dfm.align_row_offsets(ro, 16)
    assert int(n.item()) == 64
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    dfm.pad_column_indices(ro, ci, pairs, n, False, 48, status)
    assert int(status.item()) == 1
    status.zero_()
    dfm.pad_column_indices(ro, ci, pairs, n, False, 64, status)
    assert int(status.item()) == 0


@pytest.mark.parametrize("pa,pb", [(8, 4), (16, 8)])
def test_separate_entry_points_equal_fused_pack(cuda, pa, pb):
    """mcDeviceAlignRowOffsets + mcDevicePadColumnIndices +
    mcDevicePackSpmmValues + mcDeviceSortedRowSwizzle == one mcDevicePack."""
    V = 4
    m = synth.normal_mask(777, 900, V, 0.9, seed=pa + pb)
    vals = synth.random_bytes(m.nnz_vec * V * pa // 8, 4)
    ro, ci, dv = _dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), _dev(vals, cuda)
    chunk = formats.spmm_chunk(pa, pb)
    fused = dfm.prepare_spmm(ro, ci, dv, V, m.ncols, pa, pb)
    pairs, n = dfm.align_row_offsets(ro, chunk)
    cap = int(n.item())
    cols = dfm.pad_column_indices(ro, ci, pairs, n, chunk == 32, cap)
    packed = dfm.pack_spmm_values(ro, pairs, n, dv, V, pa, pb, cap)
    order = dfm.sorted_row_swizzle(ro)
    assert torch.equal(pairs, fused.row_offsets)
    assert torch.equal(cols, fused.col_indices)
    assert torch.equal(packed, fused.values)
    assert torch.equal(order, fused.row_indices)


def test_unsorted_rows_keep_identity_order(cuda):
    m = synth.normal_mask(100, 300, 8, 0.8, seed=5)
    d = dfm.prepare_sddmm(_dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), 8, m.ncols, sort_rows=False)
    np.testing.assert_array_equal(d.row_indices.cpu().numpy(), np.arange(100, dtype=np.int32))


@pytest.mark.parametrize("V", [2, 4, 8])
def test_unaligned_values_pointer_takes_generic_path(cuda, V):
    """8-bit values at an odd address: the byte-gather path, same bytes."""
    m = synth.normal_mask(50, 400, V, 0.8, seed=V)
    vals = synth.random_bytes(m.nnz_vec * V, 6)
    h = formats.prepare_spmm(m, vals, 8, 8)
    buf = torch.zeros(vals.size + 1, dtype=torch.uint8, device=cuda)
    buf[1:] = _dev(vals, cuda)
    d = dfm.prepare_spmm(_dev(m.row_offsets, cuda), _dev(m.col_indices, cuda), buf[1:], V, m.ncols, 8, 8)
    np.testing.assert_array_equal(d.values.cpu().numpy(), h.values)
