"""SDDMM parity on the GPU: the CUDA library against the CPU oracle (bit-exact)."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

PAIRS = [(4, 4), (8, 8), (16, 8), (16, 16)]
RAGGED = [0, 1, 7, 8, 9, 15, 16, 17, 33, 64, 100, 5, 250, 0, 31, 40]


def _case(pa, pb, V, K, N, lengths, seed):
    mask = synth.lengths_mask(lengths, N, V, seed=seed)
    lhs = synth.random_bytes(mask.rows * K * pa // 8, seed + 1)
    rhs = synth.random_bytes(N * K * pb // 8, seed + 2)
    return mask, lhs, rhs


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("K", [64, 192])
@pytest.mark.parametrize("vecmajor", [False, True])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
@pytest.mark.parametrize("variant", [_lib.KERNEL_PER_ROW, _lib.KERNEL_AUTO])
def test_sddmm_ragged(cuda, pa, pb, V, signed, K, vecmajor, mma, variant):
    N = 256
    mask, lhs, rhs = _case(pa, pb, V, K, N, RAGGED, seed=pa + pb + V + K)
    align = 16 if vecmajor else 8
    hm = formats.prepare_sddmm(mask, alignment=align)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb,
                    signed=signed, vecmajor=vecmajor, mma_kind=mma, variant=variant)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, pa, pb,
                            oracle.SIGNED if signed else oracle.UNSIGNED, alignment=8,
                            layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
def test_sddmm_extreme_values_large_k(cuda, pa, pb, signed, fill, mma):
    """Extreme lane values with K = 1024 (four f32 flush intervals on the f16 path)."""
    V, K, N = 8, 1024, 128
    mask = synth.lengths_mask([128, 3, 17, 0, 64, 8, 100, 1], N, V, seed=19)
    nl, nr = mask.rows * K * pa // 8, N * K * pb // 8
    if fill == "alt":
        lhs = np.tile(np.array([0x80, 0x7F], np.uint8), nl // 2 + 1)[:nl]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        lhs, rhs = np.full(nl, fill, np.uint8), np.full(nr, fill, np.uint8)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb, signed=signed,
                    mma_kind=mma)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, pa, pb,
                            oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
@pytest.mark.parametrize("V", [2, 8])
@pytest.mark.parametrize("mma", [_lib.MMA_INT8, _lib.MMA_F16])
@pytest.mark.parametrize("vecmajor", [False, True])
def test_sddmm_streaming_many_tasks(cuda, pa, pb, V, mma, vecmajor):
    """Far more tasks than resident warps: each warp streams many rows."""
    K, N, B = 64, 1024, 4
    lengths = np.random.default_rng(pa + pb + V).integers(0, 60, size=1024)
    lengths[::29] = 0
    lengths[3] = 1024
    mask = synth.lengths_mask(lengths, N, V, seed=29)
    hm = formats.prepare_sddmm(mask, alignment=16 if vecmajor else 8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs_all = [synth.random_bytes(mask.rows * K * pa // 8, 70 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(N * K * pb // 8, 80 + b) for b in range(B)]
    out = ops.sddmm(dm, torch.from_numpy(np.concatenate(lhs_all)).to(cuda),
                    torch.from_numpy(np.concatenate(rhs_all)).to(cuda), K, pa, pb, signed=True, batch=B,
                    vecmajor=vecmajor, mma_kind=mma, variant=_lib.KERNEL_STREAM)
    for b in range(B):
        ref = oracle.sddmm_host(lhs_all[b], rhs_all[b], hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N,
                                pa, pb, oracle.SIGNED,
                                layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", PAIRS)
def test_sddmm_batched(cuda, pa, pb):
    V, K, N, B = 8, 64, 512, 3
    mask = synth.normal_mask(16, N, V, 0.8, seed=3)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs_all = [synth.random_bytes(mask.rows * K * pa // 8, 30 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(N * K * pb // 8, 40 + b) for b in range(B)]
    out = ops.sddmm(dm, torch.from_numpy(np.concatenate(lhs_all)).to(cuda),
                    torch.from_numpy(np.concatenate(rhs_all)).to(cuda), K, pa, pb, signed=True, batch=B)
    for b in range(B):
        ref = oracle.sddmm_host(lhs_all[b], rhs_all[b], hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N,
                                pa, pb, oracle.SIGNED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", [(4, 4), (8, 8)])
def test_sddmm_half_vecmajor(cuda, pa, pb):
    V, K, N, scale = 8, 64, 256, 36.0 * 36.0
    mask, lhs, rhs = _case(pa, pb, V, K, N, RAGGED, seed=9)
    hm = formats.prepare_sddmm(mask, alignment=16)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb, signed=True,
                    vecmajor=True, out_half=True, scale=scale)
    acc = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, pa, pb, oracle.SIGNED,
                            layout=oracle.OUT_VECMAJOR)
    ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    got = out.cpu().numpy()
    # padding slots (never written by either side) are compared only where the oracle wrote
    written = np.zeros(acc.size, bool)
    for i in range(mask.m_vec):
        s, e = hm.row_offsets[2 * i], hm.row_offsets[2 * i + 1]
        written[s * V:e * V] = True
    np.testing.assert_array_equal(got[written].view(np.uint16), ref[written].view(np.uint16))


@pytest.mark.parametrize("name,bits", [("4b", 4), ("8b", 8), ("16b", 16)])
def test_reference_entry_points(cuda, name, bits):
    """mcWmmaSddmm_<P>: reference argument list, unsigned lanes, blocked output."""
    V, K, N = 8, 128, 256
    mask, lhs, rhs = _case(bits, bits, V, K, N, RAGGED, seed=13)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lt, rt = torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda)
    out = torch.zeros(hm.aligned_nnz * V, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    fn = getattr(_lib.lib(), f"mcWmmaSddmm_{name}")
    _lib.check(fn(mask.m_vec, K, N, dm.row_indices.data_ptr(), dm.row_offsets.data_ptr(), dm.col_indices.data_ptr(),
                  lt.data_ptr(), rt.data_ptr(), out.data_ptr(), V), name)
    torch.cuda.synchronize()
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, bits, bits,
                            oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


DP4A_PAIRS = [(4, 4), (8, 8)]


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("K", [64, 192])
@pytest.mark.parametrize("vecmajor", [False, True])
def test_sddmm_dp4a_ragged(cuda, pa, pb, V, signed, K, vecmajor):
    """The CUDA-core dp4a path: bit-exact against the oracle on ragged rows
    (empty, shorter than a tile, odd lengths), every V, both layouts."""
    N = 256
    mask, lhs, rhs = _case(pa, pb, V, K, N, RAGGED, seed=pa + pb + V + K + 1)
    hm = formats.prepare_sddmm(mask, alignment=16 if vecmajor else 8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb,
                    signed=signed, vecmajor=vecmajor, mma_kind=_lib.MMA_DP4A)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, pa, pb,
                            oracle.SIGNED if signed else oracle.UNSIGNED, alignment=8,
                            layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
@pytest.mark.parametrize("V", [2, 8])
def test_sddmm_dp4a_extreme_values(cuda, pa, pb, signed, fill, V):
    """Extreme lane values with K = 1024: the int32 dp4a chains hold every
    exact sum."""
    K, N = 1024, 128
    mask = synth.lengths_mask([128, 3, 17, 0, 64, 8, 100, 1], N, V, seed=19)
    nl, nr = mask.rows * K * pa // 8, N * K * pb // 8
    if fill == "alt":
        lhs = np.tile(np.array([0x80, 0x7F], np.uint8), nl // 2 + 1)[:nl]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        lhs, rhs = np.full(nl, fill, np.uint8), np.full(nr, fill, np.uint8)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb, signed=signed,
                    mma_kind=_lib.MMA_DP4A)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, pa, pb,
                            oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("vecmajor", [False, True])
def test_sddmm_dp4a_many_tasks_batched(cuda, V, vecmajor):
    """Many rows per launch (one row 1024 long), several batch entries, row
    split chosen by the library."""
    pa = pb = 8
    K, N, B = 64, 1024, 3
    lengths = np.random.default_rng(V).integers(0, 60, size=1024)
    lengths[::29] = 0
    lengths[3] = 1024
    mask = synth.lengths_mask(lengths, N, V, seed=31)
    hm = formats.prepare_sddmm(mask, alignment=16 if vecmajor else 8)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs_all = [synth.random_bytes(mask.rows * K * pa // 8, 90 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(N * K * pb // 8, 95 + b) for b in range(B)]
    out = ops.sddmm(dm, torch.from_numpy(np.concatenate(lhs_all)).to(cuda),
                    torch.from_numpy(np.concatenate(rhs_all)).to(cuda), K, pa, pb, signed=True, batch=B,
                    vecmajor=vecmajor, mma_kind=_lib.MMA_DP4A)
    for b in range(B):
        ref = oracle.sddmm_host(lhs_all[b], rhs_all[b], hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N,
                                pa, pb, oracle.SIGNED,
                                layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
        np.testing.assert_array_equal(out[b].cpu().numpy(), ref)


@pytest.mark.parametrize("pa,pb", DP4A_PAIRS)
@pytest.mark.parametrize("V", [2, 4, 8])
def test_sddmm_dp4a_half_equals_int8_path(cuda, pa, pb, V):
    """Half output (the attention scores): the same bits as the int8 MMA path."""
    K, N, scale = 64, 256, 36.0 * 36.0
    mask, lhs, rhs = _case(pa, pb, V, K, N, RAGGED, seed=41 + V)
    hm = formats.prepare_sddmm(mask, alignment=16)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    args = (dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, pa, pb)
    a = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, mma_kind=_lib.MMA_DP4A)
    b = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, mma_kind=_lib.MMA_INT8)
    written = np.zeros(hm.aligned_nnz * V, bool)
    for i in range(mask.m_vec):
        written[hm.row_offsets[2 * i] * V:hm.row_offsets[2 * i + 1] * V] = True
    np.testing.assert_array_equal(a.cpu().numpy().view(np.uint16)[written], b.cpu().numpy().view(np.uint16)[written])


def test_sddmm_dp4a_rejects_16_bit(cuda):
    V, K, N = 8, 64, 128
    mask, lhs, rhs = _case(16, 8, V, K, N, [8, 16], seed=3)
    dm = ops.DeviceSddmmMask.from_host(formats.prepare_sddmm(mask), cuda)
    with pytest.raises(_lib.MagicubeError, match="dp4a"):
        ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, 16, 8, signed=True,
                  mma_kind=_lib.MMA_DP4A)


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x88, 0x77, 0xFF, 0x00, 0x8F, "alt"])
@pytest.mark.parametrize("V", [2, 8])
def test_sddmm_k64_extreme_4bit(cuda, signed, fill, V):
    """L4-R4 at k = 64 on the pipelined kernel, whose int8 MMA takes each
    nibble as 16 x its value and shifts the sums back: the largest products
    (-8 x -8, 15 x 15 unsigned) and mixed signs stay exact."""
    K, N = 64, 256
    mask = synth.lengths_mask([256, 3, 17, 0, 64, 8, 100, 1, 255], N, V, seed=23)
    nl, nr = mask.rows * K // 2, N * K // 2
    if fill == "alt":
        lhs = np.tile(np.array([0x87, 0x78], np.uint8), nl // 2 + 1)[:nl]
        rhs = np.tile(np.array([0x7F, 0x80, 0xF8, 0x08], np.uint8), nr // 4 + 1)[:nr]
    else:
        lhs, rhs = np.full(nl, fill, np.uint8), np.full(nr, fill, np.uint8)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, 4, 4, signed=signed,
                    mma_kind=_lib.MMA_INT8, variant=_lib.KERNEL_STREAM)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, V, K, N, 4, 4,
                            oracle.SIGNED if signed else oracle.UNSIGNED)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
