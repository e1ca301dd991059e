"""The resident-slice SpMM (MC_KERNEL_RESIDENT: each CTA holds a K x 64-byte
column slice of B in shared memory and gathers its rows with ldmatrix), 8-bit
and 4-bit B, every A precision, against the CPU oracle bit for bit and
against the TMA-gather kernel."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

RAGGED = [0, 1, 3, 4, 5, 15, 16, 17, 31, 32, 33, 64, 100, 7, 200, 3, 48, 0, 250, 2]
RES = _lib.KERNEL_RESIDENT


def _vals(mask, V, pa, seed):
    return synth.random_bytes(mask.nnz_vec * V * formats.lane_bits(pa) // 8, seed)


def _run(cuda, mask, vals, rhs, pa, pb, N, signed, variant=RES, **kw):
    h = formats.prepare_spmm(mask, vals, pa, pb)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    return ops.spmm(d, torch.from_numpy(rhs).to(cuda), N, signed=signed, variant=variant, **kw)


def _ref(mask, vals, rhs, V, K, N, pa, pb, signed):
    return oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                            16 if pa == 12 else pa, pb, oracle.SIGNED if signed else oracle.UNSIGNED,
                            **({"preA_cut": 12} if pa == 12 else {}))


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (12, 8)])
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [64, 192, 256])
def test_resident_ragged(cuda, pa, pb, V, signed, N):
    """Row lengths around every group-of-4, 16-slot and 32-slot boundary,
    empty rows included; N = 192 runs three 64-column slices."""
    if pa == 12 and signed:
        pytest.skip("12-bit lanes are unsigned")
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V + 3)
    vals = _vals(mask, V, pa, 130 + V)
    rhs = synth.random_bytes(K * N, 131 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, pa, pb, signed))


@pytest.mark.parametrize("pa,pb", [(4, 4), (8, 4), (16, 4), (12, 4)])
@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [128, 384])
def test_resident_ragged_4bit_rhs(cuda, pa, pb, V, signed, N):
    """4-bit B (128 columns per 64-byte slice row; column indices shuffled
    within groups of 8 by the packer), every A precision."""
    if pa == 12 and signed:
        pytest.skip("12-bit lanes are unsigned")
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V + 4)
    vals = _vals(mask, V, pa, 132 + V)
    rhs = synth.random_bytes(K * N // 2, 133 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, pa, pb, signed))


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4)])
@pytest.mark.parametrize("K", [40, 300, 1000, 3584])
def test_resident_slice_heights(cuda, pa, pb, K):
    """k from well under one 256-row box to the largest accepted (14 boxes),
    and k not a multiple of 256 (the last box reaches past the tensor's end
    or into the next batch entry, rows that no column index names); three
    batch entries with their own B."""
    V, B = 8, 3
    N = 128 if pb == 8 else 256
    lengths = np.random.default_rng(K + pa).integers(0, min(K, 300) + 1, size=40)
    lengths[0], lengths[1] = K, 0
    mask = synth.lengths_mask(lengths, K, V, seed=K)
    vals_all = [_vals(mask, V, pa, 140 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 150 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size, variant=RES)
    for b in range(B):
        np.testing.assert_array_equal(out[b].cpu().numpy(), _ref(mask, vals_all[b], rhs_all[b], V, K, N, pa, pb, True))


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4)])
@pytest.mark.parametrize("shared_rhs", [False, True])
def test_resident_many_slices(cuda, pa, pb, shared_rhs):
    """Far more (slice, vector-row) units than resident CTAs, so CTA ranges
    start and end inside slices and cross several; per-entry values, B per
    entry or shared (rhs_stride 0)."""
    V, K, B = 8, 512, 6
    N = 256 if pb == 8 else 512
    lengths = np.random.default_rng(pa + pb).integers(0, 90, size=700)
    lengths[::29] = 0
    lengths[3] = 512
    mask = synth.lengths_mask(lengths, K, V, seed=42)
    vals_all = [_vals(mask, V, pa, 160 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 170 + b) for b in range(B)]
    if shared_rhs:
        rhs_all = [rhs_all[0]] * B
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(rhs_all[0] if shared_rhs else np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size,
                   rhs_stride=0 if shared_rhs else K * N * pb // 8, variant=RES)
    for b in (0, 2, B - 1):
        np.testing.assert_array_equal(out[b].cpu().numpy(), _ref(mask, vals_all[b], rhs_all[b], V, K, N, pa, pb, True))


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4), (16, 4)])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
def test_resident_extreme_values_long_rows(cuda, pa, pb, signed, fill):
    V, K = 8, 2048
    N = 64 if pb == 8 else 128
    mask = synth.lengths_mask([2048, 1000, 257, 256, 255, 0, 31, 1], K, V, seed=18)
    nv, nr = mask.nnz_vec * V * pa // 8, K * N * pb // 8
    if fill == "alt":
        vals = np.tile(np.array([0x80, 0x7F], np.uint8), nv // 2 + 1)[:nv]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        vals, rhs = np.full(nv, fill, np.uint8), np.full(nr, fill, np.uint8)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, pa, pb, signed))


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4)])
@pytest.mark.parametrize("V", [2, 4, 8])
def test_resident_half_output_equals_tma(cuda, pa, pb, V):
    """Dequantised half output on the softmax value layout, bit-identical to
    the TMA kernel and to the oracle's integer result / scale."""
    K, N, scale = 512, 256, 36.0 * 32.0
    mask = synth.lengths_mask(RAGGED, K, V, seed=80 + V)
    vals = _vals(mask, V, pa, 81)
    rhs = synth.random_bytes(K * N * pb // 8, 82)
    h = formats.prepare_spmm(mask, vals, pa, pb, layout=formats.VALUES_SOFTMAX)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    r = torch.from_numpy(rhs).to(cuda)
    outs = [ops.spmm(d, r, N, signed=True, out_half=True, scale=scale, variant=v)
            for v in (RES, _lib.KERNEL_TMA)]
    assert torch.equal(outs[0], outs[1])
    acc = oracle.spmm_host(vals, rhs, mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb, oracle.SIGNED)
    with np.errstate(over="ignore"):  # 16-bit A: sums beyond the half range round to inf, as on the GPU
        ref = (acc.astype(np.float32) / np.float32(scale)).astype(np.float16)
    np.testing.assert_array_equal(outs[0].cpu().numpy().view(np.uint16), ref.view(np.uint16))


def test_resident_equals_tma_at_1024x1024x256(cuda):
    """A 1024 x 1024 V=8 sparsity-0.9 operand times 1024 x 256, 64 batch
    entries: identical int32 results from the two kernels, two entries
    against the oracle."""
    M = K = 1024
    N, V, B = 256, 8, 64
    mask = synth.uniform_mask(M // V, K, V, 0.9, seed=7)
    vals = synth.random_bytes(mask.nnz_vec * V, 8)
    h = formats.prepare_spmm(mask, vals, 8, 8)
    d = ops.DeviceSpmmLhs.from_host(h, cuda)
    d.values = d.values.repeat(B)
    rhs = torch.randint(0, 256, (B, K * N), dtype=torch.uint8, device=cuda)
    outs = [ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=h.values.size, variant=v)
            for v in (RES, _lib.KERNEL_TMA)]
    assert torch.equal(outs[0], outs[1])
    for b in (0, B - 1):
        ref = oracle.spmm_host(vals, rhs[b].cpu().numpy(), mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N,
                               8, 8, oracle.SIGNED)
        np.testing.assert_array_equal(outs[0][b].cpu().numpy(), ref)


def test_resident_rejects_ineligible(cuda):
    V = 8
    for pa, pb, N, K, mma in ((8, 8, 96, 256, _lib.MMA_INT8), (8, 4, 192, 256, _lib.MMA_INT8),
                              (8, 8, 128, 256, _lib.MMA_F16), (16, 16, 128, 256, _lib.MMA_INT8),
                              (8, 8, 128, 3585, _lib.MMA_INT8)):
        mask = synth.lengths_mask([5, 40], K, V, seed=3)
        vals = _vals(mask, V, pa, 1)
        rhs = synth.random_bytes(K * N * pb // 8, 2)
        with pytest.raises(_lib.MagicubeError):
            _run(cuda, mask, vals, rhs, pa, pb, N, True, mma_kind=mma)


def test_resident_no_timeouts(cuda):
    torch.cuda.synchronize()
    assert _lib.lib().mcTensorCoreTimeouts() == 0


@pytest.mark.parametrize("pa,pb", [(8, 8), (8, 4), (4, 4)])
@pytest.mark.parametrize("V", [2, 4])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("N", [128, 256])
def test_resident_dp4a_ragged(cuda, pa, pb, V, signed, N):
    """The dp4a consumers of the resident-slice kernel (MC_MMA_DP4A, V = 2
    and 4): row lengths around every boundary, empty rows, bit-exact."""
    K = 256
    mask = synth.lengths_mask(RAGGED, K, V, seed=pa * 10 + V + 9)
    vals = _vals(mask, V, pa, 190 + V)
    rhs = synth.random_bytes(K * N * pb // 8, 191 + V)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, signed, mma_kind=_lib.MMA_DP4A)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, pa, pb, signed))


@pytest.mark.parametrize("pa,pb", [(8, 8), (8, 4), (4, 4)])
@pytest.mark.parametrize("V", [2, 4])
@pytest.mark.parametrize("fill", [0x80, 0x7F, 0xFF])
def test_resident_dp4a_extreme_values_long_rows(cuda, pa, pb, V, fill):
    K = 2048
    N = 64 if pb == 8 else 128
    mask = synth.lengths_mask([2048, 1000, 257, 256, 255, 0, 31, 1], K, V, seed=19)
    vals = np.full(mask.nnz_vec * V * pa // 8, fill, np.uint8)
    rhs = np.full(K * N * pb // 8, fill, np.uint8)
    out = _run(cuda, mask, vals, rhs, pa, pb, N, True, mma_kind=_lib.MMA_DP4A)
    np.testing.assert_array_equal(out.cpu().numpy(), _ref(mask, vals, rhs, V, K, N, pa, pb, True))


def test_resident_dp4a_many_slices(cuda):
    V, K, B, N = 4, 1024, 5, 256
    lengths = np.random.default_rng(5).integers(0, 200, size=900)
    mask = synth.lengths_mask(lengths, K, V, seed=43)
    vals_all = [_vals(mask, V, 8, 200 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N, 210 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, 8, 8) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(np.concatenate(rhs_all)).to(cuda)
    out = ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size, variant=RES,
                   mma_kind=_lib.MMA_DP4A)
    for b in (0, B - 1):
        np.testing.assert_array_equal(out[b].cpu().numpy(), _ref(mask, vals_all[b], rhs_all[b], V, K, N, 8, 8, True))


CONFIGS = [_lib.RESIDENT_S64_W8, _lib.RESIDENT_S64_W16, _lib.RESIDENT_S128_W16]


def _config_built(cfg, pa, pb, V):
    if cfg == _lib.RESIDENT_S64_W8:
        return True
    if V != 8:
        return False
    return not (pa == 16 and pb == 4) if cfg == _lib.RESIDENT_S64_W16 else pa <= 8


@pytest.mark.parametrize("pa,pb", [(8, 8), (16, 8), (4, 4), (8, 4), (16, 4)])
@pytest.mark.parametrize("cfg", CONFIGS)
@pytest.mark.parametrize("K", [300, 1792])
def test_resident_every_config(cuda, pa, pb, cfg, K):
    """Every slice width and CTA size, ragged rows, two batch entries with
    their own B, N a multiple of the widest slice: bit-exact against the
    oracle; configurations not built for a pair are rejected."""
    V, B = 8, 2
    N = 256 if pb == 8 else 512
    lengths = np.array(RAGGED * 6) % (K + 1)
    lengths[0] = K
    mask = synth.lengths_mask(lengths, K, V, seed=cfg * 7 + K)
    vals_all = [_vals(mask, V, pa, 220 + b) for b in range(B)]
    rhs_all = [synth.random_bytes(K * N * pb // 8, 230 + b) for b in range(B)]
    packed = [formats.prepare_spmm(mask, v, pa, pb) for v in vals_all]
    d = ops.DeviceSpmmLhs.from_host(packed[0], cuda)
    d.values = torch.from_numpy(np.concatenate([p.values for p in packed])).to(cuda)
    rhs = torch.from_numpy(np.concatenate(rhs_all)).to(cuda)
    run = lambda: ops.spmm(d, rhs, N, signed=True, batch=B, values_stride=packed[0].values.size, variant=RES,
                           config=cfg)
    if not _config_built(cfg, pa, pb, V):
        with pytest.raises(_lib.MagicubeError):
            run()
        return
    out = run()
    for b in range(B):
        np.testing.assert_array_equal(out[b].cpu().numpy(), _ref(mask, vals_all[b], rhs_all[b], V, K, N, pa, pb, True))


def test_resident_config_limits(cuda):
    """128-byte slices: k above 1792 and n not a multiple of the slice width
    are rejected; an invalid configuration number too."""
    V = 8
    for K, N, cfg in ((1800, 256, _lib.RESIDENT_S128_W16), (256, 192, _lib.RESIDENT_S128_W16), (256, 256, 4),
                      (256, 256, -1)):
        mask = synth.lengths_mask([5, 40], K, V, seed=3)
        vals = _vals(mask, V, 8, 1)
        rhs = synth.random_bytes(K * N, 2)
        with pytest.raises(_lib.MagicubeError):
            _run(cuda, mask, vals, rhs, 8, 8, N, True, config=cfg)
