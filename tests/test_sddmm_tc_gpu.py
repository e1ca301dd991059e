"""The tcgen05 SDDMM (MC_MMA_TCGEN05: L8-R8, k = 64, f16 operands in shared
memory, f32 accumulators in TMEM) against the CPU oracle, bit for bit: every
vector length, both lane semantics, both output layouts, half output,
extreme values, rows longer than one 128-nonzero chunk, batches."""
import numpy as np
import pytest
import torch

import oracle
from magicube_gb300 import _lib, formats, ops, synth

pytestmark = pytest.mark.gpu

K = 64
TC = _lib.MMA_TCGEN05
RAGGED = [0, 1, 7, 8, 9, 15, 16, 17, 33, 64, 100, 5, 250, 0, 31, 40, 127, 128, 129, 300]


def _run(cuda, mask, lhs, rhs, N, signed, vecmajor=False):
    align = 16 if vecmajor else 8
    hm = formats.prepare_sddmm(mask, alignment=align)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    out = ops.sddmm(dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, 8, 8, signed=signed,
                    vecmajor=vecmajor, mma_kind=TC)
    ref = oracle.sddmm_host(lhs, rhs, hm.row_offsets, hm.col_indices, mask.m_vec, mask.vec_length, K, N, 8, 8,
                            oracle.SIGNED if signed else oracle.UNSIGNED, alignment=8,
                            layout=oracle.OUT_VECMAJOR if vecmajor else oracle.OUT_BLOCKED)
    return out, ref


@pytest.mark.parametrize("V", [2, 4, 8])
@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("vecmajor", [False, True])
def test_tc_sddmm_ragged(cuda, V, signed, vecmajor):
    N = 512
    mask = synth.lengths_mask(RAGGED, N, V, seed=V + 3)
    lhs = synth.random_bytes(mask.rows * K, V + 4)
    rhs = synth.random_bytes(N * K, V + 5)
    out, ref = _run(cuda, mask, lhs, rhs, N, signed, vecmajor)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    assert _lib.lib().mcTensorCoreTimeouts() == 0


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("fill", [0x00, 0xFF, 0x80, 0x7F, "alt"])
def test_tc_sddmm_extreme_values(cuda, signed, fill):
    """Every lane at an extreme: the largest sums the f32 accumulator sees
    (unsigned 64 x 255 x 255 < 2^24)."""
    V, N = 8, 512
    mask = synth.lengths_mask([512, 3, 17, 0, 64, 8, 100, 1, 256, 129], N, V, seed=19)
    nl, nr = mask.rows * K, N * K
    if fill == "alt":
        lhs = np.tile(np.array([0x80, 0x7F], np.uint8), nl // 2 + 1)[:nl]
        rhs = np.tile(np.array([0x7F, 0x80, 0xFF, 0x00], np.uint8), nr // 4 + 1)[:nr]
    else:
        lhs, rhs = np.full(nl, fill, np.uint8), np.full(nr, fill, np.uint8)
    out, ref = _run(cuda, mask, lhs, rhs, N, signed)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_tc_sddmm_equals_int8_path_on_headline_shape(cuda):
    """4096 x 4096 V=8 mask at sparsity 0.9, 4 batch entries: the tcgen05 and
    the int8 mma.sync paths give the same integers."""
    V, N, B = 8, 4096, 4
    mask = synth.uniform_mask(N // V, N, V, 0.9, seed=42)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs = torch.randint(0, 256, (B, N * K), dtype=torch.uint8, device=cuda)
    rhs = torch.randint(0, 256, (B, N * K), dtype=torch.uint8, device=cuda)
    a = ops.sddmm(dm, lhs, rhs, K, 8, 8, signed=True, batch=B, mma_kind=TC)
    b = ops.sddmm(dm, lhs, rhs, K, 8, 8, signed=True, batch=B, mma_kind=_lib.MMA_INT8)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert _lib.lib().mcTensorCoreTimeouts() == 0


@pytest.mark.parametrize("V", [2, 8])
def test_tc_sddmm_half_vecmajor(cuda, V):
    """Dequantised half output in the extension's vector-major layout."""
    N, scale = 256, 36.0 * 36.0
    mask = synth.lengths_mask(RAGGED[:12], N, V, seed=11)
    lhs = synth.random_bytes(mask.rows * K, 12)
    rhs = synth.random_bytes(N * K, 13)
    hm = formats.prepare_sddmm(mask, alignment=16)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    args = (dm, torch.from_numpy(lhs).to(cuda), torch.from_numpy(rhs).to(cuda), K, 8, 8)
    a = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, mma_kind=TC)
    b = ops.sddmm(*args, signed=True, vecmajor=True, out_half=True, scale=scale, mma_kind=_lib.MMA_INT8)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_tc_sddmm_rejects_other_shapes(cuda):
    mask = synth.lengths_mask([5, 9], 64, 8, seed=1)
    hm = formats.prepare_sddmm(mask)
    dm = ops.DeviceSddmmMask.from_host(hm, cuda)
    lhs = torch.zeros(16 * 128, dtype=torch.uint8, device=cuda)
    rhs = torch.zeros(64 * 128, dtype=torch.uint8, device=cuda)
    with pytest.raises(_lib.MagicubeError):
        ops.sddmm(dm, lhs, rhs, 128, 8, 8, signed=True, mma_kind=TC)  # k != 64
    with pytest.raises(_lib.MagicubeError):
        ops.sddmm(dm, lhs, rhs, 64, 4, 4, signed=True, mma_kind=TC)  # 4-bit


@pytest.mark.parametrize("n", [16, 64, 256])
def test_tcgen05_throughput_probe(cuda, n):
    """The tcgen05 probe runs to completion (no wait ran out) and reports a
    positive rate."""
    import ctypes
    timeouts = torch.zeros(1, dtype=torch.int32, device=cuda)
    ms, ops = ctypes.c_float(), ctypes.c_double()
    _lib.check(_lib.probe_lib().mcProbeTensorCorePeak(n, 200, ctypes.byref(ms), ctypes.byref(ops), timeouts.data_ptr(),
                                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "mcProbeTensorCorePeak")
    torch.cuda.synchronize()
    assert int(timeouts.item()) == 0
    assert ms.value > 0 and ops.value == 2.0 * 128 * n * 16 * 4 * 200 * torch.cuda.get_device_properties(0).multi_processor_count
