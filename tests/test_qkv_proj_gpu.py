"""mcQkvProjectQuantize (tcgen05 projection + fused quantization) against a
float64 restatement of the reference's fp16 F.linear + bquantization, and
against the unfused path on the GPU (cuBLAS F.linear + mcQuantize).

Tolerance: the kernel accumulates in f32 in its own order, so an element whose
half rounding or truncation falls on a boundary may land one quantization step
away; at most 0.1 % of the elements may differ, each by exactly one step."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from magicube_gb300 import _lib
from magicube_gb300.projection import qkv_project_quantize

pytestmark = pytest.mark.gpu


def _ref(x, w, b, heads, bits, scale):
    y = x.double() @ w.double().T
    if b is not None:
        y = y + b.double()
    lo, hi = (-128, 127) if bits == 8 else (-8, 7)
    q = torch.trunc(torch.clamp(y.half().double() * scale, lo, hi)).to(torch.int64)
    T, N = q.shape
    E = N // 3
    return q.view(T, 3, heads, E // heads).permute(1, 2, 0, 3).contiguous()


def _unpack(out, T, heads, d, bits):
    raw = out.contiguous().view(torch.uint8).cpu().numpy().reshape(3, heads, -1)
    if bits == 8:
        v = raw.view(np.int8).astype(np.int64)
    else:
        lo = (raw & 0xF).astype(np.int64)
        hi = (raw >> 4).astype(np.int64)
        v = np.stack([lo, hi], axis=-1).reshape(3, heads, -1)
        v = np.where(v >= 8, v - 16, v)
    return torch.from_numpy(v.reshape(3, heads, T, d))


def _check(got, ref):
    diff = (got - ref).abs()
    assert int(diff.max()) <= 1, f"max diff {int(diff.max())}"
    frac = float((diff != 0).double().mean())
    assert frac <= 1e-3, f"{frac:.2e} of the elements differ"
    return frac


def _case(dev, T, E, heads, bits, bias, seed):
    g = torch.Generator().manual_seed(seed)
    x = (torch.randn(T, E, generator=g) * 0.5).half()
    w = (torch.randn(3 * E, E, generator=g) * (1.0 / E ** 0.5)).half()
    b = (torch.randn(3 * E, generator=g) * 0.1).half() if bias else None
    scale = (127.0 if bits == 8 else 7.0) / 2.0
    return x, w, b, scale


@pytest.mark.parametrize("T", [1, 77, 128, 129, 1000, 4099])
@pytest.mark.parametrize("bits", [8, 4])
def test_projection_matches_fp64_reference(cuda, T, bits):
    E, heads = 256, 4
    x, w, b, scale = _case(cuda, T, E, heads, bits, True, T + bits)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    out = qkv_project_quantize(x.to(cuda), w.to(cuda), b.to(cuda), heads, bits, scale, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    _check(_unpack(out, T, heads, E // heads, bits), _ref(x, w, b, heads, bits, scale))


@pytest.mark.parametrize("E,heads", [(64, 1), (128, 2), (192, 3), (256, 1), (256, 4)])
@pytest.mark.parametrize("bias", [True, False])
def test_projection_shapes(cuda, E, heads, bias):
    T = 300
    x, w, b, scale = _case(cuda, T, E, heads, 8, bias, E + heads)
    out = qkv_project_quantize(x.to(cuda), w.to(cuda), b.to(cuda) if bias else None, heads, 8, scale)
    _check(_unpack(out, T, heads, E // heads, 8), _ref(x, w, b, heads, 8, scale))


def test_projection_matches_unfused_gpu_path(cuda):
    """cuBLAS fp16 F.linear + permute + mcQuantize vs the fused kernel."""
    T, E, heads = 2048, 256, 4
    x, w, b, scale = _case(cuda, T, E, heads, 8, True, 5)
    x, w, b = x.to(cuda), w.to(cuda), b.to(cuda)
    qkv = F.linear(x, w, b).view(T, 3, heads, E // heads).permute(1, 2, 0, 3).contiguous()
    ref = torch.empty((3, heads, T * (E // heads) // 4), dtype=torch.int32, device=cuda)
    import ctypes
    _lib.check(_lib.lib().mcQuantize(qkv.data_ptr(), ref.data_ptr(), qkv.numel(), 8, float(scale),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "mcQuantize")
    out = qkv_project_quantize(x, w, b, heads, 8, scale)
    _check(_unpack(out, T, heads, E // heads, 8), _unpack(ref, T, heads, E // heads, 8))


def test_projection_saturates_and_handles_extremes(cuda):
    """Large activations clamp to the int8 range exactly like the reference."""
    T, E, heads = 256, 256, 4
    x, w, b, _ = _case(cuda, T, E, heads, 8, True, 9)
    scale = 500.0
    out = qkv_project_quantize(x.to(cuda), w.to(cuda), b.to(cuda), heads, 8, scale)
    got = _unpack(out, T, heads, E // heads, 8)
    ref = _ref(x, w, b, heads, 8, scale)
    assert int((got == 127).sum()) > 0 and int((got == -128).sum()) > 0
    _check(got, ref)


def test_projection_rejects_bad_shapes(cuda):
    x = torch.zeros(16, 96, dtype=torch.float16, device=cuda)
    w = torch.zeros(288, 96, dtype=torch.float16, device=cuda)
    with pytest.raises(_lib.MagicubeError):
        qkv_project_quantize(x, w, None, 2, 8, 1.0)


def test_encoder_layer_fused_projection_matches_unfused(cuda):
    from magicube_gb300 import batched, synth
    from magicube_gb300.model import SparseEncoderLayer
    torch.manual_seed(0)
    lens = [256, 512]
    masks = [synth.band_random_mask(L, 8, 64, 0.8, seed=i) for i, L in enumerate(lens)]
    mega, _ = batched.block_diagonal(masks)
    mask = batched.to_device(mega, 8, cuda)
    layer = SparseEncoderLayer().to(cuda).half().eval()
    x = (torch.randn(sum(lens), 256, device=cuda) * 0.5).half()
    assert layer.fused_projection
    with torch.no_grad():
        a = layer(x, mask)
        layer.fused_projection = False
        b = layer(x, mask)
    torch.cuda.synchronize()
    err = float((a.float() - b.float()).abs().max())
    assert err <= 2e-2 * float(b.float().abs().max()), err
