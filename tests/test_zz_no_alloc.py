"""mcDeviceAlignRowOffsetsNoAlloc against the allocating mcDeviceAlignRowOffsets.

The no-allocation entry point serves callers that may not allocate device
memory (a server that reserved its HBM up front, a host framework whose
allocator owns the device): its scratch is a fixed file-scope device array.
The file name puts it last in collection order: it runs after every other
test of a full run, and alone."""
import ctypes

import numpy as np
import pytest
import torch

from magicube_gb300 import _lib
from magicube_gb300 import device_format as dfm
from magicube_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_ROWS = 16_744_448


def _no_alloc(ro: torch.Tensor, alignment: int) -> tuple[torch.Tensor, torch.Tensor]:
    m_vec = ro.numel() - 1
    pairs = torch.full((max(2 * m_vec, 2),), -7, dtype=torch.int32, device=ro.device)
    n = torch.full((1,), -7, dtype=torch.int32, device=ro.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(_lib.lib().mcDeviceAlignRowOffsetsNoAlloc(m_vec, ro.data_ptr(), alignment, pairs.data_ptr(),
                                                         n.data_ptr(), stream), "mcDeviceAlignRowOffsetsNoAlloc")
    return pairs[:2 * m_vec], n


@pytest.mark.parametrize("alignment", [8, 16, 32])
def test_no_alloc_align_equals_allocating_entry_point_twice(cuda, alignment):
    """Two calls in a row (different sizes, the first across several scan
    tiles), each equal to the allocating entry point."""
    for m_vec, seed in ((5000, 1), (37, 2)):
        m = synth.normal_mask(m_vec, 700, 8, 0.9, seed=seed + alignment)
        ro = torch.from_numpy(np.ascontiguousarray(m.row_offsets)).to(cuda)
        p_ref, n_ref = dfm.align_row_offsets(ro, alignment)
        p, n = _no_alloc(ro, alignment)
        torch.cuda.synchronize()
        assert torch.equal(p, p_ref)
        assert int(n.item()) == int(n_ref.item()) > 0


def test_no_alloc_align_reports_bad_offsets_then_recovers(cuda):
    """The flag word that must start at zero is cleared on every call: a
    non-monotone call (-1) followed by a valid one."""
    bad = torch.tensor([0, 5, 3, 9], dtype=torch.int32, device=cuda)
    _, n = _no_alloc(bad, 16)
    assert int(n.item()) == -1
    good = torch.tensor([0, 5, 9, 9, 30], dtype=torch.int32, device=cuda)
    p, n = _no_alloc(good, 16)
    p_ref, n_ref = dfm.align_row_offsets(good, 16)
    assert torch.equal(p, p_ref) and int(n.item()) == int(n_ref.item()) == 64


def test_no_alloc_align_rejects_oversize(cuda):
    """More vector-rows than the static scratch holds: rejected before any
    launch or memory access."""
    ro = torch.zeros(2, dtype=torch.int32, device=cuda)
    pairs = torch.empty(2, dtype=torch.int32, device=cuda)
    n = torch.empty(1, dtype=torch.int32, device=cuda)
    rc = _lib.lib().mcDeviceAlignRowOffsetsNoAlloc(MAX_ROWS + 1, ro.data_ptr(), 16, pairs.data_ptr(),
                                                   n.data_ptr(), None)
    assert rc == 1
    assert b"static scratch" in _lib.lib().mcGetLastErrorString()


def test_no_alloc_align_at_the_largest_accepted_size(cuda):
    """m_vec at the limit fills the static scratch to its last tile sum and
    the flag word right after it; all-zero offsets give no slots.  A second
    call of a small size right after it is still correct."""
    ro = torch.zeros(MAX_ROWS + 1, dtype=torch.int32, device=cuda)
    p, n = _no_alloc(ro, 16)
    p_ref, n_ref = dfm.align_row_offsets(ro, 16)
    torch.cuda.synchronize()
    assert int(n.item()) == int(n_ref.item()) == 0
    assert torch.equal(p, p_ref)
    del ro, p, p_ref
    ro = torch.tensor([0, 3, 3, 20], dtype=torch.int32, device=cuda)
    p, n = _no_alloc(ro, 8)
    p_ref, n_ref = dfm.align_row_offsets(ro, 8)
    assert torch.equal(p, p_ref) and int(n.item()) == int(n_ref.item()) == 32
