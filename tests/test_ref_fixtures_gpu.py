"""The drop-in entry points on arrays packed by the reference's own host code
(tests/golden/ref_*.npz): mcWmmaSpmm_<P> / mcWmmaSddmm_<P> must reproduce the
result the reference program verified against its host routine."""
import numpy as np
import pytest
import torch

from golden_util import load, names
from magicube_gb300 import _lib

pytestmark = pytest.mark.gpu

SPMM_FN = {(4, 4): "4b", (8, 4): "8b4b", (16, 4): "16b4b", (8, 8): "8b", (16, 8): "16b8b", (12, 4): "12b4b",
           (12, 8): "12b8b", (16, 16): "16b"}
SDDMM_FN = {4: "4b", 8: "8b", 16: "16b"}


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("name", names("ref_spmm_"))
def test_spmm_on_reference_packed_arrays(cuda, name):
    d = load(name)
    V, K, N, pa, pb, m_vec = (int(d[k]) for k in ("V", "K", "N", "preA", "preB", "m_vec"))
    ri, ro, ci = _dev(d["row_indices"], cuda), _dev(d["row_offsets"], cuda), _dev(d["col_indices"], cuda)
    vals, rhs = _dev(d["values"], cuda), _dev(d["rhs"], cuda)
    out = torch.full((m_vec * V * N,), 123, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    fn = getattr(_lib.lib(), "mcWmmaSpmm_" + SPMM_FN[(pa, pb)])
    _lib.check(fn(m_vec, V, N, K, ri.data_ptr(), ro.data_ptr(), ci.data_ptr(), vals.data_ptr(), rhs.data_ptr(),
                  out.data_ptr()), name)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), d["out"])


@pytest.mark.parametrize("name", names("ref_sddmm_"))
def test_sddmm_on_reference_packed_arrays(cuda, name):
    d = load(name)
    V, K, N, bits, m_vec = (int(d[k]) for k in ("V", "K", "N", "bits", "m_vec"))
    ri, ro, ci = _dev(d["row_indices"], cuda), _dev(d["row_offsets"], cuda), _dev(d["col_indices"], cuda)
    lhs, rhs = _dev(d["lhs"], cuda), _dev(d["rhs"], cuda)
    out = torch.zeros(d["out"].size, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    fn = getattr(_lib.lib(), "mcWmmaSddmm_" + SDDMM_FN[bits])
    _lib.check(fn(m_vec, K, N, ri.data_ptr(), ro.data_ptr(), ci.data_ptr(), lhs.data_ptr(), rhs.data_ptr(),
                  out.data_ptr(), V), name)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), d["out"])
