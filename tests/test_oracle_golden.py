"""The oracle and the host packer against fixtures produced by the reference
itself (tests/golden, see make_golden.py).  CPU only."""
import numpy as np
import pytest

import oracle
from golden_util import lane_bits, load, names, unpack_spmm_values
from magicube_gb300 import formats
from magicube_gb300.formats import VectorSparse


@pytest.mark.parametrize("name", names("routine_spmm_"))
def test_oracle_literal_equals_reference_spmm_routine(name):
    """compute_ref_integers (reference, compiled from its sources) on full-range
    random data == the oracle's literal mode, bit for bit."""
    d = load(name)
    pa = int(d["preA"])
    got = oracle.spmm_host(d["values"], d["rhs"], d["row_offsets"], d["col_indices"], int(d["m_vec"]), int(d["V"]),
                           int(d["K"]), int(d["N"]), lane_bits(pa), int(d["preB"]), oracle.LITERAL, preA_cut=pa)
    np.testing.assert_array_equal(got.ravel(), d["out"])


@pytest.mark.parametrize("name", names("routine_spmm_"))
def test_reference_top_lane_quirk_is_visible(name):
    """On full-range data the reference routine's sign-extended top rhs lane
    makes it differ from purely unsigned lanes (the GPU kernels' semantics)."""
    d = load(name)
    pa = int(d["preA"])
    args = (d["values"], d["rhs"], d["row_offsets"], d["col_indices"], int(d["m_vec"]), int(d["V"]), int(d["K"]),
            int(d["N"]), lane_bits(pa), int(d["preB"]))
    lit = oracle.spmm_host(*args, oracle.LITERAL, preA_cut=pa)
    uns = oracle.spmm_host(*args, oracle.UNSIGNED, preA_cut=pa)
    if int(d["row_offsets"][-1]) > 0:
        assert not np.array_equal(lit, uns)


@pytest.mark.parametrize("name", names("routine_sddmm_"))
def test_oracle_literal_equals_reference_sddmm_routine(name):
    d = load(name)
    got = oracle.sddmm_host(d["lhs"], d["rhs"], d["row_offsets"], d["col_indices"], int(d["m_vec"]), int(d["V"]),
                            int(d["K"]), int(d["N"]), int(d["bits"]), int(d["bits"]), oracle.LITERAL)
    np.testing.assert_array_equal(got, d["out"])


@pytest.mark.parametrize("name", names("ref_spmm_"))
def test_packer_and_oracle_against_reference_spmm_program(name):
    """A run of the reference's spmm_benchmark: its host packer's device arrays
    equal ours, and its result (verified PASS by the reference itself against
    its host routine) equals the oracle on the recovered original values."""
    d = load(name)
    assert str(d["verdict"]) == "PASS"
    V, K, N, pa, pb = (int(d[k]) for k in ("V", "K", "N", "preA", "preB"))
    mask = VectorSparse(int(d["m_vec"]), V, K, d["csr_row_offsets"], d["csr_col_indices"])
    chunk = formats.spmm_chunk(pa, pb)
    pairs, n = formats.align_row_offsets(mask, chunk)
    np.testing.assert_array_equal(pairs, d["row_offsets"])
    np.testing.assert_array_equal(formats.pad_column_indices(mask, pairs, n, chunk == 32), d["col_indices"])
    np.testing.assert_array_equal(formats.sorted_row_swizzle(mask), d["row_indices"])
    orig = unpack_spmm_values(d["values"], pairs, mask.row_offsets, V, pa, pb)
    np.testing.assert_array_equal(formats.pack_spmm_values(mask, pairs, n, orig, pa, pb), d["values"])
    got = oracle.spmm_host(orig, d["rhs"], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, lane_bits(pa),
                           pb, oracle.LITERAL, preA_cut=pa)
    np.testing.assert_array_equal(got.ravel(), d["out"])


@pytest.mark.parametrize("name", names("ref_sddmm_"))
def test_oracle_against_reference_sddmm_program(name):
    d = load(name)
    assert str(d["verdict"]) == "PASS"
    V, K, N, bits = (int(d[k]) for k in ("V", "K", "N", "bits"))
    mask = VectorSparse(int(d["m_vec"]), V, N, d["csr_row_offsets"], d["csr_col_indices"])
    pairs, n = formats.align_row_offsets(mask, 8)
    np.testing.assert_array_equal(pairs, d["row_offsets"])
    np.testing.assert_array_equal(formats.pad_column_indices(mask, pairs, n, False), d["col_indices"])
    np.testing.assert_array_equal(formats.sorted_row_swizzle(mask), d["row_indices"])
    got = oracle.sddmm_host(d["lhs"], d["rhs"], pairs, d["col_indices"], mask.m_vec, V, K, N, bits, bits,
                            oracle.LITERAL)
    np.testing.assert_array_equal(got, d["out"])


@pytest.mark.parametrize("name", names("ref_sddmm_") + [n for n in names("ref_spmm_") if "R4" not in n
                                                        and "L4" not in n])
def test_oracle_aligner_equals_reference_packer(name):
    """The oracle's numpy aligner (used by the CPU baselines, which load no
    library of this package) reproduces the reference packer's aligned pairs
    and -1 padded columns (alignment 8 for SDDMM, 16 for 8/16-bit SpMM)."""
    d = load(name)
    align = 8 if name.startswith("ref_sddmm_") else 16
    pairs, n = oracle.align_pairs(d["csr_row_offsets"], align)
    np.testing.assert_array_equal(pairs, d["row_offsets"])
    np.testing.assert_array_equal(oracle.pad_columns(d["csr_row_offsets"], d["csr_col_indices"], pairs, n),
                                  d["col_indices"])


def test_oracle_aligner_edge_rows():
    """Empty rows, rows of exactly the alignment and an empty matrix."""
    ro = np.array([0, 0, 8, 9, 9, 25], np.int32)
    ci = np.arange(25, dtype=np.int32)
    pairs, n = oracle.align_pairs(ro, 8)
    np.testing.assert_array_equal(pairs, [0, 0, 0, 8, 8, 9, 16, 16, 16, 32])
    assert n == 32
    cols = oracle.pad_columns(ro, ci, pairs, n)
    np.testing.assert_array_equal(cols[:9], np.arange(9))
    assert (cols[9:16] == -1).all()
    np.testing.assert_array_equal(cols[16:], np.arange(9, 25))
    pairs0, n0 = oracle.align_pairs(np.zeros(1, np.int32), 16)
    assert pairs0.size == 0 and n0 == 0
