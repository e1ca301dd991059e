"""The C-ABI library: loads, exports every entry point the public header
declares, and rejects bad arguments before touching a GPU.  CPU only."""
import ctypes
import re
from pathlib import Path

import pytest

from magicube_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "magicube_gb300.h"
PROBE_HEADER = HEADER.with_name("magicube_gb300_probe.h")


def declared_functions(header: Path = HEADER) -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(mc[A-Z]\w*)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    names = declared_functions()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.exported_symbols())


def test_probe_library_exports_its_header_and_product_library_does_not():
    """The diagnostics live in their own library: it exports every function
    its header declares, and the product library none of them."""
    names = declared_functions(PROBE_HEADER)
    assert len(names) == 4
    probe = _lib.probe_lib()
    assert all(hasattr(probe, n) for n in names)
    import ctypes as _ct
    product = _ct.CDLL(str(_lib.LIB_PATH))
    assert not any(hasattr(product, n) for n in names)


def test_version():
    assert _lib.lib().mcVersion().decode().count(".") == 2


@pytest.mark.parametrize("field,value,msg", [
    ("vec_length", 3, b"vec_length"), ("n", 100, b"multiple of 64"), ("lhs_bits", 4, b"precision"),
    ("batch", 0, b"batch"), ("out_half", 1, b"is_signed")])
def test_spmm_argument_errors(field, value, msg):
    d = _lib.McSpmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1, scale=1.0)
    setattr(d, field, value)
    if field == "lhs_bits":
        d.rhs_bits = 8
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 1
    assert msg in _lib.lib().mcGetLastErrorString()


@pytest.mark.parametrize("field,value,msg", [
    ("k", 96, b"multiple of 64"), ("vec_length", 16, b"vec_length"), ("rhs_bits", 4, b"precision"),
    ("out_half", 1, b"half output")])
def test_sddmm_argument_errors(field, value, msg):
    d = _lib.McSddmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1, scale=1.0)
    setattr(d, field, value)
    assert _lib.lib().mcSddmm(ctypes.byref(d), None) == 1
    assert msg in _lib.lib().mcGetLastErrorString()


@pytest.mark.parametrize("field", ["lhs_stride", "rhs_stride", "out_stride"])
def test_sddmm_negative_batch_stride_rejected(field):
    """As for the SpMM: batch strides are non-negative (zero shares)."""
    d = _lib.McSddmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=2, scale=1.0,
                         row_indices=256, row_offsets=256, column_indices=256, lhs=256, rhs=256, out=256)
    setattr(d, field, -64)
    assert _lib.lib().mcSddmm(ctypes.byref(d), None) == 1
    assert b"negative stride" in _lib.lib().mcGetLastErrorString()


def test_softmax_and_fused_attention_reject_negative_strides():
    """Batch (softmax) and head (fused attention) strides are non-negative;
    both checks run before any GPU work."""
    lib = _lib.lib()
    sm = _lib.McSoftmaxDesc(m_vec=4, vec_length=8, batch=2, bits=8, scaling=0.125, scale=127.0, row_indices=256,
                            row_offsets=256, scores=256, scores_stride=-64, out=256, out_stride=64)
    assert lib.mcQuantSoftmax(ctypes.byref(sm), None) == 1
    assert b"negative stride" in lib.mcGetLastErrorString()
    a = _lib.McAttnDesc(m_vec=4, vec_length=8, heads=2, head_dim=64, max_row_nnz=32, lhs_bits=8, rhs_bits=8,
                        requant=_lib.REQUANT_FIXED, row_indices=256, row_offsets=256, column_indices=256, q=256,
                        k=256, v=256, head_stride=64, out=256, out_head_stride=-64)
    assert lib.mcSparseAttention(ctypes.byref(a), None) == 1
    assert b"negative head stride" in lib.mcGetLastErrorString()


def test_null_pointers_rejected():
    d = _lib.McSpmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1)
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 1
    assert b"null" in _lib.lib().mcGetLastErrorString()


def test_empty_matrix_is_a_no_op():
    d = _lib.McSpmmDesc(m_vec=0, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1)
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 0


@pytest.mark.parametrize("fields,msg", [
    (dict(mma_kind=_lib.MMA_DP4A, lhs_bits=16, rhs_bits=8), b"dp4a"),
    (dict(mma_kind=5), b"invalid mma_kind"),
    (dict(kernel_variant=_lib.KERNEL_TMA), b"invalid kernel_variant"),
    (dict(kernel_variant=5), b"invalid kernel_variant"),
    (dict(kernel_variant=_lib.KERNEL_DENSE_TILE, lhs_bits=4, rhs_bits=4), b"L8-R8 with k == 64"),
    (dict(kernel_variant=_lib.KERNEL_DENSE_TILE, k=128), b"L8-R8 with k == 64"),
    (dict(kernel_variant=_lib.KERNEL_DENSE_TILE), b"tile bitmap"),
])
def test_sddmm_new_path_errors(fields, msg):
    """The dp4a path and the dense-tile kernel reject what they cannot
    compute, before any device work."""
    d = _lib.McSddmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1, scale=1.0)
    for k, v in fields.items():
        setattr(d, k, v)
    assert _lib.lib().mcSddmm(ctypes.byref(d), None) == 1
    assert msg in _lib.lib().mcGetLastErrorString()


@pytest.mark.parametrize("fields,msg", [
    (dict(lhs_bits=16), b"L8-R8 with int32 output"),
    (dict(n=192), b"n % 128 == 0"),
    (dict(mma_kind=_lib.MMA_INT8), b"tcgen05 f16 path"),
    (dict(), b"chunk table"),
    (dict(batch=2, rhs_stride=64 * 128 + 16), b"rhs_stride"),
])
def test_spmm_dense_tile_errors(fields, msg):
    """The dense-tile SpMM rejects what it cannot compute, before any device
    work: other pairs, n not a multiple of 128, another tensor path, a
    missing chunk table, a B stride that is not whole rows."""
    d = _lib.McSpmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1, scale=1.0,
                        kernel_variant=_lib.KERNEL_DENSE_TILE)
    if "chunk" not in msg.decode():
        d.chunk_starts = 16
    for k, v in fields.items():
        setattr(d, k, v)
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 1
    assert msg in _lib.lib().mcGetLastErrorString()


@pytest.mark.parametrize("fields,msg", [
    (dict(rhs_bits=4), b"L8-R8 with int32 output"),
    (dict(), b"chunk table"),
])
def test_spmm_auto_with_slot_major_values_takes_dense_tile(fields, msg):
    """Slot-major values under MC_KERNEL_AUTO go to the dense-tile kernel
    (its checks answer), since no other kernel reads that layout."""
    d = _lib.McSpmmDesc(m_vec=4, vec_length=8, n=128, k=64, lhs_bits=8, rhs_bits=8, batch=1, scale=1.0,
                        kernel_variant=_lib.KERNEL_AUTO, value_layout=_lib.VALUES_SLOT_MAJOR)
    for k, v in fields.items():
        setattr(d, k, v)
    assert _lib.lib().mcSpmm(ctypes.byref(d), None) == 1
    assert msg in _lib.lib().mcGetLastErrorString()


def test_chunk_starts_count_and_argument_errors():
    lib = _lib.lib()
    assert [lib.mcSpmmChunkStartsCount(k) for k in (0, 1, 64, 65, 1024)] == [0, 2, 2, 3, 17]
    assert lib.mcSpmmChunkStarts(4, 0, None, None, None, None, None) == 1
    assert b"k > 0" in lib.mcGetLastErrorString()
    assert lib.mcSpmmChunkStarts(4, 64, None, None, None, None, None) == 1
    assert b"null status" in lib.mcGetLastErrorString()


def test_device_slot_major_pack_argument_errors():
    """The device packers take slot-major values for L8-R8 only, into a
    16-byte aligned buffer; both checks run before any GPU work."""
    lib = _lib.lib()
    one = ctypes.c_int(0)
    ro = (ctypes.c_int * 2)(0, 0)
    rc = lib.mcDevicePackSpmmValues(1, 8, 8, 4, ctypes.addressof(ro), ctypes.addressof(ro), ctypes.addressof(one),
                                    None, 64, 64, _lib.VALUES_SLOT_MAJOR, None, None)
    assert rc == 1 and b"L8-R8" in lib.mcGetLastErrorString()
    rc = lib.mcDevicePackSpmmValues(1, 8, 8, 8, ctypes.addressof(ro), ctypes.addressof(ro), ctypes.addressof(one),
                                    None, 68, 64, _lib.VALUES_SLOT_MAJOR, None, None)
    assert rc == 1 and b"16 for slot-major" in lib.mcGetLastErrorString()
    d = _lib.McDevicePackDesc(m_vec=1, vec_length=8, lhs_bits=8, rhs_bits=4, value_layout=_lib.VALUES_SLOT_MAJOR,
                              row_offsets=ctypes.addressof(ro), aligned_nnz=ctypes.addressof(one), out_cols=64,
                              aligned_pairs=64, row_indices=64, out_values=64, values_capacity_bytes=64)
    assert lib.mcDevicePack(ctypes.byref(d), None) == 1
    assert b"slot-major" in lib.mcGetLastErrorString()
    d.rhs_bits, d.out_values = 8, 68
    assert lib.mcDevicePack(ctypes.byref(d), None) == 1
    assert b"16-byte aligned" in lib.mcGetLastErrorString()


@pytest.mark.parametrize("fields,msg", [
    (dict(vec_length=3), b"vec_length"), (dict(head_dim=128), b"head_dim"), (dict(lhs_bits=4), b"pairs"),
    (dict(requant=2), b"requant"), (dict(lhs_bits=16, requant=1), b"row-max"), (dict(scale_qkv=0.0), b"scales"),
    (dict(max_batch_tokens=0), b"max_batch_tokens"), (dict(max_inflight=9), b"max_inflight"),
    (dict(hbm_reserve_bytes=-1), b"reserve"),
])
def test_attn_server_rejects_bad_descriptors(fields, msg):
    """The request server checks its descriptor before touching a GPU."""
    d = _lib.McAttnServerDesc(vec_length=8, heads=4, head_dim=64, lhs_bits=8, rhs_bits=8, requant=1,
                              scale_qkv=40.0, scale_sfmx=127.0, max_batch_tokens=4096, max_inflight=2)
    for k, v in fields.items():
        setattr(d, k, v)
    h = ctypes.c_void_p()
    assert _lib.lib().mcAttnServerCreate(ctypes.byref(d), ctypes.byref(h)) == 1
    assert msg in _lib.lib().mcGetLastErrorString()
    assert _lib.lib().mcAttnServerRun(None, None, 0, None, None) == 1
    assert _lib.lib().mcAttnServerMemory(None, None, 0, None, None) == 1


def test_tile_mask_words_and_argument_errors():
    lib = _lib.lib()
    assert [lib.mcSddmmTileMaskWords(n) for n in (0, 1, 128, 129, 4096)] == [0, 4, 4, 8, 128]
    assert lib.mcSddmmTileMask(4, 0, None, None, None, None, None, None) == 1
    assert b"n > 0" in lib.mcGetLastErrorString()
    assert lib.mcSddmmTileMask(4, 128, None, None, None, None, None, None) == 1
    assert b"null status" in lib.mcGetLastErrorString()


def test_check_entry_points_reject_bad_arguments():
    lib = _lib.probe_lib()
    assert lib.mcCheckSmallIntConversions(0, 16, None, None) == 1
    assert lib.mcCheckSmallIntConversions(16, 8, ctypes.c_void_p(8), None) == 1  # lo > hi
    assert lib.mcCheckSmallIntConversions(0, 1 << 33, ctypes.c_void_p(8), None) == 1  # past 32-bit patterns


def test_attention_batch_engine_rejects_bad_descriptors():
    """mcAttnBatchCreate validates everything before touching a GPU."""
    lib = _lib.lib()
    h = ctypes.c_void_p()
    ro = (ctypes.c_int * 3)(0, 1, 2)
    ci = (ctypes.c_int * 2)(0, 1)
    ro_p = (ctypes.c_void_p * 1)(ctypes.addressof(ro))
    ci_p = (ctypes.c_void_p * 1)(ctypes.addressof(ci))
    lens = (ctypes.c_int * 1)(16)

    def desc(**kw):
        base = dict(n_instances=1, seq_lens=ctypes.addressof(lens), row_offsets=ctypes.addressof(ro_p),
                    col_indices=ctypes.addressof(ci_p), vec_length=8, heads=1, head_dim=64, lhs_bits=8,
                    rhs_bits=8, requant=0, scale_qkv=1.0, scale_sfmx=1.0)
        base.update(kw)
        return _lib.McAttnBatchDesc(**base)

    lens12 = (ctypes.c_int * 1)(12)
    for kw, msg in ((dict(n_instances=0), b"instance"), (dict(vec_length=3), b"vec_length"),
                    (dict(head_dim=128), b"head_dim"), (dict(lhs_bits=4, rhs_bits=4), b"pairs"),
                    (dict(lhs_bits=16, requant=1), b"row-max"), (dict(scale_qkv=0.0), b"scales"),
                    (dict(seq_lens=ctypes.addressof(lens12)), b"multiple of V")):
        d = desc(**kw)
        assert lib.mcAttnBatchCreate(ctypes.byref(d), ctypes.byref(h)) == 1
        assert msg in lib.mcGetLastErrorString(), (kw, lib.mcGetLastErrorString())
    bad = (ctypes.c_int * 2)(0, 99)
    ci_bad = (ctypes.c_void_p * 1)(ctypes.addressof(bad))
    d = desc(col_indices=ctypes.addressof(ci_bad))
    assert lib.mcAttnBatchCreate(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"outside" in lib.mcGetLastErrorString()
    assert lib.mcAttnBatchReplay(None, None) == 1
