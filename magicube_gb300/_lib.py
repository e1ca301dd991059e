"""ctypes binding of libmagicube_gb300.so (the C ABI in include/magicube_gb300.h).

The library is loaded from the package directory.  There is no fallback: if
the shared object is missing every entry point raises, so a run can never
silently compute on the CPU.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name("libmagicube_gb300.so")

_c_int, _c_ll, _c_float, _c_vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_float, ctypes.c_void_p


class McSpmmDesc(ctypes.Structure):
    _fields_ = [
        ("m_vec", _c_int), ("vec_length", _c_int), ("n", _c_int), ("k", _c_int),
        ("lhs_bits", _c_int), ("rhs_bits", _c_int), ("is_signed", _c_int), ("out_half", _c_int),
        ("scale", _c_float), ("batch", _c_int),
        ("row_indices", _c_vp), ("row_offsets", _c_vp), ("column_indices", _c_vp),
        ("values", _c_vp), ("values_stride", _c_ll),
        ("rhs", _c_vp), ("rhs_stride", _c_ll),
        ("out", _c_vp), ("out_stride", _c_ll),
        ("mma_kind", _c_int), ("kernel_variant", _c_int), ("value_layout", _c_int),
        ("row_div", _c_vp), ("row_div_stride", _c_ll),
        ("kernel_config", _c_int), ("chunk_starts", _c_vp),
    ]


class McSddmmDesc(ctypes.Structure):
    _fields_ = [
        ("m_vec", _c_int), ("vec_length", _c_int), ("n", _c_int), ("k", _c_int),
        ("lhs_bits", _c_int), ("rhs_bits", _c_int), ("is_signed", _c_int), ("out_half", _c_int),
        ("out_vecmajor", _c_int), ("scale", _c_float), ("batch", _c_int), ("row_split", _c_int),
        ("row_indices", _c_vp), ("row_offsets", _c_vp), ("column_indices", _c_vp),
        ("lhs", _c_vp), ("lhs_stride", _c_ll),
        ("rhs", _c_vp), ("rhs_stride", _c_ll),
        ("out", _c_vp), ("out_stride", _c_ll),
        ("mma_kind", _c_int), ("kernel_variant", _c_int),
        ("tile_bitmap", _c_vp), ("tile_prefix", _c_vp),
    ]


class McSoftmaxDesc(ctypes.Structure):
    _fields_ = [
        ("m_vec", _c_int), ("vec_length", _c_int), ("batch", _c_int), ("bits", _c_int),
        ("scaling", _c_float), ("scale", _c_float),
        ("row_indices", _c_vp), ("row_offsets", _c_vp),
        ("scores", _c_vp), ("scores_stride", _c_ll),
        ("out", _c_vp), ("out_stride", _c_ll),
        ("requant", _c_int), ("row_div", _c_vp), ("row_div_stride", _c_ll),
    ]


class McAttnDesc(ctypes.Structure):
    _fields_ = [
        ("m_vec", _c_int), ("vec_length", _c_int), ("heads", _c_int), ("head_dim", _c_int),
        ("max_row_nnz", _c_int), ("lhs_bits", _c_int), ("rhs_bits", _c_int), ("requant", _c_int),
        ("score_scale", _c_float), ("scaling", _c_float), ("prob_scale", _c_float), ("out_scale", _c_float),
        ("row_indices", _c_vp), ("row_offsets", _c_vp), ("column_indices", _c_vp),
        ("q", _c_vp), ("k", _c_vp), ("v", _c_vp), ("head_stride", _c_ll),
        ("out", _c_vp), ("out_head_stride", _c_ll), ("status", _c_vp),
        ("warps", _c_int), ("stages", _c_int), ("ctas_per_sm", _c_int),
    ]


class McAttnServerDesc(ctypes.Structure):
    _fields_ = [
        ("vec_length", _c_int), ("heads", _c_int), ("head_dim", _c_int), ("lhs_bits", _c_int), ("rhs_bits", _c_int),
        ("requant", _c_int), ("scale_qkv", _c_float), ("scale_sfmx", _c_float), ("max_batch_tokens", _c_ll),
        ("max_inflight", _c_int), ("hbm_reserve_bytes", _c_ll),
    ]


class McAttnRequest(ctypes.Structure):
    _fields_ = [
        ("seq_len", _c_int), ("nnz_vec", _c_int), ("max_row_nnz", _c_int), ("row_offsets", _c_vp),
        ("col_indices", _c_vp), ("qkv", _c_vp), ("out", _c_vp), ("arrival_s", ctypes.c_double),
    ]


class McAttnServeStats(ctypes.Structure):
    _fields_ = [
        ("makespan_s", ctypes.c_double), ("req_per_s", ctypes.c_double), ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double), ("served", _c_int), ("rejected", _c_int),
        ("batches", _c_int), ("max_inflight_seen", _c_int), ("held_back", _c_int),
    ]


class McQkvProjDesc(ctypes.Structure):
    _fields_ = [
        ("tokens", _c_int), ("hidden", _c_int), ("heads", _c_int), ("head_dim", _c_int), ("bits", _c_int),
        ("scale", _c_float), ("x", _c_vp), ("weight", _c_vp), ("bias", _c_vp), ("out", _c_vp), ("status", _c_vp),
    ]


class McDevicePackDesc(ctypes.Structure):
    _fields_ = [
        ("m_vec", _c_int), ("vec_length", _c_int), ("lhs_bits", _c_int), ("rhs_bits", _c_int),
        ("alignment", _c_int), ("shuffle8", _c_int), ("value_layout", _c_int), ("sort_rows", _c_int),
        ("row_offsets", _c_vp), ("col_indices", _c_vp), ("values", _c_vp),
        ("aligned_pairs", _c_vp), ("aligned_nnz", _c_vp),
        ("out_cols", _c_vp), ("cols_capacity", _c_ll), ("out_values", _c_vp), ("values_capacity_bytes", _c_ll),
        ("row_indices", _c_vp), ("status", _c_vp),
    ]


class McAttnBatchDesc(ctypes.Structure):
    _fields_ = [
        ("n_instances", _c_int), ("seq_lens", _c_vp), ("row_offsets", _c_vp), ("col_indices", _c_vp),
        ("vec_length", _c_int), ("heads", _c_int), ("head_dim", _c_int), ("lhs_bits", _c_int), ("rhs_bits", _c_int),
        ("requant", _c_int), ("scale_qkv", _c_float), ("scale_sfmx", _c_float),
    ]


REQUANT_FIXED, REQUANT_ROWMAX = 0, 1
MMA_DEFAULT, MMA_INT8, MMA_F16, MMA_TCGEN05, MMA_DP4A = 0, 1, 2, 3, 4
KERNEL_AUTO, KERNEL_PER_ROW, KERNEL_STREAM, KERNEL_TMA, KERNEL_DENSE_TILE, KERNEL_RESIDENT = 0, 1, 2, 3, 4, 5
RESIDENT_AUTO, RESIDENT_S64_W8, RESIDENT_S64_W16, RESIDENT_S128_W16 = 0, 1, 2, 3
VALUES_PACKED, VALUES_SOFTMAX, VALUES_SLOT_MAJOR = 0, 1, 2

# name -> (restype, argtypes)
_IP = ctypes.POINTER(ctypes.c_int)
_SIGNATURES = {
    "mcGetLastErrorString": (ctypes.c_char_p, []),
    "mcVersion": (ctypes.c_char_p, []),
    "mcSetDefaultMmaKind": (_c_int, [_c_int]),
    "mcTensorCoreTimeouts": (ctypes.c_uint, []),
    "mcSpmm": (_c_int, [ctypes.POINTER(McSpmmDesc), _c_vp]),
    "mcSddmm": (_c_int, [ctypes.POINTER(McSddmmDesc), _c_vp]),
    "mcSddmmTileMaskWords": (_c_int, [_c_int]),
    "mcSddmmTileMask": (_c_int, [_c_int, _c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "mcSpmmChunkStartsCount": (_c_int, [_c_int]),
    "mcSpmmChunkStarts": (_c_int, [_c_int, _c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "mcQuantize": (_c_int, [_c_vp, _c_vp, _c_ll, _c_int, _c_float, _c_vp]),
    "mcQuantSoftmax": (_c_int, [ctypes.POINTER(McSoftmaxDesc), _c_vp]),
    "mcSparseAttention": (_c_int, [ctypes.POINTER(McAttnDesc), _c_vp]),
    "mcAlignRowOffsets": (_c_int, [_c_int, _c_vp, _c_int, _c_vp]),
    "mcPadColumnIndices": (_c_int, [_c_int, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_vp]),
    "mcPackSpmmValues": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_vp, _c_vp, _c_int, _c_vp, _c_vp]),
    "mcPackSpmmValuesEx": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_int]),
    "mcSortedRowSwizzle": (_c_int, [_c_int, _c_vp, _c_vp]),
    "mcIdentityRowSwizzle": (_c_int, [_c_int, _c_vp]),
    "mcDeviceAlignRowOffsets": (_c_int, [_c_int, _c_vp, _c_int, _c_vp, _c_vp, _c_vp]),
    "mcDeviceAlignRowOffsetsNoAlloc": (_c_int, [_c_int, _c_vp, _c_int, _c_vp, _c_vp, _c_vp]),
    "mcDevicePadColumnIndices": (_c_int, [_c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_ll, _c_vp, _c_vp]),
    "mcDevicePackSpmmValues": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_ll,
                                        _c_int, _c_vp, _c_vp]),
    "mcDeviceSortedRowSwizzle": (_c_int, [_c_int, _c_vp, _c_vp, _c_vp]),
    "mcDevicePack": (_c_int, [ctypes.POINTER(McDevicePackDesc), _c_vp]),
    "mcQkvProjectQuantize": (_c_int, [ctypes.POINTER(McQkvProjDesc), _c_vp]),
    "mcAttnBatchCreate": (_c_int, [ctypes.POINTER(McAttnBatchDesc), ctypes.POINTER(_c_vp)]),
    "mcAttnBatchTokens": (_c_int, [_c_vp, ctypes.POINTER(_c_ll)]),
    "mcAttnBatchRun": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "mcAttnBatchTune": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _IP, _IP, _IP]),
    "mcAttnBatchCapture": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "mcAttnBatchReplay": (_c_int, [_c_vp, _c_vp]),
    "mcAttnBatchStatus": (_c_int, [_c_vp, _IP]),
    "mcAttnBatchDestroy": (None, [_c_vp]),
    "mcAttnServerCreate": (_c_int, [ctypes.POINTER(McAttnServerDesc), ctypes.POINTER(_c_vp)]),
    "mcAttnServerRun": (_c_int, [_c_vp, ctypes.POINTER(McAttnRequest), _c_int, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(McAttnServeStats)]),
    "mcAttnServerMemory": (_c_int, [_c_vp, ctypes.POINTER(McAttnRequest), _c_int, ctypes.POINTER(_c_ll),
                                    ctypes.POINTER(_c_ll)]),
    "mcAttnServerDestroy": (None, [_c_vp]),
}
# the diagnostics library (include/magicube_gb300_probe.h)
_PROBE_SIGNATURES = {
    "mcProbeTensorPeak": (_c_int, [_c_int, _c_vp, _c_ll, _c_int, ctypes.POINTER(ctypes.c_float),
                                   ctypes.POINTER(ctypes.c_double), _c_vp]),
    "mcCheckQuotients": (_c_int, [_c_float, _c_ll, _c_ll, _c_vp, _c_vp]),
    "mcCheckSmallIntConversions": (_c_int, [ctypes.c_ulonglong, ctypes.c_ulonglong, _c_vp, _c_vp]),
    "mcProbeTensorCorePeak": (_c_int, [_c_int, _c_int, ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_double), _c_vp, _c_vp]),
}
for _p in ("4b", "8b4b", "12b4b", "16b4b", "8b", "12b8b", "16b8b", "16b"):
    _SIGNATURES[f"mcWmmaSpmm_{_p}"] = (_c_int, [_c_int, _c_int, _c_int, _c_int] + [_c_vp] * 6)
for _p in ("4b", "8b", "16b"):
    _SIGNATURES[f"mcWmmaSddmm_{_p}"] = (_c_int, [_c_int, _c_int, _c_int] + [_c_vp] * 6 + [_c_int])

_lock = threading.Lock()
_handle: ctypes.CDLL | None = None


class MagicubeError(RuntimeError):
    """A C-ABI call returned a nonzero status."""


def lib() -> ctypes.CDLL:
    """The loaded library (raises if it has not been built)."""
    global _handle
    if _handle is None:
        with _lock:
            if _handle is None:
                if not LIB_PATH.exists():
                    raise ImportError(
                        f"{LIB_PATH} is missing: build it with `python -m magicube_gb300.build` "
                        "(the CUDA library is required; there is no CPU fallback)")
                h = ctypes.CDLL(str(LIB_PATH))
                for name, (res, args) in _SIGNATURES.items():
                    fn = getattr(h, name)
                    fn.restype = res
                    fn.argtypes = args
                _handle = h
    return _handle


_probe: ctypes.CDLL | None = None
PROBE_PATH = LIB_PATH.with_name("libmagicube_gb300_probe.so")


def probe_lib() -> ctypes.CDLL:
    """The diagnostics library (tensor-peak probes, arithmetic checks); it
    reports errors through the main library's mcGetLastErrorString."""
    global _probe
    if _probe is None:
        with _lock:
            if _probe is None:
                lib()
                if not PROBE_PATH.exists():
                    raise ImportError(f"{PROBE_PATH} is missing: build it with `python -m magicube_gb300.build`")
                h = ctypes.CDLL(str(PROBE_PATH))
                for name, (res, args) in _PROBE_SIGNATURES.items():
                    fn = getattr(h, name)
                    fn.restype = res
                    fn.argtypes = args
                _probe = h
    return _probe


def check(rc: int, what: str) -> None:
    """Raise MagicubeError for a nonzero C-ABI status."""
    if rc != 0:
        msg = lib().mcGetLastErrorString().decode() or f"CUDA error {rc}"
        raise MagicubeError(f"{what} failed: {msg} (status {rc})")


def exported_symbols() -> list[str]:
    """Names of every entry point the binding declares."""
    return sorted(_SIGNATURES)
