"""ctypes binding of libpakman_gb300.so (the C ABI declared in include/pakman_gb300.h).

The library is the only compute path: if it is missing or no CUDA device is
present, calls raise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
from ctypes import POINTER, byref, c_char_p, c_float, c_int, c_int32, c_uint32, c_uint64, c_void_p

from . import build as _build

LIB_PATH = _build.LIB
HEADER = os.path.join(_build.INCLUDE, "pakman_gb300.h")

PK_OK = 0
PK_ERR_INVALID = 1
PK_ERR_FORMAT = 2
PK_ERR_EMPTY = 3
PK_ERR_NOMEM = 4
PK_ERR_CUDA = 5
PK_ERR_STATE = 6
PK_ERR_LIMIT = 7
PK_ERR_DEVICE = 8
PK_ERR_BUSY = 9
PK_ERR_NO_DEVICE = 10
PK_ERR_IO = 11
PK_ERR_CANCELLED = 12

# pk_batch_set_input_mode
PK_BATCH_INPUT_IN_GRAPH = 0
PK_BATCH_INPUT_BEFORE = 1


class PkParams(ctypes.Structure):
    _fields_ = [("k", c_int32), ("lmer_length", c_int32), ("num_buckets", c_int32),
                ("coverage", c_int32), ("read_length", c_int32), ("drop_n", c_int32),
                ("batch_kmers", c_uint64), ("bucket_bits", c_int32), ("mn_units", c_int32),
                ("chunking", c_int32), ("reserved", c_int32 * 5)]


class PkSummary(ctypes.Structure):
    _fields_ = [("n_reads", c_uint64), ("n_windows", c_uint64), ("n_unique", c_uint64),
                ("n_kept", c_uint64), ("n_nodes", c_uint64), ("cutoff", c_uint32),
                ("key_bytes", c_int32)]


class PkRequest(ctypes.Structure):
    _fields_ = [("fasta", c_void_p), ("fasta_bytes", c_uint64), ("params", PkParams),
                ("mn_keys", c_void_p), ("mn_suffix", c_void_p), ("mn_prefix", c_void_p),
                ("mn_capacity", c_uint64), ("keep_on_device", c_int32), ("reserved", c_int32 * 3)]


class PkRequestInfo(ctypes.Structure):
    _fields_ = [("status", c_int), ("done", c_int32), ("summary", PkSummary),
                ("submit_ns", c_uint64), ("start_ns", c_uint64), ("end_ns", c_uint64),
                ("attempts", c_uint32), ("reserved", c_uint32)]


class PkServerStats(ctypes.Structure):
    _fields_ = [(n, c_uint64) for n in ("submitted", "completed", "failed", "queued", "running",
                                        "admitted_bytes", "peak_admitted_bytes", "requeued", "cancelled",
                                        "resident_bytes", "resident_jobs", "count_ns", "cutoff_ns", "mn_ns",
                                        "copyout_ns", "release_ns", "pin_ns")]


class PkServerConfig(ctypes.Structure):
    _fields_ = [("small_bytes", c_uint64), ("reserved_small", c_int32), ("aging_ms", c_int32),
                ("small_sms", c_int32), ("reserved", c_int32 * 3)]


class PkBatchSet(ctypes.Structure):
    _fields_ = [("fasta", c_void_p), ("fasta_bytes", c_uint64), ("params", PkParams)]


class PkBatchResult(ctypes.Structure):
    _fields_ = [("status", c_int), ("rerun", c_int32), ("summary", PkSummary), ("mn_first", c_uint64)]


class PkBatchStats(ctypes.Structure):
    _fields_ = [("graph_launches", c_uint64), ("graph_captures", c_uint64),
                ("kernels_per_launch", c_uint64), ("reruns", c_uint64), ("tuned_classes", c_uint64),
                ("total_nodes", c_uint64), ("last_graph_ms", ctypes.c_double), ("tune_ms", ctypes.c_double)]


class PkWiring(ctypes.Structure):
    _fields_ = [("n_suffixes", c_int32), ("n_prefixes", c_int32), ("terminal_suffix_visit", c_int32),
                ("terminal_prefix_visit", c_int32), ("n_wires", c_int32), ("wire", (c_int32 * 3) * 9),
                ("prefix_begin", (c_int32 * 2) * 5)]


class PkCompactionInfo(ctypes.Structure):
    _fields_ = [("n_nodes", c_uint64), ("n_entries", c_uint64), ("n_contigs", c_uint64),
                ("ext_bases", c_uint64), ("contig_bases", c_uint64), ("rounds", c_int32),
                ("key_bytes", c_int32)]


class PkWalkInfo(ctypes.Structure):
    _fields_ = [("n_begins", c_uint64), ("n_contigs", c_uint64), ("contig_bases", c_uint64),
                ("max_depth", c_uint32), ("reserved", c_uint32)]


class PakmanError(RuntimeError):
    """A failed C-ABI call; `status` is the pk_status code."""

    def __init__(self, status: int, func: str, detail: str):
        super().__init__(f"{func}: {status_string(status)} ({detail})" if detail else
                         f"{func}: {status_string(status)}")
        self.status = status


class FormatError(PakmanError):
    """A record start is not '>' (the reference asserts)."""


class EmptyAfterCutoff(PakmanError):
    """No k-mer reaches the histogram cutoff (the reference calls MPI_Abort)."""


class OutOfMemory(PakmanError):
    pass


class Busy(PakmanError):
    pass


class Cancelled(PakmanError):
    """The served request was cancelled (pk_cancel)."""


class InputFileError(PakmanError):
    """The FASTA file cannot be opened or read (the reference exits with status 2)."""


_ERR_CLASSES = {PK_ERR_FORMAT: FormatError, PK_ERR_EMPTY: EmptyAfterCutoff,
                PK_ERR_NOMEM: OutOfMemory, PK_ERR_BUSY: Busy, PK_ERR_IO: InputFileError,
                PK_ERR_CANCELLED: Cancelled}

_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "pk_params_default": (None, [POINTER(PkParams)]),
    "pk_status_string": (c_char_p, [c_int]),
    "pk_last_error": (c_char_p, []),
    "pk_version": (c_char_p, []),
    "pk_kernel_launches": (c_uint64, []),
    "pk_ctx_create": (c_int, [c_int, c_uint64, POINTER(c_void_p)]),
    "pk_ctx_destroy": (None, [c_void_p]),
    "pk_ctx_memory": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "pk_job_create": (c_int, [c_void_p, c_void_p, POINTER(c_void_p)]),
    "pk_job_destroy": (None, [c_void_p]),
    "pk_job_reset": (c_int, [c_void_p]),
    "pk_job_sync": (c_int, [c_void_p]),
    "pk_job_memory": (c_int, [c_void_p, POINTER(c_uint64)]),
    "pk_count": (c_int, [c_void_p, c_void_p, c_uint64, POINTER(PkParams)]),
    "pk_count_device": (c_int, [c_void_p, c_void_p, c_uint64, POINTER(PkParams)]),
    "pk_count_file": (c_int, [c_void_p, c_char_p, c_int32, c_int32, POINTER(PkParams)]),
    "pk_fasta_slice": (c_int, [c_char_p, c_int32, c_int32, c_int32, POINTER(c_uint64), POINTER(c_uint64)]),
    "pk_table_load": (c_int, [c_void_p, c_void_p, c_void_p, c_uint64, POINTER(PkParams)]),
    "pk_table_info": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64)]),
    "pk_count_pieces": (c_int, [c_void_p, POINTER(c_uint32)]),
    "pk_copy_table": (c_int, [c_void_p, c_void_p, c_void_p, c_uint64]),
    "pk_copy_table_packed": (c_int, [c_void_p, c_void_p, c_uint64]),
    "pk_table_device": (c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p)]),
    "pk_cutoff": (c_int, [c_void_p, c_int32, POINTER(c_uint32), c_void_p, POINTER(c_uint64)]),
    "pk_build_macro_nodes": (c_int, [c_void_p, c_uint32, POINTER(c_uint64)]),
    "pk_copy_macro_nodes": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "pk_macro_nodes_device": (c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p),
                                      POINTER(c_void_p)]),
    "pk_run": (c_int, [c_void_p, c_void_p, c_uint64, POINTER(PkParams), POINTER(PkSummary)]),
    "pk_run_device": (c_int, [c_void_p, c_void_p, c_uint64, POINTER(PkParams),
                              POINTER(PkSummary)]),
    "pk_summary_get": (c_int, [c_void_p, POINTER(PkSummary)]),
    "pk_wire_macro_nodes": (c_int, [c_void_p, c_int32]),
    "pk_copy_wiring": (c_int, [c_void_p, c_void_p, c_uint64]),
    "pk_wiring_device": (c_int, [c_void_p, POINTER(c_void_p)]),
    "pk_compact": (c_int, [c_void_p, c_uint64, c_int32, POINTER(PkCompactionInfo)]),
    "pk_compaction_get_info": (c_int, [c_void_p, POINTER(PkCompactionInfo)]),
    "pk_copy_compacted": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pk_copy_partial_contigs": (c_int, [c_void_p, c_void_p, c_void_p]),
    "pk_walk": (c_int, [c_void_p, POINTER(PkWalkInfo)]),
    "pk_copy_walk_contigs": (c_int, [c_void_p, c_void_p, c_void_p]),
    "pk_job_enable_timing": (c_int, [c_void_p, c_int]),
    "pk_job_set_wait_limit": (c_int, [c_void_p, c_uint32, c_int32]),
    "pk_job_stage_times": (c_int, [c_void_p, POINTER(c_float), c_int, POINTER(c_int)]),
    "pk_stage_name": (c_char_p, [c_int]),
    "pk_cutoff_noalloc": (c_int, [c_void_p, c_uint64, c_int32, c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "pk_server_create": (c_int, [c_void_p, c_int32, POINTER(c_void_p)]),
    "pk_server_config_default": (None, [POINTER(PkServerConfig), c_int32]),
    "pk_server_create_config": (c_int, [c_void_p, c_int32, POINTER(PkServerConfig), POINTER(c_void_p)]),
    "pk_cancel": (c_int, [c_void_p, c_uint64]),
    "pk_server_cache_release": (None, []),
    "pk_server_partition": (c_int, [c_void_p, POINTER(c_int32), POINTER(c_int32)]),
    "pk_batch_set_input_mode": (c_int, [c_void_p, c_int32]),
    "pk_next_done": (c_int, [c_void_p, ctypes.c_int64, POINTER(c_uint64), POINTER(PkRequestInfo)]),
    "pk_result_job": (c_int, [c_void_p, c_uint64, POINTER(c_void_p)]),
    "pk_server_destroy": (None, [c_void_p]),
    "pk_submit": (c_int, [c_void_p, POINTER(PkRequest), POINTER(c_uint64)]),
    "pk_poll": (c_int, [c_void_p, c_uint64, POINTER(PkRequestInfo)]),
    "pk_wait": (c_int, [c_void_p, c_uint64, ctypes.c_int64, POINTER(PkRequestInfo)]),
    "pk_result_get": (c_int, [c_void_p, c_uint64, POINTER(c_void_p), POINTER(c_void_p),
                              POINTER(c_void_p), POINTER(c_uint64)]),
    "pk_result_release": (c_int, [c_void_p, c_uint64]),
    "pk_server_get_stats": (c_int, [c_void_p, POINTER(PkServerStats)]),
    "pk_request_footprint": (c_uint64, [POINTER(PkRequest)]),
    "pk_batch_create": (c_int, [c_void_p, c_int32, POINTER(c_void_p)]),
    "pk_batch_destroy": (None, [c_void_p]),
    "pk_batch_run": (c_int, [c_void_p, POINTER(PkBatchSet), c_int32, POINTER(PkBatchResult)]),
    "pk_batch_copy_macro_nodes": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64]),
    "pk_batch_get_stats": (c_int, [c_void_p, POINTER(PkBatchStats)]),
    "pk_batch_tuned_bits": (c_int32, [c_void_p, c_uint64, c_int32]),
    "pk_batch_tuned_shape": (c_int, [c_void_p, c_uint64, c_int32, POINTER(c_int32), POINTER(c_int32),
                                     POINTER(c_int32)]),
    "pk_host_alloc": (c_int, [c_uint64, POINTER(c_void_p)]),
    "pk_host_free": (None, [c_void_p]),
}


def header_functions():
    """Names of the functions declared in include/*.h (parsed from the headers)."""
    names = []
    inc = os.path.dirname(HEADER)
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(inc, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(pk_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def lib():
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -m pakman_plus_gb300.build` "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(s: int) -> str:
    return lib().pk_status_string(s).decode()


def last_error() -> str:
    return lib().pk_last_error().decode()


def check(status: int, func: str):
    if status != PK_OK:
        cls = _ERR_CLASSES.get(status, PakmanError)
        raise cls(status, func, last_error())


def default_params(**kw) -> PkParams:
    p = PkParams()
    lib().pk_params_default(byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown parameter {k}")
        setattr(p, k, int(v))
    return p
