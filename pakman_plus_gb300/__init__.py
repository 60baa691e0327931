"""GB300-native PaKman k-mer counting -> histogram cutoff -> macro-node path.

Compute runs only in the sm_103a kernels of ``libpakman_gb300.so`` behind the C
ABI in ``include/pakman_gb300.h``; this package is the host-side mirror of the
reference's interface for that path.  There is no CPU fallback.
"""
from .api import (KEY128, KMERPAIRS64, KMERPAIRS128, Batch, BatchResult, Compaction, Context,  # noqa: F401
                  EmptyAfterCutoff,
                  FormatError, InputFileError, Job, MacroNodeTable, PakmanError, PakmanSession, RequestInfo,
                  Server, Summary,
                  default_params, fasta_slice, key_dtype, to_key128)
from .capi import lib as load_library  # noqa: F401

__all__ = ["Context", "Job", "Compaction", "Server", "Batch", "BatchResult", "RequestInfo", "PakmanSession", "MacroNodeTable", "Summary", "default_params",
           "PakmanError", "FormatError", "EmptyAfterCutoff", "KEY128", "KMERPAIRS64",
           "KMERPAIRS128", "key_dtype", "to_key128", "load_library"]
