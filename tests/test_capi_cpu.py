"""C-ABI library checks that need no GPU: it loads, exports every function the
public headers declare, and fails loudly (no CPU fallback) without a device."""
import ctypes

import pytest

import pakman_plus_gb300 as pk
from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import capi


@pytest.fixture(scope="module")
def lib():
    pkbuild.build()
    return capi.lib()


def test_every_declared_function_is_exported(lib):
    names = capi.header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(capi._SIGS), set(names) ^ set(capi._SIGS)


def test_params_layout_matches_c(lib):
    p = capi.default_params()
    assert ctypes.sizeof(capi.PkParams) == 64
    assert ctypes.sizeof(capi.PkSummary) == 48
    assert (p.k, p.lmer_length, p.num_buckets, p.batch_kmers) == (32, 8, 21, 100_000_000)


def test_status_strings(lib):
    assert capi.status_string(capi.PK_OK) == "ok"
    assert "'>'" in capi.status_string(capi.PK_ERR_FORMAT)
    assert capi.status_string(99) == "unknown status"


def test_null_arguments_are_rejected(lib):
    assert lib.pk_job_sync(None) == capi.PK_ERR_INVALID
    assert lib.pk_count(None, None, 0, None) == capi.PK_ERR_INVALID
    assert lib.pk_cutoff(None, 21, None, None, None) == capi.PK_ERR_INVALID
    assert lib.pk_ctx_create(0, 0, None) == capi.PK_ERR_INVALID
    info = capi.PkCompactionInfo()
    assert lib.pk_compact(None, 100, 0, ctypes.byref(info)) == capi.PK_ERR_INVALID
    assert lib.pk_compaction_get_info(None, ctypes.byref(info)) == capi.PK_ERR_INVALID
    assert lib.pk_copy_compacted(None, None, None, None, None, None, None) == capi.PK_ERR_INVALID
    assert lib.pk_copy_partial_contigs(None, None, None) == capi.PK_ERR_INVALID
    assert lib.pk_walk(None, None) == capi.PK_ERR_INVALID
    assert lib.pk_copy_walk_contigs(None, None, None) == capi.PK_ERR_INVALID


def test_compaction_structs_match_c(lib):
    """pk_compaction_info, pk_compact_entry and pk_walk_info as the header lays them out."""
    import pakman_plus_gb300.api as api
    assert ctypes.sizeof(capi.PkCompactionInfo) == 5 * 8 + 2 * 4
    assert api.COMPACT_ENTRY.itemsize == 32
    assert [api.COMPACT_ENTRY.fields[f][1] for f in ("ext_offset", "ext_length", "count", "visit", "terminal",
                                                     "prefix_pos", "num_wires")] == [0, 8, 12, 16, 20, 24, 28]
    assert ctypes.sizeof(capi.PkWalkInfo) == 3 * 8 + 2 * 4


def test_no_cpu_fallback_without_device(lib):
    n = ctypes.c_int()
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(pk.PakmanError) as e:
        pk.Context(0)
    assert e.value.status == capi.PK_ERR_NO_DEVICE


def test_serving_structs_and_footprint(lib):
    # pk_request: pointer, size, 64-byte params, three pointers, capacity
    assert ctypes.sizeof(capi.PkRequest) == 8 + 8 + 64 + 8 * 3 + 8 + 4 * 4
    assert ctypes.sizeof(capi.PkRequestInfo) == 8 + 48 + 8 * 3 + 8
    assert ctypes.sizeof(capi.PkServerStats) == 17 * 8
    assert ctypes.sizeof(capi.PkServerConfig) == 8 + 4 + 4 + 4 * 4
    cfg = capi.PkServerConfig()
    lib.pk_server_config_default(ctypes.byref(cfg), 8)
    assert (cfg.small_bytes, cfg.reserved_small, cfg.aging_ms, cfg.small_sms) == (32 << 20, 1, 2000, 0)
    assert lib.pk_server_partition(None, None, None) == capi.PK_ERR_INVALID
    # batch input modes: copies inside the graph (default) or before it
    assert (capi.PK_BATCH_INPUT_IN_GRAPH, capi.PK_BATCH_INPUT_BEFORE) == (0, 1)
    assert lib.pk_batch_set_input_mode(None, capi.PK_BATCH_INPUT_BEFORE) == capi.PK_ERR_INVALID
    assert lib.pk_cancel(None, 1) == capi.PK_ERR_INVALID
    assert lib.pk_result_job(None, 1, None) == capi.PK_ERR_INVALID
    assert capi.status_string(capi.PK_ERR_CANCELLED) == "cancelled"
    r = capi.PkRequest()
    r.params = capi.default_params(k=32)
    r.fasta_bytes = 1 << 20
    small = lib.pk_request_footprint(ctypes.byref(r))
    r.fasta_bytes = 1 << 24
    big = lib.pk_request_footprint(ctypes.byref(r))
    r.params = capi.default_params(k=63)
    wide = lib.pk_request_footprint(ctypes.byref(r))
    assert small < big < wide
    assert big >= (1 << 24) * (1 + 2 * 8 + 4)  # FASTA + two key arrays + counts at N = F
    assert lib.pk_request_footprint(None) == 0
    # with the input at hand the window count is estimated from its first records
    reads = b"".join(b">r%d\n" % i + b"ACGT" * 25 + b"\n" for i in range(20000))
    buf = ctypes.create_string_buffer(reads, len(reads))
    r = capi.PkRequest()
    r.params = capi.default_params(k=32)
    r.fasta = ctypes.cast(buf, ctypes.c_void_p)
    r.fasta_bytes = len(reads)
    sampled = lib.pk_request_footprint(ctypes.byref(r))
    r.fasta = None
    bound = lib.pk_request_footprint(ctypes.byref(r))
    windows = 20000 * 69
    assert sampled < bound
    assert sampled >= len(reads) + windows * (2 * 8 + 4)
    assert lib.pk_server_create(None, 2, None) == capi.PK_ERR_INVALID
    assert lib.pk_submit(None, None, None) == capi.PK_ERR_INVALID


def test_batch_structs(lib):
    assert ctypes.sizeof(capi.PkBatchSet) == 8 + 8 + 64
    assert ctypes.sizeof(capi.PkBatchResult) == 4 + 4 + 48 + 8
    assert ctypes.sizeof(capi.PkBatchStats) == 6 * 8 + 2 * 8
    assert lib.pk_batch_create(None, 2, None) == capi.PK_ERR_INVALID
    assert lib.pk_batch_tuned_bits(None, 100, 32) == 0
