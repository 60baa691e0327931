"""pk_cutoff_noalloc: the histogram cutoff for callers that cannot allocate device
memory (their own allocator owns every device allocation, or an allocation could block
a latency-critical loop, or the device budget is already committed).  It must give the
same histogram, cutoff and kept-row count as pk_cutoff, call after call, from its static
scratch array.  Collected last so a failure here does not hide the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_cutoff_matches_pk_cutoff_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import pakman_plus_gb300 as pk
    from golden_cases import load
    from pakman_plus_gb300 import build as pkbuild
    from pakman_plus_gb300 import capi

    pkbuild.build()
    L = capi.lib()
    g = load("k32_ragged")
    with pk.Context(0) as ctx, pk.Job(ctx) as job:
        job.count(g.fasta, pk.default_params(k=g.k, num_buckets=g.t, coverage=g.coverage))
        n_rows, _, _ = job.table_info()
        _, d_counts = job.table_device()
        stream = torch.cuda.current_stream().cuda_stream
        # two calls in a row; the second uses a smaller t, so bins the first call filled
        # must not leak into it
        for t in (40, 7):
            try:
                ref_cut, ref_hist, ref_kept = job.cutoff(t)
            except pk.EmptyAfterCutoff as e:
                ref_cut, ref_hist, ref_kept = e.cutoff, e.hist, e.kept
            d_cut = torch.zeros(1, dtype=torch.int32, device="cuda")
            d_hist = torch.full((t,), -1, dtype=torch.int64, device="cuda")
            d_kept = torch.zeros(1, dtype=torch.int64, device="cuda")
            st = L.pk_cutoff_noalloc(ctypes.c_void_p(d_counts), n_rows, t, d_cut.data_ptr(),
                                     d_hist.data_ptr(), d_kept.data_ptr(), ctypes.c_void_p(stream))
            assert st == capi.PK_OK, capi.last_error()
            torch.cuda.synchronize()
            assert int(d_cut.item()) == ref_cut
            assert np.array_equal(d_hist.cpu().numpy().astype(np.uint64), ref_hist)
            assert int(d_kept.item()) == ref_kept


def test_noalloc_cutoff_rejects_more_bins_than_its_scratch():
    from pakman_plus_gb300 import build as pkbuild
    from pakman_plus_gb300 import capi

    pkbuild.build()
    L = capi.lib()
    dummy = ctypes.c_void_p(1 << 20)
    assert L.pk_cutoff_noalloc(None, 0, 4097, dummy, None, None, None) == capi.PK_ERR_INVALID
    assert "4096" in capi.last_error()
    assert L.pk_cutoff_noalloc(None, 0, 0, dummy, None, None, None) == capi.PK_ERR_INVALID
