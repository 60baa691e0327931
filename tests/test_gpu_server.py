"""Serving path (pk_submit / pk_poll): each request's result equals the same read
set run alone, in any mix of sizes and k, with failures isolated to their request and
admission held within the context's HBM budget."""
import numpy as np
import pytest

import pakman_plus_gb300 as pk
from gpu_helpers import assert_mn_equal, ctx, run_gpu
from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


def _mix():
    cases = []
    for i, (k, glen, nreads, t) in enumerate([(32, 20000, 6000, 21), (31, 5000, 1500, 12),
                                              (63, 12000, 4000, 10), (32, 60000, 20000, 30),
                                              (17, 3000, 900, 8), (63, 3000, 800, 5)]):
        lens = np.random.default_rng(9000 + i).integers(90, 152, nreads)
        rs = synth.small_case(9100 + i, genome_len=glen, n_reads=nreads, read_len=lens, err=0.005,
                              k=k, coverage=20)
        cases.append((rs.fasta, k, t, 20))
    return cases


def _params(k, t, cov):
    return pk.default_params(k=k, num_buckets=t, coverage=cov)


def test_requests_match_jobs_run_alone():
    cases = _mix()
    alone = [run_gpu(f, k, t, cov) for f, k, t, cov in cases]
    with pk.Server(ctx(), workers=3) as srv:
        tickets = [srv.submit(f, _params(k, t, cov)) for f, k, t, cov in cases]
        for tk, (s, _, _, _, mn, err) in zip(tickets, alone):
            assert err is None
            info = srv.wait(tk)
            assert info.done and info.status == 0
            assert info.summary.n_windows == s.n_windows
            assert info.summary.n_unique == s.n_unique
            assert info.summary.cutoff == s.cutoff
            assert info.summary.n_nodes == s.n_nodes
            got = srv.result(tk)
            ref = pk.to_key128(mn.keys)
            assert_mn_equal(got, ref, mn.suffix_counts, mn.prefix_counts)
            assert info.submit_ns <= info.start_ns <= info.end_ns
            srv.release(tk)
        st = srv.stats()
        assert st["completed"] == len(cases) and st["failed"] == 0


def test_caller_buffers_and_capacity_limit():
    f, k, t, cov = _mix()[0]
    s, _, _, _, mn, _ = run_gpu(f, k, t, cov)
    m = s.n_nodes
    keys = np.zeros(m + 5, np.uint64)
    suf = np.zeros((m + 5, 4), np.uint32)
    pre = np.zeros((m + 5, 4), np.uint32)
    small = (np.zeros(m - 1, np.uint64), np.zeros((m - 1, 4), np.uint32), np.zeros((m - 1, 4), np.uint32))
    with pk.Server(ctx(), workers=2) as srv:
        a = srv.submit(f, _params(k, t, cov), out=(keys, suf, pre))
        b = srv.submit(f, _params(k, t, cov), out=small)
        got = srv.result(a)
        assert_mn_equal(got, pk.to_key128(mn.keys), mn.suffix_counts, mn.prefix_counts)
        with pytest.raises(pk.PakmanError) as e:
            srv.wait(b)
        assert e.value.status == pk.capi.PK_ERR_LIMIT
        assert srv.poll(b).summary.n_nodes == m


def test_failed_request_does_not_disturb_others():
    cases = _mix()[:3]
    # a record that does not start with '>' (the reference asserts)
    bad = cases[0][0].replace(b"\n>r150\n", b"\nxr150\n", 1)
    assert bad != cases[0][0]
    with pk.Server(ctx(), workers=2) as srv:
        t_ok = [srv.submit(f, _params(k, t, cov)) for f, k, t, cov in cases]
        t_bad = srv.submit(bad, _params(32, 21, 20))
        with pytest.raises(pk.FormatError):
            srv.wait(t_bad)
        for tk, (f, k, t, cov) in zip(t_ok, cases):
            s = run_gpu(f, k, t, cov)[0]
            assert srv.wait(tk).summary.n_nodes == s.n_nodes
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 3


def test_admission_stays_within_budget():
    pkbuild.build()
    cases = _mix()
    fp = []
    for f, k, t, cov in cases:
        r = pk.capi.PkRequest()
        r.fasta_bytes = len(f)
        r.params = _params(k, t, cov)
        fp.append(pk.capi.lib().pk_request_footprint(r))
    budget = max(fp) + min(fp)  # the largest job plus the smallest fit together, no more
    with pk.Context(0, hbm_budget=budget) as c, pk.Server(c, workers=4) as srv:
        tickets = [srv.submit(f, _params(k, t, cov)) for f, k, t, cov in cases]
        for tk, (f, k, t, cov) in zip(tickets, cases):
            s = run_gpu(f, k, t, cov)[0]
            assert srv.wait(tk).summary.n_nodes == s.n_nodes
        st = srv.stats()
        assert st["peak_admitted_bytes"] <= budget
        assert st["completed"] == len(cases)
        used, _ = c.memory()
        assert used == 0


def _sized(seed, glen, nreads, k=32):
    rs = synth.small_case(seed, genome_len=glen, n_reads=nreads, read_len=100, err=0.005, k=k, coverage=20)
    return rs.fasta


def test_small_requests_overtake_queued_large_ones():
    """One worker: after the first large request, the queued small ones start before the
    second large one (least estimated work first), whatever the submission order."""
    large = [_sized(9300 + i, 400000, 160000) for i in range(2)]
    small = [_sized(9310 + i, 3000, 900) for i in range(4)]
    p = _params(32, 5, 20)
    with pk.Server(ctx(), workers=1, reserved_small=0) as srv:
        tl = [srv.submit(f, p) for f in large]
        ts = [srv.submit(f, p) for f in small]
        infos = {t: srv.wait(t) for t in tl + ts}
    assert max(infos[t].end_ns for t in ts) < infos[tl[1]].end_ns
    assert infos[tl[0]].start_ns < min(infos[t].start_ns for t in ts)


def test_aging_zero_serves_in_submission_order():
    """An aging bound of 0 ms makes every queued request the oldest first: plain FIFO."""
    fs = [_sized(9320 + i, 3000 + 4000 * (i % 3), 900 + 1200 * (i % 3)) for i in range(6)]
    p = _params(32, 5, 20)
    with pk.Server(ctx(), workers=1, reserved_small=0, aging_ms=0) as srv:
        ts = [srv.submit(f, p) for f in reversed(fs)]
        infos = [srv.wait(t) for t in ts]
    starts = [i.start_ns for i in infos]
    assert starts == sorted(starts)


def test_cancel_queued_and_running_requests():
    large = _sized(9330, 400000, 160000)
    small = [_sized(9331 + i, 3000, 900) for i in range(3)]
    p = _params(32, 5, 20)
    ref = [run_gpu(f, 32, 5, 20)[0] for f in small]
    with pk.Server(ctx(), workers=1, reserved_small=0) as srv:
        t_run = srv.submit(large, p)
        t_q = [srv.submit(f, p) for f in small]
        srv.cancel(t_q[1])  # still queued behind the running large request
        info = srv.poll(t_q[1])
        assert info.done and info.status == pk.capi.PK_ERR_CANCELLED
        with pytest.raises(pk.capi.Cancelled):
            srv.wait(t_q[1])
        srv.cancel(t_run)  # running: ends at its next stage boundary (or has finished)
        try:
            srv.wait(t_run)
        except pk.capi.Cancelled:
            pass
        assert srv.poll(t_run).status in (0, pk.capi.PK_ERR_CANCELLED)
        for i in (0, 2):
            assert srv.wait(t_q[i]).summary.n_nodes == ref[i].n_nodes
        with pytest.raises(pk.PakmanError) as e:
            srv.cancel(t_q[0])  # finished
        assert e.value.status == pk.capi.PK_ERR_STATE
        st = srv.stats()
        assert st["cancelled"] >= 1 and st["completed"] >= 2


def test_keep_on_device_hands_over_the_resident_job():
    """A keep_on_device request leaves its table and macro-nodes in HBM for further
    calls on the returned job (here the table and a compaction), counted against the
    budget until released."""
    f, k, t, cov = _mix()[0]
    s, keys, counts, hist, mn, err = run_gpu(f, k, t, cov)
    with pk.Context(0) as c, pk.Server(c, workers=2) as srv:
        tk = srv.submit(f, _params(k, t, cov), keep_on_device=True)
        info = srv.wait(tk)
        assert info.summary.n_nodes == s.n_nodes
        st = srv.stats()
        assert st["resident_jobs"] == 1 and st["resident_bytes"] > 0
        used, _ = c.memory()
        assert used >= st["resident_bytes"]
        job = srv.job(tk)
        k2, c2 = job.table()
        assert np.array_equal(pk.to_key128(k2), keys) and np.array_equal(c2, counts)
        got = job.macro_nodes(cov)
        assert_mn_equal(got, pk.to_key128(mn.keys), mn.suffix_counts, mn.prefix_counts)
        comp = job.compact(1000, cov)
        assert comp.n_nodes <= 1000
        with pytest.raises(pk.PakmanError):
            srv.result(tk)  # not kept in host memory
        srv.release(tk)
        st = srv.stats()
        assert st["resident_jobs"] == 0 and st["resident_bytes"] == 0
    # another request still runs normally on the same server afterwards is covered above


def test_next_done_hands_out_every_request_once_in_completion_order():
    cases = _mix()
    with pk.Server(ctx(), workers=3) as srv:
        tickets = [srv.submit(f, _params(k, t, cov)) for f, k, t, cov in cases]
        got = []
        for _ in tickets:
            info = srv.next_done()
            assert info.done
            got.append(info)
            srv.release(info.ticket)
        assert sorted(i.ticket for i in got) == sorted(tickets)
        ends = [i.end_ns for i in got]
        assert ends == sorted(ends)
        with pytest.raises(pk.capi.Busy):
            srv.next_done(timeout=0.05)


def test_sm_partition_for_small_requests():
    """With small_sms the device is split into two SM partitions (green contexts): small
    requests run on their own SMs, the others on the rest, and every result still equals
    the read set run alone (results copied out and kept on the device alike)."""
    cases = _mix()
    alone = [run_gpu(f, k, t, cov) for f, k, t, cov in cases]
    with pk.Server(ctx(), workers=2) as whole:  # no partition: the device's SMs twice
        total, again = whole.partition()
        assert total == again and total > 16
    try:
        srv = pk.Server(ctx(), workers=3, small_bytes=1 << 20, small_sms=16)
    except pk.PakmanError as ex:
        if ex.status == pk.capi.PK_ERR_CUDA:
            pytest.skip(f"SM partitions unavailable here: {ex}")
        raise
    with srv:
        small, large = srv.partition()
        assert small >= 16 and large > 0
        assert small + large <= total
        tickets = [srv.submit(f, _params(k, t, cov), keep_on_device=(i % 2 == 1))
                   for i, (f, k, t, cov) in enumerate(cases)]
        for i, (tk, (s, _, _, _, mn, err)) in enumerate(zip(tickets, alone)):
            info = srv.wait(tk)
            assert info.status == 0
            assert (info.summary.n_windows, info.summary.n_unique, info.summary.cutoff, info.summary.n_nodes) == \
                (s.n_windows, s.n_unique, s.cutoff, s.n_nodes)
            if i % 2 == 0:
                assert_mn_equal(srv.result(tk), pk.to_key128(mn.keys), mn.suffix_counts, mn.prefix_counts)
            srv.release(tk)
