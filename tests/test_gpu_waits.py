"""Bounded device waits: a wait that runs out ends the call with PK_ERR_DEVICE and
leaves the context usable.

The fault is injected on the host side: one macro-node work unit is told to publish no
look-back word, so the units after it wait for a word that nothing writes.  With a short
poll limit those waits give up within microseconds, set the look-back error bit and
return; nothing hangs and no kernel faults."""
import numpy as np
import pytest

import pakman_plus_gb300 as pk
from gpu_helpers import assert_mn_equal, assert_table_equal, ctx
from oracle import pk_oracle as po
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


def _case():
    rs = synth.small_case(4711, genome_len=40000, n_reads=24000, read_len=100, err=0.005, k=32)
    return rs, po.run(rs.fasta, 32, 21)


def test_withheld_lookback_word_fails_the_call_and_the_job_recovers():
    rs, ora = _case()
    # small units (mn_units=1: one partition bucket each) so that many units follow unit 3
    p = pk.default_params(k=32, num_buckets=21, coverage=30, bucket_bits=8, mn_units=1)
    with pk.Job(ctx()) as job:
        job.set_wait_limit(spins=256, withhold_unit=3)
        job.count(rs.fasta, p)
        job.cutoff(21)
        with pytest.raises(pk.PakmanError) as ei:
            job.build_macro_nodes(0)
        assert ei.value.status == pk.capi.PK_ERR_DEVICE
        assert "look-back" in str(ei.value)
        # the same job, the fault switched off: the whole path is right again
        job.set_wait_limit(0, -1)
        s = job.run(rs.fasta, p)
        keys, counts = job.table()
        mn = job.macro_nodes()
    assert_table_equal(pk.to_key128(keys), counts, ora.table.keys, ora.table.counts)
    assert s.cutoff == ora.cutoff
    assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)
    # and a new job on the same context
    with pk.Job(ctx()) as job2:
        s2 = job2.run(rs.fasta, p)
        mn2 = job2.macro_nodes()
    assert s2.n_nodes == ora.mn.keys.size
    assert np.array_equal(mn2.suffix_counts, ora.mn.suf)


def test_short_wait_limit_alone_is_harmless_or_reported():
    """A short limit with nothing withheld either finishes (every predecessor published
    in time) or reports the expired wait; it never returns a wrong result as PK_OK."""
    rs, ora = _case()
    p = pk.default_params(k=32, num_buckets=21, coverage=30, bucket_bits=8, mn_units=1)
    with pk.Job(ctx()) as job:
        job.set_wait_limit(spins=64)
        try:
            job.run(rs.fasta, p)
        except pk.PakmanError as e:
            assert e.status == pk.capi.PK_ERR_DEVICE
            return
        mn = job.macro_nodes()
    assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)
