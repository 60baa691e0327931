"""The plain-C oracle against the golden fixtures produced by the reference's own
binaries (CPU only)."""
import numpy as np
import pytest

from golden_cases import load, names
from oracle import pk_oracle as po


@pytest.mark.parametrize("name", names())
def test_oracle_matches_reference_fixture(name):
    g = load(name)
    if g.expect == "format":
        with pytest.raises(po.OracleError) as e:
            po.count(g.fasta, g.k, g.drop_n)
        assert e.value.code == po.PKO_EFORMAT
        return
    tab = po.count(g.fasta, g.k, g.drop_n)
    assert np.array_equal(tab.keys, g.table_keys)
    assert np.array_equal(tab.counts, g.table_counts)
    assert int(tab.counts.sum(dtype=np.uint64)) == tab.n_windows == g.n_windows
    hist, cut = po.cutoff(tab.counts, g.t)
    assert cut == g.cutoff
    if g.expect == "empty_after_cutoff":
        with pytest.raises(po.OracleError) as e:
            po.macro_nodes(tab, g.k, cut)
        assert e.value.code == po.PKO_EEMPTY
        return
    assert np.array_equal(hist, g.hist)
    mn = po.macro_nodes(tab, g.k, cut)
    assert mn.n_kept == g.n_kept
    assert np.array_equal(mn.keys, g.mn_keys)
    assert np.array_equal(mn.suf, g.mn_suf)
    assert np.array_equal(mn.pre, g.mn_pre)


def test_visit_value_is_ceil_division():
    for c in range(1, 200):
        for cov in (1, 7, 30, 80):
            assert po.visit(c, cov) == -(-c // cov)


def test_window_count_matches_table_sum():
    g = load("k32_ragged")
    w, reads = po.count_windows(g.fasta, g.k)
    assert w == g.n_windows
    assert reads == g.fasta.count(b">")


@pytest.mark.parametrize("k", [11, 32, 63])
def test_threaded_port_equals_serial_oracle(k):
    """The multi-threaded restatement (CPU baseline) builds the same table."""
    from pakman_plus_gb300 import synth
    lens = np.random.default_rng(k).integers(40, 151, 4000)
    rs = synth.small_case(500 + k, genome_len=8000, n_reads=4000, read_len=lens, err=0.01, k=k)
    a = po.count(rs.fasta, k)
    for threads in (2, 5, 16):
        b = po.count(rs.fasta, k, threads=threads)
        assert np.array_equal(a.keys, b.keys) and np.array_equal(a.counts, b.counts)
        assert (a.n_windows, a.n_reads) == (b.n_windows, b.n_reads)
