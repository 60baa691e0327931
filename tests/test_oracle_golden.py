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


def _wiring_in_bases(w, sext, pext):
    """A node's wiring with list indices replaced by base codes (4 = terminal)."""
    wires = [(int(sext[w["wire"][j][0]]), int(w["wire"][j][1]), int(w["wire"][j][2])) for j in range(w["nw"])]
    begin = {int(pext[p]): (int(w["begin"][p][0]), int(w["begin"][p][1])) for p in range(w["np"])}
    return wires, begin, int(w["term_suf"]), int(w["term_pre"])


@pytest.mark.parametrize("name", [n for n in names() if load(n).expect == "ok"])
def test_wiring_restatement_matches_reference(name):
    """The initial wiring restatement against the reference's own initiate_mnode_wiring
    (src/wire.cpp), dumped into the fixtures.  Lists in the reference's order equal the
    canonical order (present bases ascending, terminal last) -> identical; otherwise
    identical once list indices are read as bases, unless equal-ranked prefixes were
    left in another order by the reference's unstable sort."""
    g = load(name)
    w = g.wiring
    ours = po.wire(g.mn_suf, g.mn_pre, g.coverage)
    assert ours.size == w["w_ns"].size
    exact = mapped = tied = 0
    for i in range(ours.size):
        ref = np.zeros(1, po.WIRE_DTYPE)[0]
        for f in ("ns", "np", "term_suf", "term_pre", "nw", "wire", "begin"):
            ref[f] = w["w_" + f][i]
        sext = [e for e in w["w_sext"][i] if e >= 0]
        pext = [e for e in w["w_pext"][i] if e >= 0]
        cs = sorted(e for e in sext if e != 4) + [4]
        cp = sorted(e for e in pext if e != 4) + [4]
        if sext == cs and pext == cp:
            for f in ("ns", "np", "term_suf", "term_pre", "nw"):
                assert ours[i][f] == ref[f], (name, i, f)
            assert np.array_equal(ours[i]["wire"], ref["wire"]) and np.array_equal(ours[i]["begin"], ref["begin"])
            exact += 1
            continue
        a = _wiring_in_bases(ours[i], cs, cp)
        b = _wiring_in_bases(ref, sext, pext)
        if a == b:
            mapped += 1
            continue
        # only a reordering of prefixes with equal (visit, count) may differ
        vis = lambda c: -(-int(c) // g.coverage)  # noqa: E731
        ranks = [(vis(g.mn_pre[i][e]), int(g.mn_pre[i][e])) for e in range(4) if g.mn_pre[i][e]]
        assert len(ranks) != len(set(ranks)), (name, i, a, b)
        assert a[0] == b[0] and a[2:] == b[2:]
        tied += 1
    assert exact > 0
