"""GPU path against the reference's golden fixtures and the oracle (bit-exact)."""
import os

import numpy as np
import pytest

import pakman_plus_gb300 as pk
from golden_cases import load, names
from gpu_helpers import assert_mn_equal, assert_table_equal, ctx, run_gpu
from oracle import pk_oracle as po
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", names())
def test_golden_fixture(name):
    g = load(name)
    if g.expect == "format":
        with pytest.raises(pk.FormatError):
            run_gpu(g.fasta, g.k, g.t, g.coverage, g.drop_n)
        return
    s, keys, counts, hist, mn, err = run_gpu(g.fasta, g.k, g.t, g.coverage, g.drop_n)
    assert_table_equal(keys, counts, g.table_keys, g.table_counts)
    assert s.n_windows == g.n_windows
    assert s.n_reads == g.fasta.count(b">")
    if g.expect == "empty_after_cutoff":
        assert err == "empty_after_cutoff"
        return
    assert err is None
    assert s.cutoff == g.cutoff
    assert np.array_equal(hist, g.hist)
    assert s.n_kept == g.n_kept
    assert_mn_equal(mn, g.mn_keys, g.mn_suf, g.mn_pre)
    assert np.array_equal(mn.suffix_visits, g.mn_suf_visit)
    assert np.array_equal(mn.prefix_visits, g.mn_pre_visit)


@pytest.mark.parametrize("bucket_bits", [2, 3, 6, 11, 15, 16, 18])
@pytest.mark.parametrize("name", ["k32_basic", "k63_basic", "k11_dense", "k32_ragged"])
def test_golden_with_forced_partition(name, bucket_bits):
    """Few, large buckets force the multi-pass (split) path of the bucket kernel; deep
    partitions (above 15 digits) take their fine bucket sizes from a count over the
    coarse regions."""
    g = load(name)
    s, keys, counts, hist, mn, err = run_gpu(g.fasta, g.k, g.t, g.coverage, g.drop_n,
                                             bucket_bits=bucket_bits)
    assert_table_equal(keys, counts, g.table_keys, g.table_counts)
    if g.expect == "ok":
        assert s.cutoff == g.cutoff
        assert_mn_equal(mn, g.mn_keys, g.mn_suf, g.mn_pre)


def _compare_with_oracle(rs, t=21, bucket_bits=0, threads=1):
    ora = po.run(rs.fasta, rs.k, t, rs.drop_n, threads=threads)
    s, keys, counts, hist, mn, err = run_gpu(rs.fasta, rs.k, t, rs.coverage, rs.drop_n,
                                             bucket_bits=bucket_bits)
    assert_table_equal(keys, counts, ora.table.keys, ora.table.counts)
    assert s.n_windows == ora.table.n_windows
    assert s.cutoff == ora.cutoff
    if ora.mn is None:
        assert err == "empty_after_cutoff"
        return s
    assert np.array_equal(hist, ora.hist)
    assert s.n_kept == ora.mn.n_kept
    assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)
    return s


def test_plain_1mbp_30x_k32_full_size():
    """1 Mbp genome, 300k x 100 bp reads at 30x, 1% errors, k=32 (full size)."""
    s = _compare_with_oracle(synth.config1())
    assert s.n_windows == 300_000 * 69


def test_bacterial_80x_k32_scaled():
    """4.6 Mbp/80x workload scaled to 460 kbp (same coverage, errors, repeats)."""
    _compare_with_oracle(synth.config2(0.1))


def test_longk_k63_dropn_scaled():
    """50 Mbp/40x k=63 workload scaled to 1 Mbp, N windows dropped."""
    _compare_with_oracle(synth.config3(0.02), t=21)


@pytest.mark.slow
def test_longk_k63_dropn_quarter_scale():
    """The long-k workload at a quarter of its size (12.5 Mbp genome, 3.33M x 150 bp
    reads at 40x, 0.3% substitutions, 0.05% N, k=63 as 128-bit keys, N windows dropped;
    about 280M windows): table, histogram, cutoff and macro-nodes equal the oracle's
    threaded restatement, which equals the serial oracle."""
    _compare_with_oracle(synth.config3(0.25), t=21, threads=os.cpu_count() or 1)


@pytest.mark.parametrize("k", [2, 5, 16, 17, 31, 33, 47, 48, 49, 50, 62, 64])
def test_every_key_width(k):
    rs = synth.small_case(100 + k, genome_len=3000, n_reads=600, read_len=120, err=0.01,
                          n_rate=0.003, lowercase=0.02, k=k)
    ora = po.count(rs.fasta, k)
    p = pk.default_params(k=k)
    with pk.Job(ctx()) as job:
        job.count(rs.fasta, p)
        keys, counts = job.table()
    assert_table_equal(pk.to_key128(keys), counts, ora.keys, ora.counts)


def _low_complexity_fasta(n_reads, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    reads = []
    for i in range(n_reads):
        kind = i % 3
        if kind == 0:
            s = np.resize(np.frombuffer(b"AC", np.uint8), 150)
        elif kind == 1:
            s = np.full(150, ord("A"), np.uint8)
        else:
            s = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 150)]
        m = rng.random(150) < 0.01
        s = np.where(m, np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 150)], s)
        reads.append(s.astype(np.uint8))
    return synth.reads_to_fasta(reads)


def test_skewed_low_complexity_input():
    """Tandem repeats and homopolymers: a few buckets hold most windows."""
    fa = _low_complexity_fasta(3000)
    for k, bb in ((32, 0), (32, 4), (63, 0)):
        ora = po.run(fa, k, 21)
        s, keys, counts, hist, mn, err = run_gpu(fa, k, 21, 10, bucket_bits=bb)
        assert_table_equal(keys, counts, ora.table.keys, ora.table.counts)
        assert s.cutoff == ora.cutoff
        if ora.mn is not None:
            assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)


@pytest.mark.parametrize("k,bb", [(32, 0), (32, 2), (63, 0), (21, 3)])
def test_giant_buckets(k, bb):
    """Buckets of hundreds of thousands of keys (a homopolymer, a dinucleotide repeat and
    their error variants) are reduced chunk by chunk by many CTAs to (key, count) pairs
    before the bucket is counted; with 2 or 3 partition digits every bucket is giant and
    the chunks of random k-mers stay raw (too many distinct keys)."""
    fa = _low_complexity_fasta(36000, seed=6)
    ora = po.run(fa, k, 21)
    s, keys, counts, hist, mn, err = run_gpu(fa, k, 21, 10, bucket_bits=bb)
    assert_table_equal(keys, counts, ora.table.keys, ora.table.counts)
    assert s.cutoff == ora.cutoff
    if ora.mn is not None:
        assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)


def test_cutoff_with_other_t_and_explicit_min_count():
    g = load("k32_ragged")
    p = pk.default_params(k=g.k, num_buckets=g.t, coverage=g.coverage)
    tab = po.count(g.fasta, g.k)
    with pk.Job(ctx()) as job:
        job.count(g.fasta, p)
        for t in (2, 7, 40):
            hist, cut = po.cutoff(tab.counts, t)
            kept_ref = int((tab.counts >= cut).sum())
            try:
                c2, h2, kept = job.cutoff(t)
            except pk.EmptyAfterCutoff as e:
                assert kept_ref == 0
                c2, h2, kept = e.cutoff, e.hist, e.kept
            assert c2 == cut and np.array_equal(h2, hist) and kept == kept_ref
        # "freq > threshold" of the PaK-Graph builder = min_count threshold+1
        m = job.build_macro_nodes(3)
        mn = job.macro_nodes()
        ref = po.macro_nodes(tab, g.k, 3)
        assert m == ref.keys.size
        assert_mn_equal(mn, ref.keys, ref.suf, ref.pre)


def test_packed_table_and_session_api():
    g = load("k32_basic")
    sess = pk.PakmanSession(k=g.k, num_buckets=g.t, coverage=g.coverage, ctx=ctx())
    sess.perform_kmer_counting(g.fasta)
    buf = sess.kmer_proc_buf
    assert buf.dtype.itemsize == 12
    assert np.array_equal(buf["seq"], g.table_keys["lo"])
    assert np.array_equal(buf["k_count"], g.table_counts.astype(np.int32))
    hist, mb = sess.construct_kmer_histogram()
    assert mb == g.cutoff
    mn = sess.begin_mnode_construction()
    assert_mn_equal(mn, g.mn_keys, g.mn_suf, g.mn_pre)
    node = mn.node(0)
    assert len(node["k_1_mer"]) == g.k - 1
    sess.close()


def test_empty_input_and_no_record():
    for fa in (b"", b"no header here\nACGT\n", b">only-header"):
        with pytest.raises(pk.EmptyAfterCutoff):
            run_gpu_strict(fa)


def run_gpu_strict(fa):
    p = pk.default_params(k=32)
    with pk.Job(ctx()) as job:
        s = job.run(fa, p)
    return s


def test_job_reuse_is_deterministic():
    rs = synth.small_case(77, genome_len=5000, n_reads=2000, k=32)
    p = pk.default_params(k=32, num_buckets=21, coverage=20)
    with pk.Job(ctx()) as job:
        s1 = job.run(rs.fasta, p)
        k1, c1 = job.table()
        m1 = job.macro_nodes()
        s2 = job.run(rs.fasta, p)
        k2, c2 = job.table()
        m2 = job.macro_nodes()
    assert s1 == s2
    assert np.array_equal(k1, k2) and np.array_equal(c1, c2)
    assert np.array_equal(m1.keys, m2.keys) and np.array_equal(m1.suffix_counts, m2.suffix_counts)


def test_hbm_budget_is_enforced():
    rs = synth.small_case(78, genome_len=5000, n_reads=2000, k=32)
    small = pk.Context(0, hbm_budget=1 << 16)
    with pk.Job(small) as job:
        with pytest.raises(pk.capi.OutOfMemory):
            job.count(rs.fasta, pk.default_params(k=32))
    small.close()


@pytest.mark.parametrize("mn_units", [1, 2, 3, 5])
@pytest.mark.parametrize("name,bucket_bits", [("k32_basic", 8), ("k63_basic", 9), ("k11_dense", 11),
                                              ("k32_ragged", 12), ("k32_t1", 7)])
def test_golden_with_macro_node_units(name, bucket_bits, mn_units):
    """Macro-node work units spanning 4^level partition buckets give the same nodes."""
    g = load(name)
    p = pk.default_params(k=g.k, num_buckets=g.t, coverage=g.coverage, drop_n=int(g.drop_n),
                          bucket_bits=bucket_bits, mn_units=mn_units)
    with pk.Job(ctx()) as job:
        job.count(g.fasta, p)
        job.cutoff(g.t)
        job.build_macro_nodes(0)
        mn = job.macro_nodes(g.coverage)
    assert_mn_equal(mn, g.mn_keys, g.mn_suf, g.mn_pre)
