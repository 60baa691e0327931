"""Counting in -b pieces (the reference's batch flush, src/kmer_counting.cpp:3022-3139):
a host input counted in record-aligned pieces whose tables are merged on the device
gives the oracle's table, histogram, cutoff and macro-nodes, whether the pieces are asked
for (pk_params.chunking = 1) or forced by an HBM budget below the whole input's
footprint (chunking = 0), and pkmer -b honours them."""
import subprocess

import numpy as np
import pytest

import pakman_plus_gb300 as pk
from golden_cases import load
from gpu_helpers import assert_mn_equal, assert_table_equal, ctx
from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


def _pieces(job):
    n = pk.capi.c_uint32()
    pk.capi.check(pk.capi.lib().pk_count_pieces(job.handle, pk.capi.byref(n)), "pk_count_pieces")
    return n.value


def _run_and_compare(context, fasta, k, t, cov, drop_n=False, **params):
    ora = po.run(fasta, k, t, drop_n)
    p = pk.default_params(k=k, num_buckets=t, coverage=cov, drop_n=int(drop_n), **params)
    with pk.Job(context) as job:
        job.count(fasta, p)
        pieces = _pieces(job)
        keys, counts = job.table()
        s = job.summary()
        assert_table_equal(pk.to_key128(keys), counts, ora.table.keys, ora.table.counts)
        assert s.n_windows == ora.table.n_windows
        assert s.n_reads == fasta.count(b">") - (len(fasta) - len(fasta.lstrip(b"\x00")))
        if ora.mn is None:
            with pytest.raises(pk.EmptyAfterCutoff):
                job.cutoff(t)
            return pieces
        cut, hist, kept = job.cutoff(t)
        assert cut == ora.cutoff and np.array_equal(hist, ora.hist) and kept == ora.mn.n_kept
        job.build_macro_nodes(0)
        mn = job.macro_nodes(cov)
    assert_mn_equal(mn, ora.mn.keys, ora.mn.suf, ora.mn.pre)
    return pieces


@pytest.mark.parametrize("name", ["k32_basic", "k63_basic", "k31_lower_n", "k32_ragged", "k63_dropn"])
@pytest.mark.parametrize("piece", [3000, 40000])
def test_requested_pieces_on_fixtures(name, piece):
    g = load(name)
    pieces = _run_and_compare(ctx(), g.fasta, g.k, g.t, g.coverage, g.drop_n, chunking=1, batch_kmers=piece)
    assert pieces >= len(g.fasta) // (piece + 400)


def test_one_record_per_piece_and_a_sequence_line_starting_with_gt():
    """With a one-byte -b every record is a piece; a sequence line that begins with '>'
    (a sequence line in the reference, whose '>' is a base code) is never a cut."""
    rs = synth.small_case(91, genome_len=3000, n_reads=300, read_len=100, err=0.01, k=32)
    lines = rs.fasta.split(b"\n")[:-1]  # header, sequence, header, ...
    lines = lines[:20] + [b">h_odd", b">" + lines[11]] + lines[20:]
    fasta = b"\n".join(lines) + b"\n"
    pieces = _run_and_compare(ctx(), fasta, 32, 21, 10, chunking=1, batch_kmers=1)
    assert pieces == 301  # one per record; the sequence line's '>' starts no piece


def test_bad_record_in_a_later_piece():
    g = load("k32_bad_record")
    p = pk.default_params(k=32, num_buckets=21, coverage=10, chunking=1, batch_kmers=2000)
    with pk.Job(ctx()) as job:
        with pytest.raises(pk.FormatError):
            job.count(g.fasta, p)


def test_budget_below_the_whole_input_switches_to_pieces():
    """The bacterial workload at 0.05 scale with an HBM budget too small for counting the
    whole input at once: the job counts in -b pieces by itself."""
    rs = synth.config2(0.05)
    # counting at once needs about 13 bytes per FASTA byte (keys twice, counts); the
    # pieces need the merged table (about 1.3 bytes per FASTA byte here) three times over
    # plus one piece's working set
    budget = 8 * len(rs.fasta)
    small = pk.Context(0, hbm_budget=budget)
    try:
        pieces = _run_and_compare(small, rs.fasta, rs.k, rs.t, rs.coverage, batch_kmers=len(rs.fasta) // 10)
        assert pieces > 1
    finally:
        small.close()
    with pk.Context(0, hbm_budget=budget) as small2, pk.Job(small2) as job:
        with pytest.raises(pk.capi.OutOfMemory):
            job.count(rs.fasta, pk.default_params(k=32, chunking=2))


def test_pkmer_b_counts_in_pieces(tmp_path):
    """pkmer -b with an HBM budget (-M) below the whole input's footprint: the run counts
    in -b pieces and its dumps equal the oracle's table and macro-nodes."""
    rs = synth.config2(0.01)
    fa = tmp_path / "in.fa"
    fa.write_bytes(rs.fasta)
    out = str(tmp_path / "out")
    pkbuild.build()
    exe = pkbuild.build_pkmer()
    r = subprocess.run([exe, "-f", str(fa), "-r", "100", "-c", str(rs.coverage), "-t", str(rs.t), "-k", str(rs.k),
                        "-b", str(len(rs.fasta) // 10), "-M", str(8 * len(rs.fasta)), "-o", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    it = [ln for ln in r.stdout.splitlines() if ln.startswith("Number of batch iterations:")]
    assert it and int(it[0].split(":")[1]) > 1, r.stdout
    ora = po.run(rs.fasta, rs.k, rs.t)
    k, keys, counts = po.read_table_dump(out + ".table")
    assert np.array_equal(keys, ora.table.keys)
    assert np.array_equal(counts, ora.table.counts.astype(np.int64))
    mk, suf, pre, sv, pv, k1_ok = po.read_mn_dump(out + ".mn", rs.coverage)
    assert np.array_equal(mk, ora.mn.keys)
    assert np.array_equal(suf, ora.mn.suf) and np.array_equal(pre, ora.mn.pre)
