"""Device iterative compaction (pk_compact) and walk (pk_walk) against the oracle
restatement of the reference's begin_iterative_compaction and traverse_pakgraph
(oracle/pk_compact.py, pinned to the reference's own runs in
tests/test_compact_oracle.py): the map left at the node threshold -- every prefix and
suffix list with its extensions, counts, visits and terminal flags, the wiring and
prefix begin slots -- the partial contigs in emission order, and the walk's contigs in
begin then depth-first order, exactly."""
import os
import subprocess

import pytest

import pakman_plus_gb300 as pk
from golden_cases import load_compact
from gpu_helpers import ctx
from oracle import pk_compact as pc
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu

def _golden(name):
    g = load_compact(name)
    k, rl, cov, t = g["params"]
    return g["fasta"], k, cov, t, [r[0] for r in g["runs"]]


def _device(fasta, k, cov, t, thr, drop_n=False):
    p = pk.default_params(k=k, num_buckets=t, coverage=cov, drop_n=int(drop_n))
    with pk.Job(ctx()) as job:
        job.count(fasta, p)
        job.cutoff(t)
        job.build_macro_nodes(0)
        mn = job.macro_nodes(cov)
        res = job.compact(thr, cov)
        res.walk_contigs = job.walk()
    return mn, res


def _oracle(mn, k, cov, thr):
    nodes = pc.initial_nodes(mn.keys, mn.suffix_counts, mn.prefix_counts, k, cov)
    return pc.compact(nodes, k, thr)


def _check(res, ora, k=None):
    assert res.rounds == ora.rounds
    assert res.state_view() == pc.state_view(ora.nodes)
    assert res.contigs() == ora.contigs
    if k is not None:
        assert res.walk_contigs == pc.walk(ora.nodes, k)


@pytest.mark.parametrize("name", ["k32_small", "k32_bact", "k32_tandem", "k63_longk"])
def test_golden_inputs(name):
    fasta, k, cov, t, thrs = _golden(name)
    for thr in thrs:
        mn, res = _device(fasta, k, cov, t, thr)
        _check(res, _oracle(mn, k, cov, thr), k)


def test_bacterial_scaled_143k_nodes():
    """92 kbp of the 4.6 Mbp / 80x workload: 143k macro-nodes down to 100 in 27 rounds."""
    rs = synth.config2(0.02)
    mn, res = _device(rs.fasta, rs.k, rs.coverage, rs.t, 100)
    assert res.rounds > 10
    assert len(res.walk_contigs) > 0
    _check(res, _oracle(mn, rs.k, rs.coverage, 100), rs.k)


def test_longk_dropn_scaled():
    rs = synth.config3(0.003)
    mn, res = _device(rs.fasta, rs.k, rs.coverage, rs.t, 20, rs.drop_n)
    _check(res, _oracle(mn, rs.k, rs.coverage, 20), rs.k)


@pytest.mark.parametrize("k", [17, 21, 31, 33, 48, 64])
def test_key_widths(k):
    rs = synth.small_case(300 + k, genome_len=4000, n_reads=3000, read_len=120, err=0.005, k=k,
                          coverage=40)
    mn, res = _device(rs.fasta, k, 40, 21, 5)
    _check(res, _oracle(mn, k, 40, 5), k)


def test_threshold_above_node_count_is_the_initial_wiring():
    rs = synth.small_case(5, genome_len=3000, n_reads=1500, k=32, coverage=20)
    p = pk.default_params(k=32, coverage=20)
    with pk.Job(ctx()) as job:
        job.count(rs.fasta, p)
        job.cutoff(21)
        m = job.build_macro_nodes(0)
        w = job.wire(20)
        res = job.compact(m, 20)
    assert res.rounds == 0 and res.n_nodes == m and not res.contigs()
    view = res.state_view()
    for row, (key, suf, pre, wires, begin) in zip(w, view):
        assert len(suf) == row["ns"] and len(pre) == row["np"]
        assert suf[-1][2] == row["term_suf"] and pre[-1][2] == row["term_pre"]
        used = [x for x in wires if x[2]]
        assert len(used) == row["nw"]
        assert used == [tuple(int(v) for v in r) for r in row["wire"][:len(used)]]
        assert begin == [tuple(int(v) for v in r) for r in row["begin"][:len(begin)]]


def test_compact_twice_and_state_errors():
    rs = synth.small_case(6, genome_len=4000, n_reads=2500, k=32, coverage=25)
    p = pk.default_params(k=32, coverage=25)
    with pk.Job(ctx()) as job:
        with pytest.raises(pk.PakmanError) as e:
            job.compact(10)
        assert e.value.status == pk.capi.PK_ERR_STATE
        with pytest.raises(pk.PakmanError) as e:
            job.walk()
        assert e.value.status == pk.capi.PK_ERR_STATE
        job.count(rs.fasta, p)
        job.cutoff(21)
        job.build_macro_nodes(0)
        mn = job.macro_nodes(25)
        a = job.compact(50, 25)
        b = job.compact(3, 25)
        a2 = job.compact(50, 25)
    assert a.state_view() == a2.state_view() and a.contigs() == a2.contigs()
    _check(b, _oracle(mn, 32, 25, 3))


def test_walk_of_a_larger_map():
    """The walk straight after a shallow compaction (threshold 5000 of 143k nodes):
    many begins, long branching walks."""
    rs = synth.config2(0.02)
    mn, res = _device(rs.fasta, rs.k, rs.coverage, rs.t, 5000)
    ora = _oracle(mn, rs.k, rs.coverage, 5000)
    _check(res, ora, rs.k)


def _fa(partial, walk):
    """The reference's two contig files for these contigs (src/walk.cpp:198-227,
    488-515): contigs longer than 400 bases, numbered across both files."""
    sym = b"ACTG"
    n = 0
    files = []
    for lst in (partial, walk):
        out = []
        for c in lst:
            if len(c) > 400:
                n += 1
                out.append(b">contig_%d_l_%d_r_0\n%s\n" % (n, len(c), bytes(sym[x] for x in c)))
        files.append(b"".join(out))
    return files


# inputs whose canonical start order gives the reference's own map (no prefix-order tie
# decides a wire), so the files must equal the reference's byte for byte
SAME_AS_REFERENCE = {"k32_small", "k32_tandem", "k63_longk"}


@pytest.mark.parametrize("name", ["k32_small", "k32_bact", "k32_tandem", "k63_longk"])
def test_pkmer_contig_generation_files(name, tmp_path):
    """pkmer -g: count, cutoff, macro-nodes, compaction, walk, contig files."""
    from pakman_plus_gb300 import build as pkbuild
    from oracle import pk_oracle as po
    g = load_compact(name)
    k, rl, cov, t = g["params"]
    fa = tmp_path / "in.fa"
    fa.write_bytes(g["fasta"])
    exe = os.path.join(os.path.dirname(pkbuild.LIB), "bin", "pkmer")
    ora = po.run(g["fasta"], k, t)
    for thr, after, contigs, rounds, walk_fa, partial_fa in g["runs"]:
        d = tmp_path / ("n%d" % thr)
        d.mkdir()
        p = subprocess.run([exe, "-f", str(fa), "-r", str(rl), "-c", str(cov), "-t", str(t), "-n", str(thr),
                            "-k", str(k), "-g"], cwd=str(d), capture_output=True, text=True)
        assert p.returncode == 0, p.stdout + p.stderr
        par = (d / "contigs_par_r0.fa").read_bytes()
        out = (d / "contigs_out_r0.fa").read_bytes()
        nodes = pc.initial_nodes(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, cov)
        o = pc.compact(nodes, k, thr)
        exp_par, exp_out = _fa(o.contigs, pc.walk(o.nodes, k))
        assert par == exp_par and out == exp_out
        if name in SAME_AS_REFERENCE:
            assert par == partial_fa and out == walk_fa
