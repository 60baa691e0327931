"""The compaction and walk oracle (oracle/pk_compact.py) against the reference's own
iterative compaction and walk: golden dumps made by tests/golden/make_compact_golden.py,
a live run of the reference built here when its sources are present, and libstdc++'s
std::sort for the wiring's unstable ranking."""
import os
import subprocess

import numpy as np
import pytest

from golden_cases import compact_names, load_compact
from oracle import pk_compact as pc
from oracle import pk_oracle as po
from pakman_plus_gb300 import synth

CASES = compact_names()
load = load_compact


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_compaction(name):
    g = load(name)
    for thr, after, contigs, rounds, _, _ in g["runs"]:
        k, before = pc.parse_state(g["before"])
        o = pc.compact(before, k, thr)
        _, ref_after = pc.parse_state(after)
        assert o.rounds == rounds
        assert len(o.nodes) <= thr < len(before)
        assert pc.state_view(o.nodes) == pc.state_view(ref_after)
        assert o.contigs == pc.parse_contigs(contigs)


@pytest.mark.parametrize("name", CASES)
def test_oracle_walk_reproduces_reference_contig_files(name):
    """The walk on the compacted map: the reference writes, with one thread, its walk
    contigs and its partial contigs longer than 400 bases in generation order."""
    g = load(name)
    for thr, after, contigs, rounds, walk_fa, partial_fa in g["runs"]:
        k, nodes = pc.parse_state(after)
        w = pc.walk(nodes, k)
        assert [c for c in w if len(c) > 400] == pc.read_fasta_contigs(walk_fa)
        assert [c for c in pc.parse_contigs(contigs) if len(c) > 400] == pc.read_fasta_contigs(partial_fa)


@pytest.mark.parametrize("name", CASES)
def test_canonical_start_matches_initial_wiring(name):
    """The oracle's own start state (lists in ascending base order) has the initial
    wiring that the C oracle's pko_wire_nodes (pinned to src/wire.cpp) computes."""
    g = load(name)
    k, rl, cov, t = g["params"]
    ora = po.run(g["fasta"], k, t)
    nodes = pc.initial_nodes(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, cov)
    w = po.wire(ora.mn.suf, ora.mn.pre, cov)
    assert len(nodes) == w.size
    for nd, row in zip(nodes, w):
        assert len(nd.suf) == row["ns"] and len(nd.pre) == row["np"]
        assert nd.suf[-1][2] == row["term_suf"] and nd.pre[-1][2] == row["term_pre"]
        used = [x for x in nd.wires if x[2]]
        assert len(used) == row["nw"]
        assert [tuple(x) for x in row["wire"][:len(used)]] == used
        assert [tuple(x) for x in row["begin"][:len(nd.begin)]] == list(nd.begin)
    # the reference's own map holds the same nodes and entry multisets
    _, ref = pc.parse_state(g["before"])
    assert [nd.key for nd in ref] == [nd.key for nd in nodes]
    for a, b in zip(ref, nodes):
        assert sorted(map(tuple, (e[:4] for e in a.pre))) == sorted(map(tuple, (e[:4] for e in b.pre)))
        assert [e[:4] for e in a.suf] == [e[:4] for e in b.suf]


@pytest.fixture(scope="module")
def stdsort(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("ss") / "stdsort")
    src = os.path.join(os.path.dirname(pc.__file__), "ref", "stdsort_harness.cpp")
    try:
        subprocess.run(["g++", "-O1", "-o", exe, src], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("no C++ compiler")
    return exe


def _sort_cases(sizes, seed=11):
    rng = np.random.default_rng(seed)
    cases = []
    for n in sizes:
        for spread in (1, 2, 3, 4, 50):
            for _ in range(3):
                cases.append([(int(rng.integers(0, spread)), int(rng.integers(0, spread))) for _ in range(n)])
    return cases


def _libstdcxx(exe, cases):
    inp = "".join("%d %s\n" % (len(c), " ".join("%d %d" % vc for vc in c)) for c in cases)
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
    return [[int(x) for x in line.split()] for line in out.split("\n")[:len(cases)]]


def test_std_sort_restatement_matches_libstdcxx(stdsort):
    cases = _sort_cases(list(range(0, 40)) + [47, 64, 100, 257, 1000])
    cases.append([(3, 1)] * 70)  # all equal
    cases.append([(i // 3, 0) for i in range(90)])  # ascending runs (descending order wanted)
    cases.append([(90 - i, 2) for i in range(90)])
    for c, ref in zip(cases, _libstdcxx(stdsort, cases)):
        idx = list(range(len(c)))
        pc._std_sort(idx, lambda i, j: c[i][0] > c[j][0] or (c[i][0] == c[j][0] and c[i][1] > c[j][1]))
        assert idx == ref, c


def test_c_sort_matches_libstdcxx(stdsort):
    """The C restatement's ranking (oracle/pk_compact.c) on lists of up to 1000 entries."""
    import ctypes
    L = po.lib()
    L.pko_rank_std_sort.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    cases = _sort_cases(list(range(0, 40)) + [64, 257, 1000], seed=12)
    for c, ref in zip(cases, _libstdcxx(stdsort, cases)):
        v = np.array([x[0] for x in c] or [0], np.int32)
        k = np.array([x[1] for x in c] or [0], np.int32)
        out = np.zeros(max(1, len(c)), np.int32)
        assert L.pko_rank_std_sort(v.ctypes.data, k.ctypes.data, len(c), out.ctypes.data) == 0
        assert out[:len(c)].tolist() == ref, c


def test_device_sort_matches_libstdcxx(stdsort, tmp_path):
    """The device's ranking (pakman_plus_gb300/csrc/pk_stdsort.cuh, built for the host)
    on every list size the device ranks (0..32 entries), heavy ties included: past 16
    entries this is the introsort branch that no fixture list reaches."""
    exe = str(tmp_path / "stdsort_host")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cpp", "stdsort_host.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, src], check=True, capture_output=True)
    cases = _sort_cases(list(range(0, 33)) * 20, seed=13)
    mine = _libstdcxx(exe, cases)
    assert mine == _libstdcxx(stdsort, cases)


def test_live_reference_run():
    """A fresh seed through the reference built here (skipped without its sources)."""
    if pc.build_compact_reference(32) is None:
        pytest.skip("the reference tree is not present")
    rs = synth.small_case(91, genome_len=6000, n_reads=4000, read_len=100, err=0.01, k=32, coverage=30)
    r = pc.run_reference(rs.fasta, 32, 100, 30, 20, walk=True)
    o = pc.compact(r.before, 32, 20)
    assert pc.state_view(o.nodes) == pc.state_view(r.after)
    assert o.contigs == r.contigs
    assert [c for c in pc.walk(o.nodes, 32) if len(c) > 400] == pc.read_fasta_contigs(r.raw["walk_fa"])


@pytest.mark.parametrize("name", CASES)
def test_c_restatement_matches_the_python_oracle(name):
    """oracle/pk_compact.c (the bench's CPU baseline) gives the same map, partial
    contigs and walk contigs as oracle/pk_compact.py, through a hash of all three."""
    g = load(name)
    k, rl, cov, t = g["params"]
    ora = po.run(g["fasta"], k, t)
    for thr, *_ in g["runs"]:
        o = pc.compact(pc.initial_nodes(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, cov), k, thr)
        w = pc.walk(o.nodes, k)
        c = pc.compact_walk_c(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, cov, thr)
        assert (c.rounds, c.n_nodes, c.n_contigs, c.walk_contigs) == (o.rounds, len(o.nodes), len(o.contigs), len(w))
        assert c.hash == pc.result_hash(o.nodes, o.contigs, w)


def test_c_restatement_other_widths():
    for k in (17, 33, 48, 64):
        rs = synth.small_case(300 + k, genome_len=3000, n_reads=2500, read_len=120, err=0.005, k=k, coverage=40)
        ora = po.run(rs.fasta, k, 21)
        o = pc.compact(pc.initial_nodes(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, 40), k, 5)
        w = pc.walk(o.nodes, k)
        c = pc.compact_walk_c(ora.mn.keys, ora.mn.suf, ora.mn.pre, k, 40, 5)
        assert c.hash == pc.result_hash(o.nodes, o.contigs, w), k
