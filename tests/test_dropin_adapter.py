"""The link-level drop-in's adapter code (pakman_plus_gb300/host/pakman_dropin.cpp) run
against the device, without the reference sources.

tests/cpp/dropin_check.cpp drives the adapter in the order the reference's driver calls
it (src/distribute_kmers.cpp:147-203) and is compiled against a stand-in for the
reference header (tests/cpp/dropin_standin/distribute_kmers.h, the reference's layouts of
KmerPairs, MacroNode, WireInfo, PrefixInfo and BeginMN).  What the adapter leaves in
kmer_proc_buf and MN_map after each phase is compared with the oracle and with the
C ABI's own results on the same input: the packed table, every node's lists with
(count, visit) pairs and terminal flags, the wiring_info and prefix_begin_info the adapter
copies out of pk_wiring and pk_copy_compacted, the partial contigs and the begin k-mers
the reference's walk starts from."""
import os
import subprocess

import numpy as np
import pytest

import pakman_plus_gb300 as pk
from golden_cases import load_compact
from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "pakman_plus_gb300")


def _build(k: int, out_dir: str) -> str:
    pkbuild.build()
    exe = os.path.join(out_dir, f"dropin_check_k{k}")
    cmd = ["g++", "-O1", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(HERE, "cpp", "dropin_standin"),
           "-I", os.path.join(ROOT, "include"), f"-DWINDW_SIZE={k - 1}", "-DLMER_LENGTH=8"]
    if k > 32:
        cmd.append("-DEXTEND_KMER")
    cmd += [os.path.join(HERE, "cpp", "dropin_check.cpp"), os.path.join(PKG, "host", "pakman_dropin.cpp"),
            "-L", PKG, "-lpakman_gb300", f"-Wl,-rpath,{PKG}", "-o", exe]
    subprocess.check_call(cmd)
    return exe


@pytest.mark.parametrize("k", [32, 63])
def test_adapter_compiles_against_the_reference_layouts(tmp_path, k):
    assert os.access(_build(k, str(tmp_path)), os.X_OK)


def _key(tok: str) -> int:
    hi, lo = tok.split(":")
    return (int(hi, 16) << 64) | int(lo, 16)


def _read_map(path):
    """Per node: (key, k_1_mer, suffixes, prefixes, wires, begins); entries are
    (ext base codes, count, visit, terminal)."""
    out = []
    for line in open(path):
        t = line.split()
        key, k1 = _key(t[0]), t[1]
        i = 2
        sec = {}
        for tag in ("S", "P", "W", "B"):
            assert t[i] == tag, (t[i], tag)
            i += 1
            vals = []
            while i < len(t) and t[i] not in ("S", "P", "W", "B"):
                vals.append(t[i])
                i += 1
            sec[tag] = vals

        def ent(v):
            ext, c, vis, term = v.split(":")
            return (bytes(int(ch) for ch in ext), int(c), int(vis), bool(int(term)))
        out.append((key, k1, [ent(v) for v in sec["S"]], [ent(v) for v in sec["P"]],
                    [tuple(int(x) for x in v.split(",")) for v in sec["W"]],
                    [tuple(int(x) for x in v.split(",")) for v in sec["B"]]))
    return out


def _bases(key: int, n: int) -> str:
    return "".join(str((key >> (2 * (n - 1 - b))) & 3) for b in range(n))


def _visit(c: int, cov: int) -> int:
    return -(-c // cov)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["k32_small", "k32_bact", "k63_longk"])
def test_adapter_fills_the_reference_structures(tmp_path, name):
    g = load_compact(name)
    k, _, cov, t = g["params"]
    thr = g["runs"][0][0]
    fa = tmp_path / "in.fa"
    fa.write_bytes(g["fasta"])
    exe = _build(k, str(tmp_path))
    r = subprocess.run([exe, str(fa), str(cov), str(t), str(thr), str(tmp_path)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])

    # the C ABI on the same input
    p = pk.default_params(k=k, num_buckets=t, coverage=cov)
    with pk.Context(0) as ctx, pk.Job(ctx) as job:
        job.count(g["fasta"], p)
        job.cutoff(t)
        job.build_macro_nodes(0)
        mn = job.macro_nodes(cov)
        wiring = job.wire(cov)
        comp = job.compact(thr, cov)
    ora = po.run(g["fasta"], k, t)

    # kmer_proc_buf: the oracle's table as packed KmerPairs
    rec = np.fromfile(tmp_path / "table.bin", pk.KMERPAIRS64 if k <= 32 else pk.KMERPAIRS128)
    assert rec.size == ora.table.keys.size
    if k <= 32:
        assert np.array_equal(rec["seq"], ora.table.keys["lo"])
    else:
        assert np.array_equal(rec["seq_lo"], ora.table.keys["lo"])
        assert np.array_equal(rec["seq_hi"], ora.table.keys["hi"])
    assert np.array_equal(rec["k_count"].astype(np.int64), ora.table.counts.astype(np.int64))

    # MN_map after begin_mnode_construction: the oracle's nodes, one-base lists in
    # ascending base order with (count, ceil(count / coverage))
    built = _read_map(tmp_path / "mn_built.txt")
    keys = pk.to_key128(mn.keys)
    assert len(built) == ora.mn.keys.size == keys.size
    for i, (key, k1, suf, pre, wires, begins) in enumerate(built):
        assert key == int(ora.mn.keys["lo"][i]) | (int(ora.mn.keys["hi"][i]) << 64)
        assert k1 == _bases(key, k - 1)
        assert suf == [(bytes([e]), int(c), _visit(int(c), cov), False)
                       for e, c in enumerate(ora.mn.suf[i]) if c]
        assert pre == [(bytes([e]), int(c), _visit(int(c), cov), False)
                       for e, c in enumerate(ora.mn.pre[i]) if c]
        assert wires == [] and begins == []

    # after initiate_mnode_wiring: terminal entries (1, visit) appended, wiring_info and
    # prefix_begin_info as the device wired the node
    wired = _read_map(tmp_path / "mn_wired.txt")
    assert len(wired) == len(built)
    for i, (key, k1, suf, pre, wires, begins) in enumerate(wired):
        w = wiring[i]
        assert suf == built[i][2] + [(b"", 1, int(w["term_suf"]), True)]
        assert pre == built[i][3] + [(b"", 1, int(w["term_pre"]), True)]
        assert len(suf) == w["ns"] and len(pre) == w["np"]
        nw = int(w["ns"]) + int(w["np"]) + 1
        assert wires == [tuple(int(x) for x in w["wire"][j]) for j in range(nw)]
        assert begins == [tuple(int(x) for x in w["begin"][j]) for j in range(int(w["np"]))]

    # after begin_iterative_compaction: the device's compacted map, node for node
    compact = _read_map(tmp_path / "mn_compact.txt")
    view = comp.state_view()
    assert len(compact) == len(view)
    for (key, k1, suf, pre, wires, begins), (vkey, vsuf, vpre, vwires, vbegin) in zip(compact, view):
        assert key == vkey and k1 == _bases(key, k - 1)
        assert suf == vsuf and pre == vpre
        assert wires == vwires and begins == vbegin
    partial = [bytes(int(ch) for ch in ln.strip()) for ln in open(tmp_path / "partial.txt")]
    assert partial == comp.contigs()

    # identify_begin_kmers: every terminal prefix with visits, map order then prefix order
    want = [(key, l) for key, _, _, pre, _, _ in compact for l, e in enumerate(pre) if e[2] > 0 and e[3]]
    got = []
    for ln in open(tmp_path / "begins.txt"):
        a, b = ln.split()
        got.append((_key(a), int(b)))
    assert got == want
    if name != "k32_small":  # the small case compacts to nothing
        assert len(got) > 0
