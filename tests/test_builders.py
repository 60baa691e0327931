"""C++ builder interfaces (include/pakman_gb300.hpp): the k-mer table builder
Concurrent_Kmer_Partial_Counter (src/concurrent_kmer_counter.hpp) and the PaK-Graph
builder Pakman_Subgraph::build_graph (src/pakman_graph.hpp:592-673), driven by
tests/cpp/builders_check.cpp and compared with the oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# the builder's symbol map: A0 C1 T2 G3, everything else 0
_MAP = bytes(c if c in b"ACTG" else ord("A") for c in range(256))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    pkbuild.build()
    exe = str(tmp_path_factory.mktemp("bld") / "builders_check")
    subprocess.check_call([pkbuild.cxx(), "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "cpp", "builders_check.cpp"), "-o", exe, "-L", pkbuild.HERE,
                           "-lpakman_gb300", f"-Wl,-rpath,{pkbuild.HERE}"])
    return exe


def test_header_compiles_with_reference_call_shapes(driver):
    assert os.access(driver, os.X_OK)


# ---------------------------------------------------------------- CPU model -------
def builder_reads(buf: bytes, read_len: int, klen: int):
    """Reads as the reference's default_count_and_process walks them
    (src/concurrent_kmer_counter.hpp:2018-2060)."""
    reads, p, n = [], 0, len(buf)
    while p != n:
        q = buf.find(b">", p)
        if q < 0:
            break
        p = q + 1
        q = buf.find(b"\n", p)
        if q < 0:
            break
        p = q + 1
        rl = min(read_len, n - p)
        if rl < klen:
            continue
        reads.append(buf[p:p + rl])
    return reads


def register_kmers(read: bytes, klen: int, bases: int):
    """The builder's unmasked register after each window (last `bases` bases)."""
    mask = (1 << (2 * bases)) - 1
    x, out = 0, []
    for i, c in enumerate(read.translate(_MAP)):
        x = ((x << 2) | b"ACTG".index(c)) & mask
        if i >= klen - 1:
            out.append(x)
    return out


def as_rows(table):
    return [((int(h) << 64) | int(lo), int(c)) for (lo, h), c in zip(table.keys.tolist(), table.counts.tolist())]


def read_calls(path):
    data = open(path, "rb").read()
    off, calls = 0, []
    while off < len(data):
        n = int.from_bytes(data[off:off + 8], "little")
        off += 8
        a = np.frombuffer(data, "<u8", 3 * n, off).reshape(n, 3)
        off += 24 * n
        calls.append([((int(h) << 64) | int(lo), int(c)) for lo, h, c in a.tolist()])
    return calls


def read_graph(path):
    data = open(path, "rb").read()
    m = int.from_bytes(data[:8], "little")
    off, nodes = 8, []
    for _ in range(m):
        lo, hi = np.frombuffer(data, "<u8", 2, off)
        off += 16
        sides = []
        for _ in range(2):
            n = int.from_bytes(data[off:off + 4], "little")
            off += 4
            ent = []
            for _ in range(n):
                ch = chr(data[off])
                c = int.from_bytes(data[off + 1:off + 9], "little")
                v = int.from_bytes(data[off + 9:off + 13], "little", signed=True)
                t = data[off + 13]
                off += 14
                ent.append((ch, c, v, t))
            sides.append(ent)
        nodes.append(((int(hi) << 64) | int(lo), sides[0], sides[1]))
    return nodes


def _fasta(seed, n_reads=600, read_len=100, k=32, lens=None, n_rate=0.0, lower=0.0):
    rl = lens if lens is not None else read_len
    return synth.small_case(seed, genome_len=3000, n_reads=n_reads, read_len=rl, err=0.01, k=k,
                            n_rate=n_rate, lowercase=lower).fasta


# ---------------------------------------------------------------- GPU tests -------
@pytest.mark.gpu
@pytest.mark.parametrize("klen,wide,variant", [(32, 0, "default"), (21, 0, "default"), (32, 0, "omp_v3"),
                                               (15, 0, "omp_explicit"), (63, 1, "default"),
                                               (40, 1, "omp_v3")])
def test_table_builder_matches_model(driver, tmp_path, klen, wide, variant):
    bases = 64 if wide else 32
    # fixed 100 bp reads plus N, lowercase and short records
    lens = np.random.default_rng(klen).integers(20, 130, 600)
    fa = _fasta(100 + klen, lens=lens, n_rate=0.01, lower=0.05)
    (tmp_path / "in.fa").write_bytes(fa)
    out = str(tmp_path / "calls.bin")
    r = subprocess.run([driver, "counter", str(tmp_path / "in.fa"), str(klen), "100", "inf", str(wide),
                        variant, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    reads = builder_reads(fa, 100, klen)
    assert f"reads {len(reads)} calls 1" in r.stdout
    calls = read_calls(out)
    assert len(calls) == 1
    transformed = b"".join(b">\n" + b"A" * (bases - klen) + rd.translate(_MAP) + b"\n" for rd in reads)
    assert calls[0] == as_rows(po.count(transformed, bases))
    # the reference's unit-test invariant: total frequency = sum of windows
    assert sum(c for _, c in calls[0]) == sum(len(rd) - klen + 1 for rd in reads)


@pytest.mark.gpu
@pytest.mark.parametrize("limit", [50, 700, 5000])
def test_table_builder_partial_flushes(driver, tmp_path, limit):
    """max_kmer_count below the distinct k-mers: the map is handed over and cleared
    after the first read that takes it past the limit, as the reference does."""
    klen = 27
    fa = _fasta(77, n_reads=120)
    (tmp_path / "in.fa").write_bytes(fa)
    out = str(tmp_path / "calls.bin")
    r = subprocess.run([driver, "counter", str(tmp_path / "in.fa"), str(klen), "100", str(limit), "0",
                        "default", out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    expect, cur = [], {}
    for rd in builder_reads(fa, 100, klen):
        for x in register_kmers(rd, klen, 32):
            cur[x] = cur.get(x, 0) + 1
        if len(cur) > limit:
            expect.append(sorted(cur.items()))
            cur = {}
    expect.append(sorted(cur.items()))
    assert read_calls(out) == expect


@pytest.mark.gpu
def test_sort_variant_counts_reads_without_calling_the_processor(driver, tmp_path):
    fa = _fasta(5)
    (tmp_path / "in.fa").write_bytes(fa)
    out = str(tmp_path / "calls.bin")
    r = subprocess.run([driver, "counter", str(tmp_path / "in.fa"), "32", "100", "inf", "0", "sort", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert f"reads {len(builder_reads(fa, 100, 32))} calls 0" in r.stdout


def _expected_graph(table, k, threshold, cov):
    try:
        mn = po.macro_nodes(table, k, threshold + 1)
    except po.OracleError:
        return []
    nodes = []
    for (lo, hi), s, p in zip(mn.keys.tolist(), mn.suf.tolist(), mn.pre.tolist()):
        side = lambda cnt: [("ACTG"[e], c, -(-c // cov), 0) for e, c in enumerate(cnt) if c]
        nodes.append(((hi << 64) | lo, side(s), side(p)))
    return nodes


def _write_table(path, table):
    n = table.keys.size
    a = np.empty((n, 3), "<u8")
    a[:, 0], a[:, 1], a[:, 2] = table.keys["lo"], table.keys["hi"], table.counts
    with open(path, "wb") as f:
        f.write(np.uint64(n).tobytes())
        f.write(a.tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("k,threshold,cov,nparts", [(32, 2, 10, 3), (31, 0, 1, 1), (63, 4, 30, 4),
                                                    (25, 1000, 10, 2)])
def test_pak_graph_builder_matches_oracle(driver, tmp_path, k, threshold, cov, nparts):
    table = po.count(_fasta(300 + k, k=k, n_reads=900), k)
    _write_table(tmp_path / "t.bin", table)
    out = str(tmp_path / "g.bin")
    r = subprocess.run([driver, "graph", str(tmp_path / "t.bin"), str(k), str(threshold), str(cov),
                        str(nparts), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert read_graph(out) == _expected_graph(table, k, threshold, cov)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [32, 63])
def test_default_build_from_fasta(driver, tmp_path, k):
    fa = _fasta(900 + k, k=k, n_reads=1500)
    (tmp_path / "in.fa").write_bytes(fa)
    out = str(tmp_path / "g.bin")
    r = subprocess.run([driver, "build", str(tmp_path / "in.fa"), str(k), "2", "20", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert read_graph(out) == _expected_graph(po.count(fa, k), k, 2, 20)
