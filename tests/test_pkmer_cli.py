"""pkmer command line: the reference's options, defaults, messages and exit codes
(src/distribute_kmers.cpp:217-313), and on the GPU the same table and macro-nodes as
the reference, written in the reference dump format."""
import os
import subprocess

import numpy as np
import pytest

from golden_cases import load
from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild


@pytest.fixture(scope="module")
def pkmer():
    pkbuild.build()
    return pkbuild.build_pkmer()


def _run(exe, *args):
    return subprocess.run([exe, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                          timeout=300)


def test_missing_input_aborts_like_the_reference(pkmer):
    r = _run(pkmer, "-r", "100", "-c", "10")
    assert r.returncode == 157
    assert "Must specify an input FASTA file name with -f" in r.stderr


@pytest.mark.parametrize("args,msg", [
    (["-c", "10"], "Must specify read_length with -r"),
    (["-r", "100"], "Must specify coverage of the input data with -c"),
    (["-r", "99", "-c", "10"], "Must provide short reads of length >100 and <=250 with -r"),
    (["-r", "251", "-c", "10"], "Must provide short reads of length >100 and <=250 with -r"),
])
def test_required_options(pkmer, args, msg):
    r = _run(pkmer, "-f", "in.fa", *args)
    assert r.returncode == 157
    assert msg in r.stderr
    assert "batch size not specified with -b" in r.stdout


def test_defaults_are_announced_and_missing_file_exits_2(pkmer, tmp_path):
    r = _run(pkmer, "-f", str(tmp_path / "none.fa"), "-r", "150", "-c", "40")
    assert r.returncode == 2
    assert "Couldn't open the input FASTA file" in r.stderr
    for notice in ("MAX_KMER_COUNT=100000000", "num_buckets=21", "node_threashold=100K"):
        assert notice in r.stdout
    assert "K-mer size: 32, L-mer size: 8, Number of Processes: 1, MAX_KMER_COUNT: 100000000" in r.stdout


def test_contig_generation_flag_is_parsed(pkmer, tmp_path):
    """-g (the reference's contig-generation build) is accepted; the run then fails on
    the missing file exactly as without it."""
    r = _run(pkmer, "-f", str(tmp_path / "none.fa"), "-r", "150", "-c", "40", "-n", "500", "-g")
    assert r.returncode == 2
    assert "Couldn't open the input FASTA file" in r.stderr
    assert "node_threashold=100K" not in r.stdout


def test_unknown_option_aborts(pkmer):
    r = _run(pkmer, "-Z")
    assert r.returncode < 0 or r.returncode == 134  # SIGABRT, as the reference's assert


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["k32_basic", "k63_basic", "k31_lower_n", "k64_full_width"])
def test_dumps_match_the_reference(pkmer, tmp_path, name):
    g = load(name)
    fa = tmp_path / "in.fa"
    fa.write_bytes(g.fasta)
    out = str(tmp_path / "out")
    r = _run(pkmer, "-f", str(fa), "-r", "100", "-c", str(g.coverage), "-t", str(g.t), "-k", str(g.k),
             "-o", out)
    assert r.returncode == 0, r.stderr
    k, keys, counts = po.read_table_dump(out + ".table")
    assert k == g.k
    assert np.array_equal(keys, g.table_keys)
    assert np.array_equal(counts, g.table_counts.astype(np.int64))
    mk, suf, pre, sv, pv, k1_ok = po.read_mn_dump(out + ".mn", g.coverage)
    assert k1_ok
    assert np.array_equal(mk, g.mn_keys)
    assert np.array_equal(suf, g.mn_suf) and np.array_equal(pre, g.mn_pre)
    assert np.array_equal(sv, g.mn_suf_visit) and np.array_equal(pv, g.mn_pre_visit)
    assert f"histogram cutoff: {g.cutoff}" in r.stdout


@pytest.mark.gpu
def test_nothing_kept_aborts(pkmer, tmp_path):
    g = load("k32_nothing_kept")
    fa = tmp_path / "in.fa"
    fa.write_bytes(g.fasta)
    r = _run(pkmer, "-f", str(fa), "-r", "100", "-c", str(g.coverage), "-t", str(g.t))
    assert r.returncode == 157


@pytest.mark.gpu
def test_bad_record_aborts(pkmer, tmp_path):
    g = load("k32_bad_record")
    fa = tmp_path / "in.fa"
    fa.write_bytes(g.fasta)
    r = _run(pkmer, "-f", str(fa), "-r", "100", "-c", str(g.coverage))
    assert r.returncode == 157
    assert os.path.exists(str(fa))
