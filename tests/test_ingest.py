"""File ingest (pk_fasta_slice / pk_count_file): the rank slices follow the reference's
DivideReads (src/input_reading.cpp:68-243) -- pinned to the reference's own function
where the reference is built here -- they tile the file, and counting a file streamed
from disk gives exactly what counting the same bytes from memory gives."""
import subprocess

import numpy as np
import pytest

import pakman_plus_gb300 as pk
from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import capi, synth



@pytest.fixture(scope="module")
def lib():
    pkbuild.build()
    return capi.lib()


def _fasta(seed, n_reads=400, lo=60, hi=151, genome_len=5000):
    lens = np.random.default_rng(seed).integers(lo, hi, n_reads)
    return synth.small_case(seed, genome_len=genome_len, n_reads=n_reads, read_len=lens, err=0.01,
                            k=32).fasta


def _write(tmp_path, name, data):
    p = tmp_path / name
    p.write_bytes(data)
    return str(p)


def _slices(path, n, read_length=150):
    return [pk.fasta_slice(path, r, n, read_length) for r in range(n)]


# ------------------------------------------------------------ CPU: slice rule ------
@pytest.fixture(scope="module")
def ref_divide():
    exe = po.build_divide_reference()
    if exe is None:
        pytest.skip("the reference tree is not present: DivideReads cannot be built here")
    return exe


@pytest.mark.parametrize("seed", [5, 6])
def test_restatement_matches_reference_divide_reads(ref_divide, tmp_path, seed):
    data = _fasta(seed)
    path = _write(tmp_path, "in.fa", data)
    out = str(tmp_path / "out")
    for n in (1, 2, 3, 5, 8, 13):
        for r in range(n):
            exp = po.divide_reads(data, r, n, 250)
            assert exp is not None  # records are shorter than the overlap
            got = subprocess.run([ref_divide, path, str(r), str(n), "250", out], capture_output=True,
                                 text=True, check=True)
            ref = open(out, "rb").read()
            assert ref == exp, (n, r)
            # the harness's own last line (the reference prints its timings before it)
            assert got.stdout.strip().splitlines()[-1].split() == [str(ref.count(b">")), str(len(ref))]


@pytest.mark.parametrize("seed,n_ranks", [(7, 1), (7, 2), (8, 3), (9, 7), (10, 16)])
def test_slice_matches_divide_reads(lib, tmp_path, seed, n_ranks):
    data = _fasta(seed)
    path = _write(tmp_path, "in.fa", data)
    for r, (off, ln) in enumerate(_slices(path, n_ranks)):
        exp = po.divide_reads(data, r, n_ranks, 150 + 100)
        assert exp is not None
        assert data[off:off + ln] == exp, (r, off, ln)


@pytest.mark.parametrize("data", [
    b"",                                              # empty file
    b"ACGTACGT\nACGT\n",                              # no record at all
    b"junk\n>r0\nACGTACGTAC\n>r1\nGG\n",              # bytes before the first record
    b">r0\n" + b"A" * 5000 + b"\n>r1\nCCCC\n",        # a record longer than the overlap
    b">a\nAC\n>b\nGT\n",                              # more ranks than records
])
@pytest.mark.parametrize("n_ranks", [1, 2, 3, 9, 40])
def test_slices_tile_the_file(lib, tmp_path, data, n_ranks):
    path = _write(tmp_path, "in.fa", data)
    sl = _slices(path, n_ranks)
    pos = 0
    for off, ln in sl:
        assert off == pos
        pos += ln
    assert pos == len(data)
    for r, (off, ln) in enumerate(sl):
        if r > 0 and ln:
            assert data[off:off + 1] == b">"  # every slice but rank 0's starts at a record


def test_slice_errors(lib, tmp_path):
    with pytest.raises(pk.InputFileError) as e:
        pk.fasta_slice(str(tmp_path / "missing.fa"))
    assert e.value.status == capi.PK_ERR_IO
    assert "Couldn't open the input FASTA file" in str(e.value)
    with pytest.raises(pk.InputFileError):
        pk.fasta_slice(str(tmp_path))  # a directory
    path = _write(tmp_path, "in.fa", b">a\nACGT\n")
    for rank, n in [(1, 1), (-1, 2), (0, 0)]:
        with pytest.raises(pk.PakmanError) as e:
            pk.fasta_slice(path, rank, n)
        assert e.value.status == capi.PK_ERR_INVALID


# ------------------------------------------------------------ GPU: streamed count --
def _whole(job, k, t):
    keys, counts = job.table()
    s = job.summary()
    cut, hist, kept = job.cutoff(t)
    job.build_macro_nodes(0)
    return s, keys, counts, cut, job.macro_nodes(1)


@pytest.mark.gpu
@pytest.mark.parametrize("scale,k", [(0.1, 32), (0.02, 63)])
def test_count_file_equals_count_from_memory(tmp_path, scale, k):
    """Several 16 MiB pieces over the reader threads (and a ragged last piece)."""
    from gpu_helpers import ctx
    rs = synth.config2(scale) if k == 32 else synth.config3(scale)
    path = _write(tmp_path, "in.fa", rs.fasta)
    p = pk.default_params(k=rs.k, num_buckets=rs.t, coverage=1, drop_n=int(rs.drop_n))
    with pk.Job(ctx()) as a, pk.Job(ctx()) as b:
        a.count(rs.fasta, p)
        b.count_file(path, p)
        sa, ka, ca, cut_a, mna = _whole(a, rs.k, rs.t)
        sb, kb, cb, cut_b, mnb = _whole(b, rs.k, rs.t)
    assert (sb.n_windows, sb.n_unique, sb.n_reads) == (sa.n_windows, sa.n_unique, sa.n_reads)
    assert np.array_equal(ka, kb) and np.array_equal(ca, cb)
    assert cut_a == cut_b
    assert np.array_equal(mna.keys, mnb.keys)
    assert np.array_equal(mna.suffix_counts, mnb.suffix_counts)
    assert np.array_equal(mna.prefix_counts, mnb.prefix_counts)


@pytest.mark.gpu
@pytest.mark.parametrize("n_ranks", [2, 3, 5])
def test_count_file_rank_slices_match_the_oracle(tmp_path, n_ranks):
    from gpu_helpers import ctx
    data = _fasta(21, n_reads=3000, genome_len=20000)
    path = _write(tmp_path, "in.fa", data)
    p = pk.default_params(k=31, num_buckets=21)
    windows = 0
    for r in range(n_ranks):
        part = po.divide_reads(data, r, n_ranks, 250)
        with pk.Job(ctx()) as job:
            job.count_file(path, p, r, n_ranks)
            keys, counts = job.table()
            s = job.summary()
        ref = po.count(part, 31)
        k128 = pk.to_key128(keys)
        assert np.array_equal(k128["lo"], ref.keys["lo"]) and np.array_equal(k128["hi"], ref.keys["hi"])
        assert np.array_equal(counts, ref.counts.astype(np.uint32))
        assert s.n_reads == part.count(b">")
        windows += s.n_windows
    assert windows == po.count(data, 31).counts.sum()  # the slices split records, never windows


@pytest.mark.gpu
def test_count_file_errors(tmp_path):
    from gpu_helpers import ctx
    p = pk.default_params(k=32)
    bad = _fasta(3).replace(b"\n>r10\n", b"\nxr10\n", 1)
    assert bad != _fasta(3)
    path = _write(tmp_path, "bad.fa", bad)
    with pk.Job(ctx()) as job:
        with pytest.raises(pk.FormatError):
            job.count_file(path, p)
        with pytest.raises(pk.InputFileError):
            job.count_file(str(tmp_path / "missing.fa"), p)
        # the job is usable again afterwards
        good = _write(tmp_path, "good.fa", _fasta(4))
        job.count_file(good, p)
        assert job.summary().n_windows == po.count(_fasta(4), 32).counts.sum()


@pytest.mark.gpu
@pytest.mark.parametrize("data", [b"", b"no header here\nACGT\n", b">only-header"])
def test_count_file_without_windows(tmp_path, data):
    """Files with no k-mer window count to an empty table; the cutoff then ends the run
    as the reference's MPI_Abort does (PK_ERR_EMPTY)."""
    from gpu_helpers import ctx
    path = _write(tmp_path, "in.fa", data)
    p = pk.default_params(k=32)
    with pk.Job(ctx()) as job:
        job.count_file(path, p)
        assert job.summary().n_windows == 0
        with pytest.raises(pk.EmptyAfterCutoff):
            job.cutoff(21)
