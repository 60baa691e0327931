"""Generate the golden fixtures in this folder from the reference's own binaries.

Run from the repository root in a tree where the reference sources are present:

    python tests/golden/make_golden.py

For every case it writes ``<case>.npz`` holding the input FASTA (zlib) and what
the reference's hot path produced on it (k-mer table, histogram cutoff, number of
kept k-mers, macro-node table), after checking that the plain-C oracle produces
exactly the same.  The reference binaries are built from the reference sources by
``oracle/ref/Makefile`` (unmodified sources, single-rank MPI shim).

Cases that the reference rejects (nothing survives the cutoff -> MPI_Abort;
a record start that is not '>' -> assertion failure) are stored with
``aborted=True`` and the expected error of the GPU path.
"""
from __future__ import annotations

import os
import sys
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pk_oracle as po  # noqa: E402
from pakman_plus_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def split_at_n(fasta: bytes) -> bytes:
    """Reads split into separate records at every N/n: the reference then counts only
    N-free windows (too-short pieces yield nothing)."""
    out = []
    lines = fasta.split(b"\n")
    rid = 0
    for i in range(1, len(lines), 2):
        seq = lines[i]
        piece = bytearray()
        for c in seq:
            if c in (ord("N"), ord("n")):
                out.append(b">s%d\n%s\n" % (rid, bytes(piece)))
                rid += 1
                piece = bytearray()
            else:
                piece.append(c)
        out.append(b">s%d\n%s\n" % (rid, bytes(piece)))
        rid += 1
    return b"".join(out)


def ragged_fasta(seed: int) -> bytes:
    """Reads of 0..180 bases (some shorter than k), mixed case, N, a '\\r' inside one
    sequence line, and a last record without a trailing newline."""
    g = np.random.Generator(np.random.PCG64(seed))
    genome = synth.random_genome(g, 3000, 0.5)
    lens = g.integers(0, 181, size=400)
    lens[:5] = [0, 1, 31, 32, 33]
    lens[7] = 120
    reads = synth.sample_reads(g, genome, 400, lens, 0.01, n_rate=0.01)
    reads = [np.where(g.random(r.size) < 0.1, r | 0x20, r).astype(np.uint8) for r in reads]
    fa = synth.reads_to_fasta(reads)
    # put one carriage return inside a sequence line, drop the final newline
    i = fa.index(b"\n", fa.index(b">r7\n") + 4)
    fa = fa[:i - 3] + b"\r" + fa[i - 2:]
    return fa[:-1]


def cases():
    c = []
    rs = synth.small_case(11, genome_len=4000, n_reads=1500, read_len=100, err=0.01, k=32)
    c.append(dict(name="k32_basic", fasta=rs.fasta, k=32, r=100, cov=30, t=21,
                  variants=[dict(batch=5000), dict(variant=1, threads=4), dict(variant=5, threads=2)]))
    rs = synth.small_case(12, genome_len=3000, n_reads=1200, read_len=100, err=0.01,
                          n_rate=0.004, lowercase=0.05, k=31)
    c.append(dict(name="k31_lower_n", fasta=rs.fasta, k=31, r=100, cov=30, t=21))
    rs = synth.small_case(13, genome_len=3000, n_reads=800, read_len=150, err=0.003, k=63)
    c.append(dict(name="k63_basic", fasta=rs.fasta, k=63, r=150, cov=40, t=8))
    rs = synth.small_case(14, genome_len=2500, n_reads=800, read_len=150, err=0.003,
                          n_rate=0.002, k=63)
    c.append(dict(name="k63_dropn", fasta=rs.fasta, k=63, r=150, cov=40, t=21, drop_n=True))
    rs = synth.small_case(15, genome_len=2000, n_reads=800, read_len=100, err=0.005, k=64)
    c.append(dict(name="k64_full_width", fasta=rs.fasta, k=64, r=100, cov=30, t=8))
    rs = synth.small_case(16, genome_len=1500, n_reads=600, read_len=100, err=0.01, k=11)
    c.append(dict(name="k11_dense", fasta=rs.fasta, k=11, r=100, cov=30, t=12))
    c.append(dict(name="k32_ragged", fasta=ragged_fasta(17), k=32, r=100, cov=10, t=5))
    rs = synth.small_case(18, genome_len=2000, n_reads=500, read_len=100, err=0.01, k=32)
    c.append(dict(name="k32_t1", fasta=rs.fasta, k=32, r=100, cov=20, t=1))
    rs = synth.small_case(19, genome_len=1_000_000, n_reads=30, read_len=100, err=0.01, k=32)
    c.append(dict(name="k32_nothing_kept", fasta=rs.fasta, k=32, r=100, cov=10, t=21))
    rs = synth.small_case(20, genome_len=2000, n_reads=300, read_len=100, err=0.01, k=32)
    bad = rs.fasta.replace(b"\n>r150\n", b"\nxr150\n", 1)
    c.append(dict(name="k32_bad_record", fasta=bad, k=32, r=100, cov=10, t=21))
    return c


def main():
    po.build()
    for case in cases():
        k = case["k"]
        fa = case["fasta"]
        drop = case.get("drop_n", False)
        ref_input = split_at_n(fa) if drop else fa
        ref = po.run_reference(ref_input, k, case["r"], case["cov"], case["t"])
        assert ref is not None, "reference binaries need the reference sources"
        rec = dict(name=case["name"], k=k, read_len=case["r"], coverage=case["cov"], t=case["t"],
                   drop_n=drop, fasta_z=np.frombuffer(zlib.compress(fa, 9), np.uint8),
                   aborted=ref.aborted)
        table_ok = True
        if ref.table_keys.size or not ref.aborted:
            ora = po.count(fa, k, drop)
            table_ok = (np.array_equal(ora.keys, ref.table_keys)
                        and np.array_equal(ora.counts.astype(np.int64), ref.table_counts))
            rec.update(table_lo=ref.table_keys["lo"], table_hi=ref.table_keys["hi"],
                       table_count=ref.table_counts.astype(np.uint32), n_windows=ora.n_windows)
        if ref.aborted:
            if ref.table_keys.size:
                rec.update(expect="empty_after_cutoff", cutoff=ref.cutoff, n_kept=0)
                _, ocut = po.cutoff(ora.counts, case["t"])
                assert ocut == ref.cutoff, (case["name"], ocut, ref.cutoff)
            else:
                rec.update(expect="format")
                try:
                    po.count(fa, k, drop)
                    raise AssertionError("oracle accepted a malformed record")
                except po.OracleError as e:
                    assert e.code == po.PKO_EFORMAT
        else:
            pipe = po.run(fa, k, case["t"], drop)
            assert pipe.cutoff == ref.cutoff, (case["name"], pipe.cutoff, ref.cutoff)
            assert pipe.mn.n_kept == ref.n_kept
            assert ref.mn_k1_ok, case["name"]
            mn_ok = (np.array_equal(pipe.mn.keys, ref.mn_keys) and np.array_equal(pipe.mn.suf, ref.mn_suf)
                     and np.array_equal(pipe.mn.pre, ref.mn_pre))
            vis = np.vectorize(lambda c: po.visit(int(c), case["cov"]) if c else 0)
            visit_ok = (np.array_equal(vis(ref.mn_suf), ref.mn_suf_visit)
                        and np.array_equal(vis(ref.mn_pre), ref.mn_pre_visit))
            assert mn_ok and visit_ok, case["name"]
            rec.update(expect="ok", cutoff=ref.cutoff, n_kept=ref.n_kept, hist=pipe.hist,
                       mn_lo=ref.mn_keys["lo"], mn_hi=ref.mn_keys["hi"], mn_suf=ref.mn_suf,
                       mn_pre=ref.mn_pre, mn_suf_visit=ref.mn_suf_visit, mn_pre_visit=ref.mn_pre_visit)
            # the reference's initial wiring (src/wire.cpp) and its list orders (4 = terminal)
            rw, sexts, pexts = ref.wiring
            pad = lambda lists: np.array([l + [-1] * (5 - len(l)) for l in lists], np.int8).reshape(-1, 5)  # noqa: E731
            rec.update(w_ns=rw["ns"], w_np=rw["np"], w_term_suf=rw["term_suf"], w_term_pre=rw["term_pre"],
                       w_nw=rw["nw"], w_wire=rw["wire"], w_begin=rw["begin"], w_sext=pad(sexts),
                       w_pext=pad(pexts))
        assert table_ok, case["name"]
        # the batched flush (-b) and the concurrent counters (-p) must give the same table
        for var in case.get("variants", []):
            alt = po.run_reference(ref_input, k, case["r"], case["cov"], case["t"],
                                   batch=var.get("batch"), variant=var.get("variant"),
                                   threads=var.get("threads", 1))
            a_keys, a_cnt = alt.table_keys, alt.table_counts
            if var.get("variant") == 5:  # the async counter's table comes out unordered
                o = np.lexsort((a_keys["lo"], a_keys["hi"]))
                a_keys, a_cnt = a_keys[o], a_cnt[o]
            assert np.array_equal(a_keys, ref.table_keys), (case["name"], var)
            assert np.array_equal(a_cnt, ref.table_counts), (case["name"], var)
            assert alt.cutoff == ref.cutoff and alt.n_kept == ref.n_kept, (case["name"], var)
            print(f"  {case['name']}: reference variant {var} gives the same table")
        np.savez_compressed(os.path.join(OUT, case["name"] + ".npz"), **rec)
        print(f"{case['name']}: k={k} U={rec.get('table_count', np.empty(0)).size} "
              f"cutoff={rec.get('cutoff')} kept={rec.get('n_kept')} "
              f"M={rec.get('mn_lo', np.empty(0)).size} expect={rec['expect']}")


if __name__ == "__main__":
    main()
