"""Generate the compaction golden fixtures in this folder from the reference's own
iterative compaction.

Run from the repository root in a tree where the reference sources are present:

    python tests/golden/make_compact_golden.py

For every case it writes ``compact_<case>.npz`` holding the input FASTA (zlib), the
run's parameters and the reference's own dumps (zlib): the wired macro-node map before
compaction, the map left at the node threshold, the partial contigs, and the contig
files its walk writes (walk and partial contigs longer than 400 bases), after checking
that the oracle (oracle/pk_compact.py) reproduces them from the map before.  The
binary is built from the unmodified reference sources by ``oracle/ref/Makefile``
(``make -C oracle/ref compact``, single-rank MPI shim).
"""
from __future__ import annotations

import os
import sys
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import pk_compact as pc  # noqa: E402
from pakman_plus_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def tandem_fasta(seed: int) -> bytes:
    """8 kbp genome with a dinucleotide run, a homopolymer run and an 8-mer tandem
    array (self-loops and short cycles in the graph), 8000 reads of 100 bp at 0.5%
    errors."""
    g = np.random.Generator(np.random.PCG64(seed))
    genome = synth.random_genome(g, 8000, 0.5)
    genome[2000:2300] = np.resize(np.array([0, 1], np.uint8), 300)
    genome[5000:5200] = 2
    genome[6000:6600] = np.resize(np.array([0, 1, 2, 3, 3, 2, 1, 0], np.uint8), 600)
    return synth.reads_to_fasta(synth.sample_reads(g, genome, 8000, 100, 0.005))


def cases():
    bact = synth.config2(0.002)  # 9.2 kbp at 80x with planted repeat families
    small = synth.small_case(77, genome_len=5000, n_reads=2000, k=32)
    longk = synth.config3(0.0006)  # 30 kbp at 40x, k = 63
    tand = tandem_fasta(3)
    return [
        ("k32_bact", bact.fasta, 32, 100, bact.coverage, bact.t, (100, 2000)),
        ("k32_small", small.fasta, 32, 100, small.coverage, 21, (1,)),
        ("k32_tandem", tand, 32, 100, 100, 21, (1, 50)),
        ("k63_longk", longk.fasta, 63, 150, longk.coverage, longk.t, (50,)),
    ]


def z(b: bytes) -> np.ndarray:
    return np.frombuffer(zlib.compress(b, 9), np.uint8)


def main():
    for name, fasta, k, rl, cov, t, thrs in cases():
        arrays = {"fasta": z(fasta), "params": np.array([k, rl, cov, t], np.int64),
                  "thresholds": np.array(thrs, np.int64)}
        for thr in thrs:
            r = pc.run_reference(fasta, k, rl, cov, thr, t, walk=True)
            if r is None:
                raise SystemExit("the reference compaction cannot be built here")
            o = pc.compact(r.before, r.k, thr)
            if pc.state_view(o.nodes) != pc.state_view(r.after) or o.contigs != r.contigs:
                raise SystemExit("oracle disagrees with the reference on %s n=%d" % (name, thr))
            w = pc.walk(o.nodes, r.k)
            if [c for c in w if len(c) > 400] != pc.read_fasta_contigs(r.raw["walk_fa"]):
                raise SystemExit("oracle walk disagrees with the reference on %s n=%d" % (name, thr))
            arrays["walk_%d" % thr] = z(r.raw["walk_fa"])
            arrays["partial_fa_%d" % thr] = z(r.raw["partial_fa"])
            arrays["before"] = z(r.raw["before"])
            arrays["after_%d" % thr] = z(r.raw["after"])
            arrays["contigs_%d" % thr] = z(r.raw["contigs"])
            arrays["rounds_%d" % thr] = np.array([o.rounds], np.int64)
            print(name, "n", thr, "M0", len(r.before), "M1", len(r.after), "contigs", len(r.contigs),
                  "rounds", o.rounds, "walk", len(w), ">400", len(pc.read_fasta_contigs(r.raw["walk_fa"])))
        np.savez(os.path.join(OUT, "compact_%s.npz" % name), **arrays)


if __name__ == "__main__":
    main()
