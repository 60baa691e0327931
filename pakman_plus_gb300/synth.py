"""Seeded synthetic genomes and read sets in PaKman's FASTA layout.

The reference benchmarks on real read sets (chimp, black bear, elephant, human)
that are not available here; these generators stand in for them with seeded
synthetic reads of the same shapes: one FASTA record per read, a ``>r<i>``
header line followed by exactly one sequence line, the layout the reference's
reader accepts (src/kmer_counting.cpp:2920-2935 expects '>' at every record
start and one sequence line per record).

All randomness comes from ``numpy.random.Generator(PCG64(seed))``.  Bases are
generated as codes 0..3 = A, C, G, T; substitutions pick one of the three other
bases uniformly; the reverse strand is the reverse complement.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

_ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
_N = ord("N")


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def random_genome(rng: np.random.Generator, length: int, gc: float = 0.5) -> np.ndarray:
    """Genome as base codes (0=A 1=C 2=G 3=T) with the given GC fraction."""
    at = (1.0 - gc) / 2.0
    cg = gc / 2.0
    return rng.choice(4, size=length, p=[at, cg, cg, at]).astype(np.uint8)


def plant_repeat_families(rng, genome, families: int, unit_len: int, copies_lo: int,
                          copies_hi: int, gc: float) -> float:
    """Overwrite ``families`` random units, each at ``copies_lo..copies_hi`` random
    positions.  Returns the fraction of genome positions covered by a copy."""
    covered = np.zeros(genome.size, dtype=bool)
    for _ in range(families):
        unit = random_genome(rng, unit_len, gc)
        copies = int(rng.integers(copies_lo, copies_hi + 1))
        for _ in range(copies):
            pos = int(rng.integers(0, genome.size - unit_len + 1))
            genome[pos:pos + unit_len] = unit
            covered[pos:pos + unit_len] = True
    return float(covered.mean())


def plant_tandem_and_interspersed(rng, genome, fraction: float, period_lo: int, period_hi: int,
                                  gc: float) -> float:
    """Cover about ``fraction`` of the genome with repeats: half as tandem arrays of a
    unit whose period is log-uniform in [period_lo, period_hi], half as interspersed
    copies of such units.  Returns the achieved covered fraction."""
    covered = np.zeros(genome.size, dtype=bool)
    target = fraction * genome.size
    planted = 0
    tandem_half = True
    while planted < target:
        period = int(round(math.exp(rng.uniform(math.log(period_lo), math.log(period_hi)))))
        period = max(period_lo, min(period_hi, period))
        unit = random_genome(rng, period, gc)
        if tandem_half:
            span = int(rng.integers(max(2 * period, 200), max(4 * period, 2000) + 1))
            arr = np.resize(unit, span)
            pos = int(rng.integers(0, genome.size - span + 1))
            genome[pos:pos + span] = arr
            covered[pos:pos + span] = True
            planted += span
        else:
            copies = int(rng.integers(3, 11))
            for _ in range(copies):
                pos = int(rng.integers(0, genome.size - period + 1))
                genome[pos:pos + period] = unit
                covered[pos:pos + period] = True
                planted += period
        tandem_half = not tandem_half
    return float(covered.mean())


def sample_reads(rng, genome: np.ndarray, n_reads: int, read_len, err: float,
                 random_strand: bool = True, n_rate: float = 0.0) -> List[np.ndarray]:
    """Reads as ASCII uint8 rows.  ``read_len`` is an int or an (n_reads,) array."""
    lens = np.broadcast_to(np.asarray(read_len, dtype=np.int64), (n_reads,))
    out: List[np.ndarray] = []
    chunk = 1 << 18
    for c0 in range(0, n_reads, chunk):
        c1 = min(n_reads, c0 + chunk)
        ln = lens[c0:c1]
        lmax = int(ln.max())
        starts = rng.integers(0, genome.size - ln + 1)
        idx = starts[:, None] + np.arange(lmax)[None, :]
        idx = np.minimum(idx, genome.size - 1)
        codes = genome[idx]
        if err > 0:
            m = rng.random(codes.shape) < err
            codes = np.where(m, (codes + rng.integers(1, 4, size=codes.shape)) & 3, codes)
        if random_strand:
            rev = rng.random(c1 - c0) < 0.5
            # reverse complement of the first ln bases: complement code = 3 - code
            rc = 3 - codes[:, ::-1]
            # after reversing, the valid bases of a short row sit at the end; shift them
            shift = lmax - ln
            rows = np.arange(c1 - c0)[:, None]
            cols = (np.arange(lmax)[None, :] + shift[:, None]) % lmax
            rc = rc[rows, cols]
            codes = np.where(rev[:, None], rc, codes)
        asc = _ACGT[codes]
        if n_rate > 0:
            nm = rng.random(asc.shape) < n_rate
            asc = np.where(nm, np.uint8(_N), asc)
        for i in range(c1 - c0):
            out.append(asc[i, : ln[i]])
    return out


def _header_block(first_index: int, n: int):
    """Concatenated b">r<i>\n" headers and their lengths, built without a Python loop."""
    ids = np.arange(first_index, first_index + n, dtype=np.int64)
    nd = np.ones(n, dtype=np.int64)
    x = ids.copy()
    while True:
        x //= 10
        more = x > 0
        if not more.any():
            break
        nd += more
    hl = nd + 3  # '>' 'r' digits '\n'
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(hl, out=off[1:])
    hb = np.empty(int(off[-1]), dtype=np.uint8)
    hb[off[:-1]] = ord(">")
    hb[off[:-1] + 1] = ord("r")
    hb[off[1:] - 1] = ord("\n")
    v = ids.copy()
    for d in range(int(nd.max())):
        has = nd > d
        pos = off[:-1] + 2 + nd - 1 - d
        hb[pos[has]] = (48 + v[has] % 10).astype(np.uint8)
        v //= 10
    return hb, hl


def matrix_to_fasta(mat: np.ndarray, first_index: int = 0) -> bytes:
    """FASTA for equal-length reads given as an (n, L) uint8 ASCII matrix.  Reads whose
    ids have the same number of digits form a regular block of records, so each block
    is filled as a 2-D array."""
    n, L = mat.shape
    if n == 0:
        return b""
    parts = []
    lo = first_index
    end = first_index + n
    while lo < end:
        d = len(str(lo))
        hi = min(end, 10 ** d)
        m = hi - lo
        rec = np.empty((m, 3 + d + L + 1), dtype=np.uint8)
        rec[:, 0] = ord(">")
        rec[:, 1] = ord("r")
        v = np.arange(lo, hi, dtype=np.int64)
        for c in range(d - 1, -1, -1):
            rec[:, 2 + c] = 48 + (v % 10)
            v //= 10
        rec[:, 2 + d] = ord("\n")
        rec[:, 3 + d:3 + d + L] = mat[lo - first_index:hi - first_index]
        rec[:, -1] = ord("\n")
        parts.append(rec.reshape(-1))
        lo = hi
    return np.concatenate(parts).tobytes()


def sample_read_matrix(rng, genome: np.ndarray, n_reads: int, read_len: int, err: float,
                       random_strand: bool = True, n_rate: float = 0.0) -> np.ndarray:
    """Equal-length reads as an (n, L) ASCII matrix: uniform start positions, random
    strand, iid substitutions to one of the three other bases."""
    out = np.empty((n_reads, read_len), dtype=np.uint8)
    win = np.lib.stride_tricks.sliding_window_view(genome, read_len)
    chunk = 1 << 18
    for c0 in range(0, n_reads, chunk):
        c1 = min(n_reads, c0 + chunk)
        m = c1 - c0
        starts = rng.integers(0, genome.size - read_len + 1, size=m)
        codes = win[starts]
        flat = codes.reshape(-1)
        if err > 0:
            ne = int(rng.binomial(flat.size, err))
            pos = rng.integers(0, flat.size, size=ne)
            flat[pos] = (flat[pos] + rng.integers(1, 4, size=ne).astype(np.uint8)) & 3
        if random_strand:
            rev = rng.random(m) < 0.5
            codes[rev] = 3 - codes[rev, ::-1]
        asc = _ACGT[codes]
        if n_rate > 0:
            af = asc.reshape(-1)
            nn = int(rng.binomial(af.size, n_rate))
            af[rng.integers(0, af.size, size=nn)] = _N
        out[c0:c1] = asc
    return out


def reads_to_fasta(reads: Sequence[np.ndarray], first_index: int = 0) -> bytes:
    """One ``>r<i>`` header line and one sequence line per read."""
    n = len(reads)
    if n == 0:
        return b""
    ids = np.arange(first_index, first_index + n)
    heads = [b">r%d\n" % i for i in ids]
    hl = np.fromiter((len(h) for h in heads), dtype=np.int64, count=n)
    sl = np.fromiter((r.size for r in reads), dtype=np.int64, count=n)
    rec = hl + sl + 1
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(rec, out=off[1:])
    buf = np.empty(int(off[-1]), dtype=np.uint8)
    hb = np.frombuffer(b"".join(heads), dtype=np.uint8)
    hoff = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(hl, out=hoff[1:])
    # scatter headers
    hpos = np.repeat(off[:-1] - hoff[:-1], hl) + np.arange(hb.size)
    buf[hpos] = hb
    sb = np.concatenate(reads) if n else np.empty(0, np.uint8)
    soff = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(sl, out=soff[1:])
    spos = np.repeat(off[:-1] + hl - soff[:-1], sl) + np.arange(sb.size)
    buf[spos] = sb
    buf[off[1:] - 1] = ord("\n")
    return buf.tobytes()


@dataclasses.dataclass
class ReadSet:
    """A synthetic read set and the run parameters it is meant for."""
    name: str
    fasta: bytes
    k: int
    coverage: int
    read_len: int
    n_reads: int
    genome_len: int
    drop_n: bool = False
    t: int = 21
    batch: int = 100_000_000
    repeat_fraction: float = 0.0

    def n_windows(self) -> int:
        """Number of k-mer windows in the reference's sense (one per position of each
        sequence line with k bases available); 'N' windows included."""
        return windows_in_fasta(self.fasta, self.k, drop_n=self.drop_n)


def windows_in_fasta(fasta: bytes, k: int, drop_n: bool = False) -> int:
    """Count valid k-mer windows (host-side, independent of any counter)."""
    a = np.frombuffer(fasta, dtype=np.uint8)
    first = fasta.find(b">")
    if first < 0:
        return 0
    a = a[first:]
    nl = np.flatnonzero(a == 10)
    starts = np.concatenate(([0], nl + 1))
    ends = np.concatenate((nl, [a.size]))
    seq_s = starts[1::2]
    seq_e = ends[1::2][: seq_s.size]
    if not drop_n:
        return int(np.maximum(seq_e - seq_s - k + 1, 0).sum())
    total = 0
    isn = (a == ord("N")) | (a == ord("n"))
    for s, e in zip(seq_s, seq_e):
        seg = isn[s:e]
        cut = np.flatnonzero(seg)
        bounds = np.concatenate(([-1], cut, [e - s]))
        run = np.diff(bounds) - 1
        total += int(np.maximum(run - k + 1, 0).sum())
    return total


# --------------------------------------------------------------------------------------
# The five workloads (sizes as named in the project's workload list).
# --------------------------------------------------------------------------------------

def config1(scale: float = 1.0) -> ReadSet:
    """1 Mbp uniform genome, 100 bp reads at 30x, 1% errors, random strand, k=32."""
    g = _rng(1001)
    glen = int(1_000_000 * scale)
    genome = random_genome(g, glen, 0.5)
    n = int(round(30 * glen / 100))
    mat = sample_read_matrix(_rng(2001), genome, n, 100, 0.01)
    return ReadSet("plain-1Mbp-30x-k32", matrix_to_fasta(mat), 32, 30, 100, n, glen)


def config2(scale: float = 1.0) -> ReadSet:
    """4.6 Mbp genome at 50% GC with 20 planted 5 kb repeat families (3-6 copies);
    100 bp reads at 80x, 0.5% errors; k=32, -b 100000000, -t 21."""
    g = _rng(1002)
    glen = int(4_600_000 * scale)
    genome = random_genome(g, glen, 0.5)
    unit = min(5000, max(200, glen // 200))
    frac = plant_repeat_families(g, genome, 20, unit, 3, 6, 0.5)
    n = int(round(80 * glen / 100))
    mat = sample_read_matrix(_rng(2002), genome, n, 100, 0.005)
    return ReadSet("bacterial-4.6Mbp-80x-k32", matrix_to_fasta(mat), 32, 80, 100, n, glen,
                   repeat_fraction=frac)


def config3(scale: float = 1.0) -> ReadSet:
    """50 Mbp genome at 45% GC with 10% tandem/interspersed repeats (period 2-500 bp);
    150 bp reads at 40x, 0.3% substitutions + 0.05% N; k=63, N windows dropped."""
    g = _rng(1003)
    glen = int(50_000_000 * scale)
    genome = random_genome(g, glen, 0.45)
    frac = plant_tandem_and_interspersed(g, genome, 0.10, 2, 500, 0.45)
    n = int(round(40 * glen / 150))
    mat = sample_read_matrix(_rng(2003), genome, n, 150, 0.003, n_rate=0.0005)
    return ReadSet("longk-50Mbp-40x-k63", matrix_to_fasta(mat), 63, 40, 150, n, glen,
                   drop_n=True, repeat_fraction=frac)


def config4_set(index: int, scale: float = 1.0) -> ReadSet:
    """One of the 256 batching sets: genome log-uniform in [20 kb, 5 Mbp], read length
    uniform in 100..150, coverage uniform in [20, 80], 0.5% errors, k=32."""
    g = _rng(4_000_000 + index)
    glen = int(math.exp(g.uniform(math.log(20_000), math.log(5_000_000))) * scale)
    glen = max(glen, 400)
    rl = int(g.integers(100, 151))
    cov = int(g.integers(20, 81))
    genome = random_genome(g, glen, 0.5)
    n = max(1, int(round(cov * glen / rl)))
    mat = sample_read_matrix(g, genome, n, rl, 0.005)
    return ReadSet(f"batch-set-{index}", matrix_to_fasta(mat), 32, cov, rl, n, glen)


def config5_job(index: int, scale: float = 1.0) -> ReadSet:
    """One serving job: genome log-uniform in [10 kb, 20 Mbp], 100 bp reads at 30-80x,
    0.5% errors, k drawn from {31, 32, 63}."""
    g = _rng(5_000_000 + index)
    glen = int(math.exp(g.uniform(math.log(10_000), math.log(20_000_000))) * scale)
    glen = max(glen, 400)
    cov = int(g.integers(30, 81))
    k = int(g.choice([31, 32, 63]))
    genome = random_genome(g, glen, 0.5)
    n = max(1, int(round(cov * glen / 100)))
    mat = sample_read_matrix(g, genome, n, 100, 0.005)
    return ReadSet(f"serve-job-{index}", matrix_to_fasta(mat), k, cov, 100, n, glen)


def small_case(seed: int, genome_len: int = 2000, n_reads: int = 300, read_len=100,
               err: float = 0.01, n_rate: float = 0.0, lowercase: float = 0.0,
               k: int = 32, coverage: int = 10) -> ReadSet:
    """Small seeded read set for exact tests (optionally with N and lowercase bases)."""
    g = _rng(seed)
    genome = random_genome(g, genome_len, 0.5)
    reads = sample_reads(g, genome, n_reads, read_len, err, n_rate=n_rate)
    if lowercase > 0:
        reads = [np.where(g.random(r.size) < lowercase, r | 0x20, r).astype(np.uint8)
                 for r in reads]
    rl = int(np.max(read_len)) if np.ndim(read_len) else int(read_len)
    return ReadSet(f"small-{seed}", reads_to_fasta(reads), k, coverage, rl, n_reads, genome_len)
