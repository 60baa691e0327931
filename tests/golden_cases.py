"""Loader for the committed golden fixtures (tests/golden/*.npz)."""
import glob
import os
import zlib
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEY_DTYPE = np.dtype([("lo", "<u8"), ("hi", "<u8")])


@dataclass
class Golden:
    name: str
    fasta: bytes
    k: int
    read_len: int
    coverage: int
    t: int
    drop_n: bool
    expect: str  # "ok" | "empty_after_cutoff" | "format"
    table_keys: Optional[np.ndarray]
    table_counts: Optional[np.ndarray]
    n_windows: Optional[int]
    cutoff: Optional[int]
    n_kept: Optional[int]
    hist: Optional[np.ndarray]
    mn_keys: Optional[np.ndarray]
    mn_suf: Optional[np.ndarray]
    mn_pre: Optional[np.ndarray]
    mn_suf_visit: Optional[np.ndarray]
    mn_pre_visit: Optional[np.ndarray]
    wiring: Optional[dict] = None  # the reference's initial wiring: w_* arrays, list orders


def _keys(lo, hi):
    k = np.empty(lo.size, KEY_DTYPE)
    k["lo"], k["hi"] = lo, hi
    return k


def load(name: str) -> Golden:
    z = np.load(os.path.join(HERE, name + ".npz"))
    g = lambda f: z[f] if f in z.files else None  # noqa: E731
    tk = _keys(z["table_lo"], z["table_hi"]) if "table_lo" in z.files else None
    mk = _keys(z["mn_lo"], z["mn_hi"]) if "mn_lo" in z.files else None
    return Golden(str(z["name"]), zlib.decompress(z["fasta_z"].tobytes()), int(z["k"]),
                  int(z["read_len"]), int(z["coverage"]), int(z["t"]), bool(z["drop_n"]),
                  str(z["expect"]), tk, g("table_count"),
                  int(z["n_windows"]) if "n_windows" in z.files else None,
                  int(z["cutoff"]) if "cutoff" in z.files else None,
                  int(z["n_kept"]) if "n_kept" in z.files else None, g("hist"), mk, g("mn_suf"),
                  g("mn_pre"), g("mn_suf_visit"), g("mn_pre_visit"),
                  {f: z[f] for f in z.files if f.startswith("w_")} or None)


def names():
    """The hot-path cases (compact_*.npz hold the compaction fixtures)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "*.npz"))
                  if not os.path.basename(p).startswith("compact_"))


def compact_names():
    """The compaction cases (compact_<name>.npz, made by make_compact_golden.py)."""
    return sorted(os.path.basename(p)[len("compact_"):-4] for p in glob.glob(os.path.join(HERE, "compact_*.npz")))


def load_compact(name):
    """A compaction case: the FASTA, (k, read_length, coverage, t), the reference's wired
    map before compaction, and per node threshold (threshold, map after, partial contigs,
    rounds, walk contig file, partial contig file) -- the reference's own dumps."""
    import zlib
    z = np.load(os.path.join(HERE, "compact_%s.npz" % name))
    unz = lambda a: zlib.decompress(a.tobytes())  # noqa: E731
    out = {"fasta": unz(z["fasta"]), "params": [int(x) for x in z["params"]],
           "before": unz(z["before"]), "runs": []}
    for thr in z["thresholds"]:
        thr = int(thr)
        out["runs"].append((thr, unz(z["after_%d" % thr]), unz(z["contigs_%d" % thr]),
                            int(z["rounds_%d" % thr][0]), unz(z["walk_%d" % thr]),
                            unz(z["partial_fa_%d" % thr])))
    return out
