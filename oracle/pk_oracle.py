"""Python face of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, always as the checker of the GPU path.  It
wraps:

* ``pk_oracle.c`` -- the plain-C restatement of the reference algorithm, built
  into ``oracle/_build/libpk_oracle.so`` by :func:`build`;
* the reference's own hot path compiled from its sources into
  ``oracle/_ref/pakman_ref_k<K>`` by ``oracle/ref/Makefile`` (only where the
  reference tree is present), plus readers for the dump files it writes.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import tempfile
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "libpk_oracle.so")
# The reference source tree: $PAKMAN_REFERENCE, else where this project's build
# container mounts it.  Absent on machines that only run the prebuilt oracle.
REFERENCE_TREE = os.environ.get("PAKMAN_REFERENCE", "/root/reference")

PKO_OK, PKO_EFORMAT, PKO_EARG, PKO_ENOMEM, PKO_EEMPTY = 0, -1, -2, -3, -4


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with oracle status {code}")
        self.code = code


def build(force: bool = False) -> str:
    """Compile pk_oracle.c and pk_compact.c (gcc, -O2) into oracle/_build/libpk_oracle.so."""
    srcs = [os.path.join(HERE, "pk_oracle.c"), os.path.join(HERE, "pk_compact.c")]
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(x) for x in srcs):
        tmp = LIB + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-pthread", "-shared", "-fPIC", "-o", tmp, *srcs])
        os.replace(tmp, LIB)
    return LIB


def build_reference(k: int) -> Optional[str]:
    """Build oracle/_ref/pakman_ref_k<k> from the reference sources, if present."""
    exe = os.path.join(REF_OUT, f"pakman_ref_k{k}")
    if os.path.exists(exe):
        return exe
    if not os.path.isdir(REFERENCE_TREE):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"K={k}", f"REF={REFERENCE_TREE}", "-j8"],
                          stdout=subprocess.DEVNULL)
    return exe if os.path.exists(exe) else None


def build_divide_reference() -> Optional[str]:
    """Build oracle/_ref/divide_reads_ref (the reference's DivideReads called alone for
    any rank and rank count), if the reference tree is present."""
    exe = os.path.join(REF_OUT, "divide_reads_ref")
    if os.path.exists(exe):
        return exe
    if not os.path.isdir(REFERENCE_TREE):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), "divide", "K=32", f"REF={REFERENCE_TREE}", "-j8"],
                          stdout=subprocess.DEVNULL)
    return exe if os.path.exists(exe) else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.pko_count.argtypes = [vp, sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp),
                                ctypes.POINTER(vp), ctypes.POINTER(sz), ctypes.POINTER(sz),
                                ctypes.POINTER(sz)]
        L.pko_count_mt.argtypes = [vp, sz, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp),
                                   ctypes.POINTER(vp), ctypes.POINTER(sz), ctypes.POINTER(sz),
                                   ctypes.POINTER(sz)]
        L.pko_count_windows.argtypes = [vp, sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(sz),
                                        ctypes.POINTER(sz)]
        L.pko_cutoff.argtypes = [vp, sz, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_int)]
        L.pko_macro_nodes.argtypes = [vp, vp, sz, ctypes.c_int, ctypes.c_uint32,
                                      ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                      ctypes.POINTER(sz), ctypes.POINTER(sz)]
        L.pko_visit.argtypes = [ctypes.c_int, ctypes.c_int]
        L.pko_wire_nodes.argtypes = [vp, vp, sz, ctypes.c_int, vp]
        L.pko_free.argtypes = [vp]
        _lib = L
    return _lib


def _take(ptr: int, count: int, dtype) -> np.ndarray:
    """Copy a malloc'd C array into numpy and free it."""
    L = lib()
    if count == 0:
        if ptr:
            L.pko_free(ptr)
        return np.empty(0, dtype=dtype)
    nbytes = count * np.dtype(dtype).itemsize
    buf = (ctypes.c_char * nbytes).from_address(ptr)
    out = np.frombuffer(buf, dtype=dtype).copy()
    L.pko_free(ptr)
    return out


KEY_DTYPE = np.dtype([("lo", "<u8"), ("hi", "<u8")])


@dataclass
class Table:
    keys: np.ndarray  # KEY_DTYPE, ascending
    counts: np.ndarray  # uint32
    n_windows: int
    n_reads: int


@dataclass
class MacroNodes:
    keys: np.ndarray  # KEY_DTYPE, ascending
    suf: np.ndarray  # (M, 4) uint32 counts by ext code, 0 = absent
    pre: np.ndarray  # (M, 4) uint32
    n_kept: int


def count(fasta: bytes, k: int, drop_n: bool = False, threads: int = 1) -> Table:
    """Sorted unique (k-mer, count) table.  threads > 1 uses the owner-partitioned
    multi-threaded restatement (valid input only; same table)."""
    L = lib()
    arr = np.frombuffer(fasta, dtype=np.uint8)
    kp, cp = ctypes.c_void_p(), ctypes.c_void_p()
    u, w, r = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    if threads > 1:
        rc = L.pko_count_mt(arr.ctypes.data, arr.size, k, int(drop_n), int(threads), ctypes.byref(kp),
                            ctypes.byref(cp), ctypes.byref(u), ctypes.byref(w), ctypes.byref(r))
    else:
        rc = L.pko_count(arr.ctypes.data, arr.size, k, int(drop_n), ctypes.byref(kp),
                         ctypes.byref(cp), ctypes.byref(u), ctypes.byref(w), ctypes.byref(r))
    if rc != PKO_OK:
        raise OracleError(rc, "pko_count")
    keys = _take(kp.value, u.value, KEY_DTYPE)
    cnts = _take(cp.value, u.value, np.uint32)
    return Table(keys, cnts, w.value, r.value)


def count_windows(fasta: bytes, k: int, drop_n: bool = False):
    L = lib()
    buf = ctypes.create_string_buffer(fasta, len(fasta))
    w, r = ctypes.c_size_t(), ctypes.c_size_t()
    rc = L.pko_count_windows(ctypes.addressof(buf), len(fasta), k, int(drop_n), ctypes.byref(w),
                             ctypes.byref(r))
    if rc != PKO_OK:
        raise OracleError(rc, "pko_count_windows")
    return w.value, r.value


def cutoff(counts: np.ndarray, t: int):
    L = lib()
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    hist = np.zeros(max(t, 1), dtype=np.uint64)
    c = ctypes.c_int()
    rc = L.pko_cutoff(counts.ctypes.data, counts.size, t, hist.ctypes.data, ctypes.byref(c))
    if rc != PKO_OK:
        raise OracleError(rc, "pko_cutoff")
    return hist[:t], c.value


def macro_nodes(table: Table, k: int, cut: int) -> MacroNodes:
    L = lib()
    keys = np.ascontiguousarray(table.keys)
    cnts = np.ascontiguousarray(table.counts, dtype=np.uint32)
    nk, ns, np_ = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    m, v = ctypes.c_size_t(), ctypes.c_size_t()
    rc = L.pko_macro_nodes(keys.ctypes.data, cnts.ctypes.data, cnts.size, k, cut, ctypes.byref(nk),
                           ctypes.byref(ns), ctypes.byref(np_), ctypes.byref(m), ctypes.byref(v))
    if rc != PKO_OK:
        raise OracleError(rc, "pko_macro_nodes")
    M = m.value
    return MacroNodes(_take(nk.value, M, KEY_DTYPE), _take(ns.value, 4 * M, np.uint32).reshape(M, 4),
                      _take(np_.value, 4 * M, np.uint32).reshape(M, 4), v.value)


# one node's initial wiring (pko_wire in pk_oracle.c)
WIRE_DTYPE = np.dtype([("ns", "<i4"), ("np", "<i4"), ("term_suf", "<i4"), ("term_pre", "<i4"),
                       ("nw", "<i4"), ("wire", "<i4", (9, 3)), ("begin", "<i4", (5, 2))])


def wire(suf: np.ndarray, pre: np.ndarray, coverage: int) -> np.ndarray:
    """Initial wiring of every node of a macro-node table (suf/pre: (M, 4) counts)."""
    L = lib()
    suf = np.ascontiguousarray(suf, dtype=np.uint32)
    pre = np.ascontiguousarray(pre, dtype=np.uint32)
    m = suf.shape[0]
    out = np.zeros(max(1, m), WIRE_DTYPE)
    rc = L.pko_wire_nodes(suf.ctypes.data, pre.ctypes.data, m, int(coverage), out.ctypes.data)
    if rc != PKO_OK:
        raise OracleError(rc, "pko_wire_nodes")
    return out[:m]


def read_wire_dump(path: str):
    """The reference's wiring dump as WIRE_DTYPE rows plus each node's list order:
    (wiring, suffix_exts, prefix_exts) where *_exts[i] lists the entries' base codes
    in the reference's order (4 = terminal)."""
    data = open(path, "rb").read()
    assert data[:4] == b"PKW1"
    m = int.from_bytes(data[4:12], "little")
    off = 12
    out = np.zeros(m, WIRE_DTYPE)
    sexts, pexts = [], []
    for i in range(m):
        lists = []
        for side in range(2):
            n = int.from_bytes(data[off:off + 4], "little")
            off += 4
            ent = np.frombuffer(data, np.dtype([("ext", "u1"), ("count", "<i4"), ("visit", "<i4")]), n, off)
            off += 9 * n
            lists.append(ent)
        nw = int.from_bytes(data[off:off + 4], "little")
        off += 4
        wires = np.frombuffer(data, "<i4", 3 * nw, off).reshape(nw, 3)
        off += 12 * nw
        nb = int.from_bytes(data[off:off + 4], "little")
        off += 4
        beg = np.frombuffer(data, "<i4", 2 * nb, off).reshape(nb, 2)
        off += 8 * nb
        s, p = lists
        out[i]["ns"], out[i]["np"] = len(s), len(p)
        out[i]["term_suf"] = int(s["visit"][s["ext"] == 0xff][0])
        out[i]["term_pre"] = int(p["visit"][p["ext"] == 0xff][0])
        used = int(np.count_nonzero(wires[:, 2]))
        out[i]["nw"] = used
        out[i]["wire"][:min(9, nw)] = wires[:9]
        out[i]["begin"][:min(5, nb)] = beg[:5]
        sexts.append([4 if e == 0xff else int(e) for e in s["ext"]])
        pexts.append([4 if e == 0xff else int(e) for e in p["ext"]])
    return out, sexts, pexts


def visit(count_: int, coverage: int) -> int:
    return lib().pko_visit(int(count_), int(coverage))


@dataclass
class Pipeline:
    table: Table
    hist: np.ndarray
    cutoff: int
    mn: Optional[MacroNodes]


def run(fasta: bytes, k: int, t: int = 21, drop_n: bool = False, threads: int = 1) -> Pipeline:
    """Whole path: table, histogram/cutoff, macro-nodes (None if nothing is kept)."""
    tab = count(fasta, k, drop_n, threads)
    hist, cut = cutoff(tab.counts, t)
    try:
        mn = macro_nodes(tab, k, cut)
    except OracleError as e:
        if e.code != PKO_EEMPTY:
            raise
        mn = None
    return Pipeline(tab, hist, cut, mn)


# ----------------------------------------------------------- reference dumps ---

@dataclass
class RefRun:
    table_keys: np.ndarray
    table_counts: np.ndarray
    cutoff: Optional[int]
    n_kept: Optional[int]
    mn_keys: Optional[np.ndarray]
    mn_suf: Optional[np.ndarray]  # (M,4) counts, 0 = absent
    mn_pre: Optional[np.ndarray]
    mn_suf_visit: Optional[np.ndarray]
    mn_pre_visit: Optional[np.ndarray]
    mn_k1_ok: bool
    aborted: bool
    seconds: dict
    stdout: str
    wiring: Optional[tuple] = None  # read_wire_dump(): (WIRE_DTYPE rows, suffix exts, prefix exts)


def divide_reads(data: bytes, rank: int, size: int, overlap: int) -> Optional[bytes]:
    """One MPI rank's input data as the reference's DivideReads computes it from the
    file bytes (src/input_reading.cpp:68-243): rank r reads bytes
    [r*L, r*L + L - 1 + overlap] with L = filesize // size (the last rank up to the end
    of the file), skips the bytes before the first '>' of that chunk (ranks > 0) and
    ends at the first '>' at or after chunk offset L (every rank but the last).  The
    overlap is read_length + 100 (src/input_reading.cpp:251).  Returns None where the
    reference's scans would run past its chunk, which its loops do not bound."""
    fs = len(data)
    local = fs // size
    start = rank * local
    end = start + local - 1 + overlap
    if rank == size - 1:
        end = fs - 1
    n = end - start + 1                  # the chunk length the reference allocates
    chunk = data[start:end + 1]          # a read past the end of the file comes back short
    locstart, locend = 0, n
    if rank != 0:
        i = chunk.find(b">")
        if i < 0:
            return None
        locstart = i
    if rank != size - 1:
        i = chunk.find(b">", n - overlap)
        if i < 0:
            return None
        locend = i
    if locend < locstart:
        return None
    return chunk[locstart:locend]


def read_table_dump(path: str):
    with open(path, "rb") as f:
        assert f.read(4) == b"PKT1"
        k = int(np.frombuffer(f.read(4), "<u4")[0])
        u = int(np.frombuffer(f.read(8), "<u8")[0])
        rec = np.frombuffer(f.read(u * 20), dtype=np.dtype([("lo", "<u8"), ("hi", "<u8"),
                                                             ("count", "<i4")]))
    keys = np.empty(u, KEY_DTYPE)
    keys["lo"], keys["hi"] = rec["lo"], rec["hi"]
    return k, keys, rec["count"].astype(np.int64)


def _key_bases(lo: int, hi: int, nbases: int):
    v = (hi << 64) | lo
    return [(v >> (2 * (nbases - 1 - i))) & 3 for i in range(nbases)]


def read_mn_dump(path: str, coverage: int):
    """Parse a macro-node dump into (keys, suf, pre, suf_visit, pre_visit, k1_ok)."""
    data = open(path, "rb").read()
    assert data[:4] == b"PKM1"
    k = int.from_bytes(data[4:8], "little")
    m = int.from_bytes(data[8:16], "little")
    off = 16
    keys = np.empty(m, KEY_DTYPE)
    suf = np.zeros((m, 4), np.uint32)
    pre = np.zeros((m, 4), np.uint32)
    sv = np.zeros((m, 4), np.int64)
    pv = np.zeros((m, 4), np.int64)
    k1_ok = True
    ent = np.dtype([("ext", "u1"), ("count", "<i4"), ("visit", "<i4"), ("term", "u1")])
    for i in range(m):
        lo, hi = np.frombuffer(data, "<u8", 2, off)
        off += 16
        keys[i] = (lo, hi)
        kl = int.from_bytes(data[off:off + 4], "little")
        off += 4
        bases = list(data[off:off + kl])
        off += kl
        if bases != _key_bases(int(lo), int(hi), k - 1):
            k1_ok = False
        for side, arr, varr in ((0, suf, sv), (1, pre, pv)):
            n = int.from_bytes(data[off:off + 4], "little")
            off += 4
            e = np.frombuffer(data, ent, n, off)
            off += n * ent.itemsize
            for x in e:
                if x["term"] or x["ext"] > 3 or arr[i, x["ext"]] != 0:
                    k1_ok = False
                arr[i, x["ext"]] = x["count"]
                varr[i, x["ext"]] = x["visit"]
    return keys, suf, pre, sv, pv, k1_ok


def run_reference(fasta: bytes, k: int, read_len: int, coverage: int, t: int = 21,
                  batch: Optional[int] = None, threads: int = 1, variant: Optional[int] = None,
                  workdir: Optional[str] = None, want_mn: bool = True) -> Optional[RefRun]:
    """Run the reference's own hot path on `fasta`; None if it cannot be built here."""
    exe = build_reference(k)
    if exe is None:
        return None
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        fa = os.path.join(d, "in.fa")
        with open(fa, "wb") as f:
            f.write(fasta)
        out = os.path.join(d, "out")
        args = [exe, out, "-f", fa, "-r", str(read_len), "-c", str(coverage), "-t", str(t)]
        if batch:
            args += ["-b", str(batch)]
        if variant is not None:
            args += ["-p", str(variant)]
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        p = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, env=env)
        txt = p.stdout.decode(errors="replace")
        _, tk, tc = read_table_dump(out + ".table") if os.path.exists(out + ".table") else (
            k, np.empty(0, KEY_DTYPE), np.empty(0, np.int64))
        cut = kept = None
        for line in txt.splitlines():
            if "Total valid (>= min_bucket(" in line:
                cut = int(line.split("min_bucket(")[1].split(")")[0])
                kept = int(line.split(":")[-1].strip())
        secs = {}
        for line in txt.splitlines():
            if line.startswith("{") and "count_s" in line:
                secs = json.loads(line)
        aborted = p.returncode != 0
        if aborted or not want_mn or not os.path.exists(out + ".mn"):
            return RefRun(tk, tc, cut, kept, None, None, None, None, None, True, aborted, secs, txt)
        mk, ms, mp, sv, pv, ok = read_mn_dump(out + ".mn", coverage)
        wires = read_wire_dump(out + ".wire") if os.path.exists(out + ".wire") else None
        return RefRun(tk, tc, cut, kept, mk, ms, mp, sv, pv, ok, aborted, secs, txt, wires)
