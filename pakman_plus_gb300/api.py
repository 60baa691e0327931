"""Python host mirror of PaKman's counting / histogram / macro-node interface.

Two layers over the C ABI:

* :class:`Context` / :class:`Job` -- thin owners of ``pk_ctx`` / ``pk_job``.
* :class:`PakmanSession` -- the reference's phase functions with the reference's
  names and argument meanings: ``perform_kmer_counting(read_data)``
  (src/kmer_counting.cpp:3351) fills ``kmer_proc_buf`` (a sorted, unique
  KmerPairs table, src/distribute_kmers.cpp:87), ``construct_kmer_histogram()``
  (src/kmer_histogram.cpp:72) returns the histogram and ``min_bucket``, and
  ``begin_mnode_construction()`` (src/mn_construct.cpp:479) returns the macro-node
  map.  Failure modes follow the reference: a record start that is not '>' raises
  :class:`FormatError` (the reference asserts), no k-mer surviving the cutoff raises
  :class:`EmptyAfterCutoff` (the reference calls MPI_Abort).
"""
from __future__ import annotations

import ctypes
import os
from ctypes import byref, c_float, c_int, c_int32, c_uint32, c_uint64, c_void_p
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import capi
from .capi import EmptyAfterCutoff, FormatError, InputFileError, PakmanError, check, default_params  # noqa: F401

KEY128 = np.dtype([("lo", "<u8"), ("hi", "<u8")])
KMERPAIRS64 = np.dtype([("seq", "<u8"), ("k_count", "<i4")])  # packed, 12 bytes
KMERPAIRS128 = np.dtype([("seq_lo", "<u8"), ("seq_hi", "<u8"), ("k_count", "<i4")])  # 20 bytes
# pk_wiring: one macro-node's initial wiring
WIRING = np.dtype([("ns", "<i4"), ("np", "<i4"), ("term_suf", "<i4"), ("term_pre", "<i4"), ("nw", "<i4"),
                   ("wire", "<i4", (9, 3)), ("begin", "<i4", (5, 2))])


def key_dtype(k: int):
    return np.dtype("<u8") if k <= 32 else KEY128


def to_key128(keys: np.ndarray) -> np.ndarray:
    """Keys of either width as the (lo, hi) structured layout."""
    if keys.dtype == KEY128:
        return keys
    out = np.empty(keys.size, KEY128)
    out["lo"] = keys
    out["hi"] = 0
    return out


def fasta_slice(path: str, rank: int = 0, n_ranks: int = 1, read_length: int = 0) -> Tuple[int, int]:
    """(offset, length) of the slice of a FASTA file that rank `rank` of `n_ranks` reads
    (the reference's DivideReads rule; pk_fasta_slice).  Needs no device."""
    off, ln = c_uint64(), c_uint64()
    check(capi.lib().pk_fasta_slice(os.fsencode(path), rank, n_ranks, read_length, byref(off), byref(ln)),
          "pk_fasta_slice")
    return off.value, ln.value


class Context:
    """One device and an HBM budget (0 = unlimited)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        L = capi.lib()
        h = c_void_p()
        check(L.pk_ctx_create(device, hbm_budget, byref(h)), "pk_ctx_create")
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def memory(self) -> Tuple[int, int]:
        u, b = c_uint64(), c_uint64()
        check(capi.lib().pk_ctx_memory(self._h, byref(u), byref(b)), "pk_ctx_memory")
        return u.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().pk_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Summary:
    n_reads: int
    n_windows: int
    n_unique: int
    n_kept: int
    n_nodes: int
    cutoff: int
    key_bytes: int

    @staticmethod
    def from_c(s: capi.PkSummary) -> "Summary":
        return Summary(s.n_reads, s.n_windows, s.n_unique, s.n_kept, s.n_nodes, s.cutoff, s.key_bytes)


@dataclass
class MacroNodeTable:
    """Macro-nodes as columns: (k-1)-mer keys ascending, suffix/prefix counts by
    extension base code (A=0 C=1 T=2 G=3), 0 = absent; visit = ceil(count/coverage)."""
    keys: np.ndarray
    suffix_counts: np.ndarray
    prefix_counts: np.ndarray
    coverage: int
    k: int

    def __len__(self):
        return int(self.keys.size)

    @property
    def suffix_visits(self) -> np.ndarray:
        return _visit(self.suffix_counts, self.coverage)

    @property
    def prefix_visits(self) -> np.ndarray:
        return _visit(self.prefix_counts, self.coverage)

    def node(self, i: int) -> Dict:
        """One node in the reference MacroNode's terms (k_1_mer bases, suffixes,
        suffix_count pairs, prefixes, prefix_count pairs)."""
        key = self.keys[i]
        v = (int(key["hi"]) << 64 | int(key["lo"])) if self.keys.dtype == KEY128 else int(key)
        nb = self.k - 1
        bases = [(v >> (2 * (nb - 1 - p))) & 3 for p in range(nb)]
        sv, pv = self.suffix_visits[i], self.prefix_visits[i]
        suf = [(e, int(self.suffix_counts[i, e]), int(sv[e])) for e in range(4) if self.suffix_counts[i, e]]
        pre = [(e, int(self.prefix_counts[i, e]), int(pv[e])) for e in range(4) if self.prefix_counts[i, e]]
        return {"k_1_mer": bases, "suffixes": [s[0] for s in suf],
                "suffix_count": [(s[1], s[2]) for s in suf], "prefixes": [p[0] for p in pre],
                "prefix_count": [(p[1], p[2]) for p in pre]}


def _visit(counts: np.ndarray, coverage: int) -> np.ndarray:
    c = counts.astype(np.int64)
    cov = int(coverage)
    q = np.floor_divide(c, cov)
    q += (c - q * cov) != 0
    return np.where(c != 0, q, 0)


COMPACT_ENTRY = np.dtype([("ext_offset", "<u8"), ("ext_length", "<u4"), ("count", "<i4"),
                          ("visit", "<i4"), ("terminal", "<i4"), ("prefix_pos", "<i4"),
                          ("num_wires", "<i4")])


@dataclass
class Compaction:
    """The map left by pk_compact and the partial contigs of its rounds (host copies).
    Node i: keys[i]; entries[entry_offsets[i]:entry_offsets[i+1]] = n_prefixes[i]
    prefixes then its suffixes; wires[entry_offsets[i] + i :][:n_entries_i + 1]."""
    rounds: int
    keys: np.ndarray
    entry_offsets: np.ndarray
    n_prefixes: np.ndarray
    entries: np.ndarray
    wires: np.ndarray
    ext_bases: np.ndarray
    contig_offsets: np.ndarray
    contig_bases: np.ndarray

    @staticmethod
    def fetch(handle, info) -> "Compaction":
        n, e = info.n_nodes, info.n_entries
        kb = info.key_bytes
        keys = np.zeros(max(1, n), np.uint64 if kb == 8 else np.dtype([("lo", "<u8"), ("hi", "<u8")]))
        eo = np.zeros(n + 1, np.uint64)
        npre = np.zeros(max(1, n), np.uint32)
        ent = np.zeros(max(1, e), COMPACT_ENTRY)
        wires = np.zeros((max(1, e + n), 3), np.int32)
        xb = np.zeros(max(1, info.ext_bases), np.uint8)
        check(capi.lib().pk_copy_compacted(handle, keys.ctypes.data, eo.ctypes.data, npre.ctypes.data,
                                           ent.ctypes.data, wires.ctypes.data, xb.ctypes.data),
              "pk_copy_compacted")
        co = np.zeros(info.n_contigs + 1, np.uint64)
        cb = np.zeros(max(1, info.contig_bases), np.uint8)
        check(capi.lib().pk_copy_partial_contigs(handle, co.ctypes.data, cb.ctypes.data),
              "pk_copy_partial_contigs")
        return Compaction(info.rounds, keys[:n], eo, npre[:n], ent[:e], wires[:e + n],
                          xb[:info.ext_bases], co, cb[:info.contig_bases])

    @property
    def n_nodes(self) -> int:
        return int(self.keys.shape[0])

    def key(self, i: int) -> int:
        k = self.keys[i]
        return int(k) if self.keys.dtype.names is None else int(k["lo"]) | (int(k["hi"]) << 64)

    def contigs(self) -> List[bytes]:
        o = self.contig_offsets
        b = self.contig_bases.tobytes()
        return [b[int(o[c]):int(o[c + 1])] for c in range(o.shape[0] - 1)]

    def state_view(self):
        """Per node (key, suffixes, prefixes, wires, begin) with entries as
        (ext bytes, count, visit, terminal) -- the oracle's comparable form."""
        xb = self.ext_bases.tobytes()
        out = []
        for i in range(self.n_nodes):
            e0, e1 = int(self.entry_offsets[i]), int(self.entry_offsets[i + 1])
            npf = int(self.n_prefixes[i])
            ents = self.entries[e0:e1]

            def row(x):
                o, ln = int(x["ext_offset"]), int(x["ext_length"])
                return (xb[o:o + ln], int(x["count"]), int(x["visit"]), bool(x["terminal"]))
            pre = [row(x) for x in ents[:npf]]
            suf = [row(x) for x in ents[npf:]]
            w = self.wires[e0 + i:e1 + i + 1]
            out.append((self.key(i), suf, pre, [tuple(int(v) for v in r) for r in w],
                        [(int(x["prefix_pos"]), int(x["num_wires"])) for x in ents[:npf]]))
        return out


class Job:
    """One read set on the device: count -> cutoff -> macro-nodes; buffers stay
    resident until :meth:`reset` or :meth:`close`."""

    def __init__(self, ctx: Context, stream: Optional[int] = None, _borrowed=None):
        self.ctx = ctx
        self.params: Optional[capi.PkParams] = None
        self._pin = None
        self._owned = _borrowed is None
        if _borrowed is not None:  # a job owned by a server (keep_on_device results)
            self._h = _borrowed
            return
        h = c_void_p()
        check(capi.lib().pk_job_create(ctx.handle, c_void_p(stream) if stream else None, byref(h)),
              "pk_job_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    # -- counting
    def count(self, fasta, params: capi.PkParams):
        buf = _as_bytes_ptr(fasta)
        self.params = params
        check(capi.lib().pk_count(self._h, buf[0], buf[1], byref(params)), "pk_count")

    def count_device(self, ptr: int, n: int, params: capi.PkParams):
        self.params = params
        check(capi.lib().pk_count_device(self._h, c_void_p(ptr), n, byref(params)), "pk_count_device")

    def count_file(self, path: str, params: capi.PkParams, rank: int = 0, n_ranks: int = 1):
        """Count rank `rank`'s slice of a FASTA file (the whole file for one rank),
        streamed from disk to the device (pk_count_file)."""
        self.params = params
        check(capi.lib().pk_count_file(self._h, os.fsencode(path), rank, n_ranks, byref(params)),
              "pk_count_file")

    def load_table(self, keys: np.ndarray, counts: np.ndarray, params: capi.PkParams):
        """Use an existing ascending, unique (k-mer, count) table instead of counting."""
        self.params = params
        if keys.dtype != key_dtype(params.k):
            keys = keys.astype(key_dtype(params.k)) if params.k <= 32 else to_key128(keys)
        keys = np.ascontiguousarray(keys)
        counts = np.ascontiguousarray(counts, dtype=np.uint32)
        check(capi.lib().pk_table_load(self._h, keys.ctypes.data, counts.ctypes.data, counts.size,
                                       byref(params)), "pk_table_load")

    def table_info(self) -> Tuple[int, int, int]:
        u, w, r = c_uint64(), c_uint64(), c_uint64()
        check(capi.lib().pk_table_info(self._h, byref(u), byref(w), byref(r)), "pk_table_info")
        return u.value, w.value, r.value

    def table(self) -> Tuple[np.ndarray, np.ndarray]:
        u, _, _ = self.table_info()
        keys = np.empty(u, key_dtype(self.params.k))
        cnts = np.empty(u, np.uint32)
        check(capi.lib().pk_copy_table(self._h, keys.ctypes.data, cnts.ctypes.data, u), "pk_copy_table")
        return keys, cnts

    def table_packed(self) -> np.ndarray:
        u, _, _ = self.table_info()
        out = np.empty(u, KMERPAIRS64 if self.params.k <= 32 else KMERPAIRS128)
        check(capi.lib().pk_copy_table_packed(self._h, out.ctypes.data, u), "pk_copy_table_packed")
        return out

    def table_device(self) -> Tuple[int, int]:
        k, c = c_void_p(), c_void_p()
        check(capi.lib().pk_table_device(self._h, byref(k), byref(c)), "pk_table_device")
        return k.value, c.value

    # -- histogram cutoff
    def cutoff(self, num_buckets: int) -> Tuple[int, np.ndarray, int]:
        """(cutoff, histogram, kept rows).  Raises EmptyAfterCutoff (carrying the same
        three values as attributes) when no row reaches the cutoff."""
        cut, kept = c_uint32(), c_uint64()
        hist = np.zeros(num_buckets, np.uint64)
        try:
            check(capi.lib().pk_cutoff(self._h, num_buckets, byref(cut), hist.ctypes.data,
                                       byref(kept)), "pk_cutoff")
        except EmptyAfterCutoff as e:
            e.cutoff, e.hist, e.kept = cut.value, hist, kept.value
            raise
        return cut.value, hist, kept.value

    # -- macro-nodes
    def build_macro_nodes(self, min_count: int = 0) -> int:
        m = c_uint64()
        check(capi.lib().pk_build_macro_nodes(self._h, min_count, byref(m)), "pk_build_macro_nodes")
        return m.value

    def macro_nodes(self, coverage: Optional[int] = None, out=None) -> MacroNodeTable:
        """Copy the macro-node table to the host.  `out` = (keys, suffix, prefix) arrays
        to fill (e.g. in pinned memory), each with room for at least n_nodes rows."""
        s = self.summary()
        m = s.n_nodes
        if out is None:
            keys = np.empty(m, key_dtype(self.params.k))
            suf = np.empty((m, 4), np.uint32)
            pre = np.empty((m, 4), np.uint32)
            cap = m
        else:
            keys, suf, pre = out
            cap = min(keys.shape[0], suf.shape[0], pre.shape[0])
        check(capi.lib().pk_copy_macro_nodes(self._h, keys.ctypes.data, suf.ctypes.data,
                                             pre.ctypes.data, cap), "pk_copy_macro_nodes")
        cov = coverage if coverage is not None else self.params.coverage
        return MacroNodeTable(keys[:m], suf[:m], pre[:m], cov, self.params.k)

    # -- initial wiring
    def wire(self, coverage: int = 0) -> np.ndarray:
        """Initial wiring of every macro-node (WIRING rows, in node order)."""
        check(capi.lib().pk_wire_macro_nodes(self._h, coverage), "pk_wire_macro_nodes")
        m = self.summary().n_nodes
        out = np.zeros(max(1, m), WIRING)
        check(capi.lib().pk_copy_wiring(self._h, out.ctypes.data, m), "pk_copy_wiring")
        return out[:m]

    # -- iterative compaction
    def compact(self, node_threshold: int, coverage: int = 0) -> "Compaction":
        """Rounds of independent-set merging on the device until at most
        `node_threshold` macro-nodes remain (begin_iterative_compaction); the result is
        copied to the host."""
        info = capi.PkCompactionInfo()
        check(capi.lib().pk_compact(self._h, node_threshold, coverage, byref(info)), "pk_compact")
        return Compaction.fetch(self._h, info)

    def walk(self) -> List[bytes]:
        """Contigs of the walk over the map left by :meth:`compact` (traverse_pakgraph),
        as base codes, in begin order then depth-first order."""
        info = capi.PkWalkInfo()
        check(capi.lib().pk_walk(self._h, byref(info)), "pk_walk")
        off = np.zeros(info.n_contigs + 1, np.uint64)
        b = np.zeros(max(1, info.contig_bases), np.uint8)
        check(capi.lib().pk_copy_walk_contigs(self._h, off.ctypes.data, b.ctypes.data), "pk_copy_walk_contigs")
        raw = b.tobytes()
        return [raw[int(off[c]):int(off[c + 1])] for c in range(info.n_contigs)]

    # -- whole path
    def run(self, fasta, params: capi.PkParams) -> Summary:
        buf = _as_bytes_ptr(fasta)
        self.params = params
        s = capi.PkSummary()
        check(capi.lib().pk_run(self._h, buf[0], buf[1], byref(params), byref(s)), "pk_run")
        return Summary.from_c(s)

    def run_device(self, ptr: int, n: int, params: capi.PkParams) -> Summary:
        self.params = params
        s = capi.PkSummary()
        check(capi.lib().pk_run_device(self._h, c_void_p(ptr), n, byref(params), byref(s)),
              "pk_run_device")
        return Summary.from_c(s)

    def summary(self) -> Summary:
        s = capi.PkSummary()
        check(capi.lib().pk_summary_get(self._h, byref(s)), "pk_summary_get")
        return Summary.from_c(s)

    def sync(self):
        check(capi.lib().pk_job_sync(self._h), "pk_job_sync")

    def memory(self) -> int:
        b = c_uint64()
        check(capi.lib().pk_job_memory(self._h, byref(b)), "pk_job_memory")
        return b.value

    def enable_timing(self, on: bool = True):
        check(capi.lib().pk_job_enable_timing(self._h, int(on)), "pk_job_enable_timing")

    def set_wait_limit(self, spins: int = 0, withhold_unit: int = -1):
        """Polls before a bounded device wait gives up (0: the default, about 1-2 s), and a
        macro-node work unit that publishes nothing (-1: none) -- a host-side fault
        injection for testing the bounded waits (pk_job_set_wait_limit)."""
        check(capi.lib().pk_job_set_wait_limit(self._h, int(spins), int(withhold_unit)),
              "pk_job_set_wait_limit")

    def stage_times(self) -> Dict[str, float]:
        arr = (c_float * 16)()
        n = c_int()
        check(capi.lib().pk_job_stage_times(self._h, arr, 16, byref(n)), "pk_job_stage_times")
        return {capi.lib().pk_stage_name(i).decode(): float(arr[i]) for i in range(n.value)}

    def reset(self):
        check(capi.lib().pk_job_reset(self._h), "pk_job_reset")

    def close(self):
        if getattr(self, "_h", None):
            if self._owned:
                capi.lib().pk_job_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _as_bytes_ptr(fasta):
    """(pointer, length) of a bytes-like or numpy uint8 host buffer (kept alive by caller)."""
    if isinstance(fasta, np.ndarray):
        a = np.ascontiguousarray(fasta, dtype=np.uint8)
        return c_void_p(a.ctypes.data), a.size
    if isinstance(fasta, (bytes, bytearray, memoryview)):
        mv = memoryview(fasta)
        if mv.readonly:
            buf = ctypes.c_char_p(bytes(mv))
            return ctypes.cast(buf, c_void_p), mv.nbytes
        arr = (ctypes.c_char * mv.nbytes).from_buffer(mv)
        return ctypes.cast(arr, c_void_p), mv.nbytes
    raise TypeError("fasta must be bytes or a uint8 numpy array")


class PakmanSession:
    """The reference's counting / histogram / macro-node phases under the
    reference's names, with its globals (k, LMER_LENGTH, -t, -c, -r, -b) as
    attributes."""

    def __init__(self, k: int = 32, lmer_length: int = 8, num_buckets: int = 21, coverage: int = 1,
                 read_length: int = 100, batch: int = 100_000_000, drop_n: bool = False,
                 ctx: Optional[Context] = None, device: int = 0):
        self.ctx = ctx or Context(device)
        self.job = Job(self.ctx)
        self.params = default_params(k=k, lmer_length=lmer_length, num_buckets=num_buckets,
                                     coverage=coverage, read_length=read_length, batch_kmers=batch,
                                     drop_n=int(drop_n))
        self.min_bucket: Optional[int] = None

    def perform_kmer_counting(self, read_data) -> None:
        """Count every k-mer window of the FASTA buffer (device), table stays resident."""
        self.job.count(read_data, self.params)
        self.job.table_info()  # surfaces format errors now, as the reference's assert would

    @property
    def kmer_proc_buf(self) -> np.ndarray:
        """Sorted unique (k-mer, count) table as packed KmerPairs records."""
        return self.job.table_packed()

    def construct_kmer_histogram(self) -> Tuple[np.ndarray, int]:
        cut, hist, kept = None, None, None
        try:
            cut, hist, kept = self.job.cutoff(self.params.num_buckets)
        finally:
            pass
        self.min_bucket = cut
        return hist, cut

    def begin_mnode_construction(self) -> MacroNodeTable:
        if self.min_bucket is None:
            self.construct_kmer_histogram()
        self.job.build_macro_nodes(0)
        return self.job.macro_nodes(self.params.coverage)

    def close(self):
        self.job.close()


@dataclass
class RequestInfo:
    """State of one served request (times are CLOCK_MONOTONIC nanoseconds)."""
    ticket: int
    status: int
    done: bool
    summary: Summary
    submit_ns: int
    start_ns: int
    end_ns: int
    attempts: int

    @property
    def latency_ms(self) -> float:
        return (self.end_ns - self.submit_ns) / 1e6

    @property
    def queue_ms(self) -> float:
        return (self.start_ns - self.submit_ns) / 1e6


class Server:
    """Serving front end over ``pk_submit`` / ``pk_poll``: independent read sets run
    by ``workers`` job slots with continuous batching and HBM-budget admission (the
    context's budget).  Each request's result equals that of the same read set run
    alone in a :class:`Job`."""

    def __init__(self, ctx: Context, workers: int = 2, small_bytes: Optional[int] = None,
                 reserved_small: Optional[int] = None, aging_ms: Optional[int] = None,
                 small_sms: int = 0):
        """`small_bytes`, `reserved_small`, `aging_ms`: the scheduling knobs of
        pk_server_config (None: the library's defaults for this many workers);
        `small_sms` > 0: SMs set aside for small requests (an SM partition)."""
        self.ctx = ctx
        cfg = capi.PkServerConfig()
        capi.lib().pk_server_config_default(byref(cfg), workers)
        if small_bytes is not None:
            cfg.small_bytes = small_bytes
        if reserved_small is not None:
            cfg.reserved_small = reserved_small
        if aging_ms is not None:
            cfg.aging_ms = aging_ms
        cfg.small_sms = small_sms
        h = c_void_p()
        check(capi.lib().pk_server_create_config(ctx.handle, workers, byref(cfg), byref(h)),
              "pk_server_create_config")
        self._h = h
        self._live: Dict[int, tuple] = {}  # ticket -> (input buffer, out arrays, params)

    def partition(self) -> tuple:
        """(SMs of small requests, SMs of the others): the SM partition, or the whole
        device's count twice."""
        a, b = c_int32(), c_int32()
        check(capi.lib().pk_server_partition(self._h, byref(a), byref(b)), "pk_server_partition")
        return a.value, b.value

    def submit(self, fasta, params: capi.PkParams, out=None, keep_on_device: bool = False) -> int:
        """Queue one read set.  `fasta` stays referenced until :meth:`release`.  `out` =
        (keys, suffix, prefix) host arrays receiving the macro-node table (pinned memory
        copies fastest); without it the server keeps the table for :meth:`result`, or,
        with `keep_on_device`, keeps the whole job resident for :meth:`job`."""
        buf = _as_bytes_ptr(fasta)
        r = capi.PkRequest()
        r.fasta = buf[0]
        r.fasta_bytes = buf[1]
        r.params = params
        r.keep_on_device = int(keep_on_device)
        if out is not None:
            keys, suf, pre = out
            r.mn_keys = keys.ctypes.data
            r.mn_suffix = suf.ctypes.data
            r.mn_prefix = pre.ctypes.data
            r.mn_capacity = min(keys.shape[0], suf.shape[0], pre.shape[0])
        t = c_uint64()
        check(capi.lib().pk_submit(self._h, byref(r), byref(t)), "pk_submit")
        self._live[t.value] = (fasta, buf, out, params)
        return t.value

    @staticmethod
    def _info(ticket: int, i: capi.PkRequestInfo) -> RequestInfo:
        return RequestInfo(ticket, i.status, bool(i.done), Summary.from_c(i.summary), i.submit_ns,
                           i.start_ns, i.end_ns, i.attempts)

    def poll(self, ticket: int) -> RequestInfo:
        i = capi.PkRequestInfo()
        check(capi.lib().pk_poll(self._h, ticket, byref(i)), "pk_poll")
        return self._info(ticket, i)

    def wait(self, ticket: int, timeout: Optional[float] = None) -> RequestInfo:
        """Block until the request is done; raises the job's error if it failed."""
        i = capi.PkRequestInfo()
        ms = -1 if timeout is None else int(timeout * 1000)
        check(capi.lib().pk_wait(self._h, ticket, ms, byref(i)), "pk_wait")
        check(i.status, "request")
        return self._info(ticket, i)

    def result(self, ticket: int, coverage: Optional[int] = None) -> MacroNodeTable:
        """The macro-node table of a finished request (copied out of the server)."""
        info = self.wait(ticket)
        fasta, buf, out, params = self._live[ticket]
        m = info.summary.n_nodes
        cov = coverage if coverage is not None else params.coverage
        if out is not None:
            keys, suf, pre = out
            return MacroNodeTable(keys[:m], suf[:m], pre[:m], cov, params.k)
        kp, sp, pp, n = c_void_p(), c_void_p(), c_void_p(), c_uint64()
        check(capi.lib().pk_result_get(self._h, ticket, byref(kp), byref(sp), byref(pp), byref(n)),
              "pk_result_get")
        W = 8 if params.k <= 32 else 16
        keys = np.frombuffer((ctypes.c_char * (W * m)).from_address(kp.value), np.uint8).copy() \
            if m else np.empty(0, np.uint8)
        suf = np.frombuffer((ctypes.c_char * (16 * m)).from_address(sp.value), np.uint32).copy() \
            if m else np.empty(0, np.uint32)
        pre = np.frombuffer((ctypes.c_char * (16 * m)).from_address(pp.value), np.uint32).copy() \
            if m else np.empty(0, np.uint32)
        return MacroNodeTable(keys.view(key_dtype(params.k)), suf.reshape(m, 4), pre.reshape(m, 4), cov,
                              params.k)

    def next_done(self, timeout: Optional[float] = None) -> RequestInfo:
        """The next request to finish, in completion order (pk_next_done); its own
        status is in the returned info (not raised)."""
        t = c_uint64()
        i = capi.PkRequestInfo()
        ms = -1 if timeout is None else int(timeout * 1000)
        check(capi.lib().pk_next_done(self._h, ms, byref(t), byref(i)), "pk_next_done")
        return self._info(t.value, i)

    def cancel(self, ticket: int):
        """Cancel a queued or running request (pk_cancel)."""
        check(capi.lib().pk_cancel(self._h, ticket), "pk_cancel")

    def job(self, ticket: int) -> "Job":
        """The resident job of a finished keep_on_device request: its table and
        macro-nodes stay in HBM for further calls (table, wire, compact, walk ...) until
        :meth:`release`; the server owns it."""
        h = c_void_p()
        check(capi.lib().pk_result_job(self._h, ticket, byref(h)), "pk_result_job")
        j = Job(self.ctx, _borrowed=h)
        j.params = self._live[ticket][3]
        return j

    def release(self, ticket: int):
        check(capi.lib().pk_result_release(self._h, ticket), "pk_result_release")
        self._live.pop(ticket, None)

    def stats(self) -> Dict[str, int]:
        s = capi.PkServerStats()
        check(capi.lib().pk_server_get_stats(self._h, byref(s)), "pk_server_get_stats")
        return {n: getattr(s, n) for n, _ in capi.PkServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().pk_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class BatchResult:
    """One set of a batch: its status (0 = ok), summary and its rows of the batch's
    macro-node table; `rerun` is True when it ran again outside the graph."""
    status: int
    rerun: bool
    summary: Summary
    mn_first: int


class Batch:
    """Many independent read sets in one CUDA-graph launch (``pk_batch_run``).  The
    graph is captured on the first run of a batch shape and replayed while the shape
    stays the same; partition digits are autotuned per size class."""

    def __init__(self, ctx: Context, branches: int = 4, input_in_graph: bool = True):
        """`input_in_graph`: when every set is in page-locked host memory the graph copies
        each set itself, overlapping the other branches' work (pk_batch_set_input_mode)."""
        self.ctx = ctx
        h = c_void_p()
        check(capi.lib().pk_batch_create(ctx.handle, branches, byref(h)), "pk_batch_create")
        self._h = h
        self._keep = None
        self._k = 32
        self.set_input_in_graph(input_in_graph)

    def set_input_in_graph(self, on: bool):
        mode = capi.PK_BATCH_INPUT_IN_GRAPH if on else capi.PK_BATCH_INPUT_BEFORE
        check(capi.lib().pk_batch_set_input_mode(self._h, mode), "pk_batch_set_input_mode")

    def run(self, sets) -> list:
        """`sets`: sequence of (fasta, params).  Returns one BatchResult per set."""
        n = len(sets)
        arr = (capi.PkBatchSet * max(1, n))()
        keep = []
        for i, (fasta, params) in enumerate(sets):
            buf = _as_bytes_ptr(fasta)
            keep.append((fasta, buf))
            arr[i].fasta = buf[0]
            arr[i].fasta_bytes = buf[1]
            arr[i].params = params
            self._k = params.k
        res = (capi.PkBatchResult * max(1, n))()
        check(capi.lib().pk_batch_run(self._h, arr, n, res), "pk_batch_run")
        self._keep = keep
        return [BatchResult(r.status, bool(r.rerun), Summary.from_c(r.summary), r.mn_first) for r in res[:n]]

    def table(self, out=None):
        """(keys, suffix, prefix) of the last run, every set's rows at its mn_first."""
        m = self.stats()["total_nodes"]
        if out is None:
            keys = np.empty(m, key_dtype(self._k))
            suf = np.empty((m, 4), np.uint32)
            pre = np.empty((m, 4), np.uint32)
        else:
            keys, suf, pre = out
        check(capi.lib().pk_batch_copy_macro_nodes(self._h, keys.ctypes.data, suf.ctypes.data,
                                                   pre.ctypes.data, min(keys.shape[0], suf.shape[0],
                                                                        pre.shape[0])),
              "pk_batch_copy_macro_nodes")
        return keys[:m], suf[:m], pre[:m]

    def macro_nodes(self, result: BatchResult, table, coverage: int) -> MacroNodeTable:
        keys, suf, pre = table
        a, m = result.mn_first, result.summary.n_nodes
        return MacroNodeTable(keys[a:a + m], suf[a:a + m], pre[a:a + m], coverage, self._k)

    def stats(self) -> Dict[str, float]:
        s = capi.PkBatchStats()
        check(capi.lib().pk_batch_get_stats(self._h, byref(s)), "pk_batch_get_stats")
        return {n: getattr(s, n) for n, _ in capi.PkBatchStats._fields_}

    def tuned_bits(self, fasta_bytes: int, k: int) -> int:
        return int(capi.lib().pk_batch_tuned_bits(self._h, fasta_bytes, k))

    def tuned_shape(self, fasta_bytes: int, k: int) -> Tuple[int, int, int]:
        """(partition digits, chunk multiple, table CTAs per SM) tuned for this size class."""
        d, c, t = c_int32(), c_int32(), c_int32()
        check(capi.lib().pk_batch_tuned_shape(self._h, fasta_bytes, k, byref(d), byref(c), byref(t)),
              "pk_batch_tuned_shape")
        return d.value, c.value, t.value

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().pk_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
