"""CPU restatement of PaKman's iterative compaction (TEST INFRASTRUCTURE ONLY).

The oracle for the device compaction: only tests, the smoke check and the bench's CPU
baseline call it.  It restates, on plain Python lists and byte strings of base codes
(A=0, C=1, T=2, G=3), the reference's phase 2 as one rank runs it:

  begin_iterative_compaction   src/iterative_compaction.cpp:131-464
  generate_id_set              src/merge_mn.cpp:289-432
  iterate_and_pack_mn          src/merge_mn.cpp:433-550 (check_for_self_loops :551-558)
  retrieve_mn_pinfo / _sinfo   src/walk.cpp:117-167 / :69-115
  push_to_pred / push_to_succ  src/merge_mn.cpp:1325-1365 / :1368-1411
  MacroNode::setup_wiring      includes/distribute_kmers.h:550-657 (Comp_rev :495-506)
  identify_begin_kmers         src/iterative_compaction.cpp:65-93
  walk / traverse_pakgraph     src/walk.cpp:268-399 / :401-533

A node is keyed by its (k-1)-mer; each prefix / suffix entry is [ext, count, visit,
terminal] where ext is the extension's bases in reading order.  The packed
BasePairVector helpers the reference uses (extract = first n bases, extract_succ =
last n bases, mnode_extract_pred / _succ = the bases after the first / before the
last k-1) are restated as the string operations they compute for k-1 >= 16.

The wiring ranks entries with std::sort (not a stable sort), so ties between equal
(visit, count) pairs fall where libstdc++'s introsort puts them; `_std_sort` restates
that published algorithm (16-element insertion-sort threshold, median-of-three
pivot, unguarded partition, heap sort past a depth of 2*floor(log2 n)).

Pinned against the reference's own compaction run here (oracle/ref/compact_harness.cpp,
`make -C oracle/ref compact`): from the reference's wired map, the oracle must
reproduce its map after compaction and its partial contigs exactly.
"""
from __future__ import annotations

import os
import subprocess
import tempfile
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

EXT, CNT, VIS, TERM, NBR = 0, 1, 2, 3, 4  # entry fields (NBR: cached neighbour key)

_HERE = os.path.dirname(os.path.abspath(__file__))


class CompactionError(RuntimeError):
    pass


# ----------------------------------------------------------------- std::sort ------
def _std_sort(a: list, less) -> None:
    """libstdc++ std::sort (introsort + final insertion sort) on list `a` in place."""
    n = len(a)
    if n < 2:
        return

    def lg(x):
        return x.bit_length() - 1

    def adjust_heap(first, hole, length, value):
        top = hole
        child = hole
        while child < (length - 1) // 2:
            child = 2 * (child + 1)
            if less(a[first + child], a[first + child - 1]):
                child -= 1
            a[first + hole] = a[first + child]
            hole = child
        if (length & 1) == 0 and child == (length - 2) // 2:
            child = 2 * (child + 1)
            a[first + hole] = a[first + child - 1]
            hole = child - 1
        parent = (hole - 1) // 2
        while hole > top and less(a[first + parent], value):
            a[first + hole] = a[first + parent]
            hole = parent
            parent = (hole - 1) // 2
        a[first + hole] = value

    def heap_sort(first, last):
        length = last - first
        if length >= 2:
            parent = (length - 2) // 2
            while True:
                adjust_heap(first, parent, length, a[first + parent])
                if parent == 0:
                    break
                parent -= 1
        while last - first > 1:
            last -= 1
            value = a[last]
            a[last] = a[first]
            adjust_heap(first, 0, last - first, value)

    def move_median_to_first(res, x, y, z):
        if less(a[x], a[y]):
            if less(a[y], a[z]):
                a[res], a[y] = a[y], a[res]
            elif less(a[x], a[z]):
                a[res], a[z] = a[z], a[res]
            else:
                a[res], a[x] = a[x], a[res]
        elif less(a[x], a[z]):
            a[res], a[x] = a[x], a[res]
        elif less(a[y], a[z]):
            a[res], a[z] = a[z], a[res]
        else:
            a[res], a[y] = a[y], a[res]

    def partition_pivot(first, last):
        mid = first + (last - first) // 2
        move_median_to_first(first, first + 1, mid, last - 1)
        lo, hi = first + 1, last
        while True:
            while less(a[lo], a[first]):
                lo += 1
            hi -= 1
            while less(a[first], a[hi]):
                hi -= 1
            if not lo < hi:
                return lo
            a[lo], a[hi] = a[hi], a[lo]
            lo += 1

    def introsort(first, last, depth):
        while last - first > 16:
            if depth == 0:
                heap_sort(first, last)
                return
            depth -= 1
            cut = partition_pivot(first, last)
            introsort(cut, last, depth)
            last = cut

    def linear_insert(i):
        v = a[i]
        j = i - 1
        while less(v, a[j]):
            a[j + 1] = a[j]
            j -= 1
        a[j + 1] = v

    def insertion_sort(first, last):
        for i in range(first + 1, last):
            if less(a[i], a[first]):
                v = a[i]
                a[first + 1:i + 1] = a[first:i]
                a[first] = v
            else:
                linear_insert(i)

    introsort(0, n, 2 * lg(n))
    if n > 16:
        insertion_sort(0, 16)
        for i in range(16, n):
            linear_insert(i)
    else:
        insertion_sort(0, n)


# ----------------------------------------------------------------- state ----------
@dataclass
class Node:
    key: int
    suf: list  # [[ext, count, visit, terminal, nbr], ...]
    pre: list
    wires: list = field(default_factory=list)  # [(suffix_id, offset_in_suffix, count)]
    begin: list = field(default_factory=list)  # [(prefix_pos, num_wires)] per prefix


def key_bases(key: int, n: int) -> bytes:
    return bytes((key >> (2 * (n - 1 - i))) & 3 for i in range(n))


def bases_key(b: bytes) -> int:
    v = 0
    for x in b:
        v = (v << 2) | x
    return v


def _pred_nbr(ext: bytes, kb: bytes, L: int) -> int:
    """generate_id_set's predecessor key (src/merge_mn.cpp:320-340): the first L bases
    of ext + key; 0 for an empty extension."""
    if not ext:
        return 0
    return bases_key((ext + kb)[:L])


def _succ_nbr(ext: bytes, kb: bytes, L: int) -> int:
    if not ext:
        return 0
    return bases_key((kb + ext)[-L:])


def _entry(ext: bytes, cnt: int, vis: int, term: bool, kb: bytes, L: int, pred: bool) -> list:
    nbr = 0 if term else (_pred_nbr(ext, kb, L) if pred else _succ_nbr(ext, kb, L))
    return [ext, cnt, vis, term, nbr]


def setup_wiring(nd: Node) -> None:
    """MacroNode::setup_wiring after wiring_info / prefix_begin_info were cleared and
    resized (src/iterative_compaction.cpp:416-429; includes/distribute_kmers.h:550-657)."""
    pre, suf = nd.pre, nd.suf
    nd.wires = [(0, 0, 0)] * (len(pre) + len(suf) + 1)
    nd.begin = [(0, 0)] * len(pre)
    sc = sum(e[VIS] for e in suf if e[EXT])
    pc = sum(e[VIS] for e in pre if e[EXT])
    ns_id = np_id = -1
    for i, e in enumerate(suf):
        if not e[EXT]:
            if not e[TERM] or ns_id != -1:
                raise CompactionError("an empty suffix must be the one terminal entry")
            ns_id = i
            if e[CNT] == -1:
                e[CNT], e[VIS] = 1, max(pc - sc, 0)
    for i, e in enumerate(pre):
        if not e[EXT]:
            if not e[TERM] or np_id != -1:
                raise CompactionError("an empty prefix must be the one terminal entry")
            np_id = i
            if e[CNT] == -1:
                e[CNT], e[VIS] = 1, max(sc - pc, 0)
    if ns_id < 0 or np_id < 0:
        raise CompactionError("a node lost its terminal entry")
    if sc + suf[ns_id][VIS] != pc + pre[np_id][VIS]:
        raise CompactionError("unbalanced visits at node %x" % nd.key)  # the reference asserts

    def rank(lst):
        idx = list(range(len(lst)))
        _std_sort(idx, lambda i, j: lst[i][VIS] > lst[j][VIS] or
                  (lst[i][VIS] == lst[j][VIS] and lst[i][CNT] > lst[j][CNT]))
        return idx

    ip, is_ = rank(pre), rank(suf)
    leftover = sc + suf[ns_id][VIS]
    off = [0] * len(suf)
    top_p = top_s = var_p = var_s = 0
    wi = p_size = 0
    last_pid = begin_pos = -1
    wires = list(nd.wires)
    begin = list(nd.begin)
    while leftover > 0:
        sid, pid = is_[top_s], ip[top_p]
        c = min(pre[pid][VIS] - var_p, suf[sid][VIS] - var_s)
        wires[wi] = (sid, off[sid], c)
        if last_pid != pid:
            begin_pos = wi
            last_pid = pid
        p_size += 1
        wi += 1
        leftover -= c
        var_p += c
        var_s += c
        off[sid] += c
        if var_p == pre[pid][VIS]:
            var_p = 0
            top_p += 1
            begin[pid] = (begin_pos, p_size)
            p_size = 0
        if var_s == suf[sid][VIS]:
            var_s = 0
            top_s += 1
    nd.wires, nd.begin = wires, begin


@dataclass
class Transfer:
    target: int
    search_ext: bytes
    mn_ext: bytes
    count: Tuple[int, int]
    terminal: bool
    to_pred: bool  # True: direction P (push_to_pred), False: S (push_to_succ)


def _pack(nodes: List[Node], ids: List[int], L: int, contigs: list) -> List[Transfer]:
    """iterate_and_pack_mn (src/merge_mn.cpp:433-550) for one rank."""
    out = []
    for i in ids:
        nd = nodes[i]
        kb = key_bases(nd.key, L)
        for p, (pos, num) in enumerate(nd.begin):
            if not num:
                continue
            P = nd.pre[p]
            pkey, pext = 0, b""
            if P[EXT] and not P[TERM]:  # retrieve_mn_pinfo (src/walk.cpp:117-167)
                w = P[EXT] + kb
                pkey, pext = bases_key(w[:L]), w[L:]
            for t in range(num):
                sid, _, cnt = nd.wires[pos + t]
                S = nd.suf[sid]
                if P[TERM] and S[TERM]:
                    contigs.append(P[EXT] + kb + S[EXT])
                    continue
                skey, sext = 0, b""
                if S[EXT] and not S[TERM]:  # retrieve_mn_sinfo (src/walk.cpp:69-115)
                    w = kb + S[EXT]
                    skey, sext = bases_key(w[-L:]), w[:-L]
                self_p = (not P[TERM]) and pkey == nd.key
                self_s = (not S[TERM]) and skey == nd.key
                c = (min(P[CNT], S[CNT]), cnt)
                if not P[TERM] and not self_p:
                    out.append(Transfer(pkey, pext, S[EXT], c, bool(S[TERM] or self_s), True))
                if not S[TERM] and not self_s:
                    out.append(Transfer(skey, sext, P[EXT], c, bool(P[TERM] or self_p), False))
    return out


def _push(nd: Node, tr: Transfer, L: int) -> None:
    """push_to_pred / push_to_succ (src/merge_mn.cpp:1325-1412)."""
    kb = key_bases(nd.key, L)
    if tr.to_pred:
        lst, new_ext, pred = nd.suf, tr.search_ext + tr.mn_ext, False
    else:
        lst, new_ext, pred = nd.pre, tr.mn_ext + tr.search_ext, True
    idx = -1
    for j, e in enumerate(lst):
        if e[EXT] == tr.search_ext:
            idx = j
            break
    ent = _entry(new_ext, tr.count[0], tr.count[1], tr.terminal, kb, L, pred)
    if idx < 0 or lst[idx][TERM]:
        lst.append(ent)
    else:
        lst[idx] = ent


def id_set(nodes: List[Node]) -> List[int]:
    """generate_id_set (src/merge_mn.cpp:289-432): nodes with no non-terminal neighbour
    key above their own."""
    out = []
    for i, nd in enumerate(nodes):
        k = nd.key
        if any(e[NBR] > k for e in nd.pre) or any(e[NBR] > k for e in nd.suf):
            continue
        out.append(i)
    return out


@dataclass
class Compacted:
    nodes: List[Node]
    contigs: List[bytes]
    rounds: int


def compact(nodes: List[Node], k: int, threshold: int, max_rounds: int = 1 << 30) -> Compacted:
    """begin_iterative_compaction (src/iterative_compaction.cpp:131-464): rounds of
    ID-set merging until at most `threshold` nodes remain.  `nodes` (sorted by key,
    wired) is consumed."""
    L = k - 1
    contigs: List[bytes] = []
    rounds = 0
    while len(nodes) > threshold and rounds < max_rounds:
        rounds += 1
        ids = id_set(nodes)
        trs = _pack(nodes, ids, L, contigs)
        gone = set(ids)
        nodes = [nd for i, nd in enumerate(nodes) if i not in gone]
        pos = {nd.key: i for i, nd in enumerate(nodes)}
        touched = set()
        for tr in trs:
            j = pos.get(tr.target)
            if j is None:
                raise CompactionError("transfer to a node that is not in the map")
            _push(nodes[j], tr, L)
            touched.add(j)
        for j in sorted(touched):
            setup_wiring(nodes[j])
    return Compacted(nodes, contigs, rounds)


# ----------------------------------------------------------------- walk -----------
WALK_MAX_BASES = 500000  # the reference asserts a partial contig stays below this (src/walk.cpp:285)


def begin_kmers(nodes: List[Node]) -> List[Tuple[int, int]]:
    """identify_begin_kmers (src/iterative_compaction.cpp:65-93): every terminal prefix
    with visits, in map order then prefix-list order."""
    return [(i, p) for i, nd in enumerate(nodes) for p, e in enumerate(nd.pre) if e[VIS] > 0 and e[TERM]]


def walk(nodes: List[Node], k: int) -> List[bytes]:
    """traverse_pakgraph on one thread (src/walk.cpp:401-533): from each begin k-mer,
    the depth-first `walk` (:268-399) over the wires of the prefix it entered by, each
    wire taking its share [offset, offset + frequency) of the prefix's visits; a
    terminal suffix ends a contig.  Contigs in begin order, then depth-first order (the
    reference's order with one thread)."""
    L = k - 1
    pos = {nd.key: i for i, nd in enumerate(nodes)}
    out: List[bytes] = []
    for bi, bp in begin_kmers(nodes):
        nd = nodes[bi]
        contig = bytearray(nd.pre[bp][EXT] + key_bases(nd.key, L))
        # frame: [node, prefix, offset_in_prefix, wire index, off, freq_remaining, child share, length]
        stack = [[bi, bp, 0, 0, 0, nd.pre[bp][VIS], None, len(contig)]]
        while stack:
            f = stack[-1]
            cur = nodes[f[0]]
            bpos, num = cur.begin[f[1]]
            if f[6] is not None:  # back from the child walk
                f[5] -= f[6]
                f[6] = None
                del contig[f[7]:]
                f[4] += cur.wires[bpos + f[3]][2]
                f[3] += 1
                continue
            if f[3] >= num:
                stack.pop()
                continue
            sid, off_in_suffix, sz = cur.wires[bpos + f[3]]
            off, oip, rem = f[4], f[2], f[5]
            if off + sz <= oip or off > oip + rem:
                f[4] += sz
                f[3] += 1
                continue
            off_in_wire = 0 if oip <= off else oip - off
            next_off = off_in_suffix + off_in_wire
            share = min(rem, sz - off_in_wire)
            S = cur.suf[sid]
            f[7] = len(contig)
            contig += S[EXT]
            if S[TERM]:
                out.append(bytes(contig))
                f[5] -= share
                del contig[f[7]:]
                f[4] += sz
                f[3] += 1
                continue
            nxt_i = pos.get(S[NBR])
            if nxt_i is None:
                raise CompactionError("walk: successor node not in the map")
            nxt = nodes[nxt_i]
            search = (key_bases(cur.key, L) + S[EXT])[:len(S[EXT])]
            q = next((j for j, e in enumerate(nxt.pre) if e[EXT] == search), -1)
            if q < 0:  # the reference prints "prefix not found" and exits
                raise CompactionError("walk: no prefix of the successor matches")
            if share <= 0:  # the reference asserts freq_in_wire > 0
                raise CompactionError("walk: empty share of a wire")
            if len(contig) >= WALK_MAX_BASES:
                raise CompactionError("walk: a contig reached 500000 bases")
            f[6] = share
            stack.append([nxt_i, q, next_off, 0, 0, share, None, len(contig)])
    return out


def read_fasta_contigs(data: bytes) -> List[bytes]:
    """Sequences of a contigs_*.fa file as base codes (A=0, C=1, T=2, G=3)."""
    code = {ord("A"): 0, ord("C"): 1, ord("T"): 2, ord("G"): 3}
    return [bytes(code[c] for c in line) for line in data.split(b"\n") if line and not line.startswith(b">")]


# ----------------------------------------------------------------- C restatement --
class _CResult(__import__("ctypes").Structure):
    import ctypes as _c
    _fields_ = [("rounds", _c.c_uint64), ("n_nodes", _c.c_uint64), ("n_contigs", _c.c_uint64),
                ("walk_contigs", _c.c_uint64), ("walk_bases", _c.c_uint64), ("contig_bases", _c.c_uint64),
                ("hash", _c.c_uint64)]


def compact_walk_c(keys, suf, pre, k: int, coverage: int, threshold: int) -> _CResult:
    """The same compaction and walk in C (oracle/pk_compact.c); the result carries
    counts and a hash of everything (`result_hash`)."""
    import ctypes

    import numpy as np

    from oracle import pk_oracle as po
    L = po.lib()
    fn = L.pko_compact_walk
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                   ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_CResult)]
    m = len(keys)
    kw = np.zeros((max(1, m), 2), np.uint64)
    if m:
        if getattr(keys, "dtype", None) is not None and keys.dtype.names:
            kw[:m, 0] = keys["lo"]
            kw[:m, 1] = keys["hi"]
        else:
            kw[:m, 0] = np.asarray(keys, np.uint64)
    s = np.ascontiguousarray(suf, np.uint32).reshape(-1)
    p = np.ascontiguousarray(pre, np.uint32).reshape(-1)
    out = _CResult()
    rc = fn(kw.ctypes.data, s.ctypes.data, p.ctypes.data, m, k, coverage, threshold, ctypes.byref(out))
    if rc != 0:
        raise CompactionError("pko_compact_walk failed with %d" % rc)
    return out


def result_hash(nodes: List[Node], contigs: List[bytes], walk_contigs: List[bytes]) -> int:
    """FNV-1a 64 of a map, its partial contigs and its walk contigs, serialised the way
    oracle/pk_compact.c hashes them."""
    import struct
    M = (1 << 64) - 1

    def fnv(h, b):
        for x in b:
            h = ((h ^ x) * 1099511628211) & M
        return h

    h = 1469598103934665603
    for key, suf, pre, wires, begin in state_view(nodes):
        h = fnv(h, struct.pack("<QQ", key & M, key >> 64))
        for lst in (suf, pre):
            h = fnv(h, struct.pack("<I", len(lst)))
            for ext, c, v, t in lst:
                h = fnv(h, struct.pack("<I", len(ext)) + ext + struct.pack("<iiB", c, v, int(t)))
        h = fnv(h, struct.pack("<I", len(wires)) + b"".join(struct.pack("<iii", *w) for w in wires))
        h = fnv(h, struct.pack("<I", len(begin)) + b"".join(struct.pack("<ii", *b) for b in begin))
    h = fnv(h, struct.pack("<Q", len(contigs)))
    for c in contigs:
        h = fnv(h, struct.pack("<I", len(c)) + c)
    hw = 1469598103934665603
    for c in walk_contigs:
        hw = fnv(hw, struct.pack("<I", len(c)) + c)
    return fnv(fnv(h, struct.pack("<Q", len(walk_contigs))), struct.pack("<Q", hw))


# ----------------------------------------------------------------- construction ---
def initial_nodes(keys, suf, pre, k: int, coverage: int) -> List[Node]:
    """The wired map the reference hands to compaction, lists in canonical order:
    present one-base extensions in ascending base code, then the terminal entry
    (count -1 until wired), then MacroNode::setup_wiring on every node
    (src/wire.cpp:66-121).  keys: ints or a (lo, hi) structured array; suf / pre:
    (M, 4) k-mer counts per extension base."""
    from oracle import pk_oracle as po
    L = k - 1
    out = []
    for i in range(len(keys)):
        kv = keys[i]
        key = int(kv) if not hasattr(kv, "dtype") or kv.dtype.names is None else \
            int(kv["lo"]) | (int(kv["hi"]) << 64)
        kb = key_bases(key, L)
        s = [_entry(bytes([b]), int(c), po.visit(int(c), coverage), False, kb, L, False)
             for b, c in enumerate(suf[i]) if c]
        p = [_entry(bytes([b]), int(c), po.visit(int(c), coverage), False, kb, L, True)
             for b, c in enumerate(pre[i]) if c]
        s.append([b"", -1, -1, True, 0])
        p.append([b"", -1, -1, True, 0])
        nd = Node(key, s, p)
        setup_wiring(nd)
        out.append(nd)
    return out


# ----------------------------------------------------------------- dumps ----------
def read_state(path: str) -> Tuple[int, List[Node]]:
    """A "PKC1" map dump file of oracle/ref/compact_harness.cpp."""
    with open(path, "rb") as f:
        return parse_state(f.read())


def parse_state(data: bytes) -> Tuple[int, List[Node]]:
    """(k, nodes) of a "PKC1" map dump."""
    import struct
    if data[:4] != b"PKC1":
        raise CompactionError("not a PKC1 dump")
    k, m = struct.unpack_from("<IQ", data, 4)
    L = k - 1
    off = 16
    nodes = []
    for _ in range(m):
        lo, hi = struct.unpack_from("<QQ", data, off)
        off += 16
        key = lo | (hi << 64)
        kb = key_bases(key, L)
        lists = []
        for side in range(2):
            (n,) = struct.unpack_from("<I", data, off)
            off += 4
            lst = []
            for _ in range(n):
                (ln,) = struct.unpack_from("<I", data, off)
                off += 4
                ext = bytes(data[off:off + ln])
                off += ln
                c, v, t = struct.unpack_from("<iiB", data, off)
                off += 9
                lst.append(_entry(ext, c, v, bool(t), kb, L, side == 1))
            lists.append(lst)
        (nw,) = struct.unpack_from("<I", data, off)
        off += 4
        wires = [struct.unpack_from("<iii", data, off + 12 * j) for j in range(nw)]
        off += 12 * nw
        (nb,) = struct.unpack_from("<I", data, off)
        off += 4
        begin = [struct.unpack_from("<ii", data, off + 8 * j) for j in range(nb)]
        off += 8 * nb
        nodes.append(Node(key, lists[0], lists[1], [tuple(w) for w in wires], [tuple(b) for b in begin]))
    return k, nodes


def read_contigs(path: str) -> List[bytes]:
    with open(path, "rb") as f:
        return parse_contigs(f.read())


def parse_contigs(data: bytes) -> List[bytes]:
    """The partial contigs of a "PKP1" dump."""
    import struct
    if data[:4] != b"PKP1":
        raise CompactionError("not a PKP1 dump")
    (n,) = struct.unpack_from("<Q", data, 4)
    off = 12
    out = []
    for _ in range(n):
        (ln,) = struct.unpack_from("<I", data, off)
        off += 4
        out.append(bytes(data[off:off + ln]))
        off += ln
    return out


def state_view(nodes: List[Node]):
    """Comparable form of a map: per node (key, suffixes, prefixes, wires, begin) with
    entries as (ext, count, visit, terminal)."""
    return [(nd.key, [tuple(e[:4]) for e in nd.suf], [tuple(e[:4]) for e in nd.pre],
             [tuple(w) for w in nd.wires], [tuple(b) for b in nd.begin]) for nd in nodes]


def build_compact_reference(k: int) -> Optional[str]:
    """oracle/_ref/pakman_compact_k<k>, built from the reference sources in place; None
    when the reference tree is absent."""
    from oracle.pk_oracle import REFERENCE_TREE
    exe = os.path.join(_HERE, "_ref", "pakman_compact_k%d" % k)
    if not os.path.isdir(REFERENCE_TREE):
        return exe if os.path.exists(exe) else None
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref"), "compact", "K=%d" % k, "REF=" + REFERENCE_TREE],
                   check=True, stdout=subprocess.DEVNULL)
    return exe


@dataclass
class RefCompaction:
    k: int
    before: List[Node]
    after: List[Node]
    contigs: List[bytes]
    secs: float
    raw: dict  # the dump files' bytes: "before", "after", "contigs"


def run_reference(fasta: bytes, k: int, read_len: int, coverage: int, threshold: int,
                  t: int = 21, walk: bool = False) -> Optional[RefCompaction]:
    """The reference's compaction on `fasta` (one rank, one thread); None if it cannot
    be built here.  walk=True also runs its walk: raw["walk_fa"] / raw["partial_fa"] hold
    the contigs_out_r0.fa / contigs_par_r0.fa it writes (contigs longer than 400)."""
    import json
    exe = build_compact_reference(k)
    if exe is None or not os.path.exists(exe):
        return None
    with tempfile.TemporaryDirectory() as d:
        fa = os.path.join(d, "in.fa")
        with open(fa, "wb") as f:
            f.write(fasta)
        out = os.path.join(d, "out")
        p = subprocess.run([exe, out, "-f", fa, "-r", str(read_len), "-c", str(coverage), "-t", str(t),
                            "-n", str(threshold)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, cwd=d,
                           env=dict(os.environ, OMP_NUM_THREADS="1", PK_REF_WALK="1" if walk else "0"))
        if p.returncode != 0:
            raise CompactionError("reference compaction failed: " + p.stdout.decode(errors="replace")[-400:])
        line = [x for x in p.stdout.decode().splitlines() if x.startswith("{")][-1]
        raw = {}
        for part in ("before", "after", "contigs"):
            with open(out + "." + part, "rb") as f:
                raw[part] = f.read()
        if walk:
            for key, name in (("walk_fa", "contigs_out_r0.fa"), ("partial_fa", "contigs_par_r0.fa")):
                with open(os.path.join(d, name), "rb") as f:
                    raw[key] = f.read()
        kk, before = parse_state(raw["before"])
        _, after = parse_state(raw["after"])
        return RefCompaction(kk, before, after, parse_contigs(raw["contigs"]), json.loads(line)["compact_s"], raw)
