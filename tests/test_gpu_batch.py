"""Batching (pk_batch_run): many read sets in one CUDA-graph launch give, set by set,
exactly the results of the same sets run alone -- including sets that end without
macro-nodes, malformed sets and sets that overrun the graph's bounds and run again."""
import numpy as np
import pytest

import pakman_plus_gb300 as pk
from gpu_helpers import assert_mn_equal, ctx, run_gpu
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


def _sets(k=32, n=10, seed=700):
    out = []
    rng = np.random.default_rng(seed)
    for i in range(n):
        glen = int(rng.integers(2000, 60000))
        cov = int(rng.integers(10, 40))
        nreads = max(50, cov * glen // 100)
        lens = rng.integers(90, 151, nreads)
        rs = synth.small_case(seed + i, genome_len=glen, n_reads=nreads, read_len=lens, err=0.005, k=k,
                              coverage=cov)
        out.append((rs.fasta, pk.default_params(k=k, num_buckets=21, coverage=cov)))
    return out


def _check(batch, sets, results):
    table = batch.table()
    for (fasta, p), r in zip(sets, results):
        s, _, _, _, mn, err = run_gpu(fasta, p.k, p.num_buckets, p.coverage)
        if err == "empty_after_cutoff":
            assert r.status == pk.capi.PK_ERR_EMPTY
            assert (r.summary.n_unique, r.summary.cutoff) == (s.n_unique, s.cutoff)
            continue
        assert r.status == 0, r
        assert (r.summary.n_windows, r.summary.n_unique, r.summary.n_kept, r.summary.n_nodes,
                r.summary.cutoff) == (s.n_windows, s.n_unique, s.n_kept, s.n_nodes, s.cutoff)
        got = batch.macro_nodes(r, table, p.coverage)
        assert_mn_equal(got, pk.to_key128(mn.keys), mn.suffix_counts, mn.prefix_counts)


@pytest.mark.parametrize("k,branches", [(32, 4), (31, 1), (63, 3)])
def test_batch_matches_sets_run_alone_and_replays(k, branches):
    sets = _sets(k=k, n=9, seed=700 + k)
    with pk.Batch(ctx(), branches=branches) as b:
        res = b.run(sets)
        _check(b, sets, res)
        st = b.stats()
        assert st["graph_launches"] == 1 and st["graph_captures"] == 1
        assert st["kernels_per_launch"] >= 12 * len(sets)
        res2 = b.run(sets)  # same shape: the captured graph is replayed
        _check(b, sets, res2)
        st = b.stats()
        assert st["graph_launches"] == 2 and st["graph_captures"] == 1
        assert st["tuned_classes"] >= 1


def test_batch_statuses_and_reruns():
    sets = _sets(n=4, seed=900)
    bad = sets[0][0].replace(b"\n>r10\n", b"\nxr10\n", 1)
    assert bad != sets[0][0]
    few = synth.small_case(31, genome_len=2000, n_reads=60, read_len=100, err=0.01, k=32).fasta
    big_t1 = synth.small_case(32, genome_len=200000, n_reads=3000, read_len=100, err=0.02, k=32).fasta
    mixed = sets + [(bad, pk.default_params(k=32)),                      # malformed record
                    (few, pk.default_params(k=32, num_buckets=21)),      # nothing reaches the cutoff
                    (big_t1, pk.default_params(k=32, num_buckets=1))]    # keeps every k-mer: over the bound
    with pk.Batch(ctx(), branches=2) as b:
        res = b.run(mixed)
        assert res[len(sets)].status == pk.capi.PK_ERR_FORMAT
        assert res[len(sets) + 1].status == pk.capi.PK_ERR_EMPTY
        assert res[len(sets) + 2].rerun and res[len(sets) + 2].status == 0
        ok = [i for i in range(len(mixed)) if i != len(sets)]
        _check(b, [mixed[i] for i in ok], [res[i] for i in ok])


def test_batch_rejects_mixed_key_widths():
    s32 = _sets(k=32, n=1, seed=1)[0]
    s63 = _sets(k=63, n=1, seed=2)[0]
    with pk.Batch(ctx(), branches=2) as b:
        with pytest.raises(pk.PakmanError):
            b.run([s32, s63])


def _low_complexity(n_reads, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    kind = np.arange(n_reads) % 3
    mat = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, (n_reads, 150))].copy()
    mat[kind == 0] = np.resize(np.frombuffer(b"AC", np.uint8), 150)
    mat[kind == 1] = ord("A")
    err = rng.random((n_reads, 150)) < 0.01
    mat = np.where(err, np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, (n_reads, 150))], mat)
    return synth.matrix_to_fasta(mat.astype(np.uint8))


def test_batch_sets_with_giant_buckets():
    """Sets whose homopolymer and dinucleotide buckets hold 0.5M+ keys take the chunked
    giant-bucket path inside the captured graph, next to ordinary sets."""
    sets = _sets(n=3, seed=1200) + [(_low_complexity(36000, s), pk.default_params(k=32, num_buckets=21, coverage=10))
                                    for s in (7, 8)]
    with pk.Batch(ctx(), branches=2) as b:
        res = b.run(sets)
        _check(b, sets, res)


def test_batch_copies_pinned_inputs_inside_the_graph():
    """Inputs in page-locked host memory are copied by the graph itself (each set on its
    branch ahead of its kernels): the results equal the sets run alone, the same batch
    replays the graph, and other sets in other buffers recapture it."""
    torch = pytest.importorskip("torch")
    sets = _sets(n=6, seed=1300)
    other = _sets(n=6, seed=1400)

    def pin(fasta, size):
        t = torch.zeros(size, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:len(fasta)] = np.frombuffer(fasta, np.uint8)
        return t

    sizes = [max(len(a), len(c)) for (a, _), (c, _) in zip(sets, other)]
    bufs = [pin(f, sz) for (f, _), sz in zip(sets, sizes)]
    with pk.Batch(ctx(), branches=3) as b:
        res = b.run([(t.numpy()[:len(f)], p) for t, (f, p) in zip(bufs, sets)])
        _check(b, sets, res)
        res = b.run([(t.numpy()[:len(f)], p) for t, (f, p) in zip(bufs, sets)])  # replayed
        _check(b, sets, res)
        assert b.stats()["graph_captures"] == 1
        fresh = [pin(f, sz) for (f, _), sz in zip(other, sizes)]
        res = b.run([(t.numpy()[:len(f)], p) for t, (f, p) in zip(fresh, other)])
        _check(b, other, res)
        assert b.stats()["graph_captures"] == 2
