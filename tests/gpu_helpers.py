"""Shared helpers for the GPU tests: run the device path through the C ABI and
compare with the oracle or the golden fixtures."""
import os

import numpy as np

import pakman_plus_gb300 as pk
from pakman_plus_gb300 import build as pkbuild

_ctx = None


def ctx():
    global _ctx
    if _ctx is None:
        pkbuild.build()
        _ctx = pk.Context(0)
    return _ctx


def run_gpu(fasta: bytes, k: int, t: int = 21, coverage: int = 1, drop_n: bool = False,
            bucket_bits: int = 0, lmer: int = 8):
    """Whole path on the GPU.  Returns (summary, keys128, counts, hist, mn or None, err)."""
    p = pk.default_params(k=k, num_buckets=t, coverage=coverage, drop_n=int(drop_n),
                          bucket_bits=bucket_bits, lmer_length=lmer)
    with pk.Job(ctx()) as job:
        job.count(fasta, p)
        keys, counts = job.table()
        try:
            cut, hist, kept = job.cutoff(t)
        except pk.EmptyAfterCutoff:
            return job.summary(), pk.to_key128(keys), counts, None, None, "empty_after_cutoff"
        job.build_macro_nodes(0)
        mn = job.macro_nodes(coverage)
        s = job.summary()
        return s, pk.to_key128(keys), counts, hist, mn, None


def assert_table_equal(keys, counts, ref_keys, ref_counts):
    assert keys.size == ref_keys.size, (keys.size, ref_keys.size)
    assert np.array_equal(keys["lo"], ref_keys["lo"])
    assert np.array_equal(keys["hi"], ref_keys["hi"])
    assert np.array_equal(counts.astype(np.uint64), ref_counts.astype(np.uint64))


def assert_mn_equal(mn, ref_keys, ref_suf, ref_pre):
    k128 = pk.to_key128(mn.keys)
    assert k128.size == ref_keys.size, (k128.size, ref_keys.size)
    assert np.array_equal(k128["lo"], ref_keys["lo"])
    assert np.array_equal(k128["hi"], ref_keys["hi"])
    assert np.array_equal(mn.suffix_counts, ref_suf)
    assert np.array_equal(mn.prefix_counts, ref_pre)
