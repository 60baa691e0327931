"""Initial wiring on the GPU (pk_wire_macro_nodes) against the wiring restatement and,
through the fixtures, the reference's own initiate_mnode_wiring (src/wire.cpp)."""
import numpy as np
import pytest

import pakman_plus_gb300 as pk
from golden_cases import load, names
from gpu_helpers import ctx
from oracle import pk_oracle as po
from pakman_plus_gb300 import synth

pytestmark = pytest.mark.gpu


def _wire_gpu(fasta, k, t, cov, drop_n=False):
    with pk.Job(ctx()) as job:
        p = pk.default_params(k=k, num_buckets=t, coverage=cov, drop_n=int(drop_n))
        job.run(fasta, p)
        mn = job.macro_nodes(cov)
        return mn, job.wire()


def _assert_same(a, b):
    for f in ("ns", "np", "term_suf", "term_pre", "nw", "wire", "begin"):
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("name", [n for n in names() if load(n).expect == "ok"])
def test_wiring_matches_restatement_on_fixtures(name):
    g = load(name)
    mn, w = _wire_gpu(g.fasta, g.k, g.t, g.coverage, g.drop_n)
    ref = po.wire(g.mn_suf, g.mn_pre, g.coverage)
    _assert_same(w, ref)
    # nodes whose reference lists are in canonical order: the reference's wiring itself
    for i in range(w.size):
        sext = [e for e in g.wiring["w_sext"][i] if e >= 0]
        pext = [e for e in g.wiring["w_pext"][i] if e >= 0]
        if sext == sorted(e for e in sext if e != 4) + [4] and pext == sorted(e for e in pext if e != 4) + [4]:
            assert np.array_equal(w[i]["wire"], g.wiring["w_wire"][i])
            assert np.array_equal(w[i]["begin"], g.wiring["w_begin"][i])


@pytest.mark.parametrize("cov", [1, 7, 30])
def test_wiring_on_a_larger_set(cov):
    rs = synth.small_case(4444, genome_len=50000, n_reads=20000, read_len=120, err=0.01, k=31)
    mn, w = _wire_gpu(rs.fasta, 31, 21, cov)
    _assert_same(w, po.wire(mn.suffix_counts, mn.prefix_counts, cov))
    # flow conservation: the wires carry every suffix visit
    assert np.all(w["nw"] >= 1)


def test_wiring_requires_macro_nodes():
    with pk.Job(ctx()) as job:
        with pytest.raises(pk.PakmanError):
            job.wire()
