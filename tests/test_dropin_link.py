"""The link-level drop-in (pakman_plus_gb300/host/pakman_dropin.cpp) builds into the
reference's own pkmer driver in place of its counting, histogram and macro-node
objects, and the resulting program fails loudly (the reference's MPI_Abort(-99)) when
no GPU is present -- there is no CPU fallback.  Needs the reference sources, so it
runs where they are (it is skipped elsewhere)."""
import os
import subprocess

import pytest

from oracle import pk_oracle as po
from pakman_plus_gb300 import build as pkbuild

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(not os.path.isdir(po.REFERENCE_TREE), reason="reference sources not present")
def test_reference_driver_links_with_the_dropin(tmp_path):
    pkbuild.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "dropin", "K=32", f"REF={po.REFERENCE_TREE}", "-j8"],
                          stdout=subprocess.DEVNULL)
    exe = os.path.join(ROOT, "oracle", "_ref", "pkmer_dropin_k32")
    assert os.access(exe, os.X_OK)
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # the drop-in defines the reference's phase entry points; the reference's own
    # implementations are not linked in
    for fn in ("perform_kmer_counting(char const*, unsigned long)", "free_kmer_count_buffers()",
               "begin_mnode_construction("):
        assert fn in syms, fn
    assert "SortAndAggregate" not in syms and "construct_macro_nodes" not in syms
    fa = tmp_path / "in.fa"
    fa.write_bytes(b">r0\n" + b"ACGT" * 25 + b"\n")
    r = subprocess.run([exe, "-f", str(fa), "-r", "100", "-c", "10"], capture_output=True, text=True,
                       timeout=120)
    import torch
    if not torch.cuda.is_available():
        assert r.returncode == 157, (r.returncode, r.stderr)
        assert "[pakman-gb300] pk_ctx_create" in r.stderr
    else:
        assert r.returncode == 0, (r.returncode, r.stderr)


@pytest.mark.skipif(not os.path.isdir(po.REFERENCE_TREE), reason="reference sources not present")
def test_contig_generation_driver_links_with_the_dropin(tmp_path):
    """The reference's driver in its contig-generation build (PERFORM_CONTIG_GENERATION,
    COMPACT_PGRAGH) links with the drop-in in place of its wiring and compaction
    objects and keeps its own walk."""
    pkbuild.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "dropin_contigs", "K=32", f"REF={po.REFERENCE_TREE}",
                           "-j8"], stdout=subprocess.DEVNULL)
    exe = os.path.join(ROOT, "oracle", "_ref", "pkmer_dropin_contigs_k32")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for fn in ("initiate_mnode_wiring(", "begin_iterative_compaction(", "identify_begin_kmers(",
               "generate_compacted_pakgraph(", "traverse_pakgraph("):
        assert fn in syms, fn
    assert "generate_id_set" not in syms and "iterate_and_pack_mn" not in syms and "push_to_pred" not in syms
    fa = tmp_path / "in.fa"
    fa.write_bytes(b">r0\n" + b"ACGT" * 25 + b"\n")
    r = subprocess.run([exe, "-f", str(fa), "-r", "100", "-c", "10"], capture_output=True, text=True,
                       timeout=120, cwd=str(tmp_path))
    import torch
    if not torch.cuda.is_available():
        assert r.returncode == 157, (r.returncode, r.stderr)
        assert "[pakman-gb300] pk_ctx_create" in r.stderr
    else:
        # the reference's own walk wrote its contig files from the adapter's map
        assert r.returncode == 0, (r.returncode, r.stderr)
        assert (tmp_path / "contigs_out_r0.fa").exists()
