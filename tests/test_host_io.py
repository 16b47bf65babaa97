"""Host-side parts of librvgpu that need no GPU: BAM/BGZF decoding (the
project's own DEFLATE decoder), FASTA loading, and the exported C ABI."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bam_roundtrip(tmp_path, germline_small):
    from rabbitvar_gb300 import api, synth
    g, vs, rs = germline_small
    bam = str(tmp_path / "s.bam")
    synth.write_bam(bam, rs)
    names, lens, batches = api.read_bam(bam, threads=2)
    assert names == [rs.contig] and lens == [rs.contig_len]
    b = batches[0].arrays
    ref = api.Batch.from_readset(rs).arrays
    for k in ("pos", "flag", "mapq", "mpos", "nm", "n_cigar", "cig_off", "cigar", "l_qseq", "base_off"):
        assert np.array_equal(b[k], ref[k]), k
    for i in range(0, rs.n, 97):
        o, L = int(rs.base_off[i]), int(rs.l_qseq[i])
        assert np.array_equal(b["qual"][o:o + L], ref["qual"][o:o + L])
        assert np.array_equal(b["seq"][o // 2:o // 2 + (L + 1) // 2], ref["seq"][o // 2:o // 2 + (L + 1) // 2])


def test_bam_rejects_truncated(tmp_path, germline_small):
    import pytest
    from rabbitvar_gb300 import api, synth
    g, vs, rs = germline_small
    bam = str(tmp_path / "s.bam")
    synth.write_bam(bam, rs)
    data = open(bam, "rb").read()
    bad = str(tmp_path / "bad.bam")
    open(bad, "wb").write(data[: len(data) // 2])
    with pytest.raises(api.RvError) as e:
        api.read_bam(bad)
    assert e.value.status == -8


def test_fasta(tmp_path, germline_small):
    from rabbitvar_gb300 import api, synth
    g, vs, rs = germline_small
    fa = str(tmp_path / "r.fa")
    synth.write_fasta(fa, "ctg", g)
    assert api.read_fasta(fa) == synth.genome_str(g).encode()


def test_library_exports_every_declared_symbol():
    """librvgpu.so loads without a GPU and exports every function the public
    headers declare."""
    from rabbitvar_gb300 import api
    L = api.lib()
    declared = set()
    for h in ("rvgpu.h", "rvgpu_io.h", "rvgpu_mlp.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        declared |= set(re.findall(r"^(?:rv_status|void|const char|void \*|const char \*)\s*\**\s*(rv_[a-z_0-9]+)\s*\(",
                                   src, flags=re.M))
    assert len(declared) >= 20
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert set(api.EXPORTS) <= declared


def test_context_without_gpu_reports_cuda_error():
    """Creating a context on a host without a GPU returns an error status
    (never a silent CPU fallback)."""
    import pytest
    from rabbitvar_gb300 import api
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    with pytest.raises(api.RvError) as e:
        api.Context(api.default_params(local_realign=0))
    assert e.value.status == -2
