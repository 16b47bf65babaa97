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


def test_bam_read_mem_matches_file_decoder(tmp_path, germline_small):
    """rv_bam_read_mem (bytes already in memory) decodes the same records as
    rv_bam_read; bam_bytes' numpy records match a field-by-field rebuild."""
    import ctypes as C
    import struct
    from rabbitvar_gb300 import api, synth
    g, vs, rs = germline_small
    bam = str(tmp_path / "s.bam")
    synth.write_bam(bam, rs)
    data = open(bam, "rb").read()
    L = api.lib()
    h = C.c_void_p()
    buf = C.create_string_buffer(data, len(data))
    assert L.rv_bam_read_mem(C.cast(buf, C.c_void_p), len(data), 2, C.byref(h)) == 0
    try:
        got = api._host_batches(L, h, L.rv_bam_batch)
    finally:
        L.rv_bam_free(h)
    want = api.read_bam(bam, threads=2)
    assert got[0] == want[0] and got[1] == want[1]
    for k in ("pos", "flag", "mapq", "mpos", "nm", "n_cigar", "cig_off", "cigar", "l_qseq", "base_off"):
        assert np.array_equal(got[2][0].arrays[k], want[2][0].arrays[k]), k
    # first record rebuilt field by field
    stream = synth.bam_bytes(rs, "S")
    q = 8 + struct.unpack("<I", stream[4:8])[0]        # magic, l_text, text
    q += 4 + 4 + len(rs.contig) + 1 + 4                 # n_ref, l_name, name, l_ref
    bs = struct.unpack("<I", stream[q:q + 4])[0]
    tid, pos, lrn, mapq, _bin, nc, flag, lq, ntid, npos, tlen = struct.unpack("<iiBBHHHiiii", stream[q + 4:q + 36])
    assert (tid, pos, mapq, nc, flag, lq, npos, tlen) == (0, int(rs.pos[0]), int(rs.mapq[0]), int(rs.n_cigar[0]),
                                                          int(rs.flag[0]), int(rs.l_qseq[0]), int(rs.mpos[0]),
                                                          int(rs.isize[0]))
    assert stream[q + 36:q + 36 + lrn] == b"r%d\x00" % int(rs.name_id[0])
    assert bs == 32 + lrn + 4 * nc + (lq + 1) // 2 + lq + 7


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


def test_bam_roundtrip_hand_written_reads(tmp_path):
    """Reads of uneven length with hard clips, soft clips, insertions,
    deletions, N bases, flags 0x4/0x100/0x400/0x800 and a one-base read (the
    golden path cases) decode to the same fields, CIGARs, bases and
    qualities, read by read."""
    import importlib.util
    from rabbitvar_gb300 import api, synth
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    for make in (mg._path_reads, mg._cigar_rule_reads):
        g, rs = make()
        if make is mg._path_reads:
            assert len(set(rs.l_qseq.tolist())) > 3
        bam = str(tmp_path / "p.bam")
        synth.write_bam(bam, rs)
        _, _, batches = api.read_bam(bam, threads=2)
        b = batches[0].arrays
        ref = api.Batch.from_readset(rs).arrays
        for k in ("pos", "flag", "mapq", "mpos", "nm", "n_cigar", "l_qseq"):
            assert np.array_equal(b[k], ref[k]), k
        for i in range(rs.n):
            c0, c1, n = int(b["cig_off"][i]), int(ref["cig_off"][i]), int(rs.n_cigar[i])
            assert np.array_equal(b["cigar"][c0:c0 + n], ref["cigar"][c1:c1 + n])
            L = int(rs.l_qseq[i])
            o0, o1 = int(b["base_off"][i]), int(ref["base_off"][i])
            assert o0 % 32 == 0
            assert np.array_equal(b["qual"][o0:o0 + L], ref["qual"][o1:o1 + L])
            s0 = np.unpackbits(b["seq"][o0 // 2:o0 // 2 + (L + 1) // 2][:, None], axis=1)
            s1 = np.unpackbits(ref["seq"][o1 // 2:o1 // 2 + (L + 1) // 2][:, None], axis=1)
            assert np.array_equal(s0.ravel()[:4 * L], s1.ravel()[:4 * L])
