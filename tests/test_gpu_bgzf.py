"""BGZF/BAM decode on the GPU (rv_bam_read_gpu) against the library's host
decoder (rv_bam_read, itself checked against the generator's arrays in
test_host_io.py): identical records, fields and batch layout for every
DEFLATE block type zlib writes, member boundaries inside records, records
longer than a member, long headers, several contigs and unmapped records,
read names the record finder's plausibility check rejects; malformed input
ends in RV_ERR_FORMAT; and the pileup of a device batch equals the pileup of
the host batch."""
import os
import struct
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EOF_MEMBER = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")


def bgzf(payload: bytes, level=6, strategy=zlib.Z_DEFAULT_STRATEGY, step=0xFF00, cuts=None) -> bytes:
    """BGZF members of `payload`, cut every `step` bytes (or at `cuts`)."""
    cuts = [0] + ([c for c in cuts if 0 < c < len(payload)] if cuts else []) + [len(payload)]
    bounds = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        bounds += list(range(a, b, step))
    bounds.append(len(payload))
    out = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        data = payload[a:b]
        co = zlib.compressobj(level, zlib.DEFLATED, -15, 8, strategy)
        c = co.compress(data) + co.flush()
        hdr = struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, 66, 67, 2, len(c) + 25)
        out.append(hdr + c + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data)))
    return b"".join(out) + EOF_MEMBER


def bam_stream(rs, tids=None, contigs=None, text_pad=0, name_fn=None, big_aux=None):
    """BAM stream of a read set with per-record reference ids; `contigs` is
    [(name, length)], `big_aux` {record index: bytes of a Z tag}."""
    contigs = contigs or [(rs.contig, rs.contig_len)]
    text = "@HD\tVN:1.6\n" + "".join(f"@SQ\tSN:{n}\tLN:{l}\n" for n, l in contigs) + "@CO\t" + "x" * text_pad + "\n"
    out = [b"BAM\x01", struct.pack("<I", len(text)), text.encode(), struct.pack("<I", len(contigs))]
    for n, l in contigs:
        out += [struct.pack("<I", len(n) + 1), n.encode() + b"\x00", struct.pack("<I", l)]
    packed = rs.packed_seq()
    starts = []
    for i in range(rs.n):
        name = (name_fn(i) if name_fn else b"r%d" % i) + b"\x00"
        nc, co, L, bo = int(rs.n_cigar[i]), int(rs.cig_off[i]), int(rs.l_qseq[i]), int(rs.base_off[i])
        tid = 0 if tids is None else int(tids[i])
        aux = b"XAZ" + big_aux[i] + b"\x00" if big_aux and i in big_aux else b""
        aux += b"NMi" + struct.pack("<i", int(rs.nm[i])) if i % 7 else b"NMC" + bytes([int(rs.nm[i]) & 255])
        body = struct.pack("<iiBBHHHiiii", tid, int(rs.pos[i]), len(name), int(rs.mapq[i]), 4680, nc,
                           int(rs.flag[i]), L, tid, int(rs.mpos[i]), 0)
        rec = (body + name + rs.cigar[co:co + nc].astype("<u4").tobytes() + packed[bo // 2:bo // 2 + (L + 1) // 2]
               .tobytes() + rs.qual[bo:bo + L].tobytes() + aux)
        starts.append(sum(len(x) for x in out))
        out += [struct.pack("<I", len(rec)), rec]
    return b"".join(out), starts


def host_decode(tmp_path, data: bytes):
    from rabbitvar_gb300 import api
    p = os.path.join(tmp_path, "x.bam")
    with open(p, "wb") as f:
        f.write(data)
    return api.read_bam(p)


def same_batches(a, b):
    na, la, ba = a
    nb, lb, bb = b
    assert na == nb and la == lb
    assert sorted(ba) == sorted(bb)
    for tid in ba:
        x, y = ba[tid].arrays, bb[tid].arrays
        assert ba[tid].n_reads == bb[tid].n_reads and ba[tid].n_bases == bb[tid].n_bases
        for k in ("pos", "flag", "mapq", "mpos", "nm", "n_cigar", "cig_off", "cigar", "l_qseq", "base_off"):
            assert np.array_equal(x[k], y[k]), (tid, k)
        # bases and qualities of each read (the padding of the 32-base slots is unspecified)
        L = x["l_qseq"].astype(np.int64)
        bo = x["base_off"].astype(np.int64)
        if L.size:
            q_idx = np.repeat(bo, L) + (np.arange(L.sum()) - np.repeat(np.cumsum(L) - L, L))
            assert np.array_equal(x["qual"][q_idx], y["qual"][q_idx]), tid
            S = (L + 1) // 2
            s_idx = np.repeat(bo // 2, S) + (np.arange(S.sum()) - np.repeat(np.cumsum(S) - S, S))
            assert np.array_equal(x["seq"][s_idx], y["seq"][s_idx]), tid


@pytest.fixture(scope="module")
def mix():
    from rabbitvar_gb300 import synth
    g, _, t, n = synth.somatic_mix(0x5EED0051)
    return g, t, n


@pytest.mark.parametrize("level,strategy", [(1, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_DEFAULT_STRATEGY),
                                            (9, zlib.Z_DEFAULT_STRATEGY), (0, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_FIXED), (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)])
def test_block_types_match_host_decoder(tmp_path, mix, level, strategy):
    from rabbitvar_gb300 import api, synth
    _, t, _ = mix
    data = bgzf(synth.bam_bytes(t, "T"), level, strategy)
    db = api.DeviceBam(data)
    try:
        same_batches(db.host_batches(), host_decode(tmp_path, data))
        assert db.host_batches()[2][0].n_reads == t.n
    finally:
        db.close()


def test_contigs_long_header_long_records_odd_names(tmp_path, mix):
    """Three contigs and unmapped records, a 200 kB header text (several
    members), records of 150 kB (longer than a member), members cut at record
    starts for one file and mid-record for another, and names with a tab
    (implausible to the record finder: every chunk is re-walked)."""
    from rabbitvar_gb300 import api
    _, t, _ = mix
    n = t.n
    tids = np.zeros(n, np.int32)
    tids[n // 3:2 * n // 3] = 1
    tids[2 * n // 3:] = 2
    tids[-50:] = -1
    contigs = [("c1", t.contig_len), ("c2", t.contig_len), ("c3", t.contig_len)]
    big = {17: b"A" * 150_000, n // 2: b"C" * 70_000}
    payload, starts = bam_stream(t, tids, contigs, text_pad=200_000, big_aux=big)
    for data in (bgzf(payload, 1), bgzf(payload, 6, cuts=starts[::150])):
        db = api.DeviceBam(data)
        try:
            got = db.host_batches()
            same_batches(got, host_decode(tmp_path, data))
            assert [got[2][k].n_reads for k in range(3)] == [n // 3, 2 * n // 3 - n // 3, n - 2 * n // 3 - 50]
        finally:
            db.close()
    # names the record finder rejects; then, decoded into the same handle,
    # contigs interleaved record by record (batches gathered, not windows)
    payload, _ = bam_stream(t, name_fn=lambda i: b"r\t%d" % i)
    data = bgzf(payload, 1)
    db = api.DeviceBam(data)
    try:
        same_batches(db.host_batches(), host_decode(tmp_path, data))
        payload, _ = bam_stream(t, np.arange(n) % 2, contigs[:2])
        data = bgzf(payload, 6)
        db.reread(data)
        got = db.host_batches()
        same_batches(got, host_decode(tmp_path, data))
        assert got[2][0].n_reads == (n + 1) // 2
    finally:
        db.close()


def test_malformed_input_is_an_error(mix):
    from rabbitvar_gb300 import api, synth
    _, t, _ = mix
    data = bgzf(synth.bam_bytes(t, "T"), 6)
    # a member cut short (host-side member walk)
    with pytest.raises(api.RvError) as e:
        api.DeviceBam(data[:len(data) // 2])
    assert e.value.status == -8
    # reserved block type 3 in the second member's first block (device inflate)
    second = struct.unpack("<H", data[16:18])[0] + 1
    bad = bytearray(data)
    bad[second + 18] |= 0b110
    with pytest.raises(api.RvError) as e:
        api.DeviceBam(bytes(bad))
    assert e.value.status == -8
    # an inflated stream that ends inside a record (device record chain)
    payload = synth.bam_bytes(t, "T")
    with pytest.raises(api.RvError) as e:
        api.DeviceBam(bgzf(payload[:-100], 6))
    assert e.value.status == -8


def test_device_batch_pileup_matches_host_batch(mix):
    """A somatic pair called from device-decoded batches (bases and
    qualities never leave the GPU) gives the records of the host batches."""
    from rabbitvar_gb300 import api, synth
    g, t, n = mix
    regions = [(1, g.shape[0])]
    params = api.default_params(local_realign=1, fisher=1)
    pair = api.SomaticPair(params)
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    want = pair.call(api.Batch.from_readset(t), api.Batch.from_readset(n), regions, "T", t.contig)
    dt, dn = api.DeviceBam(bgzf(synth.bam_bytes(t, "T"), 1)), api.DeviceBam(bgzf(synth.bam_bytes(n, "N"), 1))
    try:
        got = pair.call(dt.batch(0), dn.batch(0), regions, "T", t.contig)
    finally:
        pair.close()
        dt.close()
        dn.close()
    assert len(want.splitlines()) > 100
    assert got == want
