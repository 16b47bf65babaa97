"""The native read generator's reproducibility (CPU): the deep somatic panel
and the amplicon panel are the same for any number of host threads, and a
region generated alone (`only`) carries exactly its reads of the whole panel.
The bench's records check relies on the second property: the oracle runs on
regions generated alone and the GPU on the whole panel."""
import numpy as np

FIELDS = ("pos", "flag", "mapq", "mpos", "isize", "nm", "n_cigar", "l_qseq", "qual")


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert np.array_equal(a.cigar, b.cigar)
    assert np.array_equal(a.packed, b.packed)


def test_deep_panel_same_for_any_thread_count():
    from rabbitvar_gb300 import synth
    kw = dict(n_regions=3, region_len=2000, tumor_depth=60.0, normal_depth=30.0)
    one = synth.deep_somatic_panel(threads=1, **kw)
    many = synth.deep_somatic_panel(threads=4, **kw)
    assert np.array_equal(one[0], many[0])
    assert one[4] == many[4]
    for a, b in ((one[2], many[2]), (one[3], many[3])):
        assert a.n == b.n > 1000
        _same(a, b)


def test_region_alone_equals_its_reads_in_the_whole_panel():
    from rabbitvar_gb300 import synth
    kw = dict(n_regions=4, region_len=2000, tumor_depth=60.0, normal_depth=30.0)
    g, _, t, n, regions = synth.deep_somatic_panel(**kw)
    g2, _, t2, n2, regions2 = synth.deep_somatic_panel(only=[2], **kw)
    assert np.array_equal(g, g2) and regions == regions2
    # region 2's reads in the whole panel: the same read names (pair and
    # mate), one contiguous block of the span-by-span concatenation
    for whole, alone in ((t, t2), (n, n2)):
        keys = set(zip(alone.name_id.tolist(), (alone.flag & 0xC0).tolist()))
        idx = [i for i, k in enumerate(zip(whole.name_id.tolist(), (whole.flag & 0xC0).tolist())) if k in keys]
        assert len(idx) == alone.n > 100
        a = idx[0]
        assert idx == list(range(a, a + alone.n))
        part = synth.read_range(whole, a, a + alone.n)
        for f in FIELDS:
            assert np.array_equal(getattr(alone, f), getattr(part, f)), f
        assert np.array_equal(alone.cigar, part.cigar)
        assert np.array_equal(synth.unpacked(alone).seq4, part.seq4)


def test_amplicon_panel_same_for_any_thread_count():
    from rabbitvar_gb300 import synth
    kw = dict(n_regions=20, genome_len=400_000, median_depth=40.0, max_depth=200.0, min_depth=10.0)
    one = synth.amplicon_panel_native(threads=1, **kw)
    many = synth.amplicon_panel_native(threads=3, **kw)
    assert np.array_equal(one[0], many[0])
    a, b = one[2], many[2]
    assert a.n == b.n > 500
    _same(a, b)
