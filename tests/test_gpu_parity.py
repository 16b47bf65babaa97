"""GPU path against the oracle on the same seeded inputs (-k 0).

Counts, allele keys and the emitted record set must be identical; quality
sums of multi-base alleles (fractional means summed in arbitrary order on the
GPU) agree within 1e-9 relative; the last-seen read position / quality the
reference keeps only to derive pstd/qstd are not part of the maps compared.
"""
import numpy as np
import pytest

from cmp import diff_dump, diff_records

pytestmark = pytest.mark.gpu

P_TAGS = ["P_ML", "PN", "PI", "PC", "PS5", "PS3", "PCI", "PCD", "PMN"]
R_TAGS = ["RN", "RI", "RC"]


def _gpu_ctx(**kw):
    from rabbitvar_gb300 import api
    kw.setdefault("local_realign", 0)
    return api, api.Context(api.default_params(**kw))


def _genome_bytes(g):
    from rabbitvar_gb300 import synth
    return synth.genome_str(g).encode()


def _run_gpu(ctx, api, rs, g, regions):
    ctx.upload_reference(rs.contig, _genome_bytes(g))
    batch = api.Batch.from_readset(rs)
    ctx.submit(batch, regions)
    ctx.pileup()
    p_dumps = [ctx.export_maps(i, "P") for i in range(len(regions))]
    ctx.realign()
    r_dumps = [ctx.export_maps(i, "R") for i in range(len(regions))]
    ctx.score()
    text, n = ctx.format_records("S", rs.contig)
    return p_dumps, r_dumps, text


def test_germline_single_region(germline_small):
    import oracle as O
    g, vs, rs = germline_small
    api, ctx = _gpu_ctx()
    p, r, text = _run_gpu(ctx, api, rs, g, [(1, 100000)])
    ora = O.run_region(rs, g, 1, 100000, stages="PRO", params=O.default_params(local_realign=0))
    assert diff_dump(ora, p[0], P_TAGS, rel=1e-9) == []
    assert diff_dump(ora, r[0], R_TAGS, rel=1e-9) == []
    ora_recs = [l for l in ora.splitlines() if l.startswith("S\t")]
    assert len(ora_recs) > 50
    assert diff_records(ora_recs, text.splitlines()) == []


def test_dense_multi_region():
    import oracle as O
    from rabbitvar_gb300 import synth
    g, vs, rs = synth.dense_multi()
    regions = [(1 + 6000 * i, 6000 * (i + 1)) for i in range(10)]
    api, ctx = _gpu_ctx()
    p, r, text = _run_gpu(ctx, api, rs, g, regions)
    prm = O.default_params(local_realign=0)
    for i in (0, 3, 9):
        ora = O.run_region(rs, g, regions[i][0], regions[i][1], stages="PR", params=prm)
        assert diff_dump(ora, p[i], P_TAGS, rel=1e-9) == [], f"region {i}"
        assert diff_dump(ora, r[i], R_TAGS, rel=1e-9) == [], f"region {i}"
    n, ora_text = O.run_regions(rs, g, regions, params=prm)
    assert n > 100
    assert diff_records(ora_text.splitlines(), text.splitlines()) == []


def test_fisher_records_and_unique_mode():
    import oracle as O
    from rabbitvar_gb300 import synth
    g, vs, rs = synth.dense_multi(seed=0x5EED00D1, length=30_000)
    regions = [(1, 15000), (15001, 30000)]
    api, ctx = _gpu_ctx(fisher=1, unique_fwd=1)
    _, _, text = _run_gpu(ctx, api, rs, g, regions)
    n, ora_text = O.run_regions(rs, g, regions, params=O.default_params(local_realign=0, fisher=1, unique_fwd=1))
    assert n > 20
    assert diff_records(ora_text.splitlines(), text.splitlines(), rel=1e-9) == []


def test_contig_end_in_order_path():
    """Reads reaching past the loaded reference window take the in-order
    walker (the reference's map inserts 0 for missing positions)."""
    import oracle as O
    from rabbitvar_gb300 import synth
    rng = np.random.default_rng(7)
    gen = synth.make_genome(8000, rng)
    vs = synth.plant_variants(gen, rng, 5e-3, 1e-3, lambda r: 0.5, mnv_frac=0.3, margin=20, spacing=8)
    rs = synth.simulate(gen, vs, 80.0, rng, softclip_frac=0.05)
    api, ctx = _gpu_ctx()
    p, r, text = _run_gpu(ctx, api, rs, gen, [(1, 8000)])
    ora = O.run_region(rs, gen, 1, 8000, stages="PRO", params=O.default_params(local_realign=0))
    assert diff_dump(ora, p[0], P_TAGS, rel=1e-9) == []
    assert diff_records([l for l in ora.splitlines() if l.startswith("S\t")], text.splitlines()) == []


def test_fisher_batch_matches_oracle():
    import oracle as O
    api, ctx = _gpu_ctx()
    rng = np.random.default_rng(3)
    tabs = rng.integers(0, 60, size=(400, 4)).astype(np.int32)
    tabs[:50] = rng.integers(0, 3000, size=(50, 4))
    tabs[50] = [0, 0, 0, 0]
    tabs[51] = [5000, 10, 4, 4000]
    p, ratio = ctx.fisher(tabs)
    for i, (a, b, c, d) in enumerate(tabs.tolist()):
        _, _, two = O.fisher(a, b, c, d)
        assert abs(p[i] - two) <= 1e-9 * max(abs(two), 1e-300), (i, a, b, c, d, p[i], two)


def test_somatic_depth_tiles():
    """Tumor-depth (200x) reads over BED-style 10 kb tiles: the bench shape."""
    import oracle as O
    from rabbitvar_gb300 import synth
    rng = np.random.default_rng(0x5EED0002)
    g = synth.make_genome(40_000, rng)
    germ = synth.plant_variants(g, rng, 1e-3, 1e-4, lambda r: 0.5 if r.random() < 0.7 else 1.0)
    som = synth.plant_variants(g, rng, 4e-4, 0.0, lambda r: r.uniform(0.01, 0.5), mnv_frac=0.3, avoid=germ)
    rs = synth.simulate(g, germ + som, 200.0, rng, tail_margin=300)
    regions = [(1 + 10_000 * i, 10_000 * (i + 1)) for i in range(4)]
    api, ctx = _gpu_ctx(fisher=1)
    _, _, text = _run_gpu(ctx, api, rs, g, regions)
    n, ora_text = O.run_regions(rs, g, regions, params=O.default_params(local_realign=0, fisher=1), threads=4)
    assert n > 30
    assert diff_records(ora_text.splitlines(), text.splitlines(), rel=1e-9) == []


def test_dedup_duplicate_reads():
    """-t: reads whose mate starts within the first 9 bases are deduplicated
    by (start, mate contig, mate start), in each region's read order
    (RecordPreprocessor::next_record).  Here every read starting in
    2000..4000 gets mate position 4 and two exact copies."""
    import numpy as np
    import oracle as O
    from rabbitvar_gb300 import synth
    g, vs, rs = synth.dense_multi(seed=0x5EED00D2, length=8_000)
    idx = []
    for i in range(rs.n):
        idx.append(i)
        if 2000 <= rs.pos[i] < 4000:
            idx += [i, i]
    rs2 = synth.take(rs, np.array(idx))
    sel = (rs2.pos >= 2000) & (rs2.pos < 4000)
    rs2.mpos[sel] = 4
    regions = [(1, 2000), (2001, 4000), (4001, 8000)]
    api, ctx = _gpu_ctx(dedup=1)
    _, _, text = _run_gpu(ctx, api, rs2, g, regions)
    n, ora_text = O.run_regions(rs2, g, regions, params=O.default_params(local_realign=0, dedup=1))
    assert n > 10
    assert diff_records(ora_text.splitlines(), text.splitlines()) == []
    # without -t the copies count three times
    n2, ora2 = O.run_regions(rs2, g, regions, params=O.default_params(local_realign=0))
    assert ora2 != ora_text
    api2, ctx2 = _gpu_ctx()
    _, _, text2 = _run_gpu(ctx2, api2, rs2, g, regions)
    assert diff_records(ora2.splitlines(), text2.splitlines()) == []


@pytest.mark.parametrize("case", ["germline", "dense"])
def test_local_realign_cigar_rewrite_maps(case, germline_small):
    """-k 1: the device CIGAR rewrite (CigarModifier) and the -k 1 branches of
    the walk give the same maps after the pileup (P) as the oracle, which
    matches the reference's own -k 1 maps."""
    import oracle as O
    from rabbitvar_gb300 import synth
    if case == "germline":
        g, vs, rs = germline_small
        regions = [(1, 100000)]
    else:
        g, vs, rs = synth.dense_multi()
        regions = [(1 + 6000 * i, 6000 * (i + 1)) for i in range(10)]
    api, ctx = _gpu_ctx(local_realign=1)
    ctx.upload_reference(rs.contig, _genome_bytes(g))
    ctx.submit(api.Batch.from_readset(rs), regions)
    ctx.pileup()
    prm = O.default_params(local_realign=1)
    for i in range(len(regions)) if len(regions) < 4 else (0, 4, 9):
        ora = O.run_region(rs, g, regions[i][0], regions[i][1], stages="P", params=prm)
        assert diff_dump(ora, ctx.export_maps(i, "P"), P_TAGS, rel=1e-9) == [], f"region {i}"
