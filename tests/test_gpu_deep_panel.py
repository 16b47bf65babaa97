"""The deep targeted somatic panel (400 x 5 kb, tumor 5000x + normal 1000x,
low-VAF somatic SNVs / indels, C>A artifacts at Q20) through the GPU path on
a slice of four regions at full depth (0.8 M reads), somatic mode with
--fisher and the reference's default -k 1, against the oracle on the same
reads: the 63-column records must match one for one (integer and string
columns equal, %f columns within 2e-6 relative, Fisher p in FP64)."""
import pytest

from cmp import diff_records

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 0])
def test_deep_panel_slice_matches_oracle(k):
    import oracle as O
    from rabbitvar_gb300 import api, synth
    only = [0, 137, 263, 399]
    g, _, t, n, regions = synth.deep_somatic_panel(only=only)
    regs = [regions[i] for i in only]
    pair = api.SomaticPair(api.default_params(local_realign=k, fisher=1))
    pair.upload_reference(t.contig, synth.genome_str(g).encode())
    mine = pair.call(api.Batch.from_readset(t), api.Batch.from_readset(n), regs, "T", t.contig).splitlines()
    pair.close()
    _, ora = O.run_somatic_regions(synth.unpacked(t), synth.unpacked(n), g, regs, "T",
                                   O.default_params(local_realign=k, fisher=1), threads=4)
    ora = ora.splitlines()
    assert len(ora) > 10
    assert len(mine) == len(ora)
    assert diff_records(ora, mine, somatic=True) == []
