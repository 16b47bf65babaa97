"""Benchmark: reads/s of pileup + variant scoring on one GB300.

Headline workload: the deep targeted somatic panel -- a seeded synthetic
contig with 400 regions of 5 kb (2 Mb), tumor 5000x + normal 1000x 2x150 bp
pairs (~80 M reads), germline SNVs/indels in both samples, low-VAF somatic
SNVs/MNVs/indels (VAF log-uniform(0.001, 0.05)) in the tumor and C>A
artifacts at 1e-4 per C base with quality 20, called in somatic mode (the
reference's `-b 'T.bam|N.bam' -N 'T|N' --fisher` over the 400-region BED,
its default -k 1): both samples through the full per-region path (record
filters, CIGAR rewrite and walk, allele maps, the realigner, site
statistics), then the tumor/normal classification, the hard filter, three
Fisher tests per record and the 63-column record text.  One step = both
samples, all regions.

    value : reads/s with the read batches already resident in HBM
    e2e   : reads/s through the C ABI from pinned host batches, including
            the host->device copy of the reads and the device->host copy of
            the scored candidates every step
Inputs (~22 GB of reads) exceed the 129 MB L2, so no flush is needed
between steps.  `parity` compares the GPU's records of four regions with
the oracle's on the same reads (the CPU baseline sample); a mismatch fails
the run.  Secondary keys: the 1 Mb somatic pair at 200x/100x
(`somatic_pair_1mb`, with its BAM-decode leg), the batched 10,000-region
amplicon panel against region-by-region calls (`panel`), the other -k
setting, the learned filter.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
    python bench.py --bam-decode      # BAM decode alone, GPU vs host decoder
    python bench.py --panel N         # batched amplicon panel of N regions
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TILE = 10_000
CONTIG = 1_000_000
# algorithmic bytes per unit (the scope table's figures): per read
# 4 pos + 4 n_cigar words + L/4 bases + L/8 N mask + L quals + 1 mapq + 2 flag
# + 4 mpos + 1 NM; per covered site 256 B of count record; per string-keyed
# allele 64 B; plus 1 B per reference base
BYTES_PER_READ_FIXED = 4 + 1 + 2 + 4 + 1


def read_alg_bytes(rs) -> float:
    L = rs.l_qseq.astype(float)
    return float((BYTES_PER_READ_FIXED + 4 * rs.n_cigar.astype(float) + L / 4 + L / 8 + L).sum())


def make_workload(seed_offset: int = 0):
    from rabbitvar_gb300 import synth
    g, _, tumor, normal = synth.somatic_pair(seed=0x5EED0001 + seed_offset, length=CONTIG)
    regions = [(1 + TILE * i, TILE * (i + 1)) for i in range(CONTIG // TILE)]
    return g, tumor, normal, regions


class Clocks:
    """nvidia-smi sampling (every 200 ms) started before the warm-up, so that
    its start-up does not fall in a timed region; the samples taken inside the
    timed regions (marked with window()) are the ones reported."""

    def __init__(self, index: int = 0):
        self.p = None
        self.windows = []
        self.path = f"/tmp/rv_clocks_{os.getpid()}.csv"
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={index}",
                 "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def window(self, t0: float, t1: float):
        """A timed region, in time.time() seconds."""
        self.windows.append((t0, t1))

    def stop(self) -> dict:
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for ln in f:
                c = [x.strip() for x in ln.split(",")]
                if len(c) < 9:
                    continue
                try:
                    ts = time.mktime(time.strptime(c[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                    ts += float("0." + c[0].split(".")[1]) if "." in c[0] else 0.0
                    rows.append((ts, float(c[1]), float(c[2]), c[5:9]))
                except (ValueError, IndexError):
                    continue
        os.unlink(self.path)
        inside = [r for r in rows if any(a - 0.25 <= r[0] <= b + 0.25 for a, b in self.windows)]
        use = inside or rows
        reasons = set()
        for r in use:
            for n, v in zip(names, r[3]):
                if v.lower() == "active":
                    reasons.add(n)
        sm = [r[1] for r in use]
        mx = [r[2] for r in use]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(use),
                "window": "timed regions" if inside else "whole run (no sample fell inside the timed regions)"}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def dist_init():
    n = int(os.environ.get("WORLD_SIZE", "1"))
    if n <= 1:
        return 0, 1, None
    import torch.distributed as dist
    backend = "nccl"
    try:
        import torch
        if not torch.cuda.is_available():
            backend = "gloo"
    except ImportError:
        backend = "gloo"
    dist.init_process_group(backend)
    return dist.get_rank(), dist.get_world_size(), dist


def barrier_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(k: int) -> str:
    return (f"somatic mode (-b 'T|N' -N 'T|N' --fisher -f 0.01 -k {k}): synthetic 1 Mb contig, "
            "tumor 200x + normal 100x 2x150, 100 x 10 kb BED tiles")


def deep_workload_name(k: int, n_regions: int = 400) -> str:
    return (f"somatic mode (-b 'T|N' -N 'T|N' --fisher -f 0.01 -k {k}): deep targeted panel, {n_regions} x 5 kb "
            "regions, tumor 5000x + normal 1000x 2x150, somatic VAF log-U(0.001,0.05), C>A 1e-4/base at Q20")


METRIC = "reads/s pileup+var scoring (deep somatic panel 400 x 5 kb, T5000x+N1000x)"
PANEL_REGIONS = 400
# the oracle's sample of the panel: the CPU baseline and the records check
PARITY_REGIONS = [0, 137, 263, 399]
# the reference arm's sample (all host threads): 16 regions, ~3.2 M reads
REF_REGIONS = list(range(0, PANEL_REGIONS, 25))
CPU_TILES = 40   # 1 Mb pair: CPU sample of 40 of the 100 tiles
# DRAM bytes (read + write) per read of one k_pileup_tiles launch, from one
# ncu capture of a tumor launch of the deep panel on a 16-region slice
# (2.67 M reads, 1541.7 MB read + 1368.3 MB written); the headline launch's
# traffic is this times its reads
PILEUP_TRAFFIC_PER_READ = (1541.7e6 + 1368.3e6) / 2666656


def deep_workload(rank: int = 0, world: int = 1, only=None):
    """The deep panel (400 x world regions, LPT-partitioned across ranks by
    expected reads: each rank generates and calls its own share) or the
    regions `only`; returns (genome, tumor, normal, regions of the reads)."""
    from rabbitvar_gb300 import shard, synth
    n_reg = PANEL_REGIONS * world
    if only is None and world > 1:
        only = shard.partition([1] * n_reg, world)[rank]
    g, _, t, n, regions = synth.deep_somatic_panel(n_regions=n_reg, only=only)
    regs = regions if only is None else [regions[i] for i in sorted(only)]
    return g, t, n, regs


def oracle_regions(g, tumor, normal, regions, k: int, threads: int = 1):
    """The oracle on `regions` of a read set whose regions are separated by
    more than a read pair (each region's reads sliced out): returns (record
    text, reads, seconds)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from rabbitvar_gb300 import synth
    p = O.default_params(local_realign=k, fisher=1)
    sl = []
    for rs in (tumor, normal):
        lo = [int(np.searchsorted(rs.pos, a - 1 - 1000)) for a, _ in regions]
        hi = [int(np.searchsorted(rs.pos, b + 1000)) for _, b in regions]
        if rs.seq4 is not None:
            sl.append(synth.take(rs, np.concatenate([np.arange(a, b) for a, b in zip(lo, hi)])))
        else:
            sl.append(_slices(rs, lo, hi))
    reads = sl[0].n + sl[1].n
    t0 = time.perf_counter()
    _, text = O.run_somatic_regions(sl[0], sl[1], g, regions, "T", p, threads=threads)
    return text, reads, time.perf_counter() - t0


def _slices(rs, lo, hi):
    """Concatenation of the read ranges [lo[i], hi[i]) (ascending, disjoint)
    of a packed read set, unpacked."""
    import dataclasses
    import numpy as np
    from rabbitvar_gb300 import synth
    parts = [synth.read_range(rs, a, b) for a, b in zip(lo, hi)]
    cig = np.concatenate([p.cigar for p in parts])
    ncig = np.concatenate([p.n_cigar for p in parts])
    cig_off = np.zeros(ncig.shape[0], np.uint32)
    cig_off[1:] = np.cumsum(ncig[:-1].astype(np.uint64)).astype(np.uint32)
    n = ncig.shape[0]
    stride = 160
    cat = lambda f: np.concatenate([getattr(p, f) for p in parts])  # noqa: E731
    return dataclasses.replace(parts[0], pos=cat("pos"), flag=cat("flag"), mapq=cat("mapq"), mpos=cat("mpos"),
                               isize=cat("isize"), nm=cat("nm"), n_cigar=ncig, cig_off=cig_off, cigar=cig,
                               l_qseq=cat("l_qseq"), base_off=np.arange(n, dtype=np.uint64) * np.uint64(stride),
                               seq4=cat("seq4"), qual=cat("qual"), name_id=cat("name_id"))


def region_records(text: str, contig: str, regions) -> list[str]:
    """Records of `text` whose region column names one of `regions`."""
    keys = {f"\t{contig}:{a}-{b}\t" for a, b in regions}
    return [ln for ln in text.splitlines() if any(k in ln for k in keys)]


def cpu_baseline_run(g, tumor, normal, regions, threads: int, n_regions: int, k: int):
    """The oracle's CPU restatement of the path in somatic mode (OpenMP over
    regions, as the reference's BED mode) on a bounded sample of the
    workload's regions; returns reads/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    p = O.default_params(local_realign=k, fisher=1)
    sub = regions[:n_regions]
    lo, hi = sub[0][0], sub[-1][1]
    reads = sum(int(((rs.pos >= lo - 1) & (rs.pos < hi)).sum()) for rs in (tumor, normal))
    t0 = time.perf_counter()
    O.run_somatic_regions(tumor, normal, g, sub, "T", p, threads=threads)
    dt = time.perf_counter() - t0
    return reads / dt, dt, reads


def other_k_leg(g, tumor, normal, regions, k: int, steps: int, warmup: int, device: int) -> dict:
    """The same workload with the other -k setting (reported beside the
    main line): device-resident reads/s, end-to-end reads/s and the host
    realigner's time per step."""
    from rabbitvar_gb300 import api, synth
    pair = api.SomaticPair(api.default_params(local_realign=k, fisher=1), device=device)
    pair.upload_reference(tumor.contig, synth.genome_str(g).encode())
    batches = [api.Batch.from_readset(rs, pinned=True) for rs in (tumor, normal)]
    n_reads = tumor.n + normal.n

    def step(submit: bool):
        if submit:
            pair.submit(batches[0], batches[1], regions)
        t = time.perf_counter()
        pair.pileup_realign()
        dt = time.perf_counter() - t
        pair.score()
        _, n = pair.format_records("T", "ctg")
        return dt, n

    # end to end: the same stream of batches as the main line
    stream = api.SomaticStream(api.default_params(local_realign=k, fisher=1), device=device)
    stream.upload_reference(tumor.contig, synth.genome_str(g).encode())
    job = (batches[0], batches[1], regions)
    stream.run([job] * max(1, warmup), "T", "ctg")
    t0 = time.perf_counter()
    stream.run([job] * steps, "T", "ctg")
    e2e_dt = time.perf_counter() - t0
    stream.close()
    pair.submit(batches[0], batches[1], regions)
    for _ in range(warmup):
        step(False)
    t0 = time.perf_counter()
    re_ms, recs = 0.0, 0
    for _ in range(steps):
        dt, recs = step(False)
        re_ms += dt * 1e3
    dev_dt = time.perf_counter() - t0
    pair.close()
    return {"workload": workload(k), "value": n_reads * steps / dev_dt, "e2e": n_reads * steps / e2e_dt,
            "unit": "reads/s", "ms_per_step": dev_dt / steps * 1e3, "pileup_realign_ms_per_step": re_ms / steps,
            "records_per_step": recs, "steps": steps, "warmup": warmup}


def bgzf_bytes(payload: bytes, level: int = 1) -> bytes:
    """BGZF members (zlib level 1, 0xFF00 bytes of stream each) + EOF member."""
    import struct
    import zlib
    from rabbitvar_gb300 import synth
    parts = []
    for i in range(0, len(payload), 0xFF00):
        d = payload[i:i + 0xFF00]
        co = zlib.compressobj(level, zlib.DEFLATED, -15)
        c = co.compress(d) + co.flush()
        parts.append(struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, 66, 67, 2, len(c) + 25) + c +
                     struct.pack("<II", zlib.crc32(d) & 0xFFFFFFFF, len(d)))
    return b"".join(parts) + synth._BGZF_EOF


def bam_leg(g, tumor, normal, regions, k: int, steps: int, warmup: int, device: int, want_text: str) -> dict:
    """End to end from BGZF-compressed BAM bytes in pinned host memory: each
    step decodes both samples on the GPU (rv_bam_reread_gpu into reused
    buffers, contig batches as windows of the decoded layout) and calls the
    pair on those batches; beside it the same step with the library's host
    decoder (all host threads) feeding pinned host batches."""
    import ctypes as C
    from rabbitvar_gb300 import api, synth
    L = api.lib()
    data = [bgzf_bytes(synth.bam_bytes(rs, name)) for rs, name in ((tumor, "T"), (normal, "N"))]
    ptrs = []
    for d in data:
        p = L.rv_alloc_pinned(len(d))
        C.memmove(p, d, len(d))
        ptrs.append(p)
    n_reads = tumor.n + normal.n
    pair = api.SomaticPair(api.default_params(local_realign=k, fisher=1), device=device)
    pair.upload_reference(tumor.contig, synth.genome_str(g).encode())
    dbams = [api.DeviceBam(d, device) for d in data]
    dec_ms = []

    def gpu_step():
        t = time.perf_counter()
        for db, d, p in zip(dbams, data, ptrs):
            db.reread(d, pinned_ptr=p)
        bt, bn = dbams[0].batch(0), dbams[1].batch(0)
        dec_ms.append((time.perf_counter() - t) * 1e3)
        return pair.call(bt, bn, regions, "T", "ctg")

    for _ in range(max(1, warmup)):
        gpu_step()
    dec_ms.clear()
    t0 = time.perf_counter()
    texts = [gpu_step() for _ in range(steps)]
    gpu_dt = time.perf_counter() - t0
    host_dec = []

    def host_step():
        t = time.perf_counter()
        hs, bs = [], []
        for d, p in zip(data, ptrs):
            h = C.c_void_p()
            st = L.rv_bam_read_mem(p, len(d), 0, C.byref(h))
            if st != 0:
                raise api.RvError(st, "rv_bam_read_mem")
            rb = api.ReadBatch()
            L.rv_bam_batch(h, 0, C.byref(rb))
            hs.append(h)
            bs.append(type("HostBatch", (), {"struct": lambda self, rb=rb: rb, "n_reads": rb.n_reads})())
        host_dec.append((time.perf_counter() - t) * 1e3)
        text = pair.call(bs[0], bs[1], regions, "T", "ctg")
        for h in hs:
            L.rv_bam_free(h)
        return text

    host_step()
    host_dec.clear()
    host_steps = max(1, min(steps, 3))
    t0 = time.perf_counter()
    htexts = [host_step() for _ in range(host_steps)]
    host_dt = time.perf_counter() - t0
    for db in dbams:
        db.close()
    pair.close()
    for p in ptrs:
        L.rv_free_pinned(p)
    same = all(t == want_text for t in texts + htexts)
    return {"value": n_reads * steps / gpu_dt, "unit": "reads/s", "steps": steps,
            "bgzf_bytes_per_step": sum(len(d) for d in data),
            "decode_ms_per_step": statistics.mean(dec_ms),
            "host_decoder": {"value": n_reads * host_steps / host_dt, "unit": "reads/s", "steps": host_steps,
                             "decode_ms_per_step": statistics.mean(host_dec), "threads": os.cpu_count()},
            "records_equal_to_batch_path": same,
            "note": "BGZF level-1 members of the synthetic BAMs in pinned host memory; decode + pileup + scoring + records"}


def run_bam_decode(args):
    """`--bam-decode`: BGZF/BAM decode of the workload's tumor sample (1.33 M
    reads, BGZF level 1) on the GPU (rv_bam_reread_gpu into reused buffers,
    then its contig batch) against the library's host decoder with all host
    threads (rv_bam_read_mem + rv_bam_batch); one JSON line."""
    import ctypes as C
    from rabbitvar_gb300 import api, synth
    g, tumor, normal, regions = make_workload()
    payload = synth.bam_bytes(tumor, "T")
    data = bgzf_bytes(payload)
    L = api.lib()
    ptr = L.rv_alloc_pinned(len(data))
    C.memmove(ptr, data, len(data))
    h = C.c_void_p()
    if L.rv_bam_read_gpu(ptr, len(data), int(os.environ.get("LOCAL_RANK", "0")), C.byref(h)) != 0:
        raise RuntimeError("rv_bam_read_gpu failed")
    gpu = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = L.rv_bam_reread_gpu(h, ptr, len(data))
        rb = api.ReadBatch()
        st2 = L.rv_bam_batch(h, 0, C.byref(rb))
        if st or st2 or rb.n_reads != tumor.n:
            raise RuntimeError("device decode failed")
        if i >= args.warmup:
            gpu.append((time.perf_counter() - t0) * 1e3)
    L.rv_bam_free(h)
    host = []
    for i in range(1 + min(args.steps, 3)):
        t0 = time.perf_counter()
        hh = C.c_void_p()
        if L.rv_bam_read_mem(ptr, len(data), 0, C.byref(hh)) != 0:
            raise RuntimeError("host decode failed")
        rb = api.ReadBatch()
        L.rv_bam_batch(hh, 0, C.byref(rb))
        if i:
            host.append((time.perf_counter() - t0) * 1e3)
        L.rv_bam_free(hh)
    L.rv_free_pinned(ptr)
    gms, hms = statistics.median(gpu), statistics.median(host)
    print(json.dumps({"metric": "BAM decode (BGZF inflate + records -> read batch)", "value": tumor.n / (gms * 1e-3),
                      "unit": "reads/s", "ms": gms, "steps": args.steps, "warmup": args.warmup,
                      "host_decoder": {"value": tumor.n / (hms * 1e-3), "ms": hms, "threads": os.cpu_count()},
                      "bgzf_bytes": len(data), "stream_bytes": len(payload), "reads": tumor.n,
                      "stream_GBps": len(payload) / (gms * 1e-3) / 1e9}))


def learned_filter_leg():
    """The learned filter against the hard filter at the shapes of the three
    calling workloads (deep somatic panel slices, amplicon panel slices,
    200x tumors; learn.shape_samples): trained on three seeds, evaluated on
    three held-out seeds one by one (planted truth), F1 and precision at the
    hard filter's recall per seed and their spread, plus the training step
    time and the inference rate (features already built)."""
    import numpy as np
    from rabbitvar_gb300 import learn, mlp
    t0 = time.perf_counter()
    xtr, ytr, _, _ = learn.dataset_shapes([401, 402, 403])
    xte, yte, hte, bounds = learn.dataset_shapes([501, 502, 503])
    data_s = time.perf_counter() - t0
    m = mlp.Mlp(batch=4096, seed=3)
    t0 = time.perf_counter()
    m.train(xtr, ytr, epochs=20, lr=1e-3)
    train_s = time.perf_counter() - t0
    m.predict(xte)
    t0 = time.perf_counter()
    scores = m.predict(xte)
    pred_s = time.perf_counter() - t0
    per_seed = []
    for (a, b) in bounds:
        r = learn.compare(scores[a:b], yte[a:b], hte[a:b])
        per_seed.append({"candidates": r["candidates"], "true": r["true"], "hard_f1": r["hard"]["f1"],
                         "learned_f1_at_hard_recall": r["learned"]["f1"],
                         "learned_recall_at_hard_precision": r["learned_at_hard_precision"]["recall"],
                         "hard_recall": r["hard"]["recall"], "hard_precision": r["hard"]["precision"]})
    res = learn.compare(scores, yte, hte)
    gain = [p["learned_f1_at_hard_recall"] - p["hard_f1"] for p in per_seed]
    flops_per_candidate = 2 * (64 * 128 + 2 * 128 * 128 + 128)
    res.update({"train_candidates": int(len(ytr)), "epochs": 20, "train_s": train_s, "dataset_s": data_s,
                "train_step_ms": m.step_ms(), "predict_candidates_per_s": len(yte) / pred_s,
                "predict_tflops": len(yte) / pred_s * flops_per_candidate / 1e12,
                "held_out_seeds": per_seed,
                "f1_gain_at_hard_recall": {"mean": float(np.mean(gain)), "min": float(np.min(gain)),
                                           "max": float(np.max(gain))},
                "network": "40-128-128-128-1 GELU, BF16 tcgen05 GEMMs, FP32 accumulate, Adam",
                "data": "synthetic: per seed a 12-region slice of the deep somatic panel (tumor 5000x), a "
                        "150-region slice of the amplicon panel and a 300 kb 200x tumor; planted truth"})
    m.close()
    return res


def panel_leg(n_reg: int, k: int, steps: int, warmup: int, device: int = 0, per_region_sample: int = 500) -> dict:
    """Batched amplicon panel (config 2's shape: n_reg regions of U(100, 2000)
    bp, depth log-normal median 500x, amplicon reads with 0.5% exact
    duplicates, -t -u, simple mode), from pinned host batches through the C
    ABI.  Batched: all regions in one submit and one pileup launch (the
    pileup chain as a CUDA graph); region by region: one submit
    and pipeline per region (the reference's per-region stage sequence), on
    the first `per_region_sample` regions, whose records must equal the
    batched run's records for them."""
    import numpy as np
    from rabbitvar_gb300 import api, synth
    t_gen = time.perf_counter()
    g, _, rs, regions = synth.amplicon_panel_native(n_regions=n_reg, genome_len=n_reg * 5000)
    t_gen = time.perf_counter() - t_gen
    params = api.default_params(local_realign=k, dedup=1, unique_fwd=1)
    ctx = api.Context(params, device=device)
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    ctx.set_pileup_graph(True)
    batch = api.Batch.from_readset(rs, pinned=True)
    sample = regions[:min(per_region_sample, len(regions))]
    subs = []
    for a, b in sample:
        lo = int(np.searchsorted(rs.pos, a - 1 - 400))
        hi = int(np.searchsorted(rs.pos, b))
        subs.append(api.Batch.from_readset(synth.read_range(rs, lo, hi), pinned=True))
    sample_reads = sum(sb.n_reads for sb in subs)

    def batched():
        ctx.submit(batch, regions)
        ctx.pileup()
        ctx.realign()
        ctx.score()
        return ctx.format_records("S", rs.contig)[0]

    def per_region():
        out = []
        for r, b in zip(sample, subs):
            ctx.submit(b, [r])
            ctx.pileup()
            ctx.realign()
            ctx.score()
            out.append(ctx.format_records("S", rs.contig)[0])
        return "".join(out)

    for _ in range(max(1, warmup)):
        t_b = batched()
    t0 = time.perf_counter()
    for _ in range(steps):
        t_b = batched()
    dt_b = (time.perf_counter() - t0) / steps
    per_region()
    t0 = time.perf_counter()
    t_r = per_region()
    dt_r = time.perf_counter() - t0
    mine = sorted(region_records(t_b, rs.contig, sample))
    same = mine == sorted(t_r.splitlines())
    out = {"workload": f"{n_reg} regions U(100,2000) bp, depth lognormal median 500x, amplicon 2x150, "
                       f"0.5% PCR duplicates, -t -u -k {k}, simple mode",
           "value": rs.n / dt_b, "unit": "reads/s", "reads": int(rs.n), "ms_per_step": dt_b * 1e3, "steps": steps,
           "records": len(t_b.splitlines()), "generate_s": t_gen,
           "region_by_region": {"value": sample_reads / dt_r, "unit": "reads/s", "regions": len(sample),
                                "reads": int(sample_reads), "ms": dt_r * 1e3},
           "speedup_batched": (rs.n / dt_b) / (sample_reads / dt_r),
           "records_equal_region_by_region": same, "sample_records": len(mine),
           "pileup_graph": dict(zip(("launches", "instantiations"), ctx.pileup_graph_stats()))}
    ctx.close()
    batch.close()
    for sb in subs:
        sb.close()
    return out


def run_panel(args):
    """`--panel N`: the batched amplicon panel leg alone, as one JSON line."""
    r = panel_leg(args.panel, args.local_realign, args.steps, args.warmup)
    out = {"metric": f"reads/s batched amplicon panel ({args.panel} regions, -t -u)", "value": r["value"],
           "unit": "reads/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": r["ms_per_step"], "higher_is_better": True, "data": "synthetic (seeded)",
           "config": {"workload": r["workload"], "reads": r["reads"]}}
    out.update({k: v for k, v in r.items() if k not in ("value", "workload", "ms_per_step", "steps")})
    print(json.dumps(out))


def run_reference(args, rank):
    """The reference arm: the oracle (the CPU restatement of the reference's
    path, pinned to the reference binary) on the machine's host cores, all
    threads, somatic mode, on a 16-region sample of the deep panel per step."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    g, tumor, normal, regs = deep_workload(only=REF_REGIONS)
    vals = []
    nr = 0
    for i in range(args.warmup + args.steps):
        _, nr, dt = oracle_regions(g, tumor, normal, regs, args.local_realign, threads=threads)
        if i >= args.warmup:
            vals.append(nr / dt)
    v = statistics.median(vals)
    sample = f"{len(REF_REGIONS)} of {PANEL_REGIONS} regions (every 25th), tumor+normal ({nr} reads), per step"
    out = {"impl": "reference", "metric": METRIC,
           "value": v, "unit": "reads/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "data": "synthetic (seeded)",
           "config": {"workload": deep_workload_name(args.local_realign), "sample": sample},
           "cpu_baseline": {"value": v, "unit": "reads/s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def measure_pair(g, tumor, normal, regions, args, dist, clocks, device: int, world: int, contig: str = "ctg",
                 roofline: bool = True) -> dict:
    """One somatic workload through the pair: e2e (a stream of pinned host
    batches uploaded every step), value (the stream on batches resident in
    HBM), the same steps one after the other (stage times, launches), and the
    tumor's pileup launch timed alone.  Returns the measurements and the
    first step's record text."""
    from rabbitvar_gb300 import api, synth
    params = api.default_params(local_realign=args.local_realign, fisher=1)
    pair = api.SomaticPair(params, device=device)
    pair.upload_reference(contig, synth.genome_str(g).encode())
    ctxs = [pair.tumor, pair.normal]
    batches = [api.Batch.from_readset(rs, pinned=True) for rs in (tumor, normal)]
    n_reads = tumor.n + normal.n
    host_ms = {"pileup+realign": 0.0, "score": 0.0, "format": 0.0}

    def kernels_of():
        return sum(c.timings()["kernels"] for c in ctxs)

    def device_step(collect=None):
        t0 = time.perf_counter()
        pair.pileup_realign()
        t2 = time.perf_counter()
        pair.score()
        t3 = time.perf_counter()
        text, n = pair.format_records("T", contig)
        t4 = time.perf_counter()
        if collect is not None:
            host_ms["pileup+realign"] += (t2 - t0) * 1e3
            host_ms["score"] += (t3 - t2) * 1e3
            host_ms["format"] += (t4 - t3) * 1e3
            collect.extend(c.stage_times() for c in ctxs)
        return kernels_of(), n

    stream = api.SomaticStream(params, device=device)
    stream.upload_reference(contig, synth.genome_str(g).encode())
    job = (batches[0], batches[1], regions)
    stream.run([job] * max(1, args.warmup), "T", contig)
    w0 = time.time()
    t0 = time.perf_counter()
    e2e_texts = stream.run([job] * args.steps, "T", contig)
    e2e_dt = barrier_max(dist, time.perf_counter() - t0)
    clocks.window(w0, time.time())
    last = stream.pairs[(args.steps - 1) % 2]
    h2d = sum(c.io_bytes()[0] for c in (last.tumor, last.normal))
    d2h = sum(c.io_bytes()[1] for c in (last.tumor, last.normal))
    resident = (None, None, regions)
    stream.run([resident] * max(1, args.warmup), "T", contig)
    w0 = time.time()
    t0 = time.perf_counter()
    res_texts = stream.run([resident] * args.steps, "T", contig)
    res_dt = barrier_max(dist, time.perf_counter() - t0)
    clocks.window(w0, time.time())
    stream.close()
    pair.submit(batches[0], batches[1], regions)
    for _ in range(args.warmup):
        device_step()
    stages = []
    w0 = time.time()
    t0 = time.perf_counter()
    kernels = 0
    recs = 0
    for _ in range(args.steps):
        k, recs = device_step(stages)
        kernels += k
    dev_dt = barrier_max(dist, time.perf_counter() - t0)
    clocks.window(w0, time.time())
    if any(t != e2e_texts[0] for t in e2e_texts + res_texts):
        raise RuntimeError("the streamed steps gave different records")
    if len(e2e_texts[0].splitlines()) != recs:
        raise RuntimeError("the streamed batches gave a different record count from the resident steps")
    out = {"value": n_reads * world * args.steps / res_dt, "ms_per_step": res_dt / args.steps * 1e3,
           "e2e": {"value": n_reads * world * args.steps / e2e_dt, "unit": "reads/s",
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "value_sequential": {"value": n_reads * world * args.steps / dev_dt, "unit": "reads/s",
                                "note": "the same steps one after the other on one context pair, no overlap"},
           "gpu_launches": kernels, "reads_per_step": n_reads * world, "records_per_step": recs,
           "stage_ms": {k: statistics.mean(s_[k] for s_ in stages) for k in stages[0]},
           "host_call_ms_per_step": {k: v / args.steps for k, v in host_ms.items()},
           "capacity": pair.tumor.capacity_stats()}
    # sites/s: region positions of both samples over the whole scoring stage
    # (device k_score plus the host's allele strings, MSI and record text)
    sites = 2 * sum(b - a + 1 for a, b in regions)
    score_stage_ms = (host_ms["score"] + host_ms["format"]) / args.steps
    out["sites_per_s"] = sites / (score_stage_ms * 1e-3)
    # the tumor's k_pileup_tiles launch, timed alone right after the timed
    # region on the same batch (in the timed steps both samples' kernels
    # share the GPU, one stream each)
    tile_ms_shared = statistics.mean(s_["pileup_tiles"] for s_ in stages[0::2])
    solo = []
    for _ in range(3):
        pair.tumor.pileup()
        solo.append(pair.tumor.stage_times()["pileup_tiles"])
    tile_ms = statistics.mean(solo)
    cells = sum(b - a + 1 for a, b in regions)
    window = sum(b - a + 1 + 2 * 1200 for a, b in regions)
    per_launch_bytes = read_alg_bytes(tumor) + cells * 256 + window  # reads + site records + reference windows
    achieved = per_launch_bytes / (tile_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    out["tumor_tile_launch"] = {"launch_ms": tile_ms, "reads": int(tumor.n), "achieved_gbs": achieved,
                                "frac": achieved / peak, "peak_kind": peak_kind}
    if roofline:
        traffic = PILEUP_TRAFFIC_PER_READ * tumor.n if PILEUP_TRAFFIC_PER_READ else None
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                           "kernel": "k_pileup_tiles", "launch": f"tumor sample, {tumor.n} reads, timed alone",
                           "alg_bytes_per_launch": per_launch_bytes, "launch_ms": tile_ms,
                           "launch_ms_sharing_gpu": tile_ms_shared}
    pair.close()
    for b in batches:
        b.close()
    out["text"] = e2e_texts[0]
    return out


def pair_1mb_leg(args, device: int) -> dict:
    """The 1 Mb somatic pair (tumor 200x + normal 100x): value and e2e as
    the headline, plus its BAM-decode leg."""
    from rabbitvar_gb300 import api  # noqa: F401
    g, tumor, normal, regions = make_workload()
    clocks = type("NoClocks", (), {"window": lambda self, a, b: None})()
    r = measure_pair(g, tumor, normal, regions, args, None, clocks, device, 1, roofline=False)
    out = {"workload": workload(args.local_realign), "value": r["value"], "e2e": r["e2e"]["value"],
           "unit": "reads/s", "ms_per_step": r["ms_per_step"], "reads_per_step": r["reads_per_step"],
           "records_per_step": r["records_per_step"], "host_call_ms_per_step": r["host_call_ms_per_step"],
           "tumor_tile_launch": r["tumor_tile_launch"]}
    if not args.no_bam:
        out["e2e_from_bam"] = bam_leg(g, tumor, normal, regions, args.local_realign, args.steps, args.warmup,
                                      device, r["text"])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--local-realign", "-k", type=int, default=1, choices=[0, 1],
                    help="the reference's -k (default 1, as the reference): 0 leaves out the realigner's indel passes")
    ap.add_argument("--no-other-k", action="store_true", help="skip the leg with the other -k setting")
    ap.add_argument("--no-bam", action="store_true", help="skip the leg that starts from BGZF-compressed BAM bytes")
    ap.add_argument("--no-1mb", action="store_true", help="skip the 1 Mb somatic pair leg")
    ap.add_argument("--no-panel", action="store_true", help="skip the 10,000-region amplicon panel leg")
    ap.add_argument("--regions", type=int, default=0, metavar="N",
                    help="run the headline on the first N regions of the panel only (for profiling)")
    ap.add_argument("--bam-decode", action="store_true",
                    help="only time the BAM decode of the tumor sample, GPU against the host decoder")
    ap.add_argument("--panel", type=int, default=0, metavar="N",
                    help="batched amplicon panel of N regions (-t -u): one launch for all regions vs one per region")
    args = ap.parse_args()
    rank, world, dist = dist_init()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.panel:
        run_panel(args)
        return
    if args.bam_decode:
        run_bam_decode(args)
        return
    local = int(os.environ.get("LOCAL_RANK", "0"))
    only = list(range(args.regions)) if args.regions else None
    t_gen = time.perf_counter()
    g, tumor, normal, regions = deep_workload(rank, world, only=only)
    print(f"bench: generated {tumor.n + normal.n} reads in {time.perf_counter() - t_gen:.1f} s", file=sys.stderr)
    clocks = Clocks(local)
    r = measure_pair(g, tumor, normal, regions, args, dist, clocks, local, world)
    clk = clocks.stop()
    text = r.pop("text")
    out = {
        "metric": METRIC,
        "value": r["value"], "unit": "reads/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32/fp64", "data": "synthetic (seeded)",
        "config": {"workload": deep_workload_name(args.local_realign, len(regions)),
                   "reads_per_step": r["reads_per_step"], "records_per_step": r["records_per_step"],
                   "l2": "inputs (~22 GB) larger than L2, no flush",
                   "regions_per_rank": len(regions),
                   "sharding": "regions LPT-partitioned across ranks (rabbitvar_gb300/shard.py), no collective"},
        "e2e": r["e2e"], "value_sequential": r["value_sequential"], "gpu_launches": r["gpu_launches"],
        "stage_ms": r["stage_ms"], "host_call_ms_per_step": r["host_call_ms_per_step"],
        "roofline": r["roofline"], "clocks": clk, "sites_per_s": r["sites_per_s"], "capacity": r["capacity"],
    }
    parity_ok = True
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle on four regions of the same reads, one core: the CPU
        # baseline, and the records check of the GPU's output for them
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from cmp import diff_records
        pr = [regions[i] for i in PARITY_REGIONS if i < len(regions)] if only is None and world == 1 else regions[:4]
        ora, nr, dt = oracle_regions(g, tumor, normal, pr, args.local_realign, threads=1)
        mine = region_records(text, "ctg", pr)
        problems = diff_records(ora.splitlines(), mine, somatic=True)
        parity_ok = not problems and len(mine) == len(ora.splitlines())
        out["parity"] = {"records_equal": parity_ok, "records": len(mine), "oracle_records": len(ora.splitlines()),
                         "regions": [f"ctg:{a}-{b}" for a, b in pr], "problems": problems[:3],
                         "against": "oracle (pinned to the reference binary) on the same reads"}
        out["cpu_baseline"] = {"value": nr / dt, "unit": "reads/s", "cores": 1, "kind": "port",
                               "sample": f"{len(pr)} of {len(regions)} regions, tumor+normal ({nr} reads, {dt:.1f} s)"}
    del text, tumor, normal
    if rank == 0 and not args.no_other_k:
        from types import SimpleNamespace
        a2 = SimpleNamespace(**vars(args))
        a2.local_realign = 1 - args.local_realign
        a2.steps = min(args.steps, 5)
        a2.warmup = min(args.warmup, 3)
        g2, t2, n2, regs2 = deep_workload(rank, world, only=only)
        nclk = type("NoClocks", (), {"window": lambda self, a, b: None})()
        r2 = measure_pair(g2, t2, n2, regs2, a2, None, nclk, local, 1, roofline=False)
        out["other_k"] = {"workload": deep_workload_name(a2.local_realign, len(regs2)), "value": r2["value"],
                          "e2e": r2["e2e"]["value"], "unit": "reads/s", "ms_per_step": r2["ms_per_step"],
                          "records_per_step": r2["records_per_step"], "steps": a2.steps, "warmup": a2.warmup,
                          "host_call_ms_per_step": r2["host_call_ms_per_step"]}
        del t2, n2
    if rank == 0 and not args.no_1mb:
        out["somatic_pair_1mb"] = pair_1mb_leg(args, local)
    if rank == 0 and not args.no_panel:
        out["panel"] = panel_leg(10_000, args.local_realign, min(args.steps, 3), min(args.warmup, 2), local)
        parity_ok = parity_ok and out["panel"]["records_equal_region_by_region"]
    if rank == 0 and not args.no_learned:
        out["learned_filter"] = learned_filter_leg()
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    if not parity_ok:
        sys.exit(1)


if __name__ == "__main__":
    main()
