"""Benchmark: reads/s of pileup + variant scoring on one GB300.

Workload (the somatic-pair shape the reference's metric is quoted on): a
seeded synthetic 1 Mb contig, tumor 200x + normal 100x 2x150 bp pairs
(~2.0 M reads), germline SNVs 1e-3/bp and indels 1e-4/bp in both samples,
somatic SNV/MNV 2e-5/bp (VAF U(0.01, 0.5)) and strand-biased artifacts
5e-6/bp in the tumor, called in somatic mode (the reference's
`-b 'T.bam|N.bam' -N 'T|N' --fisher`) over 100 BED tiles of 10 kb with -k 0:
both samples through the full per-region path (record filters, CIGAR walk,
allele maps, MNP realignment, site statistics), then the tumor/normal
classification, the hard filter, three Fisher tests per record and the
63-column record text.  One step = both samples, all regions.

    value : reads/s with the read batches already resident in HBM
    e2e   : reads/s through the C ABI from pinned host batches, including
            the host->device copy of the reads and the device->host copy of
            the scored candidates every step
Inputs (~0.5 GB of reads) exceed the 129 MB L2, so no flush is needed
between steps.

    e2e_from_bam : reads/s from BGZF-compressed BAM bytes in pinned host
            memory: the BAM decode on the GPU, then the same calls

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
    python bench.py --bam-decode      # BAM decode alone, GPU vs host decoder
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
METRIC = "reads/s pileup+var scoring (somatic pair 1 Mb, T200x+N100x)"
CPU_TILES = 40   # CPU sample: 40 of the 100 tiles (~0.8 M reads, ~10 s on one core)
# DRAM bytes (read + write) of one tumor-sample k_pileup_tiles<640, 3> launch
# of this workload, from one ncu capture each (by -k:
# profiles/k_pileup_tiles_somatic1mb.md, profiles/k_pileup_tiles_somatic1mb_k1.md)
PILEUP_TRAFFIC = {0: 1301.5e6, 1: 1627.2e6}


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
    """The learned filter against the hard filter on the deep-panel shape:
    trained on 4 seeded panels, evaluated on 2 held-out ones (planted truth),
    F1 and precision at the hard filter's recall, plus the training step
    time and the inference rate (candidates/s, features already built)."""
    from rabbitvar_gb300 import learn, mlp
    xtr, ytr, _ = learn.dataset([101, 102, 103, 104], n_regions=6)
    xte, yte, hte = learn.dataset([201, 202], n_regions=6)
    m = mlp.Mlp(batch=4096, seed=3)
    t0 = time.perf_counter()
    m.train(xtr, ytr, epochs=20, lr=1e-3)
    train_s = time.perf_counter() - t0
    m.predict(xte)
    t0 = time.perf_counter()
    scores = m.predict(xte)
    pred_s = time.perf_counter() - t0
    res = learn.compare(scores, yte, hte)
    res.update({"train_candidates": int(len(ytr)), "epochs": 20, "train_s": train_s,
                "train_step_ms": m.step_ms(), "predict_candidates_per_s": len(yte) / pred_s,
                "network": "40-128-128-128-1 GELU, BF16 tcgen05 GEMMs, FP32 accumulate, Adam",
                "data": "synthetic deep panels (6 x 5 kb at 1500x, C>A artifacts 1e-4/base at Q20, planted truth)"})
    m.close()
    return res


def run_panel(args):
    """Batched amplicon panel (the 10,000-region shape, scaled to N regions):
    region lengths U(100, 2000), depth log-normal median 500x, amplicon
    reads with 0.5% exact duplicates, -t -u, simple mode.  Batched: all
    regions in one submit and one persistent pileup launch; region by
    region: one submit + pipeline per region (the reference's per-region
    stage sequence).  Both through the C ABI from pinned host batches."""
    import numpy as np
    from rabbitvar_gb300 import api, synth
    n_reg = args.panel
    g, _, rs, regions = synth.amplicon_panel(n_regions=n_reg, genome_len=n_reg * 5000)
    params = api.default_params(local_realign=args.local_realign, dedup=1, unique_fwd=1)
    ctx = api.Context(params)
    ctx.upload_reference(rs.contig, synth.genome_str(g).encode())
    # the pileup chain as a CUDA graph (updated per batch), in both legs
    ctx.set_pileup_graph(True)
    batch = api.Batch.from_readset(rs, pinned=True)
    span = rs.pos.astype(np.int64) + 150
    subs = []
    for a, b in regions:
        idx = np.nonzero((rs.pos < b) & (span > a - 1 - 200))[0]
        subs.append(api.Batch.from_readset(synth.take(rs, idx), pinned=True))

    def batched():
        ctx.submit(batch, regions)
        ctx.pileup()
        ctx.realign()
        ctx.score()
        return ctx.format_records("S", rs.contig)[0]

    def per_region():
        out = []
        for r, b in zip(regions, subs):
            ctx.submit(b, [r])
            ctx.pileup()
            ctx.realign()
            ctx.score()
            out.append(ctx.format_records("S", rs.contig)[0])
        return "".join(out)

    for _ in range(args.warmup):
        t_b = batched()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t_b = batched()
    dt_b = (time.perf_counter() - t0) / args.steps
    t_r = per_region()
    t0 = time.perf_counter()
    t_r = per_region()
    dt_r = time.perf_counter() - t0
    same = sorted(t_b.splitlines()) == sorted(t_r.splitlines())
    out = {"metric": f"reads/s batched amplicon panel ({n_reg} regions, -t -u)", "value": rs.n / dt_b,
           "unit": "reads/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt_b * 1e3, "higher_is_better": True, "data": "synthetic",
           "config": {"workload": f"{n_reg} regions U(100,2000) bp, depth lognormal median 500x, amplicon 2x150, "
                                  f"0.5% PCR duplicates, -t -u -k {args.local_realign}, simple mode", "reads": int(rs.n)},
           "region_by_region": {"value": rs.n / dt_r, "unit": "reads/s", "ms": dt_r * 1e3},
           "speedup_batched": dt_r / dt_b, "records": len(t_b.splitlines()), "records_equal": same,
           "pileup_graph": dict(zip(("launches", "instantiations"), ctx.pileup_graph_stats()))}
    print(json.dumps(out))
    ctx.close()


def run_reference(args, rank):
    if rank != 0:
        return
    g, tumor, normal, regions = make_workload()
    threads = os.cpu_count() or 1
    n_reg = CPU_TILES
    vals = []
    for _ in range(args.warmup):
        cpu_baseline_run(g, tumor, normal, regions, threads, n_reg, args.local_realign)
    for _ in range(args.steps):
        v, dt, nr = cpu_baseline_run(g, tumor, normal, regions, threads, n_reg, args.local_realign)
        vals.append(v)
    v = statistics.median(vals)
    out = {"impl": "reference", "metric": METRIC,
           "value": v, "unit": "reads/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "data": "synthetic",
           "config": {"workload": workload(args.local_realign), "sample": f"first {n_reg} of 100 tiles, both samples"},
           "cpu_baseline": {"value": v, "unit": "reads/s", "cores": threads, "kind": "port",
                            "sample": f"first {n_reg} of 100 10-kb tiles, tumor+normal ({nr} reads), per step"},
           "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


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
    import numpy as np
    from rabbitvar_gb300 import api, synth
    local = int(os.environ.get("LOCAL_RANK", "0"))
    g, tumor, normal, regions = make_workload(seed_offset=rank)
    samples = [("T", tumor), ("N", normal)]
    params = api.default_params(local_realign=args.local_realign, fisher=1)
    pair = api.SomaticPair(params, device=local)
    pair.upload_reference(tumor.contig, synth.genome_str(g).encode())
    ctxs = [pair.tumor, pair.normal]
    batches = [api.Batch.from_readset(rs, pinned=True) for _, rs in samples]
    n_reads = sum(rs.n for _, rs in samples)
    alg_read_bytes = sum(read_alg_bytes(rs) for _, rs in samples)

    host_ms = {"pileup+realign": 0.0, "score": 0.0, "format": 0.0}

    def kernels_of():
        return sum(c.timings()["kernels"] for c in ctxs)

    def device_step(collect=None):
        t0 = time.perf_counter()
        pair.pileup_realign()
        t2 = time.perf_counter()
        pair.score()
        t3 = time.perf_counter()
        text, n = pair.format_records("T", "ctg")
        t4 = time.perf_counter()
        if collect is not None:
            host_ms["pileup+realign"] += (t2 - t0) * 1e3
            host_ms["score"] += (t3 - t2) * 1e3
            host_ms["format"] += (t4 - t3) * 1e3
            collect.extend(c.stage_times() for c in ctxs)
        return kernels_of(), n

    io = {"h2d": 0, "d2h": 0}
    # e2e: a stream of batches through rv_call_somatic_stream (two context
    # pairs: one pair's records are formatted on a host thread while the
    # other pair's next batch is uploaded and piled up); every step uploads
    # its pinned host batches and reads back its records
    stream = api.SomaticStream(params, device=local)
    stream.upload_reference(tumor.contig, synth.genome_str(g).encode())
    job = (batches[0], batches[1], regions)
    clocks = Clocks(local)
    stream.run([job] * max(1, args.warmup), "T", "ctg")
    w0 = time.time()
    t0 = time.perf_counter()
    e2e_texts = stream.run([job] * args.steps, "T", "ctg")
    e2e_dt = barrier_max(dist, time.perf_counter() - t0)
    clocks.window(w0, time.time())
    last = stream.pairs[(args.steps - 1) % 2]
    io["h2d"] = sum(c.io_bytes()[0] for c in (last.tumor, last.normal))
    io["d2h"] = sum(c.io_bytes()[1] for c in (last.tumor, last.normal))
    # value: the same stream on the batches both pairs now hold (inputs
    # resident in HBM; no upload in the timed region)
    resident = (None, None, regions)
    stream.run([resident] * max(1, args.warmup), "T", "ctg")
    w0 = time.time()
    t0 = time.perf_counter()
    res_texts = stream.run([resident] * args.steps, "T", "ctg")
    res_dt = barrier_max(dist, time.perf_counter() - t0)
    clocks.window(w0, time.time())
    stream.close()
    pair.submit(batches[0], batches[1], regions)
    # the same steps one after the other on one pair (no overlap between
    # steps): stage times, launch counts, and `value_sequential`
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
    clk = clocks.stop()
    if any(len(t.splitlines()) != recs for t in e2e_texts + res_texts):
        raise RuntimeError("the streamed batches gave a different record count from the resident steps")
    ms_per_step = res_dt / args.steps * 1e3
    value = n_reads * world * args.steps / res_dt
    value_seq = n_reads * world * args.steps / dev_dt
    e2e = n_reads * world * args.steps / e2e_dt
    # roofline of the dominant kernel: the tumor sample's k_pileup_tiles
    # launch (1.33 M reads), event-timed on its stream.  In the timed steps
    # the two samples' kernels share the GPU (one stream each), so the launch
    # is also timed alone, right after the timed region, on the same batch.
    tile_ms_shared = statistics.mean(s["pileup_tiles"] for s in stages[0::2])
    solo = []
    for _ in range(3):
        pair.tumor.pileup()
        solo.append(pair.tumor.stage_times()["pileup_tiles"])
    tile_ms = statistics.mean(solo)
    cells = sum(r[1] - r[0] + 1 for r in regions)
    per_launch_bytes = read_alg_bytes(tumor) + cells * 256 + CONTIG  # reads + site records + reference window
    achieved = per_launch_bytes / (tile_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    h2d = sum(b.nbytes for b in batches)
    out = {
        "metric": METRIC,
        "value": value, "unit": "reads/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32/fp64", "data": "synthetic (seeded)",
        "config": {"workload": workload(args.local_realign), "reads_per_step": n_reads * world, "l2": "inputs (~0.5 GB) larger than L2, no flush",
                   "records_per_step": recs},
        "e2e": {"value": e2e, "unit": "reads/s", "h2d_bytes_per_step": io["h2d"],
                "d2h_bytes_per_step": io["d2h"]},
        "value_sequential": {"value": value_seq, "unit": "reads/s",
                             "note": "the same steps one after the other on one context pair, no overlap"},
        "gpu_launches": kernels,
        "stage_ms": {k: statistics.mean(s[k] for s in stages) for k in stages[0]},
        "host_call_ms_per_step": {k: v / args.steps for k, v in host_ms.items()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": PILEUP_TRAFFIC[args.local_realign], "peak_kind": peak_kind,
                     "kernel": "k_pileup_tiles", "launch": "tumor sample, 1.33 M reads, timed alone",
                     "alg_bytes_per_launch": per_launch_bytes, "launch_ms": tile_ms,
                     "launch_ms_sharing_gpu": tile_ms_shared},
        "clocks": clk,
    }
    # sites/s: region positions of both samples scored per second of k_score
    score_ms = statistics.mean(s["score"] for s in stages)
    out["sites_per_s"] = (sum(r[1] - r[0] + 1 for r in regions)) / (score_ms * 1e-3)
    pair.close()
    if rank == 0 and not args.no_bam:
        out["e2e_from_bam"] = bam_leg(g, tumor, normal, regions, args.local_realign, args.steps, args.warmup, local,
                                      e2e_texts[0])
    if rank == 0 and not args.no_other_k:
        out["other_k"] = other_k_leg(g, tumor, normal, regions, 1 - args.local_realign, args.steps,
                                     args.warmup, local)
    if rank == 0 and not args.no_learned:
        out["learned_filter"] = learned_filter_leg()
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, nr = cpu_baseline_run(g, tumor, normal, regions, 1, CPU_TILES, args.local_realign)
        out["cpu_baseline"] = {"value": v, "unit": "reads/s", "cores": 1, "kind": "port",
                               "sample": f"first {CPU_TILES} of 100 10-kb tiles, tumor+normal ({nr} reads, {dt:.1f} s)"}
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
