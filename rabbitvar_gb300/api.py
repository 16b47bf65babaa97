"""Python front end of librvgpu (ctypes over the C ABI in include/rvgpu.h).

The call sequence mirrors the reference's per-region stages
(src/modes/simpleMode.cpp:18-64): submit a batch of reads and regions, pile
them up (CigarParser), realign MNPs (VariationRealigner), score sites
(ToVarsBuilder + isGoodVar + Fisher) and format the tab-delimited records
(SimpleMode::output).  Every error status raises RvError; nothing here
falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librvgpu.so")

STATUS = {0: "OK", -1: "ERR_ARG", -2: "ERR_CUDA", -3: "ERR_CAPACITY", -4: "ERR_TIMEOUT", -5: "ERR_UNSUPPORTED",
          -6: "ERR_STATE", -7: "ERR_COLLISION", -8: "ERR_FORMAT"}


class RvError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("goodq", C.c_double), ("vext", C.c_int32), ("mismatch", C.c_int32), ("local_realign", C.c_int32),
                ("freq", C.c_double), ("minr", C.c_int32), ("read_pos_filter", C.c_int32), ("qratio", C.c_double),
                ("mapq_filter", C.c_double), ("min_mapq", C.c_int32), ("lofreq", C.c_double), ("bias", C.c_double),
                ("min_bias_reads", C.c_int32), ("samfilter", C.c_int32), ("ref_extension", C.c_int32),
                ("extend_nt", C.c_int32), ("trim_bases_after", C.c_int32), ("minmatch", C.c_int32),
                ("dedup", C.c_int32), ("unique_fwd", C.c_int32), ("unique_first", C.c_int32),
                ("do_pileup", C.c_int32), ("fisher", C.c_int32), ("move_indels_3", C.c_int32),
                ("svminlen", C.c_int32), ("somatic", C.c_int32)]


class ReadBatch(C.Structure):
    _fields_ = [("n_reads", C.c_int64), ("pos", C.c_void_p), ("flag", C.c_void_p), ("mapq", C.c_void_p),
                ("mpos", C.c_void_p), ("nm", C.c_void_p), ("n_cigar", C.c_void_p), ("cig_off", C.c_void_p),
                ("cigar", C.c_void_p), ("n_cigar_words", C.c_int64), ("l_qseq", C.c_void_p),
                ("base_off", C.c_void_p), ("seq", C.c_void_p), ("qual", C.c_void_p), ("n_bases", C.c_int64)]


class Region(C.Structure):
    _fields_ = [("start", C.c_int32), ("end", C.c_int32)]


class SomaticJob(C.Structure):
    _fields_ = [("tumor", C.POINTER(ReadBatch)), ("normal", C.POINTER(ReadBatch)), ("regions", C.POINTER(Region)),
                ("n_regions", C.c_int), ("sample", C.c_char_p), ("gene", C.c_char_p)]


SomaticSink = C.CFUNCTYPE(None, C.c_void_p, C.c_int64, C.POINTER(C.c_char), C.c_size_t, C.c_int64)


class Candidate(C.Structure):
    _fields_ = [("region", C.c_int32), ("position", C.c_int32), ("hard_pass", C.c_int32), ("key_len", C.c_int32),
                ("key", C.c_char * 48)]


class SiteRecord(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in ("region", "position", "start", "end", "total_cov", "var_cov", "ref_fwd",
                                          "ref_rev", "alt_fwd", "alt_rev")] +
                [(n, C.c_double) for n in ("freq", "pmean", "qual", "mapq", "qratio", "hifreq", "extrafreq", "msi",
                                           "nm")] +
                [(n, C.c_int32) for n in ("pstd", "qstd", "shift3", "msint", "hicnt", "hicov")] +
                [("fisher_p", C.c_double), ("fisher_ratio", C.c_double)])


EXPORTS = ["rv_default_params", "rv_create", "rv_destroy", "rv_last_error", "rv_upload_reference",
           "rv_submit_batch", "rv_pileup", "rv_realign", "rv_score", "rv_format_records", "rv_fetch_records",
           "rv_call_regions", "rv_score_candidates", "rv_candidates", "rv_score_pair", "rv_pileup_realign_pair", "rv_format_somatic", "rv_call_somatic", "rv_call_somatic_stream", "rv_export_maps", "rv_last_timings", "rv_stage_times", "rv_set_pileup_graph", "rv_pileup_graph_stats", "rv_set_capacities", "rv_capacity_stats", "rv_io_bytes", "rv_fisher_batch", "rv_bam_read",
           "rv_bam_contigs", "rv_bam_batch", "rv_bam_read_mem", "rv_bam_read_gpu", "rv_bam_reread_gpu", "rv_bam_batch_host", "rv_bam_free", "rv_fasta_read", "rv_free", "rv_alloc_pinned",
           "rv_free_pinned", "rv_mlp_create", "rv_mlp_destroy", "rv_mlp_last_error", "rv_mlp_set_params",
           "rv_mlp_get_params", "rv_mlp_train", "rv_mlp_gradients", "rv_mlp_predict", "rv_mlp_step_ms"]

_lib = None


def lib():
    """Load librvgpu.so (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
    L.rv_default_params.argtypes = [C.POINTER(Params)]
    L.rv_create.argtypes = [C.POINTER(vp), C.POINTER(Params), C.c_int, sz]
    L.rv_destroy.argtypes = [vp]
    L.rv_last_error.argtypes = [vp]
    L.rv_last_error.restype = C.c_char_p
    L.rv_upload_reference.argtypes = [vp, C.c_char_p, C.c_char_p, i64]
    L.rv_submit_batch.argtypes = [vp, C.POINTER(ReadBatch), C.POINTER(Region), C.c_int, vp]
    L.rv_pileup.argtypes = [vp, vp]
    L.rv_realign.argtypes = [vp, vp]
    L.rv_score.argtypes = [vp, vp]
    L.rv_format_records.argtypes = [vp, C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(sz),
                                    C.POINTER(i64)]
    L.rv_fetch_records.argtypes = [vp, C.POINTER(SiteRecord), sz, C.POINTER(sz)]
    L.rv_score_pair.argtypes = [vp, vp]
    L.rv_pileup_realign_pair.argtypes = [vp, vp]
    L.rv_call_somatic_stream.argtypes = [vp, vp, vp, vp, C.POINTER(SomaticJob), i64, SomaticSink, vp]
    L.rv_score_candidates.argtypes = [vp, C.c_int]
    L.rv_candidates.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    L.rv_format_somatic.argtypes = [vp, vp, C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(sz),
                                    C.POINTER(i64)]
    L.rv_export_maps.argtypes = [vp, C.c_int, C.c_char_p, C.POINTER(vp), C.POINTER(sz)]
    L.rv_last_timings.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(i64)]
    L.rv_fisher_batch.argtypes = [vp, vp, i64, vp, vp]
    L.rv_stage_times.argtypes = [vp, vp, C.c_int]
    L.rv_set_pileup_graph.argtypes = [vp, C.c_int]
    L.rv_pileup_graph_stats.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
    L.rv_set_capacities.argtypes = [vp, sz, sz, sz, sz]
    L.rv_capacity_stats.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]
    L.rv_io_bytes.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
    L.rv_bam_read.argtypes = [C.c_char_p, C.c_int, C.POINTER(vp)]
    L.rv_bam_contigs.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(vp), C.POINTER(vp)]
    L.rv_bam_batch.argtypes = [vp, C.c_int, C.POINTER(ReadBatch)]
    L.rv_bam_read_gpu.argtypes = [vp, sz, C.c_int, C.POINTER(vp)]
    L.rv_bam_batch_host.argtypes = [vp, C.c_int, C.POINTER(ReadBatch)]
    L.rv_bam_reread_gpu.argtypes = [vp, vp, sz]
    L.rv_bam_read_mem.argtypes = [vp, sz, C.c_int, C.POINTER(vp)]
    L.rv_bam_free.argtypes = [vp]
    L.rv_fasta_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp), C.POINTER(i64)]
    L.rv_free.argtypes = [vp]
    L.rv_alloc_pinned.argtypes = [sz]
    L.rv_alloc_pinned.restype = vp
    L.rv_free_pinned.argtypes = [vp]
    _lib = L
    return L


def default_params(**kw) -> Params:
    p = Params()
    lib().rv_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Batch:
    """Host structure-of-arrays read batch (keeps its arrays alive).

    With pinned=True the arrays are allocated in page-locked memory."""

    FIELDS = [("pos", np.int32), ("flag", np.uint16), ("mapq", np.uint8), ("mpos", np.int32), ("nm", np.int32),
              ("n_cigar", np.uint16), ("cig_off", np.uint32), ("cigar", np.uint32), ("l_qseq", np.int32),
              ("base_off", np.uint64), ("seq", np.uint8), ("qual", np.uint8)]

    def __init__(self, arrays: dict, pinned: bool = False):
        self._pinned = []
        self.arrays = {}
        for name, dt in self.FIELDS:
            a = np.ascontiguousarray(arrays[name], dtype=dt)
            if pinned:
                ptr = lib().rv_alloc_pinned(max(a.nbytes, 1))
                if not ptr:
                    raise RvError(-2, "pinned allocation failed")
                self._pinned.append(ptr)
                buf = (C.c_uint8 * max(a.nbytes, 1)).from_address(ptr)
                b = np.frombuffer(buf, dtype=dt, count=a.size)
                b[...] = a
                a = b
            self.arrays[name] = a
        self.n_reads = int(self.arrays["pos"].size)
        self.n_bases = int(arrays.get("n_bases", self.arrays["qual"].size))
        self.nbytes = sum(a.nbytes for a in self.arrays.values())

    @classmethod
    def from_readset(cls, rs, pinned: bool = False) -> "Batch":
        arrs = dict(pos=rs.pos, flag=rs.flag, mapq=rs.mapq, mpos=rs.mpos, nm=rs.nm, n_cigar=rs.n_cigar,
                    cig_off=rs.cig_off, cigar=rs.cigar, l_qseq=rs.l_qseq, base_off=rs.base_off,
                    seq=rs.packed_seq(), qual=rs.qual, n_bases=rs.qual.size)
        return cls(arrs, pinned=pinned)

    def struct(self) -> ReadBatch:
        b = ReadBatch()
        b.n_reads = self.n_reads
        for name, _ in self.FIELDS:
            setattr(b, name, self.arrays[name].ctypes.data)
        b.n_cigar_words = int(self.arrays["cigar"].size)
        b.n_bases = self.n_bases
        return b

    def close(self):
        for p in self._pinned:
            lib().rv_free_pinned(p)
        self._pinned = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One GPU context (rv_ctx): device memory, stream, and the last results."""

    def __init__(self, params: Params | None = None, device: int = 0, budget: int = 0):
        self.L = lib()
        self.params = params or default_params(local_realign=0)
        self.h = C.c_void_p()
        st = self.L.rv_create(C.byref(self.h), C.byref(self.params), device, budget)
        self._check(st)

    def _check(self, st: int):
        if st != 0:
            msg = self.L.rv_last_error(self.h).decode() if self.h else ""
            raise RvError(st, msg)

    def close(self):
        if self.h:
            self.L.rv_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_reference(self, chr_name: str, bases: bytes):
        self._check(self.L.rv_upload_reference(self.h, chr_name.encode(), bases, len(bases)))

    def submit(self, batch: Batch, regions: list[tuple[int, int]]):
        # the batch's arrays stay referenced until the next submit: with -k 1
        # the realigner reads the alignments again from them
        self._batch = batch
        self._batch_struct = batch.struct()
        self._regions = (Region * max(len(regions), 1))(*[Region(a, b) for a, b in regions])
        self._check(self.L.rv_submit_batch(self.h, C.byref(self._batch_struct), self._regions, len(regions), None))

    def pileup(self):
        self._check(self.L.rv_pileup(self.h, None))

    def realign(self):
        self._check(self.L.rv_realign(self.h, None))

    def score(self):
        self._check(self.L.rv_score(self.h, None))

    def format_records(self, sample: str = "S", gene: str | None = None) -> tuple[str, int]:
        t = C.c_char_p()
        n = C.c_size_t()
        nrec = C.c_int64()
        self._check(self.L.rv_format_records(self.h, sample.encode(), gene.encode() if gene else None,
                                             C.byref(t), C.byref(n), C.byref(nrec)))
        return C.string_at(t, n.value).decode(), nrec.value

    def records(self) -> list[SiteRecord]:
        n = C.c_size_t()
        self._check(self.L.rv_fetch_records(self.h, None, 0, C.byref(n)))
        arr = (SiteRecord * max(n.value, 1))()
        self._check(self.L.rv_fetch_records(self.h, arr, n.value, C.byref(n)))
        return list(arr[:n.value])

    def call(self, batch: Batch, regions, sample: str = "S", gene: str | None = None) -> str:
        self.submit(batch, regions)
        self.pileup()
        self.realign()
        self.score()
        return self.format_records(sample, gene)[0]

    def export_maps(self, region: int = 0, stages: str = "P") -> str:
        t = C.c_void_p()
        n = C.c_size_t()
        self._check(self.L.rv_export_maps(self.h, region, stages.encode(), C.byref(t), C.byref(n)))
        return C.string_at(t, n.value).decode()

    def timings(self) -> dict:
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        k = C.c_int64()
        self._check(self.L.rv_last_timings(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(k)))
        return dict(pileup_ms=a.value, score_ms=b.value, total_ms=c.value, kernels=k.value)

    def io_bytes(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        self._check(self.L.rv_io_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    STAGES = ["reset", "region_spans", "pileup_tiles", "edge_walk", "deferred_link_check", "ins_adjust", "score",
              "pileup_variant"]

    def stage_times(self) -> dict:
        ms = np.zeros(8)
        self._check(self.L.rv_stage_times(self.h, ms.ctypes.data, 8))
        return {k: float(ms[i]) for i, k in enumerate(self.STAGES)}

    def set_pileup_graph(self, enable: bool = True):
        """rv_pileup launches its kernel chain as a CUDA graph once the
        kernel variant is settled."""
        self._check(self.L.rv_set_pileup_graph(self.h, int(bool(enable))))

    def pileup_graph_stats(self) -> tuple[int, int]:
        """(graph launches, graph instantiations) since the context was made."""
        a, b = C.c_int64(), C.c_int64()
        self._check(self.L.rv_pileup_graph_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_capacities(self, hash_slots: int = 0, arena_bytes: int = 0, deferred: int = 0, order_fix: int = 0):
        """Table capacities for the next submit (0 = automatic); a table that
        overflows grows and the pileup runs again."""
        self._check(self.L.rv_set_capacities(self.h, hash_slots, arena_bytes, deferred, order_fix))

    def capacity_stats(self) -> dict:
        r, h, a = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.L.rv_capacity_stats(self.h, C.byref(r), C.byref(h), C.byref(a)))
        return {"retries": r.value, "hash_slots": h.value, "arena_bytes": a.value}

    def score_candidates(self, min_count: int = 2):
        self._check(self.L.rv_score_candidates(self.h, min_count))

    def candidates(self):
        """Features [n][40] (float32) and the candidate table of the last
        scoring call: list of (region, position, key, hard_pass)."""
        n = C.c_int64()
        self._check(self.L.rv_candidates(self.h, None, None, 0, C.byref(n)))
        feats = np.zeros((max(n.value, 1), 40), np.float32)
        arr = (Candidate * max(n.value, 1))()
        self._check(self.L.rv_candidates(self.h, feats.ctypes.data, arr, n.value, C.byref(n)))
        table = [(c.region, c.position, c.key.decode(), c.hard_pass) for c in arr[:n.value]]
        return feats[:n.value], table

    def fisher(self, tables: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        t = np.ascontiguousarray(tables, dtype=np.int32).reshape(-1, 4)
        p = np.zeros(t.shape[0])
        r = np.zeros(t.shape[0])
        self._check(self.L.rv_fisher_batch(self.h, t.ctypes.data, t.shape[0], p.ctypes.data, r.ctypes.data))
        return p, r


class SomaticPair:
    """Somatic mode (a tumor/normal pair, the reference's `-b 'T.bam|N.bam'`):
    one context per sample, created with somatic = 1, sharing the contig and
    the region list."""

    def __init__(self, params: Params | None = None, device: int = 0, budget: int = 0):
        p = params or default_params(local_realign=0)
        p.somatic = 1
        self.tumor = Context(p, device, budget)
        self.normal = Context(p, device, budget)

    def close(self):
        self.tumor.close()
        self.normal.close()

    def upload_reference(self, chr_name: str, bases: bytes):
        self.tumor.upload_reference(chr_name, bases)
        self.normal.upload_reference(chr_name, bases)

    def submit(self, tumor: Batch, normal: Batch, regions):
        self.tumor.submit(tumor, regions)
        self.normal.submit(normal, regions)

    def pileup(self):
        self.tumor.pileup()
        self.normal.pileup()

    def realign(self):
        self.tumor.realign()
        self.normal.realign()

    def pileup_realign(self):
        """pileup() then realign(), overlapped: the tumor's host realigner
        runs while the normal's pileup kernels are on the device."""
        self.tumor._check(self.tumor.L.rv_pileup_realign_pair(self.tumor.h, self.normal.h))

    def score(self):
        self.tumor._check(self.tumor.L.rv_score_pair(self.tumor.h, self.normal.h))

    def format_records(self, sample: str = "T", gene: str | None = None) -> tuple[str, int]:
        t = C.c_char_p()
        n = C.c_size_t()
        nrec = C.c_int64()
        self.tumor._check(self.tumor.L.rv_format_somatic(self.tumor.h, self.normal.h, sample.encode(),
                                                         gene.encode() if gene else None, C.byref(t), C.byref(n),
                                                         C.byref(nrec)))
        return C.string_at(t, n.value).decode(), nrec.value

    def call(self, tumor: Batch, normal: Batch, regions, sample: str = "T", gene: str | None = None) -> str:
        self.submit(tumor, normal, regions)
        self.pileup()
        self.realign()
        self.score()
        return self.format_records(sample, gene)[0]


class SomaticStream:
    """Somatic calling over a sequence of batches with two tumor/normal
    context pairs (rv_call_somatic_stream): while one pair's records are
    formatted on a host thread, the other pair's next batch is uploaded and
    piled up.  The records are those of one SomaticPair.call per batch."""

    def __init__(self, params: Params | None = None, device: int = 0, budget: int = 0):
        self.pairs = [SomaticPair(params, device, budget), SomaticPair(params, device, budget)]

    def close(self):
        for p in self.pairs:
            p.close()

    def upload_reference(self, chr_name: str, bases: bytes):
        for p in self.pairs:
            p.upload_reference(chr_name, bases)

    def run(self, jobs, sample: str = "T", gene: str | None = None) -> list[str]:
        """jobs: (tumor Batch, normal Batch, regions) per batch; returns the
        record text of each, in order."""
        keep = []
        arr = (SomaticJob * max(1, len(jobs)))()
        for i, (tb, nb, regions) in enumerate(jobs):
            # (None, None, regions): run again on the batch the pair holds
            ts = tb.struct() if tb is not None else None
            ns = nb.struct() if nb is not None else None
            rg = (Region * max(len(regions), 1))(*[Region(a, b) for a, b in regions])
            keep += [ts, ns, rg]
            arr[i] = SomaticJob(C.pointer(ts) if ts is not None else C.POINTER(ReadBatch)(),
                                C.pointer(ns) if ns is not None else C.POINTER(ReadBatch)(),
                                C.cast(rg, C.POINTER(Region)), len(regions),
                                sample.encode(), gene.encode() if gene else None)
        out = [None] * len(jobs)

        def sink(_user, k, text, n, _nrec):
            out[k] = C.string_at(text, n).decode()

        cb = SomaticSink(sink)
        t0, n0 = self.pairs[0].tumor, self.pairs[0].normal
        t1, n1 = self.pairs[1].tumor, self.pairs[1].normal
        t0._check(t0.L.rv_call_somatic_stream(t0.h, n0.h, t1.h, n1.h, arr, len(jobs), cb, None))
        return out


def _host_batches(L, h, batch_fn):
    n = C.c_int()
    names = C.c_void_p()
    lens = C.c_void_p()
    L.rv_bam_contigs(h, C.byref(n), C.byref(names), C.byref(lens))
    nm = [C.cast(names, C.POINTER(C.c_char_p))[i].decode() for i in range(n.value)]
    ln = [C.cast(lens, C.POINTER(C.c_int32))[i] for i in range(n.value)]
    out = {}
    for tid in range(n.value):
        rb = ReadBatch()
        st = batch_fn(h, tid, C.byref(rb))
        if st != 0:
            raise RvError(st, "rv_bam_batch")
        nr = rb.n_reads

        def arr(ptr, dt, count):
            if count == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         shape=(count,)).copy()
        arrays = dict(pos=arr(rb.pos, np.int32, nr), flag=arr(rb.flag, np.uint16, nr),
                      mapq=arr(rb.mapq, np.uint8, nr), mpos=arr(rb.mpos, np.int32, nr),
                      nm=arr(rb.nm, np.int32, nr), n_cigar=arr(rb.n_cigar, np.uint16, nr),
                      cig_off=arr(rb.cig_off, np.uint32, nr), cigar=arr(rb.cigar, np.uint32, rb.n_cigar_words),
                      l_qseq=arr(rb.l_qseq, np.int32, nr), base_off=arr(rb.base_off, np.uint64, nr),
                      seq=arr(rb.seq, np.uint8, (rb.n_bases + 1) // 2), qual=arr(rb.qual, np.uint8, rb.n_bases),
                      n_bases=rb.n_bases)
        out[tid] = Batch(arrays)
    return nm, ln, out


def read_bam(path: str, threads: int = 0):
    """Decode a BAM file with the library's host decoder; returns
    (contig names, lengths, {tid: Batch}) with copies of the arrays."""
    L = lib()
    h = C.c_void_p()
    st = L.rv_bam_read(path.encode(), threads, C.byref(h))
    if st != 0:
        raise RvError(st, f"cannot decode {path}")
    try:
        return _host_batches(L, h, L.rv_bam_batch)
    finally:
        L.rv_bam_free(h)


class DeviceBatch:
    """A read batch of a BAM decoded on the GPU: bases and qualities in device
    memory, the other arrays in pinned host memory (owned by the DeviceBam)."""

    def __init__(self, owner: "DeviceBam", rb: ReadBatch):
        self._owner = owner
        self._rb = rb
        self.n_reads = int(rb.n_reads)
        self.n_bases = int(rb.n_bases)
        self.nbytes = 0

    def struct(self) -> ReadBatch:
        return self._rb


class DeviceBam:
    """BGZF/BAM decode on the GPU (rv_bam_read_gpu) of a file's bytes."""

    def __init__(self, data: bytes | str, device: int = 0):
        self.L = lib()
        if isinstance(data, str):
            with open(data, "rb") as f:
                data = f.read()
        self.compressed_bytes = len(data)
        ptr = self.L.rv_alloc_pinned(max(len(data), 1))
        if not ptr:
            raise RvError(-2, "pinned allocation failed")
        try:
            C.memmove(ptr, data, len(data))
            self.h = C.c_void_p()
            st = self.L.rv_bam_read_gpu(ptr, len(data), device, C.byref(self.h))
        finally:
            self.L.rv_free_pinned(ptr)
        if st != 0:
            raise RvError(st, "rv_bam_read_gpu")
        n = C.c_int()
        names = C.c_void_p()
        lens = C.c_void_p()
        self.L.rv_bam_contigs(self.h, C.byref(n), C.byref(names), C.byref(lens))
        self.names = [C.cast(names, C.POINTER(C.c_char_p))[i].decode() for i in range(n.value)]
        self.lens = [C.cast(lens, C.POINTER(C.c_int32))[i] for i in range(n.value)]

    def reread(self, data: bytes, pinned_ptr: int | None = None):
        """Decode another file into this handle's buffers (earlier batches
        become invalid); `pinned_ptr` may point at a pinned copy of `data`."""
        ptr = pinned_ptr
        if ptr is None:
            ptr = self.L.rv_alloc_pinned(max(len(data), 1))
            if not ptr:
                raise RvError(-2, "pinned allocation failed")
            C.memmove(ptr, data, len(data))
        try:
            st = self.L.rv_bam_reread_gpu(self.h, ptr, len(data))
        finally:
            if pinned_ptr is None:
                self.L.rv_free_pinned(ptr)
        if st != 0:
            raise RvError(st, "rv_bam_reread_gpu")

    def batch(self, tid: int = 0) -> DeviceBatch:
        rb = ReadBatch()
        st = self.L.rv_bam_batch(self.h, tid, C.byref(rb))
        if st != 0:
            raise RvError(st, "rv_bam_batch")
        return DeviceBatch(self, rb)

    def host_batches(self):
        """(names, lengths, {tid: Batch}) with host copies of every array."""
        return _host_batches(self.L, self.h, self.L.rv_bam_batch_host)

    def close(self):
        if self.h:
            self.L.rv_bam_free(self.h)
            self.h = C.c_void_p()


def read_fasta(path: str, name: str | None = None) -> bytes:
    L = lib()
    p = C.c_void_p()
    n = C.c_int64()
    st = L.rv_fasta_read(path.encode(), name.encode() if name else None, C.byref(p), C.byref(n))
    if st != 0:
        raise RvError(st, f"cannot read {path}")
    try:
        return C.string_at(p, n.value)
    finally:
        L.rv_free(p)
