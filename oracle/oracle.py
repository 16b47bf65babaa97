"""Oracle test infrastructure -- not part of the product.

ctypes front end to the CPU restatement in rv_oracle.cpp (built by
oracle/Makefile into oracle/_ref/librvoracle.so) and to the reference's own
binaries in oracle/_ref/ (built from the unmodified reference sources; present
only where the reference tree was available at build time).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(REF_DIR, "librvoracle.so")
REF_BIN = os.path.join(REF_DIR, "RabbitVar")
REF_DUMP = os.path.join(REF_DIR, "rvref_dump")


class Reads(C.Structure):
    _fields_ = [("n", C.c_int64), ("pos", C.c_void_p), ("flag", C.c_void_p), ("mapq", C.c_void_p),
                ("mpos", C.c_void_p), ("nm", C.c_void_p), ("n_cigar", C.c_void_p), ("cig_off", C.c_void_p),
                ("cigar", C.c_void_p), ("l_qseq", C.c_void_p), ("base_off", C.c_void_p), ("seq4", C.c_void_p),
                ("qual", C.c_void_p)]


class Params(C.Structure):
    _fields_ = [("goodq", C.c_double), ("vext", C.c_int), ("mismatch", C.c_int), ("local_realign", C.c_int),
                ("freq", C.c_double), ("minr", C.c_int), ("read_pos_filter", C.c_int), ("qratio", C.c_double),
                ("mapq_filter", C.c_double), ("min_mapq", C.c_int), ("lofreq", C.c_double), ("bias", C.c_double),
                ("min_bias_reads", C.c_int), ("samfilter", C.c_int), ("ref_extension", C.c_int),
                ("extend_nt", C.c_int), ("trim_bases_after", C.c_int), ("minmatch", C.c_int), ("dedup", C.c_int),
                ("unique_fwd", C.c_int), ("unique_first", C.c_int), ("do_pileup", C.c_int), ("fisher", C.c_int),
                ("move_indels_3", C.c_int), ("svminlen", C.c_int)]


_lib = None


def build() -> None:
    """Compile the oracle library (and the reference binaries when the
    reference tree is present)."""
    targets = ["oracle"]
    if os.path.isdir("/root/reference/src"):
        targets.append("ref")
    subprocess.run(["make", "-s", "-j8"] + targets, cwd=HERE, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-j8", "oracle"], cwd=HERE, check=True)
        L = C.CDLL(LIB_PATH)
        L.rvo_default_params.argtypes = [C.POINTER(Params)]
        L.rvo_run_region.argtypes = [C.POINTER(Reads), C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int,
                                     C.c_char_p, C.POINTER(Params), C.c_char_p, C.POINTER(C.c_void_p),
                                     C.POINTER(C.c_size_t)]
        L.rvo_run_regions.argtypes = [C.POINTER(Reads), C.c_char_p, C.c_int, C.c_char_p, C.c_void_p, C.c_void_p,
                                      C.c_int, C.c_char_p, C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_size_t)]
        L.rvo_run_regions.restype = C.c_long
        L.rvo_run_somatic.argtypes = [C.POINTER(Reads), C.POINTER(Reads), C.c_char_p, C.c_int, C.c_char_p, C.c_int,
                                      C.c_int, C.c_char_p, C.POINTER(Params), C.c_char_p, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_size_t)]
        L.rvo_run_somatic_regions.argtypes = [C.POINTER(Reads), C.POINTER(Reads), C.c_char_p, C.c_int, C.c_char_p,
                                              C.c_void_p, C.c_void_p, C.c_int, C.c_char_p, C.POINTER(Params),
                                              C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        L.rvo_run_somatic_regions.restype = C.c_long
        L.rvo_free.argtypes = [C.c_void_p]
        L.rvo_fisher.argtypes = [C.c_int] * 4 + [C.POINTER(C.c_double)] * 3
        L.rvo_fisher.restype = C.c_double
        _lib = L
    return _lib


def default_params(**kw) -> Params:
    p = Params()
    lib().rvo_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _reads_struct(rs, keep: list) -> Reads:
    arrs = dict(pos=np.ascontiguousarray(rs.pos, np.int32), flag=np.ascontiguousarray(rs.flag, np.uint16),
                mapq=np.ascontiguousarray(rs.mapq, np.uint8), mpos=np.ascontiguousarray(rs.mpos, np.int32),
                nm=np.ascontiguousarray(rs.nm, np.int32), n_cigar=np.ascontiguousarray(rs.n_cigar, np.uint16),
                cig_off=np.ascontiguousarray(rs.cig_off, np.uint32), cigar=np.ascontiguousarray(rs.cigar, np.uint32),
                l_qseq=np.ascontiguousarray(rs.l_qseq, np.int32), base_off=np.ascontiguousarray(rs.base_off, np.uint64),
                seq4=np.ascontiguousarray(rs.seq4, np.uint8), qual=np.ascontiguousarray(rs.qual, np.uint8))
    keep.append(arrs)
    r = Reads()
    r.n = rs.n
    for k, a in arrs.items():
        setattr(r, k, a.ctypes.data)
    return r


def _genome_bytes(genome) -> bytes:
    if isinstance(genome, (bytes, bytearray)):
        return bytes(genome)
    return np.frombuffer(b"ACGT", dtype=np.uint8)[genome].tobytes()


def run_region(rs, genome, start: int, end: int, stages: str = "PRVO", sample: str = "S",
               params: Params | None = None) -> str:
    """Run the restated pipeline on region [start, end] (1-based)."""
    keep: list = []
    r = _reads_struct(rs, keep)
    g = _genome_bytes(genome)
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_size_t()
    lib().rvo_run_region(C.byref(r), g, len(g), rs.contig.encode(), start, end, sample.encode(), C.byref(p),
                         stages.encode(), C.byref(out), C.byref(n))
    s = C.string_at(out, n.value).decode()
    lib().rvo_free(out)
    return s


def run_regions(rs, genome, regions, sample: str = "S", params: Params | None = None, threads: int = 1):
    keep: list = []
    r = _reads_struct(rs, keep)
    g = _genome_bytes(genome)
    p = params or default_params()
    st = np.ascontiguousarray([a for a, _ in regions], np.int32)
    en = np.ascontiguousarray([b for _, b in regions], np.int32)
    out = C.c_void_p()
    n = C.c_size_t()
    cnt = lib().rvo_run_regions(C.byref(r), g, len(g), rs.contig.encode(), st.ctypes.data, en.ctypes.data,
                                len(regions), sample.encode(), C.byref(p), threads, C.byref(out), C.byref(n))
    s = C.string_at(out, n.value).decode()
    lib().rvo_free(out)
    return cnt, s


def run_somatic(tumor, normal, genome, start: int, end: int, stages: str = "O", sample: str = "T",
                params: Params | None = None) -> str:
    """Somatic mode on region [start, end] (1-based) of a tumor/normal pair."""
    keep: list = []
    rt = _reads_struct(tumor, keep)
    rn = _reads_struct(normal, keep)
    g = _genome_bytes(genome)
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_size_t()
    lib().rvo_run_somatic(C.byref(rt), C.byref(rn), g, len(g), tumor.contig.encode(), start, end, sample.encode(),
                          C.byref(p), stages.encode(), C.byref(out), C.byref(n))
    s = C.string_at(out, n.value).decode()
    lib().rvo_free(out)
    return s


def run_somatic_regions(tumor, normal, genome, regions, sample: str = "T", params: Params | None = None,
                        threads: int = 1):
    keep: list = []
    rt = _reads_struct(tumor, keep)
    rn = _reads_struct(normal, keep)
    g = _genome_bytes(genome)
    p = params or default_params()
    st = np.ascontiguousarray([a for a, _ in regions], np.int32)
    en = np.ascontiguousarray([b for _, b in regions], np.int32)
    out = C.c_void_p()
    n = C.c_size_t()
    cnt = lib().rvo_run_somatic_regions(C.byref(rt), C.byref(rn), g, len(g), tumor.contig.encode(), st.ctypes.data,
                                        en.ctypes.data, len(regions), sample.encode(), C.byref(p), threads,
                                        C.byref(out), C.byref(n))
    s = C.string_at(out, n.value).decode()
    lib().rvo_free(out)
    return cnt, s


def fisher(a: int, b: int, c: int, d: int):
    l, r, t = C.c_double(), C.c_double(), C.c_double()
    lib().rvo_fisher(a, b, c, d, C.byref(l), C.byref(r), C.byref(t))
    return l.value, r.value, t.value


def have_reference() -> bool:
    return os.path.exists(REF_DUMP) and os.path.exists(REF_BIN)


def reference_dump(fasta: str, bam: str, region: str, extra: list[str] | None = None, stages: str = "PRV") -> str:
    cmd = [REF_DUMP, "-G", fasta, "-b", bam, "-R", region, "-stage", stages] + (extra or [])
    return subprocess.run(cmd, check=True, capture_output=True, text=True).stdout


def reference_records(fasta: str, bam: str, region: str, out_path: str, extra: list[str] | None = None,
                      sample: str = "S") -> list[str]:
    """Records of the reference binary; `bam` may be a 'T.bam|N.bam' pair with
    `sample` 'T|N' (somatic mode)."""
    cmd = [REF_BIN, "-G", fasta, "-b", bam, "-N", sample, "-R", region, "--out", out_path] + (extra or [])
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    with open(out_path) as f:
        return f.read().splitlines()
