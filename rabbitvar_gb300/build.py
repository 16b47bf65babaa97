"""In-tree build of librvgpu.so for sm_103a (nvcc + g++, compiled in parallel).

    python -m rabbitvar_gb300.build        # or rabbitvar_gb300.build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librvgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["rv_pileup.cu", "rv_score.cu", "rv_util.cu", "rv_prep.cu", "rv_noalloc.cu", "rv_mlp.cu", "rv_bgzf.cu"]
CPP = ["rv_capi.cpp", "rv_host.cpp", "rv_realign.cpp", "rv_records.cpp", "rv_somatic.cpp", "rv_bam.cpp", "rv_pool.cpp"]
# the native generator of the large synthetic workloads (host only, its own library)
SYNTH_SRC = "rv_synth.cpp"
SYNTH_LIB = os.path.join(HERE, "librvsynth.so")


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _needs(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "rvgpu.h"))
    jobs = []
    objs = []
    for f in CU:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if _needs(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "--expt-relaxed-constexpr"] + inc + ["-c", src, "-o", obj])
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if _needs(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-g", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(cuda, "include")] + inc +
                        ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    synth_src = os.path.join(CSRC, SYNTH_SRC)
    if _needs(SYNTH_LIB, [synth_src]):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", synth_src, "-o", SYNTH_LIB])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(run, jobs))
    if _needs(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
