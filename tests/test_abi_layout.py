"""The C ABI as its callers see it, without a GPU.

A C compiler lays out every public struct of include/rvgpu.h; the ctypes
mirrors in rabbitvar_gb300/api.py must have the same size and field offsets
(a mismatch would hand the library shifted fields).  rv_default_params must
give RabbitVar's Configuration defaults (include/Configuration.h)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _structs():
    from rabbitvar_gb300 import api
    return {"rv_params": api.Params, "rv_read_batch": api.ReadBatch, "rv_region": api.Region,
            "rv_site_record": api.SiteRecord, "rv_somatic_job": api.SomaticJob, "rv_candidate": api.Candidate}


def test_struct_layouts_match_ctypes_mirrors(tmp_path):
    import ctypes as C
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = _structs()
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rvgpu.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    seen = 0
    for line in filter(None, out):
        cname, fname, value = line.split()
        cls = structs[cname]
        want = C.sizeof(cls) if fname == "sizeof" else getattr(cls, fname).offset
        assert int(value) == want, f"{cname}.{fname}: C {value}, ctypes {want}"
        seen += 1
    assert seen == sum(len(c._fields_) + 1 for c in structs.values())


def test_default_params_are_the_reference_defaults():
    from rabbitvar_gb300 import api
    p = api.default_params()
    # include/Configuration.h: goodq :173, vext :177, mismatch :165, -k :185,
    # freq :210, minr :201, readPosFilter :228, qratio :232, mapq :236,
    # mappingQuality :157, lofreq :244, bias :193, minBiasReads :197,
    # samfilter "0x504" :219, referenceExtension :320, SVMINLEN :316;
    # the flags (-x -T -M -t -u -UN -p --fisher -3) default to off
    want = dict(goodq=22.5, vext=2, mismatch=8, local_realign=1, freq=0.01, minr=2, read_pos_filter=5, qratio=1.5,
                mapq_filter=0.0, min_mapq=0, lofreq=0.05, bias=0.05, min_bias_reads=2, samfilter=0x504,
                ref_extension=1200, extend_nt=0, trim_bases_after=0, minmatch=0, dedup=0, unique_fwd=0,
                unique_first=0, do_pileup=0, fisher=0, move_indels_3=0, svminlen=1000, somatic=0)
    assert {k: getattr(p, k) for k in want} == want
    assert {f for f, _ in api.Params._fields_} == set(want)


def test_cpp_caller_compiles_and_links(tmp_path):
    """A C++ translation unit like the reference's would-be GpuSimpleMode
    includes the three headers, links librvgpu.so and calls through the C
    ABI (without a GPU rv_create reports a CUDA error; with one it succeeds)."""
    from rabbitvar_gb300 import api
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    lib = api.lib()._name
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include "rvgpu.h"
#include "rvgpu_io.h"
#include "rvgpu_mlp.h"
#include <cstdio>
int main() {
    rv_params p;
    rv_default_params(&p);
    p.local_realign = 0;
    p.fisher = 1;
    rv_ctx *ctx = nullptr;
    rv_status st = rv_create(&ctx, &p, 0, 0);
    std::printf("%d %d %s\n", st, p.samfilter, st == RV_OK ? "ok" : rv_last_error(ctx));
    rv_destroy(ctx);
    return 0;
}
''')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(lib)
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), "-L", libdir, "-l:" + os.path.basename(lib), "-Wl,-rpath," + libdir],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    st, samfilter = int(out[0]), int(out[1])
    assert samfilter == 0x504
    assert st in (0, -2)  # RV_OK with a GPU, RV_ERR_CUDA without one
    assert len(out) > 2


def test_product_code_does_not_use_the_oracle():
    """The library and its Python front end neither import, load nor link
    anything under oracle/ (the oracle is test infrastructure only)."""
    import re
    pkg = os.path.join(ROOT, "rabbitvar_gb300")
    files = [os.path.join(pkg, f) for f in os.listdir(pkg) if f.endswith(".py")]
    files += [os.path.join(pkg, "csrc", f) for f in os.listdir(os.path.join(pkg, "csrc"))]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    bad = re.compile(r"import\s+oracle|from\s+oracle|librvoracle|oracle/|rvo_[a-z]|#include\s+\"rv_oracle")
    hits = [f for f in files if os.path.isfile(f) and bad.search(open(f, errors="replace").read())]
    assert hits == []


def test_graph_entry_points_reject_a_null_context():
    import ctypes as C
    from rabbitvar_gb300 import api
    L = api.lib()
    n = C.c_int64(-1)
    assert L.rv_set_pileup_graph(None, 1) == -1          # RV_ERR_ARG
    assert L.rv_pileup_graph_stats(None, C.byref(n), None) == -1
    assert n.value == -1


def test_capacity_entry_points_check_their_arguments():
    """rv_set_capacities / rv_capacity_stats without a GPU: a null context and
    out-of-range capacities are argument errors; valid ones are accepted on a
    context whose device set-up failed (no device memory is touched)."""
    import ctypes as C
    from rabbitvar_gb300 import api
    L = api.lib()
    assert L.rv_set_capacities(None, 1, 1, 1, 1) == -1
    assert L.rv_capacity_stats(None, None, None, None) == -1
    h = C.c_void_p()
    p = api.default_params()
    st = L.rv_create(C.byref(h), C.byref(p), 0, 0)
    assert st in (0, -2) and h
    try:
        assert L.rv_set_capacities(h, 0, 0, 1 << 40, 0) == -1      # deferred above INT32_MAX
        assert L.rv_set_capacities(h, 0, 0, 0, 1 << 40) == -1      # order-fix entries above INT32_MAX
        assert L.rv_set_capacities(h, (1 << 32) + 1, 0, 0, 0) == -1  # more slots than 32-bit indexes reach
        assert L.rv_set_capacities(h, 64, 256, 4, 4) == 0
        r, hs, ab = C.c_int64(-1), C.c_int64(-1), C.c_int64(-1)
        assert L.rv_capacity_stats(h, C.byref(r), C.byref(hs), C.byref(ab)) == 0
        assert r.value == 0
    finally:
        L.rv_destroy(h)
