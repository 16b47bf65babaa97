"""Comparison helpers for map dumps and records (shared by the tests)."""
from __future__ import annotations

# command-line options of the reference (src/Launcher.cpp:299-470) -> the
# rv_params / oracle parameter names (both mirror Configuration)
VALUED = {"-k": ("local_realign", int), "-f": ("freq", float), "-q": ("goodq", float), "-X": ("vext", int),
          "-m": ("mismatch", int), "-Q": ("min_mapq", int), "-T": ("trim_bases_after", int), "-M": ("minmatch", int),
          "-O": ("mapq_filter", float), "-P": ("read_pos_filter", int), "-o": ("qratio", float),
          "-B": ("min_bias_reads", int), "-x": ("extend_nt", int), "-r": ("minr", int), "-V": ("lofreq", float),
          "-Y": ("ref_extension", int)}
SWITCHES = {"-u": "unique_fwd", "-t": "dedup", "--fisher": "fisher", "-3": "move_indels_3", "--UN": "unique_first",
            "-p": "do_pileup"}


def flag_params(flags) -> dict:
    """Parameter values of a reference command line (default -k 1)."""
    kw = {"local_realign": 1}
    i = 0
    while i < len(flags):
        if flags[i] in SWITCHES:
            kw[SWITCHES[flags[i]]] = 1
            i += 1
        else:
            name, ty = VALUED[flags[i]]
            kw[name] = ty(flags[i + 1])
            i += 2
    return kw


def widened(a, b, flags):
    """The -R region as the reference's region builder widens it by -x
    (src/RegionBuilder.cpp:187-188)."""
    x = int(flags[flags.index("-x") + 1]) if "-x" in flags else 0
    return a - x, b + x


# column index (0-based, tag first) of pp and pq in stat lines: the last-seen
# read position / quality the reference keeps only to derive pstd/qstd
STAT_SKIP = (14, 15)


def parse(text: str) -> dict:
    d: dict = {}
    for ln in text.splitlines():
        f = ln.split("\t")
        d.setdefault(f[0], []).append(f)
    return d


def diff_dump(a_text: str, b_text: str, tags, skip=STAT_SKIP, rel=1e-6, key_cols=2):
    """Compares two dumps tag by tag.  Integer fields must match exactly;
    fields with a decimal point match within `rel` relative tolerance.
    Returns a list of human-readable problems (empty = equal)."""
    A, B = parse(a_text), parse(b_text)
    problems = []
    for t in tags:
        a, b = A.get(t, []), B.get(t, [])
        kk = (lambda x: tuple(x[1:1 + key_cols]))
        ka = {kk(x): x for x in a}
        kb = {kk(x): x for x in b}
        miss = sorted(set(ka) - set(kb))[:5]
        extra = sorted(set(kb) - set(ka))[:5]
        if miss:
            problems.append(f"{t}: {len(set(ka) - set(kb))} missing, e.g. {miss}")
        if extra:
            problems.append(f"{t}: {len(set(kb) - set(ka))} extra, e.g. {extra}")
        nbad = 0
        for k in set(ka) & set(kb):
            x, y = ka[k], kb[k]
            for i, (u, v) in enumerate(zip(x, y)):
                if i in skip or u == v:
                    continue
                try:
                    fu, fv = float(u), float(v)
                    if ("." in u or "." in v or "e" in u or "e" in v) and abs(fu - fv) <= rel * max(1.0, abs(fu)):
                        continue
                except ValueError:
                    pass
                nbad += 1
                if nbad <= 5:
                    problems.append(f"{t} {k} col {i}: {u} != {v}")
                break
        if nbad > 5:
            problems.append(f"{t}: {nbad} differing entries")
    return problems


def diff_records(ra: list[str], rb: list[str], rel=2e-6, somatic: bool = False):
    """Emitted record sets: same (start, ref, alt) keys (plus the label column
    for somatic records), integer and string columns equal, %f-formatted
    columns within rel (plus one unit in the sixth decimal)."""
    def key(f):
        k = (f[2], int(f[3]), f[5], f[6])
        return k + (f[-11] if len(f) > 60 else f[-7],) if somatic else k
    A = {key(l.split("\t")): l.split("\t") for l in ra if l}
    B = {key(l.split("\t")): l.split("\t") for l in rb if l}
    problems = []
    if somatic and (len(A) != len([l for l in ra if l]) or len(B) != len([l for l in rb if l])):
        problems.append("duplicate record keys")
    if set(A) != set(B):
        problems.append(f"record keys differ: missing {sorted(set(A) - set(B))[:5]} extra {sorted(set(B) - set(A))[:5]}")
    for k in set(A) & set(B):
        for i, (u, v) in enumerate(zip(A[k], B[k])):
            if u == v:
                continue
            try:
                fu, fv = float(u), float(v)
                if "." in u and abs(fu - fv) <= rel * max(1.0, abs(fu)) + 1.5e-6:
                    continue
            except ValueError:
                pass
            problems.append(f"record {k} col {i}: {u} != {v}")
            break
    return problems


def diff_vcf(va: str, vb: str, rel=2e-6):
    """VCF texts: same header, same body lines in the same (CHROM, POS) order,
    each line's fields equal or, where numeric with a decimal point, within
    rel (plus one unit in the sixth decimal)."""
    import re
    ha = [l for l in va.splitlines() if l.startswith("#")]
    hb = [l for l in vb.splitlines() if l.startswith("#")]
    a = [l for l in va.splitlines() if l and not l.startswith("#")]
    b = [l for l in vb.splitlines() if l and not l.startswith("#")]
    problems = [] if ha == hb else ["headers differ"]
    if len(a) != len(b):
        return problems + [f"{len(a)} != {len(b)} body lines"]

    def key(l):
        f = l.split("\t")
        return (f[0], int(f[1]), f[3], f[4], f[7].split(";")[0])
    if [key(l)[:2] for l in a] != [key(l)[:2] for l in b]:
        problems.append("line order differs")
    A, B = {key(l): l for l in a}, {key(l): l for l in b}
    if set(A) != set(B):
        return problems + [f"line keys differ: {sorted(set(A) ^ set(B))[:5]}"]
    for k in A:
        ta, tb = re.split(r"[\t;:,=]", A[k]), re.split(r"[\t;:,=]", B[k])
        if len(ta) != len(tb):
            problems.append(f"{k}: field counts differ")
            continue
        for u, v in zip(ta, tb):
            if u == v:
                continue
            try:
                if "." in u and abs(float(u) - float(v)) <= rel * max(1.0, abs(float(u))) + 1.5e-6:
                    continue
            except ValueError:
                pass
            problems.append(f"{k}: {u} != {v}")
            break
    return problems
