"""Generate coef_tables.c: the Gauss-coefficient data of the field models.

The internal-field tables (IGRF-9..14 from IAGA, the historical model and
CALS10k.2; lib/internal/coefs/*.h) and the CHAOS-7.16 lithospheric table
(lib/chaos/coefs/chaos_7_16.h) are published geophysical data.  This script
reads them from the reference's headers once and writes them in this
project's own layout: one array per epoch, an epoch list per model, and the
CHAOS table packed as the lower triangle (m <= n) that chaos_geo reads.
Each value is written as the shortest decimal that round-trips, so the
compiled doubles equal the reference's.

Usage: python gen_coef_tables.py REFERENCE_ROOT   (or COR_REFERENCE_ROOT set)
"""
from __future__ import annotations

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# Model registry order and display names: src/models.c:22-84,110
MODELS = [
    ("igrf14", "IGRF-14", "igrf_14_coefs.h", "_IGRF_14", "IGRF_14_COEFS"),
    ("igrf13", "IGRF-13", "igrf_13_coefs.h", "_IGRF_13", "IGRF_13_COEFS"),
    ("igrf12", "IGRF-12", "igrf_12_coefs.h", "_IGRF_12", "IGRF_12_COEFS"),
    ("igrf11", "IGRF-11", "igrf_11_coefs.h", "_IGRF_11", "IGRF_11_COEFS"),
    ("igrf10", "IGRF-10", "igrf_10_coefs.h", "_IGRF_10", "IGRF_10_COEFS"),
    ("igrf9", "IGRF-9", "igrf_9_coefs.h", "_IGRF_9", "IGRF_9_COEFS"),
    ("hist", "Historical (0-1968 CE)", "hist_coefs.h", "_HIST", "HIST_COEFS"),
    ("cals10k.2", "Historical (CALS10k.2)", "cals10k_2_coefs.h", "_CALS10K_2", "CALS10K_2_COEFS"),
]

ARRAY_RE = re.compile(r"const\s+double\s+(\w+)\s*\[[^\]]*\]\s*=\s*\{([^}]*)\}\s*;", re.S)
LIST_RE = re.compile(r"const\s+double\s*\*\s*(\w+)\s*\[\s*\]\s*=\s*\{([^}]*)\}\s*;", re.S)
STRUCT_RE = re.compile(r"const\s+InternalModelCoefs\s+(\w+)\s*=\s*\{([^}]*)\}\s*;", re.S)


def _num(tok: str) -> float:
    return float(tok.strip())


def _fmt(x: float) -> str:
    s = repr(x)
    if s in ("0.0", "-0.0"):
        return "0" if s == "0.0" else "-0.0"
    return s


def parse_internal(root: str):
    cdir = os.path.join(root, "lib", "internal", "coefs")
    arrays: dict[str, list[float]] = {}
    lists: dict[str, list[str]] = {}
    structs: dict[str, dict[str, str]] = {}
    for fn in sorted(os.listdir(cdir)):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(cdir, fn)).read()
        for name, body in ARRAY_RE.findall(txt):
            vals = [_num(t) for t in body.split(",") if t.strip()]
            if len(vals) != 105:
                raise ValueError(f"{fn}:{name} has {len(vals)} values")
            arrays[name] = vals
        for name, body in LIST_RE.findall(txt):
            lists[name] = [t.strip() for t in body.split(",") if t.strip()]
        for name, body in STRUCT_RE.findall(txt):
            fields = {}
            for part in body.split(","):
                if "=" in part:
                    k, v = part.split("=", 1)
                    fields[k.strip().lstrip(".")] = v.strip()
            structs[name] = fields
    return arrays, lists, structs


def parse_chaos(root: str):
    txt = open(os.path.join(root, "lib", "chaos", "coefs", "chaos_7_16.h")).read()
    out = {}
    for key in ("G_CHAOS_7_16", "H_CHAOS_7_16"):
        m = re.search(r"const\s+double\s+" + key + r"\s*\[186\]\s*\[186\]\s*=\s*\{(.*?)\}\s*;", txt, re.S)
        rows = re.findall(r"\{([^{}]*)\}", m.group(1))
        if len(rows) != 186:
            raise ValueError(f"{key}: {len(rows)} rows")
        table = []
        for r in rows:
            vals = [_num(t) for t in r.split(",") if t.strip()]
            if len(vals) != 186:
                raise ValueError(f"{key}: row of {len(vals)}")
            table.append(vals)
        for n in range(186):
            for m_ in range(n + 1, 186):
                if table[n][m_] != 0.0:
                    raise ValueError(f"{key}[{n}][{m_}] above the diagonal is non-zero")
        out[key] = table
    nm = re.search(r"\.nm_max\s*=\s*(\d+)", txt)
    return out["G_CHAOS_7_16"], out["H_CHAOS_7_16"], int(nm.group(1))


def _emit_array(lines: list[str], cname: str, vals: list[float], per_line: int = 8) -> None:
    lines.append(f"static const double {cname}[{len(vals)}] = {{")
    for i in range(0, len(vals), per_line):
        lines.append("    " + ", ".join(_fmt(v) for v in vals[i:i + per_line]) + ",")
    lines.append("};")


def generate(root: str) -> str:
    arrays, lists, structs = parse_internal(root)
    used = []
    for _, _, _, lname, _ in MODELS:
        for a in lists[lname]:
            if a not in used:
                used.append(a)
    lines = [
        "/* Generated by gen_coef_tables.py -- data only, do not edit.",
        " * Gauss coefficients [nT] of the internal field models (IGRF-9..14 by",
        " * IAGA, the historical model, CALS10k.2) per epoch, and the CHAOS-7.16",
        " * lithospheric coefficients packed as the lower triangle m <= n. */",
        '#include "coef_tables.h"',
        "",
    ]
    for a in used:
        _emit_array(lines, "t_" + a.lower(), arrays[a])
    lines.append("")
    for version, _, _, lname, _ in MODELS:
        cname = "l_" + version.replace(".", "_")
        lines.append(f"static const double *const {cname}[{len(lists[lname])}] = {{")
        names = ["t_" + a.lower() for a in lists[lname]]
        for i in range(0, len(names), 6):
            lines.append("    " + ", ".join(names[i:i + 6]) + ",")
        lines.append("};")
    lines.append("")
    lines.append(f"const cor_sh_table cor_sh_tables[{len(MODELS)}] = {{")
    for version, name, _, lname, sname in MODELS:
        st = structs[sname]
        n = int(st["coefs_size"])
        if n != len(lists[lname]):
            raise ValueError(f"{sname}: coefs_size {n} vs list {len(lists[lname])}")
        ext = 1 if st["extrapolate"] == "true" else 0
        cname = "l_" + version.replace(".", "_")
        lines.append(f'    {{ "{version}", "{name}", {cname}, {n}, {int(st["years_step"])}, '
                     f'{int(st["min_year"])}, {int(st["max_year"])}, {ext} }},')
    lines.append("};")
    lines.append(f"const int cor_sh_table_count = {len(MODELS)};")
    lines.append("")
    g, h, nmax = parse_chaos(root)
    tri_g = [g[n][m] for n in range(nmax) for m in range(n + 1)]
    tri_h = [h[n][m] for n in range(nmax) for m in range(n + 1)]
    _emit_array(lines, "t_chaos716_g", tri_g)
    _emit_array(lines, "t_chaos716_h", tri_h)
    lines.append(f"const cor_chaos_table cor_chaos716 = {{ \"chaos7.16\", \"CHAOS-7.16\", {nmax}, t_chaos716_g, t_chaos716_h }};")
    lines.append("")
    return "\n".join(lines)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("COR_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: gen_coef_tables.py REFERENCE_ROOT (or set COR_REFERENCE_ROOT)")
    out = os.path.join(HERE, "coef_tables.c")
    with open(out, "w") as f:
        f.write(generate(root))
    print(out, os.path.getsize(out))
