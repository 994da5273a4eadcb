"""The drop-in `cor` program on the GPU: its text output for IGRF-only scans is
byte-for-byte the reference's (golden texts made by the reference's own `cor`),
in single-INFILE mode and in the one-call batch mode."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

COR = os.path.join(ROOT, "cor-model_gb300", "bin", "cor")


def _infile(s, g) -> str:
    r0 = 1.0031391260673028
    return (f"{g['rig']!r} 1 {g['rk']!r}\n{r0!r} {s['lat']!r} {s['lon']!r}\n{s['the1']!r} {s['fi1']!r}\n"
            + " ".join(str(v) for v in g["time"]) + f"\n100 0 0 {g['del']!r}\n")


def test_cli_output_is_the_references(tmp_path):
    g = golden("scan_config0.json")
    done = 0
    for s in g["sites"]:
        if "text" not in s:
            continue
        f = tmp_path / "site.in"
        f.write_text(_infile(s, g))
        out = subprocess.run([COR, "-p", "-i", "igrf14", str(f)], capture_output=True, text=True, check=True).stdout
        assert out == s["text"], (s["lat"], s["lon"])
        done += 1
    assert done >= 5


def test_cli_batch_manifest(tmp_path):
    g = golden("scan_config0.json")
    sites = [s for s in g["sites"] if "text" in s]
    lines = []
    for k, s in enumerate(sites):
        f = tmp_path / f"site{k}.in"
        f.write_text(_infile(s, g))
        lines.append(f"{f} {tmp_path / f'site{k}.out'}")
    man = tmp_path / "manifest"
    man.write_text("\n".join(lines) + "\n")
    subprocess.run([COR, "-i", "igrf14", "-b", str(man)], capture_output=True, text=True, check=True)
    for k, s in enumerate(sites):
        assert (tmp_path / f"site{k}.out").read_text() == s["text"], k
