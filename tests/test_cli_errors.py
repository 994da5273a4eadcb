"""The drop-in `cor` program rejects malformed command lines and INFILEs
exactly as the reference does: same exit code, same message on stderr,
nothing on stdout (tests/golden/cli_errors.json, made by running the
reference's own `cor`).  Each case fails before any device work, so this
runs without a GPU."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT, golden

COR = os.path.join(ROOT, "cor-model_gb300", "bin", "cor")
CASES = golden("cli_errors.json")


@pytest.fixture(scope="module")
def cor_exe():
    if not os.path.exists(COR):
        import build_lib
        build_lib.build()
    return COR


@pytest.mark.parametrize("name", sorted(CASES))
def test_cli_rejects_like_the_reference(cor_exe, tmp_path, name):
    case = CASES[name]
    if case["infile"] is not None:
        (tmp_path / "t.in").write_text(case["infile"])
    r = subprocess.run([cor_exe, *case["args"], "t.in"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert (r.returncode, r.stderr, r.stdout) == (case["rc"], case["stderr"], case["stdout"])


CUTOFF_HEADER = "0.05 1 20\n1.0031391260673028 50 15\n50 15\n2020 1 1 1 0 0 0\n100 0 0 0.05\n"
FIELD_HEADER = "1.0 -90 0\n10 10 90 360\n2020 1 1 1 0 0 0\n"


@pytest.mark.parametrize("mode,header", [("cutoff", CUTOFF_HEADER), ("field", FIELD_HEADER)])
def test_header_cut_short_is_rejected(cor_exe, tmp_path, mode, header):
    """A header cut after any of its items is "Invalid input file".  (The
    reference rejects only an empty file and otherwise reads its unset stack
    fields: cut inside the date line it exits 0 with a garbage time.)"""
    items = header.split()
    for k in range(1, len(items)):
        (tmp_path / "t.in").write_text(" ".join(items[:k]) + "\n")
        r = subprocess.run([cor_exe, "-m", mode, "t.in"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
        assert (r.returncode, r.stderr, r.stdout) == (1, "Error: Invalid input file\n", ""), (mode, k)
