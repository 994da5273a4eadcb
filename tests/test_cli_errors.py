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
