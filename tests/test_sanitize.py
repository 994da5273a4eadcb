"""The host-side C (model set-up, INFILE and PARMOD parsing, the model
registry) and the C oracle built with AddressSanitizer and
UndefinedBehaviorSanitizer and driven by tests/sanitize_harness.c, malformed
inputs included.  Any sanitizer report fails the test (the runtime is told to
abort on the first one)."""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "cor-model_gb300", "host")
ORACLE = os.path.join(ROOT, "oracle")
SOURCES = [os.path.join(HOST, f) for f in ("setup.c", "coef_tables.c", "cli_io.c", "cli_models.c")] + \
    sorted(os.path.join(ORACLE, f) for f in os.listdir(ORACLE) if f.endswith(".c"))


def _sanitizers_available() -> bool:
    if shutil.which("gcc") is None:
        return False
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write("int main(void){return 0;}\n")
        r = subprocess.run(["gcc", "-fsanitize=address,undefined", src, "-o", os.path.join(d, "t")],
                           capture_output=True)
        return r.returncode == 0


@pytest.mark.skipif(not _sanitizers_available(), reason="gcc without ASan/UBSan runtimes")
def test_host_c_and_oracle_are_clean_under_asan_ubsan(tmp_path):
    exe = str(tmp_path / "sanitize_harness")
    cmd = ["gcc", "-std=gnu17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-pthread", os.path.join(ROOT, "tests", "sanitize_harness.c"), *SOURCES,
           "-o", exe, "-lm"]
    b = subprocess.run(cmd, capture_output=True, text=True)
    assert b.returncode == 0, b.stderr[-4000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0:halt_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and "sanitize ok" in r.stdout, (r.stdout[-2000:], r.stderr[-4000:])
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
