"""The link-in drop-in: the reference's own `cor` program with its
trajectory_simulation_cutoff (src/trajectory.h:10) replaced by
cor-model_gb300/host/trajectory_shim.c and linked against libcortrace.so
(oracle/build.py build_shim).  Built only where the reference tree is; the
reference's sources never travel, so this runs on the CPU: the program must
link, keep the reference's own main(), INFILE reader and output header, and
reach the GPU scan (where, without a GPU, it stops with the shim's message
and status 1).  The scan text itself is shared with bin/cor (scan_text.h),
whose output the GPU tests compare with the reference's byte for byte."""
from __future__ import annotations

import subprocess

import pytest

import build as obuild
import pyoracle

INFILE = "0.05 1 20\n1.0031391260673028 50.0 15.0\n50.0 15.0\n2020 1 1 1 0 0 0\n100 0 0 0.05\n"


def _built():
    if not obuild.ref_available():
        pytest.skip("the reference tree is not here")
    obuild.build_ref()
    exe = obuild.build_shim()
    if exe is None:
        pytest.skip("libcortrace.so is not built")
    return exe


def test_shim_replaces_the_reference_function():
    exe = _built()
    syms = subprocess.run(["nm", exe], capture_output=True, text=True, check=True).stdout.split("\n")
    defined = {ln.split()[-1] for ln in syms if " T " in ln}
    assert "trajectory_simulation_cutoff" in defined                     # the shim's
    assert "reference_trajectory_simulation_cutoff_replaced" in defined  # the reference's, renamed away
    assert "read_cutoff_infile_header" in defined and "main" in defined   # the reference's own host code
    assert "cor_trace_batch" not in defined                               # from libcortrace.so at run time


def test_shim_runs_the_reference_host_code_then_the_gpu_scan(tmp_path):
    exe = _built()
    f = tmp_path / "site.in"
    f.write_text(INFILE)
    got = subprocess.run([exe, "-i", "igrf14", str(f)], capture_output=True, text=True, timeout=120)
    ref = pyoracle.run_ref_cor(INFILE, ["-i", "igrf14"], parallel=False)
    # the reference's header lines, written by its own main() before the scan
    header = ref.split(" rig : v")[0]
    assert got.stdout.startswith(header.rstrip("\n")), got.stdout[:400]
    if got.returncode == 0:
        # a GPU is present: the whole text is the reference's
        assert got.stdout == ref
    else:
        assert got.returncode == 1
        assert "no usable CUDA device for the GPU scan" in got.stderr
