"""GPU parity of libcortrace against the reference (golden fixtures) and the
oracle, through the C ABI.  IGRF-only scans are bit-exact: identical
allowed/forbidden flags, identical P(S)/P(C)/P(M), identical final states."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, unhex
import cortrace as ct
import pyoracle

pytestmark = pytest.mark.gpu


def fmt5(x: float) -> str:
    return f"{x:12.5f}".strip()


def test_field_igrf_bit_exact(ctx):
    g = golden("field_kats.json")["calculate_field"]
    p = ct.internal_setup("igrf14", g["time"])
    pts = unhex(g["points_m"]).reshape(-1, 3)
    want = unhex(g["cases"]["igrf14"]["b"]).reshape(-1, 3)
    got = ctx.field_batch(pts, p)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_field_internal_geo_points_bit_exact(ctx):
    """internal_geo KATs (incl. poles and truncation edges) via an identity GSM frame."""
    g = golden("field_kats.json")["internal_geo"]
    p = ct.internal_setup(g["version"], g["time"])
    p["a1"][0], p["a2"][0], p["a3"][0] = [1, 0, 0], [0, 1, 0], [0, 0, 1]
    pts = unhex(g["points"]).reshape(-1, 3)
    want = unhex(g["b"]).reshape(-1, 3)
    got = ctx.field_batch(pts * ct.DEF_RE, p)
    # with an identity rotation calculate_field reduces to internal_geo of pos/RE
    ref = pyoracle.internal_geo((pts * ct.DEF_RE) / ct.DEF_RE, p)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    exact = np.all(((pts * ct.DEF_RE) / ct.DEF_RE) == pts, axis=1)
    assert np.array_equal(got[exact].view(np.uint64), want[exact].view(np.uint64))


def config0_jobs(sites, rig, rk, dele):
    return np.concatenate([ct.make_job(s["lat"], s["lon"], rig=rig, rk=rk, dele=dele, the1=s["the1"], fi1=s["fi1"])
                           for s in sites])


def test_scan_config0_full_matches_reference(ctx):
    """All 228 sites x 400 rigidities of the IGRF-only workload: flags and cutoffs identical."""
    g = golden("scan_config0.json")
    p = ct.internal_setup(g["model"], g["time"])
    jobs = config0_jobs(g["sites"], g["rig"], g["rk"], g["del"])
    res = ctx.trace_batch(jobs, p)
    assert res.counters["trajectories"] == 91200
    assert res.counters["watchdog"] == 0
    bad = []
    for j, s in enumerate(g["sites"]):
        st = res.status[res.offsets[j]:res.offsets[j + 1]]
        allowed = np.nonzero(st == ct.TRAJ_ALLOWED)[0].tolist()
        site = res.sites[j]
        cut = [fmt5(site["r_lower"]), fmt5(site["r_upper"]), fmt5(site["r_cutoff"])]
        if allowed != s["allowed"] or cut != s["cutoff"]:
            bad.append((s["lat"], s["lon"]))
    assert not bad, bad


def test_scan_records_equal_oracle(ctx):
    """Final positions, velocities, times, lengths and step counts equal the oracle's bit for bit."""
    g = golden("scan_config0.json")
    sites = g["sites"][5::37]
    p = ct.internal_setup(g["model"], g["time"])
    jobs = config0_jobs(sites, g["rig"], g["rk"], g["del"])
    gpu = ctx.trace_batch(jobs, p, want_records=True)
    cpu = pyoracle.scan_batch(jobs, p, threads=8, want_records=True)
    assert np.array_equal(gpu.status, cpu.status)
    for k in ("pos", "vel", "v", "time", "length"):
        assert np.array_equal(gpu.records[k].view(np.uint64), cpu.records[k].view(np.uint64)), k
    for k in ("steps", "trials", "status"):
        assert np.array_equal(gpu.records[k], cpu.records[k]), k
    assert gpu.counters["accepted_steps"] == cpu.counters["accepted_steps"]
    assert gpu.counters["trials"] == cpu.counters["trials"]


def test_scan_edge_cases(ctx):
    """Single-rigidity scan, electrons, a short step limit, and a pole site."""
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    jobs = np.concatenate([ct.make_job(50.0, 15.0, rig=5.0, rk=5.0, dele=0.1),
                           ct.make_job(90.0, 0.0, rig=0.5, rk=2.0, dele=0.5),
                           ct.make_job(-33.0, 200.0, rig=1.0, rk=3.0, dele=0.25)])
    for kw in ({}, {"particle_mass": ct.DEF_HM0_E}, {"step_limit": 300}):
        gpu = ctx.trace_batch(jobs, p, want_records=True, **kw)
        cpu = pyoracle.scan_batch(jobs, p, want_records=True, **kw)
        assert np.array_equal(gpu.status, cpu.status), kw
        assert np.array_equal(gpu.records["pos"].view(np.uint64), cpu.records["pos"].view(np.uint64)), kw
        assert np.array_equal(gpu.sites.view(np.uint8), cpu.sites.view(np.uint8)), kw


def test_empty_batch(ctx):
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    res = ctx.trace_batch(np.zeros(0, ct.JOB_DTYPE), p)
    assert len(res.sites) == 0 and res.counters["trajectories"] == 0


def test_invalid_requests_fail_cleanly(ctx):
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    j = ct.make_job(0.0, 0.0, rig=1.0, rk=2.0, dele=0.5, param_index=3)
    with pytest.raises(ct.CorError) as e:
        ctx.trace_batch(j, p)
    assert e.value.code == -1
    # the context stays usable
    res = ctx.trace_batch(ct.make_job(0.0, 0.0, rig=1.0, rk=2.0, dele=0.5), p)
    assert res.counters["trajectories"] == 3
