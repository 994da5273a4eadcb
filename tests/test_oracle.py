"""CPU tests: the oracle (CPU restatement) and the product's host set-up,
pinned against golden fixtures made by the reference itself."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import golden, unhex
import cortrace as ct
import pyoracle


def test_setup_matches_reference_bit_for_bit():
    """cor_internal_setup == internal_recalc for every model family and epoch kind."""
    for case in golden("setup_params.json")["cases"]:
        p = ct.internal_setup(case["version"], case["time"])
        for k in ("g", "h", "rec", "a1", "a2", "a3"):
            want = unhex(case[k])
            got = p[k][0].ravel()
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (case["version"], case["time"], k)


def test_setup_rejects_out_of_range_and_unknown():
    with pytest.raises(ct.CorError):
        ct.internal_setup("igrf14", [2031, 1, 1, 1, 0, 0, 0])
    with pytest.raises(ct.CorError):
        ct.internal_setup("igrf99", [2020, 1, 1, 1, 0, 0, 0])
    with pytest.raises(ct.CorError):
        ct.internal_setup("hist", [2000, 1, 1, 1, 0, 0, 0])   # year >= max_year without extrapolation


def test_oracle_internal_geo_bit_exact():
    g = golden("field_kats.json")["internal_geo"]
    p = ct.internal_setup(g["version"], g["time"])
    pts = unhex(g["points"]).reshape(-1, 3)
    want = unhex(g["b"]).reshape(-1, 3)
    got = pyoracle.internal_geo(pts, p)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_oracle_calculate_field_igrf_bit_exact():
    g = golden("field_kats.json")["calculate_field"]
    p = ct.internal_setup("igrf14", g["time"])
    pts = unhex(g["points_m"]).reshape(-1, 3)
    want = unhex(g["cases"]["igrf14"]["b"]).reshape(-1, 3)
    got = pyoracle.calculate_field(pts, p)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_oracle_chaos_bit_exact():
    g = golden("field_kats.json")["chaos_geo"]
    pts = unhex(g["points"]).reshape(-1, 3)
    want = unhex(g["b"]).reshape(-1, 3)
    G, H, nmax = ct.chaos_dense()
    lib = pyoracle.load()
    b = np.zeros(3)
    for i, (x, y, z) in enumerate(pts):
        lib.orc_chaos_geo(x, y, z, G.ctypes.data, H.ctypes.data, nmax, b[0:].ctypes.data, b[1:].ctypes.data,
                          b[2:].ctypes.data)
        assert np.array_equal(b.view(np.uint64), want[i].view(np.uint64)), i


def config0_jobs(sites, rig=0.05, rk=20.0, dele=0.05):
    jobs = np.concatenate([ct.make_job(s["lat"], s["lon"], rig=rig, rk=rk, dele=dele, the1=s["the1"], fi1=s["fi1"])
                           for s in sites])
    return jobs


def fmt5(x: float) -> str:
    return f"{x:12.5f}".strip()


def test_oracle_scan_matches_reference_config0_subset():
    """Allowed/forbidden flags and P(S)/P(C)/P(M) identical on 12 config-0 sites."""
    g = golden("scan_config0.json")
    sites = g["sites"][::19]
    p = ct.internal_setup(g["model"], g["time"])
    jobs = config0_jobs(sites, g["rig"], g["rk"], g["del"])
    res = pyoracle.scan_batch(jobs, p, threads=8)
    for j, s in enumerate(sites):
        st = res.status[res.offsets[j]:res.offsets[j + 1]]
        allowed = np.nonzero(st == ct.TRAJ_ALLOWED)[0].tolist()
        assert allowed == s["allowed"], (s["lat"], s["lon"])
        site = res.sites[j]
        assert [fmt5(site["r_lower"]), fmt5(site["r_upper"]), fmt5(site["r_cutoff"])] == s["cutoff"]


EXT_SCANS = {
    "scan_t96.json": (ct.INTERNAL_SH, ct.EXTERNAL_T96, ct.CRUSTAL_NONE, 8),
    "scan_ts05.json": (ct.INTERNAL_SH, ct.EXTERNAL_TS05, ct.CRUSTAL_NONE, 8),
    "scan_chaos.json": (ct.INTERNAL_SH, ct.EXTERNAL_NONE, ct.CRUSTAL_CHAOS, 3),
}


@pytest.mark.parametrize("name", sorted(EXT_SCANS))
def test_oracle_scan_with_external_and_crustal_fields_matches_reference(name):
    """The oracle, built with the reference's compiler flags against the same C
    library, gives the reference's own allowed/forbidden flags and P(S)/P(C)/P(M)
    lines on the T96, TS05 and CHAOS scan fixtures: every stride-th site by
    default, every site with COR_ORACLE_ALL_SITES=1 (200 + 200 + 12 sites, a
    few minutes on 8 threads)."""
    internal, external, crustal, stride = EXT_SCANS[name]
    if os.environ.get("COR_ORACLE_ALL_SITES") == "1":
        stride = 1
    g = golden(name)
    sites = g["sites"][::stride]
    p = ct.internal_setup(g["model"], g["time"], parmod=g.get("parmod"))
    jobs = config0_jobs(sites, g["rig"], g["rk"], g["del"])
    res = pyoracle.scan_batch(jobs, p, models=ct.model_set(internal, external, crustal), threads=8,
                              step_limit=g.get("step_limit", 25000))
    for j, s in enumerate(sites):
        st = res.status[res.offsets[j]:res.offsets[j + 1]]
        assert np.nonzero(st == ct.TRAJ_ALLOWED)[0].tolist() == s["allowed"], (s["lat"], s["lon"])
        site = res.sites[j]
        assert [fmt5(site["r_lower"]), fmt5(site["r_upper"]), fmt5(site["r_cutoff"])] == s["cutoff"]


def test_oracle_scans_match_reference_at_storm_conditions():
    """IGRF-14 + TS05 at 4 seeded storm-range conditions, 6 site-directions
    each (vertical and 30 deg zenith): the reference's own flags and
    P(S)/P(C)/P(M) lines."""
    g = golden("scan_storm.json")
    models = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_TS05)
    for c in g["conditions"]:
        p = ct.internal_setup(g["model"], c["time"], parmod=c["parmod"])
        jobs = config0_jobs(c["sites"], g["rig"], g["rk"], g["del"])
        res = pyoracle.scan_batch(jobs, p, models=models, threads=8)
        for j, s in enumerate(c["sites"]):
            st = res.status[res.offsets[j]:res.offsets[j + 1]]
            assert np.nonzero(st == ct.TRAJ_ALLOWED)[0].tolist() == s["allowed"], (c["time"], s["lat"], s["lon"])
            site = res.sites[j]
            assert [fmt5(site["r_lower"]), fmt5(site["r_upper"]), fmt5(site["r_cutoff"])] == s["cutoff"]


def test_oracle_flop_model():
    """The op-count model of the SH field follows the degree truncation."""
    assert pyoracle.internal_geo_flops(1.5) > pyoracle.internal_geo_flops(2.5) > pyoracle.internal_geo_flops(20.0)
    # K = 14 at R < 2: 105 (n,m) terms, 14 of them with m = 1
    assert pyoracle.internal_geo_flops(1.0) == 12 + 28 + 13 + 14 * 4 + 13 * 8 + 14 * 17 + (105 - 14) * 23


def _ext_kat(name: str, fn):
    g = golden("field_kats.json")[name]
    pm = unhex(g["parmod"])
    pts = unhex(g["points"]).reshape(-1, 3)
    want = unhex(g["b"]).reshape(-1, 3)
    b = np.zeros(3)
    for i, (x, y, z) in enumerate(pts):
        fn(pm.ctypes.data, x, y, z, b[0:].ctypes.data, b[1:].ctypes.data, b[2:].ctypes.data)
        assert np.array_equal(b.view(np.uint64), want[i].view(np.uint64)), (name, i, b, want[i])


def test_oracle_t96_bit_exact():
    _ext_kat("t96_gsm", pyoracle.load().orc_t96_gsm)


def test_oracle_ts05_bit_exact():
    _ext_kat("ts05_gsm", pyoracle.load().orc_ts05_gsm)


def test_oracle_calculate_field_external_bit_exact():
    g = golden("field_kats.json")["calculate_field"]
    pts = unhex(g["points_m"]).reshape(-1, 3)
    for key, ext in (("igrf14+t96", ct.EXTERNAL_T96), ("igrf14+ts05", ct.EXTERNAL_TS05)):
        case = g["cases"][key]
        p = ct.internal_setup("igrf14", g["time"], parmod=unhex(case["parmod"]))
        want = unhex(case["b"]).reshape(-1, 3)
        got = pyoracle.calculate_field(pts, p, models=ct.model_set(ct.INTERNAL_SH, ext))
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), key


@pytest.mark.parametrize("model", ["t96", "ts05"])
def test_oracle_external_fields_bit_exact_at_storm_conditions(model):
    """T96 / TS05 alone and composed with IGRF-14 at 8 seeded storm-range
    conditions each (Pdyn to 10 nPa, Dst to -300 nT, IMF to +-20 nT, W to 5):
    the oracle equals the reference bit for bit."""
    lib = pyoracle.load()
    fn = lib.orc_t96_gsm if model == "t96" else lib.orc_ts05_gsm
    ext = ct.EXTERNAL_T96 if model == "t96" else ct.EXTERNAL_TS05
    for case in golden("field_storm.json")[model]:
        pm = unhex(case["parmod"])
        want = unhex(case["b"]).reshape(-1, 3)
        b = np.zeros(3)
        for i, (x, y, z) in enumerate(unhex(case["points"]).reshape(-1, 3)):
            fn(pm.ctypes.data, x, y, z, b[0:].ctypes.data, b[1:].ctypes.data, b[2:].ctypes.data)
            assert np.array_equal(b.view(np.uint64), want[i].view(np.uint64)), (model, case["time"], i)
        p = ct.internal_setup("igrf14", case["time"], parmod=pm)
        got = pyoracle.calculate_field(unhex(case["points_m"]).reshape(-1, 3), p, models=ct.model_set(ct.INTERNAL_SH, ext))
        want = unhex(case["b_composed"]).reshape(-1, 3)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (model, case["time"])


def test_oracle_calculate_field_crustal_bit_exact():
    """calculate_field with the CHAOS-7.16 crustal model (chaos_7_16_calc,
    src/models.c:179-192), alone with IGRF-14 and together with T96."""
    g = golden("field_kats.json")["calculate_field"]
    pts = unhex(g["points_m"]).reshape(-1, 3)
    for key, ext in (("igrf14+chaos7.16", ct.EXTERNAL_NONE), ("igrf14+t96+chaos7.16", ct.EXTERNAL_T96)):
        case = g["cases"][key]
        p = ct.internal_setup("igrf14", g["time"], parmod=unhex(case["parmod"]))
        want = unhex(case["b"]).reshape(-1, 3)
        got = pyoracle.calculate_field(pts, p, models=ct.model_set(ct.INTERNAL_SH, ext, ct.CRUSTAL_CHAOS))
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), key


def test_oracle_window_equals_whole_scan():
    """A window of the grid that holds the penumbra gives the whole scan's
    P(S), P(C), P(M) bit for bit and the same classes on its indices; a
    window that cuts into the penumbra does not (cor_trace.h, i_first/i_count)."""
    g = golden("scan_config0.json")
    sites = [s for s in g["sites"] if float(s["cutoff"][0]) < float(s["cutoff"][1]) - 0.2][:3]
    p = ct.internal_setup(g["model"], g["time"])
    jobs = config0_jobs(sites, g["rig"], g["rk"], g["del"])
    full = pyoracle.scan_batch(jobs, p, threads=8)
    win = jobs.copy()
    for j in range(len(sites)):
        st = full.status[full.offsets[j]:full.offsets[j + 1]]
        allowed = np.nonzero(st == ct.TRAJ_ALLOWED)[0]
        forbidden = np.nonzero(st != ct.TRAJ_ALLOWED)[0]
        lo, hi = int(allowed.min()) - 3, int(forbidden.max()) + 3
        win[j]["i_first"], win[j]["i_count"] = lo, hi - lo + 1
    part = pyoracle.scan_batch(win, p, threads=8)
    for j in range(len(sites)):
        for k in ("r_lower", "r_upper", "r_cutoff", "n_forbidden"):
            assert part.sites[j][k] == full.sites[j][k], (j, k)
        a = int(full.offsets[j]) + int(win[j]["i_first"])
        assert np.array_equal(part.status[part.offsets[j]:part.offsets[j + 1]],
                              full.status[a:a + int(win[j]["i_count"])])
    # cutting the penumbra from above changes P(C)
    cut = win.copy()
    cut["i_count"] = cut["i_count"] - 6
    bad = pyoracle.scan_batch(cut, p, threads=8)
    assert any(bad.sites[j]["r_upper"] != full.sites[j]["r_upper"] for j in range(len(sites)))


def _parse_cutoff_infile(text):
    """INFILE of `cor -m cutoff|trajectory` (src/io.c:4-20) -> (job, time7)."""
    v = text.split()
    rig, zn, rk, r0, lat, lon, the1, fi1 = (float(x) for x in v[:8])
    t7 = [int(x) for x in v[8:15]]
    nk1, dele = int(v[15]), float(v[18])
    return ct.make_job(lat, lon, rig=rig, rk=rk, dele=dele if dele > 0 else 1.0, r0=r0, the1=the1, fi1=fi1, zn=zn,
                       nk1=nk1), t7


def test_oracle_trajectory_mode_matches_reference():
    """The oracle's per-step records, printed in trajectory_simulation's
    formats (src/trajectory.c:254-258), reproduce the reference's tragsm_ and
    trasph_ files byte for byte (IGRF-14, one allowed and one forbidden
    rigidity)."""
    import hashlib
    import math
    g = golden("trajectory_cli.json")
    for case in ("igrf14_allowed", "igrf14_forbidden"):
        job, t7 = _parse_cutoff_infile(g[case]["infile"])
        p = ct.internal_setup("igrf14", t7)
        steps = pyoracle.trace_steps(job, p)
        gsm_lines, sph_lines = [], []
        for s in steps:
            x, y, z = s["pos"]
            sq = x * x + y * y
            r = math.sqrt(sq + z * z)
            theta = math.atan2(math.sqrt(sq), z)
            phi = math.atan2(y, x)
            if phi < 0.:
                phi += 6.28318531
            to_rad = 3.141592654 / 180.
            row = (s["v"], s["time"], s["length"])
            gsm_lines.append("%6d%17.5f%17.5f%17.5f%14.2f%15.10f%18.2f\n" % (s["step"], *s["gsm"], *row))
            sph_lines.append("%6d%17.5f%17.5f%17.5f%14.2f%15.10f%18.2f\n"
                             % (s["step"], r / 6.3712e+06, 90. - theta / to_rad, phi / to_rad, *row))
        for pre, lines in (("tragsm_", gsm_lines), ("trasph_", sph_lines)):
            body = "".join(lines)
            assert len(lines) == g[case][pre]["lines"], (case, pre)
            assert hashlib.sha256(body.encode()).hexdigest() == g[case][pre]["sha256"], (case, pre)
