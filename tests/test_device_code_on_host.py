"""The device field code and RK step of libcortrace, compiled as host C++
(tests/device_on_host/) with the reference's floating-point flags and the host
C library, against the reference's own field vectors.

On the GPU the field models call CUDA's transcendental functions, and the
external- and crustal-field units are compiled with FMA contraction; both
change last bits, so the GPU tests hold T96/TS05 to the reference's own
one-ulp sensitivity.  Here both are taken away: the same expression trees are
evaluated with glibc and without contraction, so they must give the
reference's bits.  With COR_T96_POW5 (the reference's pow(u, 5) in r2sheet)
every golden field vector is reproduced bit for bit: IGRF, T96 and TS05,
alone and composed, at the quiet and the storm-range conditions.  The default
build, which multiplies u out, differs only in T96, by a few ulp.  The scan
kernel's per-trajectory functions (lane_init, lane_advance, lane_finish), run
trajectory by trajectory as the kernel's loop runs them, give every
trajectory's class and final record bit for bit as the reference does.  The
crustal model's warp-cooperative sum runs on 32 host threads standing for a
warp: it sums in another order than the reference, so it agrees to a few ulp,
and composed with IGRF-14 (and T96) the golden field vectors come out bit for
bit.  No GPU."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, unhex
import cortrace as ct
import pyoracle

SRC = os.path.join(ROOT, "tests", "device_on_host", "field_host.cpp")
# the reference's flags (CMakeLists.txt:17, without -march=native)
FLAGS = ["-std=c++20", "-O3", "-fno-math-errno", "-fno-trapping-math", "-ffp-contract=off", "-fPIC", "-shared",
         "-pthread", "-Wno-unknown-pragmas"]


def _build(out_dir, defines=()) -> C.CDLL:
    so = os.path.join(out_dir, "field_host%s.so" % ("".join(d.lower() for d in defines)))
    r = subprocess.run(["g++", *FLAGS, *[f"-D{d}" for d in defines], SRC, "-o", so, "-lm"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(so)
    vp = C.c_void_p
    lib.host_internal_geo.argtypes = [vp, vp, C.c_int64, vp]
    lib.host_external.argtypes = [C.c_int, vp, vp, C.c_int64, vp]
    lib.host_calculate_field.argtypes = [C.c_int, C.c_int, vp, vp, C.c_int64, vp]
    lib.host_rk_step.argtypes = [C.c_double, C.c_double, vp, vp, vp]
    lib.host_chaos.argtypes = [vp, vp, C.c_int32, vp, C.c_int64, vp]
    lib.host_calculate_field_crustal.argtypes = [C.c_int, C.c_int, vp, vp, vp, C.c_int32, vp, C.c_int64, vp]
    lib.host_trace.argtypes = [C.c_int, C.c_int, vp, vp, C.c_int32, vp, C.c_uint64, vp, C.c_int32, C.c_uint64,
                               C.c_double, C.c_double, vp, vp]
    lib.host_regroup.argtypes = [vp, vp, C.c_int32, vp]
    lib.host_tables()
    return lib


@pytest.fixture(scope="module")
def builds(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    d = str(tmp_path_factory.mktemp("device_on_host"))
    return {"default": _build(d), "reference_pow": _build(d, ["COR_T96_POW5"])}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _external(lib, ext, parmod, pts):
    out = np.zeros_like(pts)
    lib.host_external(ext, _p(parmod), _p(pts), len(pts), _p(out))
    return out


def _composed(lib, internal, ext, params, pts_m):
    out = np.zeros_like(pts_m)
    assert lib.host_calculate_field(internal, ext, _p(params), _p(pts_m), len(pts_m), _p(out)) == 0
    return out


def _cases():
    """(name, model, function of lib -> (got, want)) over every golden field vector
    the host build can evaluate (all but the crustal model)."""
    g = golden("field_kats.json")
    st = golden("field_storm.json")
    out = []
    ig = g["internal_geo"]

    def igrf(lib):
        p = ct.internal_setup(ig["version"], ig["time"])
        pts = unhex(ig["points"]).reshape(-1, 3)
        got = np.zeros_like(pts)
        lib.host_internal_geo(_p(p), _p(pts), len(pts), _p(got))
        return got, unhex(ig["b"]).reshape(-1, 3)
    out.append(("internal_geo", "igrf", igrf))
    for key, ext, model in (("t96_gsm", ct.EXTERNAL_T96, "t96"), ("ts05_gsm", ct.EXTERNAL_TS05, "ts05")):
        k = g[key]
        out.append((key, model, lambda lib, k=k, ext=ext: (
            _external(lib, ext, unhex(k["parmod"]), unhex(k["points"]).reshape(-1, 3)), unhex(k["b"]).reshape(-1, 3))))
    cf = g["calculate_field"]
    for key, ext, model in (("igrf14", ct.EXTERNAL_NONE, "igrf"), ("igrf14+t96", ct.EXTERNAL_T96, "t96"),
                            ("igrf14+ts05", ct.EXTERNAL_TS05, "ts05")):
        case = cf["cases"][key]

        def comp(lib, case=case, ext=ext):
            p = ct.internal_setup("igrf14", cf["time"], parmod=unhex(case["parmod"]))
            return (_composed(lib, 1, ext, p, unhex(cf["points_m"]).reshape(-1, 3)), unhex(case["b"]).reshape(-1, 3))
        out.append(("calculate_field " + key, model, comp))
    for model, ext in (("t96", ct.EXTERNAL_T96), ("ts05", ct.EXTERNAL_TS05)):
        for n, case in enumerate(st[model]):
            pm = unhex(case["parmod"])
            out.append((f"storm {model} {n}", model, lambda lib, case=case, pm=pm, ext=ext: (
                _external(lib, ext, pm, unhex(case["points"]).reshape(-1, 3)), unhex(case["b"]).reshape(-1, 3))))

            def scomp(lib, case=case, pm=pm, ext=ext):
                p = ct.internal_setup("igrf14", case["time"], parmod=pm)
                return (_composed(lib, 1, ext, p, unhex(case["points_m"]).reshape(-1, 3)),
                        unhex(case["b_composed"]).reshape(-1, 3))
            out.append((f"storm igrf14+{model} {n}", model, scomp))
    return out


def _bits_equal(a, b):
    return (a.view(np.uint64) == b.view(np.uint64)).all(axis=1)


def test_device_field_code_is_the_references_arithmetic(builds):
    """With the reference's pow(u, 5): every point of every golden field case bit for bit."""
    lib = builds["reference_pow"]
    n = 0
    for name, _, fn in _cases():
        got, want = fn(lib)
        eq = _bits_equal(got, want)
        assert eq.all(), (name, int((~eq).sum()), len(eq))
        n += len(eq)
    assert n > 2800   # 2,902 points: 410 IGRF, 612 T96/TS05, 600 composed, 1,280 at storm conditions


def test_default_build_differs_only_in_t96_r2sheet(builds):
    """The device's own form: IGRF and TS05 stay bit for bit; T96 (u^5 by
    multiplication) stays within 1e-14 of |B|."""
    lib = builds["default"]
    for name, model, fn in _cases():
        got, want = fn(lib)
        if model != "t96":
            assert _bits_equal(got, want).all(), name
        else:
            rel = np.linalg.norm(got - want, axis=1) / np.maximum(np.linalg.norm(want, axis=1), 1e-300)
            assert rel.max() <= 1e-14, (name, rel.max())


def test_rk_step_is_the_oracles(builds):
    """rk_velocity + rk_position against the oracle's restatement of
    calculate_position_and_speed (src/trajectory.c:275-356), bit for bit."""
    lib = builds["default"]
    olib = pyoracle.load()
    rng = np.random.default_rng(5)
    for _ in range(2000):
        h = 10.0 ** rng.uniform(-6, -1)
        d = rng.uniform(-1, 1) * 10.0 ** rng.uniform(-3, 3)
        f = rng.normal(0, 3e4, 3)
        v = rng.normal(0, 1e8, 3)
        x = rng.normal(0, 3e7, 3)
        v1, x1, v2, x2 = v.copy(), x.copy(), v.copy(), x.copy()
        lib.host_rk_step(h, d, _p(f), _p(v1), _p(x1))
        olib.orc_rk_step(h, d, _p(f), _p(v2), _p(x2))
        assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64)) and \
            np.array_equal(x1.view(np.uint64), x2.view(np.uint64))


def _host_scan(lib, internal, external, jobs, params, step_limit=25000):
    """host_trace one job per call, 8 calls at a time (ctypes releases the GIL;
    the host build reads no mutable global)."""
    from concurrent.futures import ThreadPoolExecutor
    n, off = ct.batch_offsets(jobs)
    status = np.zeros(n, np.uint8)
    rec = np.zeros(n, ct.RECORD_DTYPE)
    params = np.ascontiguousarray(params, ct.PARAMS_DTYPE)

    def one(j):
        job = np.ascontiguousarray(jobs[j:j + 1])
        trig = ct.prepare_trig(job)
        m, o1 = ct.batch_offsets(job)
        st = np.zeros(m, np.uint8)
        r = np.zeros(m, ct.RECORD_DTYPE)
        rc = lib.host_trace(internal, external, _p(job), _p(trig), 1, _p(o1), m, _p(params), len(params), step_limit,
                            0.01, ct.DEF_HM0_P, _p(st), _p(r))
        status[off[j]:off[j + 1]] = st
        rec[off[j]:off[j + 1]] = r
        return rc
    with ThreadPoolExecutor(8) as ex:
        assert all(rc == 0 for rc in ex.map(one, range(len(jobs))))
    return status, rec, off


def _scan_cases():
    """(name, internal, external, jobs, params, sites) from the golden scans."""
    out = []
    for fn, ext, stride in (("scan_config0.json", ct.EXTERNAL_NONE, 38), ("scan_t96.json", ct.EXTERNAL_T96, 100),
                            ("scan_ts05.json", ct.EXTERNAL_TS05, 100)):
        g = golden(fn)
        sites = g["sites"][::stride]
        p = ct.internal_setup(g["model"], g["time"], parmod=g.get("parmod"))
        jobs = np.concatenate([ct.make_job(s["lat"], s["lon"], rig=g["rig"], rk=g["rk"], dele=g["del"],
                                           the1=s["the1"], fi1=s["fi1"]) for s in sites])
        out.append((fn, ext, jobs, p, sites))
    g = golden("scan_storm.json")
    c = g["conditions"][0]
    sites = c["sites"][:3]                 # vertical and both oblique directions
    jobs = np.concatenate([ct.make_job(s["lat"], s["lon"], rig=g["rig"], rk=g["rk"], dele=g["del"], the1=s["the1"],
                                       fi1=s["fi1"]) for s in sites])
    out.append(("scan_storm.json", ct.EXTERNAL_TS05, jobs, ct.internal_setup(g["model"], c["time"],
                                                                             parmod=c["parmod"]), sites))
    return out


def test_device_scan_logic_is_the_references(builds):
    """Every trajectory of sites from the IGRF, T96, TS05 and storm-condition
    golden scans: the allowed/forbidden flags equal the reference's, and the
    class and final record (position, velocity, time, length, step and trial
    counts) equal the oracle's -- the reference's arithmetic -- bit for bit."""
    lib = builds["reference_pow"]
    for name, ext, jobs, p, sites in _scan_cases():
        status, rec, off = _host_scan(lib, 1, ext, jobs, p)
        for j, s in enumerate(sites):
            allowed = np.nonzero(status[off[j]:off[j + 1]] == ct.TRAJ_ALLOWED)[0].tolist()
            assert allowed == s["allowed"], (name, s["lat"], s["lon"])
        o = pyoracle.scan_batch(jobs, p, models=ct.model_set(ct.INTERNAL_SH, ext), threads=8, want_records=True)
        assert np.array_equal(status, o.status), name
        assert np.array_equal(rec.view(np.uint8), o.records.view(np.uint8)), name


def test_crustal_warp_sum_within_ulps(builds):
    """chaos_geo_warp on an emulated warp (40 points: a full warp and a partly
    idle one) against the reference's chaos_geo: per order, then across the
    lanes, instead of degree by degree -- a few ulp of the crustal field."""
    lib = builds["default"]
    g, h, nmax = ct.chaos_table()
    k = golden("field_kats.json")["chaos_geo"]
    pts = unhex(k["points"]).reshape(-1, 3)
    want = unhex(k["b"]).reshape(-1, 3)
    got = np.zeros_like(pts)
    assert lib.host_chaos(_p(g), _p(h), nmax, _p(pts), len(pts), _p(got)) == 0
    rel = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert rel.max() <= 1e-13, rel.max()


def test_crustal_model_set_composes_bit_for_bit(builds):
    """calculate_field of the crustal model set (IGRF-14 + CHAOS-7.16, with and
    without T96) at the 200 golden points: the crustal part's last bits are far
    below the total's, so the composed field is the reference's bit for bit."""
    lib = builds["reference_pow"]
    g, h, nmax = ct.chaos_table()
    cf = golden("field_kats.json")["calculate_field"]
    pts = unhex(cf["points_m"]).reshape(-1, 3)
    for key, ext in (("igrf14+chaos7.16", ct.EXTERNAL_NONE), ("igrf14+t96+chaos7.16", ct.EXTERNAL_T96)):
        case = cf["cases"][key]
        p = ct.internal_setup("igrf14", cf["time"], parmod=unhex(case["parmod"]))
        got = np.zeros_like(pts)
        assert lib.host_calculate_field_crustal(1, ext, _p(p), _p(g), _p(h), nmax, _p(pts), len(pts), _p(got)) == 0
        assert _bits_equal(got, unhex(case["b"]).reshape(-1, 3)).all(), key


@pytest.mark.parametrize("job_copy", [0, 1])
def test_lane_regrouping_permutes_the_block(builds, job_copy):
    """regroup_lanes on an emulated 256-thread block (256 host threads, a block
    barrier and per-warp ballots): the threads that take part end up holding
    exactly their original trajectories, in ascending key order (ties in
    thread order), each with all of its own fields (step, segment slot and
    sequence, rigidity, the job's zn and nk1); the others keep theirs.  In the
    stream kernel's form the job fields land in the thread's own job copy."""
    lib = builds["default"]
    rng = np.random.default_rng(11)
    for trial in range(3):
        part = (rng.uniform(size=256) < (0.95, 0.5, 0.1)[trial]).astype(np.int32)
        key = rng.integers(0, 40, size=256).astype(np.uint32)
        out = np.zeros((256, 8))
        lib.host_regroup(_p(key), _p(part), job_copy, _p(out))
        origin = out[:, 0].astype(int)
        holders = np.nonzero(part)[0]
        # the threads that took part hold a permutation of their trajectories ...
        assert sorted(origin[holders]) == sorted(holders)
        # ... in ascending (key, original thread) order
        order = sorted(holders, key=lambda t: (int(key[t]), int(t)))
        assert list(origin[holders]) == order
        # the others are untouched
        rest = np.nonzero(part == 0)[0]
        assert np.array_equal(origin[rest], rest)
        # every field travelled with its trajectory
        assert np.array_equal(out[:, 1], 1000 + origin)
        assert np.array_equal(out[:, 2], origin)
        assert np.array_equal(out[:, 3], 100000 + origin)
        assert np.array_equal(out[:, 4], origin + 0.5)
        assert np.array_equal(out[:, 5], origin + 1.0)
        assert np.array_equal(out[:, 6], 7 + origin)
        assert np.array_equal(out[:, 7], np.ones(256) if job_copy else np.zeros(256))
