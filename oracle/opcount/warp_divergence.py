"""TEST INFRASTRUCTURE: how many lanes of a warp the IGRF-14 + T96 field
evaluation keeps busy, estimated on the CPU.

A warp issues every call site that any of its lanes reaches, so its cost is
the sum over the call sites its lanes reach, and lanes that do not need a
site sit idle while it runs.  With lanes refilled from the queue as their
trajectories end, a warp's lanes hold unrelated trajectories, so in steady
state they behave like independent draws from the positions where the field
is evaluated, weighted by step.  This script
  1. samples those positions: the accepted steps of oracle trajectories of
     the bench workload (IGRF-14 + T96 at the bench condition, sites of the
     5-degree grid, vertical arrival at 20 km, 0.01-20 GV);
  2. prices every expensive T96 call site at each position with the
     op-counting oracle (t96_site_costs.cpp; weighted FP64 operations with
     the transcendental costs measured on the GPU), and the internal field by
     its degree at that radius (orc_internal_geo_flops);
  3. forms blocks of 256 positions, splits them into warps of 32 and prices
     each warp under three layouts of the field code:
       * per-band call sites: birk1tot_02 and r2_birk as the reference writes
         them (lib/t96/t96.c:619-807, :1265-1314), one call of a sub-model
         per band, so a warp whose lanes span several bands repeats them;
       * single call sites: each sub-model called once per evaluation
         (csrc/t96.cuh);
       * single call sites with the block's lanes sorted by field_band's key
         (csrc/field.cuh) before the warps are formed (the scan stream's
         sort_lanes).
Lanes per operation = the lanes' own work / the warp's issued work x 32; the
field evaluation only (the step logic around it is left out).  It also sizes
splitting a lone long trajectory's field evaluation over the SM's four FP64
pipes (tail_split).

usage: python oracle/opcount/warp_divergence.py [n_trajectories]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
sys.path[:0] = [ORACLE, os.path.join(ROOT, "cor-model_gb300")]

EXE = os.path.join(HERE, "t96_site_costs")
TIME7 = [2020, 6, 21, 173, 12, 0, 0]
PARMOD = [2.0, -20.0, 0.0, -1.0]
N_POSITIONS = 120000
RE = 6.3712e6
# column indices of t96_site_costs' output
(WHOLE, SIGMA, CYL, TAIL, B2S, IC, B1S, B1PRE, B1BAND, LX, CX, BLEND, LE1, CE1, LE2, CE2, XKSI, R2BAND, OUTER,
 SHEET, INNER, R2BIRK, B1TOT, RADIUS, RINGCURR, SHLCAR, TAILDISK, TAIL87, NCOLS) = range(29)
LONG = 5000   # accepted steps: the trajectories that make a run's tail


def build() -> str:
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + ORACLE, "-include",
                    os.path.join(HERE, "flop.hpp"), "-x", "c++", os.path.join(HERE, "t96_site_costs.cpp"),
                    "-o", EXE], check=True)
    return EXE


def _trajectory(args):
    import cortrace as ct
    import pyoracle
    lat, lon, rig = args
    p = ct.internal_setup("igrf14", TIME7, parmod=PARMOD)
    job = ct.make_job(lat, lon, rig=rig, rk=rig, dele=0.01)
    return pyoracle.trace_steps(job, p, models=ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96))["gsm"].copy()


def sample_positions(n_traj: int, seed: int = 5) -> tuple[np.ndarray, np.ndarray]:
    """-> (positions, the accepted steps of the trajectory each belongs to)."""
    rng = np.random.default_rng(seed)
    sites = [(float(a), float(b)) for a in range(-90, 91, 5) for b in range(0, 360, 5)]
    picks = [(*sites[rng.integers(len(sites))], round(0.01 * int(rng.integers(1, 2001)), 2)) for _ in range(n_traj)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        runs = pool.map(_trajectory, picks, chunksize=1)
    pts = np.concatenate(runs)
    length = np.repeat([len(r) for r in runs], [len(r) for r in runs])
    keep = np.sort(np.random.default_rng(seed + 1).choice(len(pts), min(N_POSITIONS, len(pts)), replace=False))
    return np.ascontiguousarray(pts[keep]), length[keep]


def site_costs(pos: np.ndarray) -> np.ndarray:
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "pos.bin"), os.path.join(td, "costs.bin")
        pos.astype("<f8").tofile(fi)
        subprocess.run([EXE, fi, fo, *map(str, PARMOD)], check=True)
        return np.fromfile(fo).reshape(-1, NCOLS)


def internal_costs(radius: np.ndarray) -> np.ndarray:
    import pyoracle
    table = {k: pyoracle.internal_geo_flops(float(k) + 0.5) for k in np.unique(radius.astype(int))}
    return np.array([table[k] for k in radius.astype(int)], float)


def field_band_key(pos: np.ndarray, r2band: np.ndarray) -> np.ndarray:
    """field_band<ModelSet<1,1,0>> (csrc/field.cuh) from the oracle's band."""
    x = pos / RE
    r = np.linalg.norm(x, axis=1)
    ri = np.minimum(r.astype(int), 31)
    lat = np.minimum((np.abs(x[:, 2]) / r * 12.0).astype(int), 12)
    return (r2band.astype(int) << 9) | (ri << 4) | lat


class WarpModel:
    def __init__(self, c: np.ndarray, igrf: np.ndarray):
        self.c, self.igrf = c, igrf
        self.inside = c[:, SIGMA] < 2
        b1 = c[:, B1BAND].astype(int)
        self.b1, self.r2 = b1, c[:, R2BAND].astype(int)
        # each part's own share: the birk1tot_02 work before the band decision,
        # the blend's own arithmetic, r2_birk's own arithmetic
        self.blend_pre = np.where(b1 == 2, c[:, BLEND] - c[:, LE1] - c[:, CE2],
                                  np.where(b1 == 3, c[:, BLEND] - c[:, CE1] - c[:, LE2], 0.0))
        calls = np.select([self.r2 == 0, self.r2 == 1, self.r2 == 2, self.r2 == 3, self.r2 == 4],
                          [c[:, OUTER], c[:, OUTER] + c[:, SHEET], c[:, SHEET], c[:, INNER] + c[:, SHEET],
                           c[:, INNER]])
        self.r2_pre = c[:, R2BIRK] - calls
        parts = c[:, CYL] + c[:, TAIL] + c[:, B2S] + c[:, IC] + c[:, B1TOT] + c[:, R2BIRK]
        self.pre = np.where(self.inside, c[:, WHOLE] - parts, c[:, WHOLE])
        self.lane = c[:, WHOLE] + igrf

    def warp(self, ix: np.ndarray, single_sites: bool) -> float:
        c, i, b1, r2 = self.c[ix], self.inside[ix], self.b1[ix], self.r2[ix]

        def mx(col, m):
            v = col[m]
            return float(v.max()) if len(v) else 0.0
        w = float(self.pre[ix].max()) + float(self.igrf[ix].max())
        if not i.any():
            return w
        for col in (CYL, TAIL, B2S, IC, B1S, B1PRE, XKSI):
            w += mx(c[:, col], i)
        w += mx(self.r2_pre[ix], i)
        if single_sites:
            loops = np.concatenate([c[i & (b1 == 0), LX], c[i & (b1 == 2), LE1], c[i & (b1 == 3), LE2]])
            condip = np.concatenate([c[i & (b1 == 1), CX], c[i & (b1 == 2), CE2], c[i & (b1 == 3), CE1]])
            w += (loops.max() if len(loops) else 0.0) + (condip.max() if len(condip) else 0.0)
            w += mx(self.blend_pre[ix], i & (b1 >= 2))
            w += mx(c[:, OUTER], i & (r2 <= 1)) + mx(c[:, SHEET], i & (r2 >= 1) & (r2 <= 3))
            w += mx(c[:, INNER], i & (r2 >= 3))
        else:
            w += mx(c[:, LX], i & (b1 == 0)) + mx(c[:, CX], i & (b1 == 1))
            if (i & (b1 >= 2)).any():
                # one blend call site; its two bases behind a north/south branch each
                w += mx(self.blend_pre[ix], i & (b1 >= 2))
                w += mx(c[:, LE1], i & (b1 == 2)) + mx(c[:, CE2], i & (b1 == 2))
                w += mx(c[:, CE1], i & (b1 == 3)) + mx(c[:, LE2], i & (b1 == 3))
            w += mx(c[:, OUTER], i & (r2 == 0)) + mx(c[:, OUTER], i & (r2 == 1)) + mx(c[:, SHEET], i & (r2 == 1))
            w += mx(c[:, SHEET], i & (r2 == 2)) + mx(c[:, INNER], i & (r2 == 3)) + mx(c[:, SHEET], i & (r2 == 3))
            w += mx(c[:, INNER], i & (r2 == 4))
        return w

    def layout(self, single_sites: bool, key: np.ndarray | None, blocks: int = 300, seed: int = 0) -> dict:
        rng = np.random.default_rng(seed)
        lane_work = warp_work = 0.0
        for _ in range(blocks):
            ix = rng.choice(len(self.lane), 256, replace=False)
            if key is not None:
                ix = ix[np.argsort(key[ix], kind="stable")]
            for w in range(8):
                wi = ix[32 * w:32 * w + 32]
                lane_work += float(self.lane[wi].sum())
                warp_work += self.warp(wi, single_sites)
        return {"lanes_per_op": 32.0 * lane_work / (32.0 * warp_work), "warp_work": warp_work}


def tail_split(c: np.ndarray, igrf: np.ndarray, pipes: int = 4) -> dict:
    """A lone trajectory's field evaluation split over the SM's FP64 pipes
    (one warp per pipe, each taking whole independent sub-models), priced on
    positions of long trajectories: the sub-models' mean costs, and the
    longest-first assignment's makespan against the serial sum.  Chains that
    must stay together: birk1tot_02's band decision with the basis it picks
    (and, in a band, the decision before both bases), r2_birk's xksi with the
    field it picks."""
    b1 = c[:, B1BAND].astype(int)
    r2 = c[:, R2BAND].astype(int)
    band = b1 >= 2
    blend_pre = np.where(b1 == 2, c[:, BLEND] - c[:, LE1] - c[:, CE2],
                         np.where(b1 == 3, c[:, BLEND] - c[:, CE1] - c[:, LE2], 0.0))
    pre = c[:, B1PRE] + blend_pre            # what both bases wait for (each warp that takes one repeats it)
    needs_loops, needs_condip = b1 != 1, b1 != 0
    items = {
        "internal field": igrf,
        "cylharm (dipole shield)": c[:, CYL],
        "ringcurr": c[:, RINGCURR],
        "ring-current shield": c[:, SHLCAR],
        "tail sheet (taildisk)": c[:, TAILDISK],
        "tail shield 2": c[:, SHLCAR],
        "tail87": c[:, TAIL87],
        "tail shield 3": c[:, SHLCAR],
        "birk1 band decision + loops basis": np.where(needs_loops, pre + np.select(
            [b1 == 0, b1 == 2, b1 == 3], [c[:, LX], c[:, LE1], c[:, LE2]], 0.0), 0.0),
        "birk1 band decision + conical basis": np.where(needs_condip, pre + np.select(
            [b1 == 1, b1 == 2, b1 == 3], [c[:, CX], c[:, CE2], c[:, CE1]], 0.0), 0.0),
        "birk1 shield": c[:, B1S],
        "birk2 shield": c[:, B2S],
        "r2 xksi + outer": np.where(r2 <= 1, c[:, XKSI] + c[:, OUTER], 0.0),
        "r2 xksi + sheet": np.where((r2 >= 1) & (r2 <= 3), c[:, XKSI] + c[:, SHEET], 0.0),
        "r2 xksi + inner": np.where(r2 >= 3, c[:, XKSI] + c[:, INNER], 0.0),
        "intercon": c[:, IC],
    }
    means = {k: float(v.mean()) for k, v in items.items()}
    serial = float((c[:, WHOLE] + igrf).mean())   # the unsplit evaluation
    load = [0.0] * pipes
    for v in sorted(means.values(), reverse=True):
        load[load.index(min(load))] += v
    return {"mean_cost": {k: round(v) for k, v in means.items()}, "serial": round(serial),
            "band_share": float(band.mean()), "pipes": pipes, "makespan": round(max(load)),
            "speedup": serial / max(load)}


def main(n_traj: int) -> dict:
    build()
    pos, length = sample_positions(n_traj)
    c = site_costs(pos)
    m = WarpModel(c, internal_costs(c[:, RADIUS]))
    key = field_band_key(pos, c[:, R2BAND])
    base = m.layout(False, None)
    single = m.layout(True, None)
    sorted_ = m.layout(True, key)
    ins = m.inside
    return {
        "positions": int(len(pos)), "trajectories": n_traj,
        "inside_magnetopause": float(ins.mean()),
        "birk1_bands_loops_condip_north_south": (np.bincount(m.b1[ins], minlength=4) / ins.sum()).round(4).tolist(),
        "r2_bands_outer_mix_sheet_mix_inner": (np.bincount(m.r2[ins], minlength=5) / ins.sum()).round(4).tolist(),
        "mean_cost": {"t96": float(c[:, WHOLE].mean()), "internal": float(m.igrf.mean()),
                      "r1_loops": float(c[ins, LX].mean()), "r1_condip": float(c[ins, CX].mean()),
                      "r2_outer": float(c[ins, OUTER].mean()), "r2_sheet": float(c[ins, SHEET].mean()),
                      "r2_inner": float(c[ins, INNER].mean()), "xksi (the sort key)": float(c[ins, XKSI].mean())},
        "per_band_call_sites_random_warps": {"lanes_per_op": base["lanes_per_op"]},
        "single_call_sites_random_warps": {"lanes_per_op": single["lanes_per_op"],
                                           "speedup": base["warp_work"] / single["warp_work"]},
        "single_call_sites_sorted_by_field_band": {"lanes_per_op": sorted_["lanes_per_op"],
                                                   "speedup": base["warp_work"] / sorted_["warp_work"]},
        f"tail_split_over_4_pipes (positions of trajectories >= {LONG} steps)":
            tail_split(c[length >= LONG], m.igrf[length >= LONG]),
    }


if __name__ == "__main__":
    print(json.dumps(main(int(sys.argv[1]) if len(sys.argv) > 1 else 400), indent=1))
