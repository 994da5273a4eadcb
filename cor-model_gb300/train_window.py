"""Train the learned rigidity window on cutoffs traced by the plain GPU scan.

    python cor-model_gb300/train_window.py [--external t96|ts05] [--samples N] [--val M] [--seed S] [--out FILE]

1. Seeded site-directions (uniform over the sphere; half vertical, half at
   30 deg zenith and one of 8 azimuths) and conditions (window.sample_conditions:
   Pdyn, Dst, By, Bz (and W1..W6 for TS05) over storm ranges, the tilt through
   the date), IGRF-14 + T96 or, with --external ts05, IGRF-14 + TS05.
2. Labels from the plain tracer (log GV), by one of two methods:
   * full (the default): the whole 0.01 GV scan of every sample, streamed
     through one scan stream (cor_stream_*); its R_U and R_L are exactly what
     the window has to hold;
   * coarse: a coarse scan (20 -> 0.1 GV by 0.1), then the 0.01 GV grid over
     the coarse penumbra plus a margin, about a seventh of the trajectories.
     The coarse scan cannot see penumbra structure finer than its step: over
     seeded storm-range samples, 9 of 48 came out with R_L too high (an allowed
     rigidity far below the main penumbra, up to 3.5 GV) and 1 with R_U too
     low, against the full scan.
3. The network (include/cor_window.h) is trained on the GPU with its own
   tensor-core kernels (AdamW, minibatches), on standardised features and
   targets.
4. The residual spread on the held-out samples, per band of predicted R_L
   (8 equal-count bands: the spread in log R is wide for low cutoffs, where a
   wide relative window is only a few grid points, and narrow above 4 GV),
   gives the sigma_U, sigma_L the windows are built from (prediction +- 3
   sigma).
5. With full labels, the held-out samples (drawn from their own seed) are
   scanned again through the trained windows and compared with their whole
   scans: R_C agreement, trajectories traced, and the time of both.
The result (parameters, standardisation, sigmas, provenance) goes to --out.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import cortrace as ct  # noqa: E402
import window  # noqa: E402

R0 = 1.0031391260673028          # 20 km, as the reference's INFILEs give it
COARSE = (0.1, 20.0, 0.1)
MARGIN = 20                      # fine-grid indices traced beyond the coarse penumbra


def sample_sites(rng, n):
    lat = np.degrees(np.arcsin(rng.uniform(-1, 1, n)))
    lon = rng.uniform(0, 360, n)
    vertical = rng.uniform(0, 1, n) < 0.5
    az = rng.integers(0, 8, n) * 45.0
    zen = np.where(vertical, 0.0, 30.0)
    return lat, lon, zen, np.where(vertical, 0.0, az)


def build_samples(rng, n, external="t96"):
    lat, lon, zen, az = sample_sites(rng, n)
    conds = window.sample_conditions(rng, n, external)
    params = np.concatenate([ct.internal_setup("igrf14", c["time7"], parmod=c["parmod"]) for c in conds])
    feats, dirs = [], []
    for k in range(n):
        the1, fi1 = window.arrival_direction(lat[k], lon[k], zen[k], az[k])
        dirs.append((the1, fi1))
        feats.append(window.features(lat[k], lon[k], zen[k], az[k], window.decimal_epoch(conds[k]["time7"]),
                                     conds[k]["parmod"], window.dipole_tilt(params[k:k + 1])))
    return {"lat": lat, "lon": lon, "dirs": dirs, "params": params, "features": np.array(feats)}


def _full_jobs(s, a, b):
    return np.concatenate([ct.make_job(s["lat"][k], s["lon"][k], rig=window.GRID_RIG, rk=20.0, dele=window.GRID_DEL,
                                       r0=R0, the1=s["dirs"][k][0], fi1=s["dirs"][k][1], param_index=k - a)
                           for k in range(a, b)])


STREAM_CHUNK = 400                # samples per stream segment (one parameter block each)
VAL_SEED_OFFSET = 7919            # held-out samples: seed + this


def label_stream(ctx, s, models, chunk=STREAM_CHUNK):
    """(log R_U, log R_L, R_C [GV], trajectories traced, seconds) of every
    sample from its whole 0.01 GV scan, the samples streamed through one
    scan stream in segments of `chunk` (each segment handed out lowest
    rigidity first)."""
    from collections import deque
    n = len(s["lat"])
    ru, rl, rc = np.zeros(n), np.zeros(n), np.zeros(n)
    traced = 0
    t0 = time.perf_counter()
    st = ct.Stream(ctx, models, slots=4, max_jobs=chunk, max_trajectories=chunk * window.GRID_N, max_params=chunk,
                   pool_params=8 * chunk, idle_limit_s=300.0)
    try:
        inflight = deque()
        spans = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
        nxt = 0
        while nxt < len(spans) or inflight:
            while nxt < len(spans) and len(inflight) < 4:
                a, b = spans[nxt]
                inflight.append((st.submit(_full_jobs(s, a, b), s["params"][a:b], want_status=False), a, b))
                nxt += 1
            t, a, b = inflight.popleft()
            res, _ = st.wait(t, -1)
            traced += int(res.counters["trajectories"])
            ru[a:b] = np.log(np.maximum(res.sites["r_upper"], window.GRID_RIG))
            rl[a:b] = np.log(np.maximum(res.sites["r_lower"], window.GRID_RIG))
            rc[a:b] = res.sites["r_cutoff"]
            print(f"  labelled {b}/{n} ({traced} trajectories, {time.perf_counter() - t0:.0f} s)", flush=True)
        st.drain()
    finally:
        st.close()
    return ru, rl, rc, traced, time.perf_counter() - t0


def label(ctx, s, models, chunk=4000, method="full"):
    """(log R_U, log R_L, trajectories traced) of every sample, by the
    full 0.01 GV scan or the coarse-then-fine method (module docstring),
    through ctx.trace_batch in chunks."""
    n = len(s["lat"])
    traced = 0
    ru = np.zeros(n)
    rl = np.zeros(n)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        if method == "full":
            res = ctx.trace_batch(_full_jobs(s, a, b), s["params"][a:b], models=models, want_status=False)
            traced += int(res.counters["trajectories"])
            ru[a:b] = np.log(np.maximum(res.sites["r_upper"], window.GRID_RIG))
            rl[a:b] = np.log(np.maximum(res.sites["r_lower"], window.GRID_RIG))
            print(f"  labelled {b}/{n} ({traced} trajectories)", flush=True)
            continue
        if method != "coarse":
            raise ValueError(f"label method {method!r}")
        jobs = np.concatenate([ct.make_job(s["lat"][k], s["lon"][k], rig=COARSE[0], rk=COARSE[1], dele=COARSE[2],
                                           r0=R0, the1=s["dirs"][k][0], fi1=s["dirs"][k][1], param_index=k - a)
                               for k in range(a, b)])
        res = ctx.trace_batch(jobs, s["params"][a:b], models=models, want_status=False)
        traced += int(res.counters["trajectories"])
        lo = np.array([res.sites[k]["r_lower"] for k in range(b - a)])
        hi = np.array([res.sites[k]["r_upper"] for k in range(b - a)])
        i_lo = np.clip(np.floor((lo - COARSE[2] - window.GRID_RIG) / window.GRID_DEL) - MARGIN, 0,
                       window.GRID_N - 1).astype(int)
        i_hi = np.clip(np.ceil((hi - window.GRID_RIG) / window.GRID_DEL) + MARGIN, 0, window.GRID_N - 1).astype(int)
        fine = np.concatenate([ct.make_job(s["lat"][k], s["lon"][k], rig=window.GRID_RIG, rk=20.0,
                                           dele=window.GRID_DEL, r0=R0, the1=s["dirs"][k][0], fi1=s["dirs"][k][1],
                                           param_index=k - a, i_first=int(i_lo[k - a]), i_last=int(i_hi[k - a]))
                               for k in range(a, b)])
        fr = ctx.trace_batch(fine, s["params"][a:b], models=models, want_status=False)
        traced += int(fr.counters["trajectories"])
        ru[a:b] = np.log(np.maximum(fr.sites["r_upper"], window.GRID_RIG))
        rl[a:b] = np.log(np.maximum(fr.sites["r_lower"], window.GRID_RIG))
        print(f"  labelled {b}/{n} ({traced} trajectories)", flush=True)
    return ru, rl, traced


def evaluate(ctx, wm_path, s, models, rc_full, full_seconds, full_traj):
    """The trained network's windows on held-out samples (their own seed)
    through a scan stream, against the same samples' whole scans: R_C
    agreement within 0.01 GV, trajectories traced, and the time of both."""
    wm = window.WindowModel(wm_path)
    try:
        wm.windows(s["features"][:8])
        n = len(s["lat"])
        st = ct.Stream(ctx, models, slots=8, max_jobs=n, max_trajectories=n * window.GRID_N, max_params=n,
                       pool_params=n, idle_limit_s=300.0)
        try:
            jobs = _full_jobs(s, 0, n)
            t0 = time.perf_counter()
            i_lo, i_hi = wm.windows(s["features"])   # no stream kernel runs yet: the network has the SMs
            (sites, fb, traced, _), = window.trace_windows_stream(st, [(jobs, s["params"], i_lo, i_hi)])
            st.drain()
            wall = time.perf_counter() - t0
        finally:
            st.close()
    finally:
        wm.close()
    d = np.abs(sites["r_cutoff"] - rc_full)
    return {"samples": int(n), "agree_frac_dRc_le_0.01GV": float(np.mean(d <= 0.01 + 1e-9)),
            "max_abs_dRc_GV": float(d.max()), "widened_frac": float(fb.mean()),
            "trajectories_frac_of_full_scan": traced / full_traj, "window_seconds": wall,
            "full_scan_seconds": full_seconds, "gain": full_seconds / wall}


def train(x, y, xv, yv, seed, epochs, batch=512, lr=2e-3):
    import torch
    net = window.Network(0, max_batch=max(batch, len(xv)))
    net.set_params(window.init_params(seed))
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    yd = torch.from_numpy(y.astype(np.float32)).cuda()
    rng = np.random.default_rng(seed)
    n = len(x)
    steps = 0
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
        tot = 0.0
        for a in range(0, n - batch + 1, batch):
            idx = perm[a:a + batch]
            tot += net.train_step(xd[idx], yd[idx], lr=lr_ep, weight_decay=1e-4)
            steps += 1
        if ep % 10 == 0 or ep == epochs - 1:
            pv = net.forward(torch.from_numpy(xv.astype(np.float32)).cuda()).cpu().numpy()
            print(f"  epoch {ep}: train loss {tot / max(1, n // batch):.4f}, val mse {np.mean((pv - yv) ** 2):.4f}",
                  flush=True)
    params = net.get_params()
    pv = net.forward(torch.from_numpy(xv.astype(np.float32)).cuda()).cpu().numpy()
    net.close()
    return params, pv, steps


EXTERNALS = {"t96": ct.EXTERNAL_T96, "ts05": ct.EXTERNAL_TS05}


def default_paths(external: str, label_method: str) -> tuple[str, str]:
    """(network file, labels file) for a field model and label method:
    window_<ext>.npz, and window_<ext>_labels.npz (coarse) or
    window_<ext>_labels_full.npz (full)."""
    labels = f"window_{external}_labels.npz" if label_method == "coarse" else f"window_{external}_labels_full.npz"
    return os.path.join(HERE, f"window_{external}.npz"), os.path.join(HERE, labels)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--external", default="t96", choices=sorted(EXTERNALS),
                    help="external field model of the samples and labels (IGRF-14 is the internal one)")
    ap.add_argument("--samples", type=int, default=8000)
    ap.add_argument("--val", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--out", default=None, help="default: window_<external>.npz")
    ap.add_argument("--label-method", default="full", choices=["full", "coarse"])
    ap.add_argument("--no-eval", action="store_true",
                    help="skip the window scan of the held-out samples against their whole scans")
    ap.add_argument("--labels", default=None,
                    help="labelled set: loaded when the file exists, else traced and saved there (default: "
                         "window_<external>_labels.npz for the coarse method, window_<external>_labels_full.npz "
                         "for full)")
    args = ap.parse_args()
    out_default, labels_default = default_paths(args.external, args.label_method)
    args.out = args.out or out_default
    args.labels = args.labels or labels_default
    rng = np.random.default_rng(args.seed)
    models = ct.model_set(ct.INTERNAL_SH, EXTERNALS[args.external])
    t0 = time.time()
    tr = build_samples(rng, args.samples, args.external)
    # the held-out set is a fresh draw from its own seed
    va = build_samples(np.random.default_rng(args.seed + VAL_SEED_OFFSET), args.val, args.external)
    vrc = None
    val_seconds = 0.0
    if args.labels and os.path.exists(args.labels):
        d = np.load(args.labels)
        assert d["features"].shape == tr["features"].shape, "labels were made for other samples"
        made = str(d["method"]) if "method" in d else "coarse"
        assert made == args.label_method, f"{args.labels} holds {made} labels"
        ru, rl, vru, vrl = d["ru"], d["rl"], d["vru"], d["vrl"]
        va["features"] = d["val_features"]        # the held-out samples the file's labels belong to
        n1, n2 = int(d["n1"]), int(d["n2"])
        if "vrc" in d:
            vrc, val_seconds = d["vrc"], float(d["val_seconds"])
    else:
        ctx = ct.Context(0)
        if args.label_method == "full":
            ru, rl, _, n1, _ = label_stream(ctx, tr, models)
            vru, vrl, vrc, n2, val_seconds = label_stream(ctx, va, models)
        else:
            ru, rl, n1 = label(ctx, tr, models, method=args.label_method)
            vru, vrl, n2 = label(ctx, va, models, method=args.label_method)
        ctx.close()
        if args.labels:
            extra = {} if vrc is None else {"vrc": vrc, "val_seconds": val_seconds}
            np.savez(args.labels, features=tr["features"], ru=ru, rl=rl, val_features=va["features"], vru=vru,
                     vrl=vrl, n1=n1, n2=n2, method=args.label_method, **extra)
    t_label = time.time() - t0
    print(f"labels: {n1 + n2} trajectories in {t_label:.0f} s", flush=True)
    fm, fs = tr["features"].mean(0), tr["features"].std(0)
    fs[fs == 0] = 1.0
    y = np.stack([ru, rl], 1)
    ym, ys = y.mean(0), y.std(0)
    x = (tr["features"] - fm) / fs
    xv = (va["features"] - fm) / fs
    yn = (y - ym) / ys
    yvn = (np.stack([vru, vrl], 1) - ym) / ys
    params, pv, steps = train(x, yn, xv, yvn, args.seed, args.epochs, batch=args.batch)
    pred = pv * ys + ym
    truth = np.stack([vru, vrl], 1)
    resid = pred - truth
    sigma = resid.std(0)
    edges, band_sigma = window.band_sigmas(pred, resid)
    b = window.band_of(pred[:, 1], edges)
    lo = np.exp(pred[:, 1] - 3 * band_sigma[b, 1])
    hi = np.exp(pred[:, 0] + 3 * band_sigma[b, 0])
    miss = np.mean((lo > np.exp(truth[:, 1])) | (hi < np.exp(truth[:, 0])))
    print(f"held-out residual sigma (log R): U {sigma[0]:.4f}, L {sigma[1]:.4f}; per band of predicted R_L "
          f"(edges {np.exp(edges).round(2).tolist()} GV): U {band_sigma[:, 0].round(3).tolist()}, "
          f"L {band_sigma[:, 1].round(3).tolist()}; held-out windows missing the penumbra: {miss:.4f}", flush=True)
    info = {"samples": args.samples, "val": args.val, "seed": args.seed, "epochs": args.epochs, "steps": steps,
            "batch": args.batch, "sigma_log_ru": float(sigma[0]), "sigma_log_rl": float(sigma[1]),
            "band_sigma": band_sigma.round(4).tolist(), "heldout_window_miss": float(miss),
            "model": f"igrf14+{args.external}", "label_method": args.label_method, "label_trajectories": n1 + n2,
            "label_seconds": t_label,
            "total_seconds": time.time() - t0}
    save = lambda: np.savez(args.out, params=params, feat_mean=fm, feat_std=fs, y_mean=ym, y_std=ys, sigma=sigma,
                            band_edges=edges, band_sigma=band_sigma, val_features=va["features"],
                            val_targets=np.stack([vru, vrl], 1), info=json.dumps(info))
    save()
    if vrc is not None and not args.no_eval and "lat" in va:
        # the held-out samples through the trained windows, against their
        # whole scans timed while labelling
        ctx = ct.Context(0)
        try:
            info["heldout_eval"] = evaluate(ctx, args.out, va, models, vrc, val_seconds, n2)
        finally:
            ctx.close()
        save()
    print(json.dumps(info), flush=True)


if __name__ == "__main__":
    main()
