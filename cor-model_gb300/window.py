"""The learned rigidity window (include/cor_window.h) on the host side.

A site-direction and its conditions become COR_MLP_IN features; the network
(trained on cutoffs the plain tracer produced) predicts log R_U and log R_L;
the scan then traces only the grid indices of the window
[exp(log R_L - k sigma_L), exp(log R_U + k sigma_U)] and falls back to the full
scan of the site whenever a boundary lands on a window edge.  The reference
has no counterpart; the plain scan judges every result.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

import cortrace as ct

N_IN, HIDDEN, LAYERS, N_OUT = 19, 256, 4, 2
N_PARAMS = 256 * 19 + 256 + 3 * (256 * 256 + 256) + 2 * 256 + 2
SHAPES = [(256, 19), (256,), (256, 256), (256,), (256, 256), (256,), (256, 256), (256,), (2, 256), (2,)]


def _bind(lib: C.CDLL) -> C.CDLL:
    if getattr(lib, "_mlp_bound", False):
        return lib
    vp, i32, f32 = C.c_void_p, C.c_int32, C.c_float
    lib.cor_mlp_create.argtypes = [C.c_int, i32, C.POINTER(vp)]
    lib.cor_mlp_destroy.argtypes = [vp]
    lib.cor_mlp_error.argtypes = [vp]
    lib.cor_mlp_error.restype = C.c_char_p
    lib.cor_mlp_set_params.argtypes = [vp, vp]
    lib.cor_mlp_get_params.argtypes = [vp, vp]
    lib.cor_mlp_forward.argtypes = [vp, vp, i32, vp, vp]
    lib.cor_mlp_train_step.argtypes = [vp, vp, vp, i32, f32, f32, vp, vp, vp]
    lib.cor_mlp_gradient.argtypes = [vp, vp, vp, i32, vp, vp, vp]
    lib._mlp_bound = True
    return lib


def init_params(seed: int) -> np.ndarray:
    """Seeded initial parameters: weights and biases uniform in
    +-1/sqrt(fan_in) of their layer."""
    rng = np.random.default_rng(seed)
    out = []
    fan_in = None
    for shp in SHAPES:
        if len(shp) == 2:
            fan_in = shp[1]
        lim = 1.0 / math.sqrt(fan_in)
        out.append(rng.uniform(-lim, lim, shp).astype(np.float32))
    return np.concatenate([a.ravel() for a in out])


def split_params(p: np.ndarray) -> list[np.ndarray]:
    out, o = [], 0
    for shp in SHAPES:
        n = int(np.prod(shp))
        out.append(p[o:o + n].reshape(shp))
        o += n
    return out


class Network:
    """cor_mlp: the network's device state (weights, AdamW moments, buffers)."""

    def __init__(self, device: int = 0, max_batch: int = 8192):
        import torch
        self.torch = torch
        self.lib = _bind(ct.load())
        h = C.c_void_p()
        rc = self.lib.cor_mlp_create(device, max_batch, C.byref(h))
        if rc != 0:
            raise ct.CorError(rc, "cannot create the network")
        self.h = h
        self.device = device
        self.max_batch = max_batch
        self.loss = torch.zeros(1, dtype=torch.float32, device=f"cuda:{device}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.cor_mlp_destroy(self.h)
            self.h = None

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise ct.CorError(rc, f"{what}: {self.lib.cor_mlp_error(self.h).decode()}")

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == N_PARAMS
        self._check(self.lib.cor_mlp_set_params(self.h, p.ctypes.data), "set_params")

    def get_params(self) -> np.ndarray:
        p = np.zeros(N_PARAMS, np.float32)
        self._check(self.lib.cor_mlp_get_params(self.h, p.ctypes.data), "get_params")
        return p

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def forward(self, x):
        """x: torch CUDA float32 (n, 19) -> (n, 2)."""
        assert x.dim() == 2 and x.shape[1] == N_IN, x.shape
        x = x.to(device=self.device, dtype=self.torch.float32).contiguous()
        y = self.torch.empty((x.shape[0], N_OUT), dtype=self.torch.float32, device=x.device)
        self._check(self.lib.cor_mlp_forward(self.h, x.data_ptr(), x.shape[0], y.data_ptr(), self._stream()),
                    "forward")
        return y

    def train_step(self, x, t, lr: float, weight_decay: float = 1e-4) -> float:
        assert x.shape[1] == N_IN and t.shape[1] == N_OUT and x.shape[0] == t.shape[0]
        x = x.to(device=self.device, dtype=self.torch.float32).contiguous()
        t = t.to(device=self.device, dtype=self.torch.float32).contiguous()
        self._check(self.lib.cor_mlp_train_step(self.h, x.data_ptr(), t.data_ptr(), x.shape[0], lr, weight_decay,
                                                self.loss.data_ptr(), None, self._stream()), "train_step")
        return float(self.loss.item())

    def gradient(self, x, t):
        """(loss, gradient in the parameter layout) without an update."""
        assert x.shape[1] == N_IN and t.shape[1] == N_OUT and x.shape[0] == t.shape[0]
        x = x.to(device=self.device, dtype=self.torch.float32).contiguous()
        t = t.to(device=self.device, dtype=self.torch.float32).contiguous()
        g = self.torch.zeros(N_PARAMS, dtype=self.torch.float32, device=x.device)
        self._check(self.lib.cor_mlp_gradient(self.h, x.data_ptr(), t.data_ptr(), x.shape[0], self.loss.data_ptr(),
                                              g.data_ptr(), self._stream()), "gradient")
        return float(self.loss.item()), g.cpu().numpy()


# ---- features of a site-direction and its conditions --------------------------
# The N_IN = 19 inputs: sin/cos latitude, sin/cos longitude, zenith [deg],
# sin/cos azimuth, decimal epoch, Pdyn, Dst, By, Bz, dipole tilt [deg], W1..W6.
# The start altitude is 20 km in every configuration, so it is not an input.
R_E_KM = 6371.2


def arrival_direction(lat: float, lon: float, zenith: float, azimuth: float) -> tuple[float, float]:
    """(the1, fi1): latitude and longitude [deg] of the outward direction a
    particle arriving from (zenith, azimuth) is backtraced along (azimuth
    from north through east); vertical incidence gives (lat, lon)."""
    if zenith == 0.0:
        return lat, lon
    la, lo, z, a = (math.radians(v) for v in (lat, lon, zenith, azimuth))
    up = np.array([math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)])
    north = np.array([-math.sin(la) * math.cos(lo), -math.sin(la) * math.sin(lo), math.cos(la)])
    east = np.array([-math.sin(lo), math.cos(lo), 0.0])
    v = math.cos(z) * up + math.sin(z) * (math.cos(a) * north + math.sin(a) * east)
    return math.degrees(math.asin(max(-1.0, min(1.0, v[2])))), math.degrees(math.atan2(v[1], v[0])) % 360.0


def dipole_tilt(p: np.ndarray) -> float:
    """Dipole tilt [deg] of a parameter block: the angle between the
    dipole axis (from g10, g11, h11) and the GSM y-z plane."""
    p = np.asarray(p).reshape(-1)[0]
    m = -np.array([p["g"][2], p["h"][2], p["g"][1]], np.float64)   # (g11, h11, g10) in the SH index order
    m /= np.linalg.norm(m)
    return math.degrees(math.asin(float(np.dot(m, np.asarray(p["a1"], np.float64)))))


def decimal_epoch(time7) -> float:
    iy, _, _, doy, ih, mi, sec = time7
    days = 366.0 if (iy % 4 == 0 and (iy % 100 != 0 or iy % 400 == 0)) else 365.0
    return iy + (doy - 1 + (ih + (mi + sec / 60.0) / 60.0) / 24.0) / days


def features(lat, lon, zenith, azimuth, epoch, parmod, tilt) -> np.ndarray:
    pm = np.zeros(10)
    pm[:len(parmod)] = parmod
    la, lo, az = math.radians(lat), math.radians(lon), math.radians(azimuth)
    f = np.array([math.sin(la), math.cos(la), math.sin(lo), math.cos(lo), zenith, math.sin(az), math.cos(az), epoch,
                  *pm[:4], tilt, *pm[4:10]], np.float64)
    assert f.size == N_IN
    return f


def time7_of(year: int, doy: int, hour: int, minute: int = 0) -> list[int]:
    """{iy, mes, ide, id, ih, min, is} for a day of the year."""
    import datetime as dt
    d = dt.date(year, 1, 1) + dt.timedelta(days=doy - 1)
    return [year, d.month, d.day, doy, hour, minute, 0]


def sample_conditions(rng: np.random.Generator, n: int, external: str = "t96") -> list[dict]:
    """Seeded storm-range conditions: Pdyn ~ U[1,10] nPa, Dst ~ U[-300,0] nT,
    By, Bz ~ U[-20,20] nT, W1..W6 ~ U[0,5] (TS05 only); the dipole tilt is
    set through the date and hour (2020), as the reference has no tilt input."""
    out = []
    for _ in range(n):
        pm = [rng.uniform(1, 10), rng.uniform(-300, 0), rng.uniform(-20, 20), rng.uniform(-20, 20)]
        if external == "ts05":
            pm += list(rng.uniform(0, 5, 6))
        out.append({"time7": time7_of(2020, int(rng.integers(1, 367)), int(rng.integers(0, 24))), "parmod": pm})
    return out


# ---- windows on the rigidity grid -------------------------------------------------
GRID_RIG, GRID_DEL, GRID_N = 0.01, 0.01, 2000     # 0.01 -> 20 GV, the scans' 0.01 GV grid


def window_indices(log_ru, log_rl, sigma_u, sigma_l, k=3.0, n=GRID_N, rig=GRID_RIG, dele=GRID_DEL):
    """Grid index windows [i_lo, i_hi] covering [R_L e^(-k sigma_L), R_U e^(k sigma_U)]."""
    lo = np.exp(np.minimum(log_rl, log_ru) - k * sigma_l)
    hi = np.exp(np.maximum(log_ru, log_rl) + k * sigma_u)
    i_lo = np.clip(np.floor((lo - rig) / dele), 0, n - 1).astype(np.int64)
    i_hi = np.clip(np.ceil((hi - rig) / dele), 0, n - 1).astype(np.int64)
    return i_lo, np.maximum(i_hi, i_lo)


def edge_hit(status_row: np.ndarray, i_lo: int, i_hi: int, n: int = GRID_N) -> bool:
    """A window scan is conclusive when its first rigidity is forbidden (or is
    the grid's first) and its last is allowed (or is the grid's last): then
    everything below is forbidden and everything above allowed as far as the
    plain scan of the window can tell.  Otherwise a boundary sits on an edge
    and the site falls back to the full scan."""
    allowed = status_row == ct.TRAJ_ALLOWED
    if i_lo > 0 and allowed[0]:
        return True
    if i_hi < n - 1 and not allowed[-1]:
        return True
    return False


def band_of(log_rl: np.ndarray, edges: np.ndarray) -> np.ndarray:
    """Band index of predicted log R_L values for the inner band edges."""
    return np.searchsorted(np.asarray(edges), np.asarray(log_rl), side="right")


def band_sigmas(pred: np.ndarray, resid: np.ndarray, n_bands: int = 8):
    """(inner edges, sigma per band): equal-count bands of predicted log R_L
    and the standard deviation of the held-out residuals (log R_U, log R_L)
    in each."""
    edges = np.quantile(pred[:, 1], np.linspace(0, 1, n_bands + 1))[1:-1]
    b = band_of(pred[:, 1], edges)
    sig = np.array([resid[b == k].std(0) if np.sum(b == k) > 1 else resid.std(0) for k in range(n_bands)])
    return edges, sig


def window_jobs(jobs: np.ndarray, i_lo: np.ndarray, i_hi: np.ndarray) -> np.ndarray:
    """The jobs restricted to grid windows [i_lo, i_hi] (inclusive)."""
    w = np.array(jobs, copy=True)
    w["i_first"] = i_lo
    w["i_count"] = i_hi - i_lo + 1
    return w


def trace_windows(ctx, jobs, params, models, i_lo, i_hi, widen: int = 3, **kw):
    """Scan every job over its window.  A job whose window had a boundary on
    an edge is scanned again over a window widened on that side (its width
    doubled there, clipped to the grid), up to `widen` times, and then over
    its whole grid: every reported cutoff comes from a window whose first
    rigidity is forbidden and whose last is allowed (or from the whole scan).
    Returns (sites, mask of jobs that needed more than one pass, trajectories
    traced, accepted steps)."""
    n_grid = (np.round((jobs["rk"] - jobs["rig"]) / jobs["del"]).astype(np.int64) + 1)
    lo = np.asarray(i_lo, np.int64).copy()
    hi = np.asarray(i_hi, np.int64).copy()
    sites = np.zeros(len(jobs), ct.SITE_DTYPE)
    redone = np.zeros(len(jobs), bool)
    todo = np.arange(len(jobs))
    traced = steps = 0
    for attempt in range(widen + 2):
        if len(todo) == 0:
            break
        if attempt == widen + 1:                 # last resort: the whole grid
            lo[todo] = 0
            hi[todo] = n_grid[todo] - 1
        res = ctx.trace_batch(window_jobs(jobs[todo], lo[todo], hi[todo]), params, models=models, **kw)
        traced += int(res.counters["trajectories"])
        steps += int(res.counters["accepted_steps"])
        again = []
        for k, j in enumerate(todo):
            st = res.status[res.offsets[k]:res.offsets[k + 1]]
            allowed = st == ct.TRAJ_ALLOWED
            low = lo[j] > 0 and allowed[0]
            high = hi[j] < n_grid[j] - 1 and not allowed[-1]
            if not (low or high):
                sites[j] = res.sites[k]
                continue
            width = hi[j] - lo[j] + 1
            if low:
                lo[j] = max(0, lo[j] - width)
            if high:
                hi[j] = min(n_grid[j] - 1, hi[j] + width)
            again.append(j)
        redone[again] = True
        todo = np.array(again, np.int64)
    return sites, redone, traced, steps


def trace_windows_stream(stream, items, widen: int = 3, poll_s: float = 0.002):
    """trace_windows for many batches at once through a scan stream
    (cortrace.Stream): items are (jobs, params, i_lo, i_hi).  Every batch's
    windows go in as one segment; a scan whose window had a boundary on an
    edge goes back in over a widened window (the same rule as trace_windows),
    so first passes and retraces are in flight together.  With a stream made
    with scan_events=1, each scan's result is taken the moment the scan is
    reduced (cor_stream_poll_scans) and its retrace goes in at once, without
    waiting for the rest of its segment.  Returns, per item, (sites, mask of
    jobs that needed more than one pass, trajectories traced, accepted steps)."""
    from collections import deque
    import time
    events = bool(stream.config.scan_events)
    state = []
    for jobs, params, i_lo, i_hi in items:
        n_grid = np.round((jobs["rk"] - jobs["rig"]) / jobs["del"]).astype(np.int64) + 1
        state.append({"jobs": jobs, "params": params, "n_grid": n_grid,
                      "lo": np.asarray(i_lo, np.int64).copy(), "hi": np.asarray(i_hi, np.int64).copy(),
                      "sites": np.zeros(len(jobs), ct.SITE_DTYPE), "redone": np.zeros(len(jobs), bool),
                      "traced": 0, "steps": 0})
    todo = deque((k, np.arange(len(it[0])), 0) for k, it in enumerate(items) if len(it[0]))
    inflight = []
    slots = int(stream.config.slots)

    def judge(S, j, first_allowed: bool, last_allowed: bool, site) -> bool:
        """Takes scan j's pass; returns whether it must be traced again."""
        low = S["lo"][j] > 0 and first_allowed
        high = S["hi"][j] < S["n_grid"][j] - 1 and not last_allowed
        if not (low or high):
            S["sites"][j] = site
            return False
        width = S["hi"][j] - S["lo"][j] + 1
        if low:
            S["lo"][j] = max(0, S["lo"][j] - width)
        if high:
            S["hi"][j] = min(S["n_grid"][j] - 1, S["hi"][j] + width)
        S["redone"][j] = True
        return True

    while todo or inflight:
        while todo and len(inflight) < slots:
            k, idx, attempt = todo.popleft()
            S = state[k]
            if attempt == widen + 1:                   # last resort: the whole grid
                S["lo"][idx] = 0
                S["hi"][idx] = S["n_grid"][idx] - 1
            try:
                t = stream.submit(window_jobs(S["jobs"][idx], S["lo"][idx], S["hi"][idx]), S["params"],
                                  want_status=not events)
            except ct.CorError as e:
                if e.code != ct.ERR_BUSY:
                    raise
                # the ring slot this segment needs still holds an older,
                # unfinished one: submit after it is collected
                todo.appendleft((k, idx, attempt))
                break
            inflight.append({"t": t, "k": k, "idx": idx, "attempt": attempt, "seen": np.zeros(len(idx), bool)})
        progressed = False
        again = {}
        for seg in list(inflight):
            S = state[seg["k"]]
            key = (seg["k"], seg["attempt"] + 1)
            if events:
                done, ev = stream.poll_scans(seg["t"])
                new = np.nonzero(done & ~seg["seen"])[0]
                for m in new:
                    j = seg["idx"][m]
                    if judge(S, j, ev[m]["first_class"] == ct.TRAJ_ALLOWED, ev[m]["last_class"] == ct.TRAJ_ALLOWED,
                             ev[m]["site"]):
                        again.setdefault(key, []).append(j)
                seg["seen"][new] = True
                progressed |= len(new) > 0
                if not seg["seen"].all():
                    continue
                res, _ = stream.wait(seg["t"], -1)
            else:
                got = stream.wait(seg["t"], 0)
                if got is None:
                    continue
                res = got[0]
                for m, j in enumerate(seg["idx"]):
                    st = res.status[res.offsets[m]:res.offsets[m + 1]]
                    if judge(S, j, st[0] == ct.TRAJ_ALLOWED, st[-1] == ct.TRAJ_ALLOWED, res.sites[m]):
                        again.setdefault(key, []).append(j)
            inflight.remove(seg)
            progressed = True
            S["traced"] += int(res.counters["trajectories"])
            S["steps"] += int(res.counters["accepted_steps"])
        for (k, attempt), js in again.items():
            todo.append((k, np.array(js, np.int64), attempt))
        if not progressed:
            time.sleep(poll_s)
    return [(S["sites"], S["redone"], S["traced"], S["steps"]) for S in state]


def trained_external(info: str) -> int | None:
    """The external field model (COR_EXTERNAL_*) a window network was trained
    with, from the provenance train_window.py stores ("igrf14+t96" ...); None
    when it names none the scan knows."""
    import json
    try:
        model = json.loads(info).get("model", "")
    except (ValueError, AttributeError):
        return None
    return {"igrf14+t96": ct.EXTERNAL_T96, "igrf14+ts05": ct.EXTERNAL_TS05, "igrf14": ct.EXTERNAL_NONE}.get(model)


class WindowModel:
    """A trained window network with its standardisation and sigmas (the
    file train_window.py writes).  `external` is the external field model it
    was trained with: its windows are meant for scans with that model only."""

    def __init__(self, path: str, device: int = 0, max_batch: int = 8192):
        d = np.load(path, allow_pickle=False)
        self.params = d["params"]
        self.feat_mean, self.feat_std = d["feat_mean"], d["feat_std"]
        self.y_mean, self.y_std = d["y_mean"], d["y_std"]
        self.sigma = d["sigma"]
        # held-out spread per band of predicted log R_L (inner edges; one
        # sigma pair per band); the global pair when absent
        self.band_edges = d["band_edges"] if "band_edges" in d else np.zeros(0)
        self.band_sigma = d["band_sigma"] if "band_sigma" in d else self.sigma[None, :]
        self.info = str(d["info"])
        self.external = trained_external(self.info)
        self.net = Network(device, max_batch=max_batch)
        self.net.set_params(self.params)
        import threading
        self.lock = threading.Lock()   # one network state: one caller at a time

    def predict(self, feats: np.ndarray) -> np.ndarray:
        """features (n, 19) -> (n, 2): log R_U, log R_L."""
        with self.lock:
            return self._predict(feats)

    def _predict(self, feats: np.ndarray) -> np.ndarray:
        import torch
        x = (np.asarray(feats, np.float64) - self.feat_mean) / self.feat_std
        out = []
        for a in range(0, len(x), self.net.max_batch):
            xb = torch.from_numpy(x[a:a + self.net.max_batch].astype(np.float32)).cuda(self.net.device)
            out.append(self.net.forward(xb).cpu().numpy())
        y = np.concatenate(out) if out else np.zeros((0, 2))
        return y * self.y_std + self.y_mean

    def windows(self, feats: np.ndarray, k: float = 3.0):
        """Grid windows: the prediction +- k sigma, sigma of the prediction's
        band of log R_L."""
        y = self.predict(feats)
        b = band_of(y[:, 1], self.band_edges)
        return window_indices(y[:, 0], y[:, 1], self.band_sigma[b, 0], self.band_sigma[b, 1], k=k)

    def close(self):
        self.net.close()
