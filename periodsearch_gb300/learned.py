"""Learned early stop of the period scan.

A small perceptron (10 -> 64 GELU -> 64 GELU -> 1, FP32) predicts the final
rms of an LM fit from its first K iterations (the screening depth, K = 8):
log(accepted chi^2 / starting chi^2) after iterations K/4, K/2, 3K/4 and K,
log10 lambda after the same iterations, log Ndata and log of the trial
period.  The target is log(final rms / rms after K iterations).  Training
data are trajectories that the engine itself records (ps_trajectories,
ps_pack_trajectories); training and inference run in the engine's own CUDA
kernels (ps_mlp_train, ps_mlp_predict, and inside the fit kernel during
screening).

The scan (ps_scan_learned) screens every fit with K iterations and keeps
its LM state, then completes periods -- all poles, resumed where the
screening stopped them -- in the order of their predicted rows until no
remaining period's predicted row, lowered by a margin, can beat the best
completed row; the fits that cannot beat the current best are stopped after
screening.  The periods around the best row are completed too, and the
minimum region is refitted in full with the plain FP64 form.

The margin is calibrated with the network: the smallest margin at which the
replayed cascade (replay_cascade, the scan's decisions on recorded full
trajectories) finds the full scan's best period on every structured training
window.  The same calibration with the zero predictor (the rms after K
iterations taken as the final rms: the method without the network) gives
the baseline that the network must beat.

    python -m periodsearch_gb300.learned --out periodsearch_gb300/stop_mlp.npy

collects trajectories of seeded synthetic objects on the GPU (packed
launches), trains the network, calibrates both margins, evaluates them on
fresh objects (the structured windows and the 2000-object survey population
of the learned stop's evaluation), and writes the weights with those
figures next to this file.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import tempfile
import time
from pathlib import Path

import numpy as np

from . import _abi

WEIGHTS = Path(__file__).resolve().parent / "stop_mlp.npy"
META = Path(__file__).resolve().parent / "stop_mlp.json"
F = _abi.MLP_FEATURES
H = 64
NP = _abi.MLP_FLOATS
# offsets (ps_engine.h kMlp*)
O_MU, O_SD = 0, F
O_W1 = 2 * F
O_B1 = O_W1 + H * F
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H
O_YMU = O_B3 + 1
O_YSD = O_YMU + 1
assert O_YSD + 1 == NP


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def init_weights(x: np.ndarray, y: np.ndarray, seed: int = 0) -> np.ndarray:
    """Standardisation constants from the data and a scaled normal start."""
    rng = np.random.default_rng(seed)
    P = np.zeros(NP, np.float32)
    P[O_MU:O_MU + F] = x.mean(axis=0)
    P[O_SD:O_SD + F] = np.maximum(x.std(axis=0), 1e-3)
    P[O_W1:O_B1] = rng.normal(0, math.sqrt(2.0 / F), H * F)
    P[O_W2:O_B2] = rng.normal(0, math.sqrt(2.0 / H), H * H)
    P[O_W3:O_B3] = rng.normal(0, math.sqrt(1.0 / H), H)
    P[O_YMU] = y.mean()
    P[O_YSD] = max(float(y.std()), 1e-3)
    return P


def zero_predictor() -> np.ndarray:
    """Weights whose prediction is 0: the final rms is taken to be the rms
    after four iterations (the scan without the learned part)."""
    P = np.zeros(NP, np.float32)
    P[O_SD:O_SD + F] = 1.0
    P[O_YSD] = 1.0
    return P


def train(x: np.ndarray, y: np.ndarray, epochs: int = 60, batch: int = 512, lr: float = 2e-3, seed: int = 0,
          device: int = 0, weights: np.ndarray | None = None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    P = np.array(init_weights(x, y, seed) if weights is None else weights, np.float32)
    hist = np.zeros(epochs, np.float32)
    st = _abi.lib().ps_mlp_train(device, _fp(P), _fp(x), _fp(y), len(y), epochs, batch, lr, seed, _fp(hist))
    _abi.check(st, "ps_mlp_train")
    return P, hist


def predict(P: np.ndarray, x: np.ndarray, device: int = 0) -> np.ndarray:
    P = np.ascontiguousarray(P, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(len(x), np.float32)
    _abi.check(_abi.lib().ps_mlp_predict(device, _fp(P), _fp(x), len(x), _fp(out)), "ps_mlp_predict")
    return out


def grad(P: np.ndarray, x: np.ndarray, y: np.ndarray, device: int = 0):
    P = np.ascontiguousarray(P, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    g = np.zeros(NP, np.float32)
    loss = C.c_float()
    _abi.check(_abi.lib().ps_mlp_grad(device, _fp(P), _fp(x), _fp(y), len(y), C.byref(loss), _fp(g)), "ps_mlp_grad")
    return loss.value, g


def load_default():
    """Committed weights and their training record, or (None, None)."""
    if not WEIGHTS.exists():
        return None, None
    meta = json.loads(META.read_text()) if META.exists() else {}
    return np.load(WEIGHTS).astype(np.float32), meta


# Screening depth of the committed network and the cascade's defaults
# (ps_learned_opts); the margin is the one calibrated with the network.
SCREEN_ITERS = 8
DEFAULT_CASCADE = {"screen_iters": SCREEN_ITERS, "margin": 0.02, "batch_periods": 0, "region_halfwidth": 2,
                   "refit_rel": 0.005, "refit_halfwidth": 2, "fill_refit_waves": 1}


def cascade_defaults() -> dict:
    """ps_learned_opts of the committed predictor: its screening depth and
    calibrated margin over DEFAULT_CASCADE."""
    out = dict(DEFAULT_CASCADE)
    if META.exists():
        meta = json.loads(META.read_text())
        for k in ("screen_iters", "margin"):
            if k in meta.get("cascade", {}):
                out[k] = meta["cascade"][k]
    return out


def trajectories(engine, conw_r: float, n_lo: int, n_hi: int, feat_iters: int | None = None) -> np.ndarray:
    """[fits][16] records of full fits (features after feat_iters
    iterations, rms after them, final rms, iterations, rms after 8/16/32)."""
    k = SCREEN_ITERS if feat_iters is None else int(feat_iters)
    n = (n_hi - n_lo + 1) * 10
    out = np.zeros((n, _abi.TRAJ_FLOATS), np.float32)
    st = engine._L.ps_trajectories(engine._ctx, conw_r, n_lo, n_hi, k, _fp(out))
    _abi.check(st, "ps_trajectories", engine._ctx)
    return out


def _usable(traj: np.ndarray) -> np.ndarray:
    devk, fin = traj[:, 10].astype(np.float64), traj[:, 11].astype(np.float64)
    return np.isfinite(traj[:, :F]).all(axis=1) & (devk > 0) & (fin > 0) & np.isfinite(devk) & np.isfinite(fin)


def samples(traj: np.ndarray):
    """Features and targets log(final rms / rms after the screening
    iterations) of the records with a finite, positive rms."""
    ok = _usable(traj)
    devk, fin = traj[ok, 10].astype(np.float64), traj[ok, 11].astype(np.float64)
    return traj[ok, :F], np.log(fin / devk).astype(np.float32), devk, fin


def pole_rank_agreement(P: np.ndarray, x, y, fin, period, device: int = 0) -> dict:
    """How often the pole with the lowest final rms of a period is the
    best-predicted pole (top1) or among the two best-predicted (top2), over
    the periods of held-out samples (`period` labels each sample's period)."""
    pred = fin * np.exp(predict(P, x, device).astype(np.float64) - y)   # rms after K iterations x exp(prediction)
    top1 = top2 = n = 0
    order = np.argsort(period, kind="stable")
    for grp in np.split(order, np.flatnonzero(np.diff(period[order])) + 1):
        if len(grp) < 2:
            continue
        truth = grp[np.argmin(fin[grp])]
        ranked = grp[np.argsort(pred[grp], kind="stable")]
        top1 += ranked[0] == truth
        top2 += truth in ranked[:2]
        n += 1
    return {"periods": n, "top1": top1 / max(n, 1), "top2": top2 / max(n, 1)}


# ---------------------------------------------------------------------------
# The cascade's decisions replayed on recorded trajectories
# ---------------------------------------------------------------------------

def replay_cascade(pred: np.ndarray, screened: np.ndarray, final: np.ndarray, margin: float, batch: int,
                   halfwidth: int = 2):
    """The completion decisions of ps_scan_learned (stages 2 and 3) for one
    window, on [periods][10] arrays of the predicted final rms, the rms
    after the screening iterations and the final rms (a completed fit ends
    exactly as the uninterrupted one: the recorded final rms).  Returns the
    completed-period mask and the index of the best row (completed periods:
    their final rows; the others: their screened rows)."""
    nper = pred.shape[0]
    R = np.where(pred > 0, pred, np.inf).min(axis=1)
    order = np.argsort(R, kind="stable")
    rows_f = final.min(axis=1)
    done = np.zeros(nper, bool)
    shrink = math.exp(-margin)
    nxt = 0
    while True:
        best = rows_f[done].min() if done.any() else np.inf
        grp = []
        while nxt < nper and len(grp) < batch:
            n = order[nxt]
            if not (R[n] * shrink <= best):
                break
            grp.append(n)
            nxt += 1
        if not grp:
            break
        done[grp] = True
    for _ in range(16):
        if not done.any():
            break
        bn = int(np.flatnonzero(done)[np.argmin(rows_f[done])])
        grp = [n for n in range(max(0, bn - halfwidth), min(nper, bn + halfwidth + 1)) if not done[n]]
        if not grp:
            break
        done[grp] = True
    rows = np.where(done, rows_f, screened.min(axis=1))
    return done, int(np.argmin(rows))


def replay_windows(windows, P, margin: float, batch: int, device: int = 0, preds=None) -> dict:
    """replay_cascade over windows (dicts with traj [periods*10][16]):
    completed fraction of the periods, how often the best period differs
    from the full scan's (misses), and how often it does by more than 0.1 %
    in rms (misses beyond a near-tie).  preds: the predicted final rms per
    window (else computed with P)."""
    done_n = per_n = miss = miss_far = 0
    evals = full_evals = 0
    for j, w in enumerate(windows):
        tr = w["traj"]
        nper = len(tr) // 10
        devk = tr[:, 10].astype(np.float64)
        fin = tr[:, 11].astype(np.float64)
        pr = preds[j] if preds is not None else devk * np.exp(predict(P, tr[:, :F], device).astype(np.float64))
        done, b = replay_cascade(pr.reshape(nper, 10), devk.reshape(nper, 10), fin.reshape(nper, 10), margin,
                                 batch)
        rows = fin.reshape(nper, 10).min(axis=1)
        full_b = int(np.argmin(rows))
        done_n += int(done.sum())
        per_n += nper
        if b != full_b:
            miss += 1
            miss_far += rows[b] > rows[full_b] * 1.001
        k = w.get("screen_iters", SCREEN_ITERS)
        it = tr[:, 12].astype(np.float64)
        evals += nper * 10 * (k + 1) + float(((it - k) + 1).reshape(nper, 10)[done].sum())
        full_evals += float((it + 1).sum())
    return {"windows": len(windows), "completed_fraction": done_n / max(per_n, 1), "misses": miss,
            "miss_rate": miss / max(len(windows), 1), "misses_beyond_0.1pct": int(miss_far),
            "evals_fraction": evals / max(full_evals, 1)}


def calibrate_margin(windows, P, batch: int, device: int = 0, grid=None) -> float:
    """The smallest margin at which the replayed cascade finds the full
    scan's best period on every window."""
    grid = grid if grid is not None else [0.0025 * i for i in range(0, 41)] + [0.125, 0.15, 0.2, 0.3, 0.5]
    preds = []
    for w in windows:
        tr = w["traj"]
        devk = tr[:, 10].astype(np.float64)
        preds.append(devk * np.exp(predict(P, tr[:, :F], device).astype(np.float64)))
    for m in grid:
        if replay_windows(windows, P, m, batch, device, preds)["misses"] == 0:
            return float(m)
    return float(grid[-1])


# ---------------------------------------------------------------------------
# Trajectory collection (packed launches)
# ---------------------------------------------------------------------------

def collect_windows(objects, periods: int, feat_iters: int, device: int = 0, around_truth=None, seed: int = 0,
                    batch_objects: int = 250):
    """Full-fit trajectories of one window of `periods` consecutive trial
    periods per object (objects: synth.SynthObject list), packed many
    objects per launch.  around_truth(k) -> True centres object k's window
    on its true period, else the window is placed at random.  Returns a list
    of dicts (traj, lo, ndata, truth) and the kernel time [ms]."""
    from . import Engine, Pack, PS_FORM_MIXED, read_input

    rng = np.random.default_rng(seed)
    out, kernel_ms = [], 0.0
    with tempfile.TemporaryDirectory() as td:
        for b0 in range(0, len(objects), batch_objects):
            batch = objects[b0:b0 + batch_objects]
            engines = []
            for j, o in enumerate(batch):
                p = Path(td) / f"o{b0 + j}"
                p.write_text(o.text)
                engines.append(Engine(read_input(p), device=device, form=PS_FORM_MIXED))
            ob, pi, po, cw, los = [], [], [], [], []
            for j, (e, o) in enumerate(zip(engines, batch)):
                n_max = int(e.info.n_max)
                width = min(periods, n_max)
                if around_truth is None or around_truth(b0 + j):
                    nt = int(round((e.info.freq_start - 1 / o.truth["period_h"]) / e.info.freq_step)) + 1
                    lo = max(1, min(n_max - width + 1, nt - width // 2))
                else:
                    lo = int(rng.integers(1, n_max - width + 2))
                los.append((lo, width))
                cw.append(e.info.conw_r0)
                for n in range(lo, lo + width):
                    ob += [j] * 10
                    pi += [n] * 10
                    po += list(range(1, 11))
            with Pack(engines, form=PS_FORM_MIXED) as pk:
                _, traj = pk.trajectories(cw, ob, pi, po, feat_iters)
                kernel_ms += pk.timing()["kernel_ms"]
            ob = np.asarray(ob)
            for j, (e, o) in enumerate(zip(engines, batch)):
                out.append({"traj": traj[ob == j], "lo": los[j][0], "ndata": int(e.info.ndata), "truth": o.truth,
                            "screen_iters": feat_iters})
            for e in engines:
                e.close()
    return out, kernel_ms


def _population(pop: str, n: int, base_seed: int, processes: int = 16):
    """Objects of a synthetic population, generated in worker processes
    (started with spawn, before the parent uses the GPU)."""
    import multiprocessing as mp

    from . import synth

    if processes <= 1:
        return [synth.population_object(pop, k, base_seed) for k in range(n)]
    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.starmap(synth.population_object, [(pop, k, base_seed) for k in range(n)], chunksize=8)


def _structured(n: int, base_seed: int):
    """c1-shaped objects (8 dense relative lightcurves and 500 sparse
    points) with fresh seeds: period landscapes with a clear minimum."""
    from . import synth

    return [synth.make_object("c1", seed=base_seed + k) for k in range(n)]


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--train-objects", type=int, default=400, help="survey-population training objects")
    ap.add_argument("--structured-train", type=int, default=24, help="c1-shaped training objects")
    ap.add_argument("--structured-eval", type=int, default=16, help="c1-shaped evaluation objects")
    ap.add_argument("--eval-objects", type=int, default=2000, help="survey-population evaluation objects")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--processes", type=int, default=16)
    ap.add_argument("--dump", default="", help="save the collected windows' trajectories (npz) here")
    ap.add_argument("--screen-iters", type=int, default=SCREEN_ITERS,
                    help="LM iterations before the prediction (a multiple of 4)")
    args = ap.parse_args()
    K = args.screen_iters
    if K < 4 or K % 4:
        ap.error("--screen-iters must be a positive multiple of 4")
    # every object is generated before the GPU is touched (spawned workers)
    pop_train = _population("c5", args.train_objects, 60000, args.processes)
    pop_eval = _population("c5", args.eval_objects, 50000, args.processes)
    st_train = _structured(args.structured_train, 100)
    st_eval = _structured(args.structured_eval, 900)
    from . import build

    build.build()
    t0 = time.time()
    w_pop, ms_a = collect_windows(pop_train, 24, K, args.device, around_truth=lambda k: k % 2 == 0, seed=1)
    w_st, ms_b = collect_windows(st_train, 200, K, args.device, seed=2)
    w_pop_ev, ms_c = collect_windows(pop_eval, 24, K, args.device, around_truth=lambda k: k % 2 == 0, seed=3)
    w_st_ev, ms_d = collect_windows(st_eval, 400, K, args.device, seed=4)
    t1 = time.time()
    if args.dump:
        arrs = {}
        for name, ws in (("pop_train", w_pop), ("st_train", w_st), ("pop_eval", w_pop_ev), ("st_eval", w_st_ev)):
            arrs[name + "_feat"] = np.concatenate([w["traj"][:, :F] for w in ws]).astype(np.float16)
            arrs[name + "_dev"] = np.concatenate([w["traj"][:, F:] for w in ws]).astype(np.float32)
            arrs[name + "_len"] = np.array([len(w["traj"]) for w in ws])
        np.savez(args.dump, **arrs)
    xs, ys = [], []
    for w in w_pop + w_st:
        x, y, _, _ = samples(w["traj"])
        xs.append(x)
        ys.append(y)
    x, y = np.concatenate(xs), np.concatenate(ys)
    P, hist = train(x, y, epochs=args.epochs, device=args.device)
    t2 = time.time()
    P0 = zero_predictor()
    batch = 15   # periods per completion launch on a 152-SM GB300 (slots / 10)
    m_net = calibrate_margin(w_st, P, batch, args.device)
    m_zero = calibrate_margin(w_st, P0, batch, args.device)
    ev = {"structured": {"network": replay_windows(w_st_ev, P, m_net, batch, args.device),
                         "without_network": replay_windows(w_st_ev, P0, m_zero, batch, args.device)},
          "survey_population": {"network": replay_windows(w_pop_ev, P, m_net, batch, args.device),
                                "without_network": replay_windows(w_pop_ev, P0, m_zero, batch, args.device)}}
    # the trade-off on the survey population at other margins
    ev["survey_population"]["margin_sweep"] = [
        {"margin": m, "network": replay_windows(w_pop_ev, P, m, batch, args.device),
         "without_network": replay_windows(w_pop_ev, P0, m, batch, args.device)} for m in (0.02, 0.05, 0.1, 0.2)]
    xv, yv = [], []
    for w in w_st_ev + w_pop_ev[:200]:
        a, b, _, _ = samples(w["traj"])
        xv.append(a)
        yv.append(b)
    xv, yv = np.concatenate(xv), np.concatenate(yv)
    pv = predict(P, xv, args.device)
    meta = {"screen_iters": K, "train_samples": int(len(y)), "epochs": args.epochs,
            "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
            "val_rmse_log": float(np.sqrt(np.mean((pv - yv) ** 2))),
            "val_rmse_log_without_network": float(np.sqrt(np.mean(yv ** 2))),
            "cascade": {**DEFAULT_CASCADE, "screen_iters": K, "margin": m_net}, "margin_without_network": m_zero,
            "windows": {"train_population": len(w_pop), "train_structured": len(w_st),
                        "eval_population": len(w_pop_ev), "eval_structured": len(w_st_ev)},
            "evaluation": ev, "collect_s": t1 - t0, "collect_kernel_s": (ms_a + ms_b + ms_c + ms_d) / 1e3,
            "train_s": t2 - t1}
    np.save(args.out, P)
    Path(args.out).with_suffix(".json").write_text(json.dumps(meta, indent=1))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
