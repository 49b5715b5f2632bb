"""Learned early stop of the period scan.

A small perceptron (10 -> 64 GELU -> 64 GELU -> 1, FP32) predicts the final
rms of an LM fit from its first four iterations: log(accepted chi^2 /
starting chi^2) after each, log10 lambda after each, log Ndata and log of the
trial period.  The target is log(final rms / rms after four iterations).
Training data are trajectories that the engine itself records
(ps_trajectories); training and inference run in the engine's own CUDA
kernels (ps_mlp_train, ps_mlp_predict, and inside the fit kernel during
screening).

The scan (ps_scan_learned) screens every fit with four iterations, completes
in full the best-predicted poles of every period, then every pole of the
periods near the best row, and refits the minimum region in full with the
plain FP64 form.

    python -m periodsearch_gb300.learned --out periodsearch_gb300/stop_mlp.npy

trains on seeded synthetic objects, measures the prediction error on
held-out objects, compares the learned scan with the full scans and with the
same cascade ranked without the network on fresh objects, and writes the
weights (with those figures) next to this file.
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


def trajectories(engine, conw_r: float, n_lo: int, n_hi: int) -> np.ndarray:
    """[fits][16] records of full fits (features, rms after 4 iterations,
    final rms, iterations)."""
    n = (n_hi - n_lo + 1) * 10
    out = np.zeros((n, _abi.TRAJ_FLOATS), np.float32)
    st = engine._L.ps_trajectories(engine._ctx, conw_r, n_lo, n_hi, _fp(out))
    _abi.check(st, "ps_trajectories", engine._ctx)
    return out


def _usable(traj: np.ndarray) -> np.ndarray:
    dev4, fin = traj[:, 10].astype(np.float64), traj[:, 11].astype(np.float64)
    return np.isfinite(traj[:, :F]).all(axis=1) & (dev4 > 0) & (fin > 0) & np.isfinite(dev4) & np.isfinite(fin)


def samples(traj: np.ndarray):
    """Features and targets log(final rms / rms after 4 iterations) of the
    records with a finite, positive rms."""
    ok = _usable(traj)
    dev4, fin = traj[ok, 10].astype(np.float64), traj[ok, 11].astype(np.float64)
    return traj[ok, :F], np.log(fin / dev4).astype(np.float32), dev4, fin


def pole_rank_agreement(P: np.ndarray, x, y, fin, period, device: int = 0) -> dict:
    """How often the pole with the lowest final rms of a period is the
    best-predicted pole (top1) or among the two best-predicted (top2), over
    the periods of held-out samples (`period` labels each sample's period)."""
    pred = fin * np.exp(predict(P, x, device).astype(np.float64) - y)   # rms after 4 iterations x exp(prediction)
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


def _object_periods(eng, truth_period_h: float, n_random: int, rng) -> list[tuple[int, int]]:
    n_max = int(eng.info.n_max)
    n_truth = int(round((eng.info.freq_start - 1 / truth_period_h) / eng.info.freq_step)) + 1
    spans = [(max(1, n_truth - 8), min(n_max, n_truth + 8))]
    for n0 in rng.choice(max(n_max - 8, 1), size=n_random, replace=False):
        spans.append((int(n0) + 1, min(n_max, int(n0) + 8)))
    return spans


def build_training_set(seeds, configs=("c0", "c1"), n_random: int = 12, device: int = 0, form=None, dump=None):
    """Trajectory samples of seeded synthetic objects: the window around the
    true period and random 8-period spans of each scan.  Returns features,
    targets, final rms, a label of every sample's (object, period) and the
    (config, seed) of every object."""
    from . import Engine, PS_FORM_MIXED, read_input, synth

    form = PS_FORM_MIXED if form is None else form
    xs, ys, fins, objs, meta = [], [], [], [], []
    for cfg in configs:
        for seed in seeds:
            with tempfile.TemporaryDirectory() as td:
                obj = synth.write_object(Path(td) / "period_search_in", cfg, seed=seed)
                with Engine(read_input(Path(td) / "period_search_in"), device=device, form=form) as eng:
                    conw_r, _ = eng.precalc_conw()
                    rng = np.random.default_rng(seed)
                    for lo, hi in _object_periods(eng, obj.truth["period_h"], n_random, rng):
                        tr = trajectories(eng, conw_r, lo, hi)
                        x, y, _, fin = samples(tr)
                        xs.append(x)
                        ys.append(y)
                        fins.append(fin)
                        fit = np.flatnonzero(_usable(tr))
                        objs.append(len(meta) * 1_000_000 + lo + fit // 10)
                        if dump is not None:
                            fit = np.arange(len(tr))
                            dump.append(np.column_stack([np.full(len(tr), len(meta)), lo + fit // 10, fit % 10 + 1,
                                                         tr]))
            meta.append((cfg, seed))
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(fins), np.concatenate(objs), meta


CASCADE = {"top_k": 1, "region_rel": 0.03, "region_halfwidth": 2, "refit_rel": 0.005, "refit_halfwidth": 2}


def evaluate_gain(P, P0, seeds, cfg="c1", half_window=100, device: int = 0, **opts):
    """On fresh objects, a window of 2*half_window periods around the true
    period: the full scans of the mixed and the FP64 form against the
    learned scan with the trained predictor and with the zero predictor (the
    rms after four iterations, i.e. the same cascade without the network).
    Best period (index) of each, evaluations and kernel time."""
    from . import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input, synth

    opts = {**CASCADE, **opts}
    out = []
    for seed in seeds:
        with tempfile.TemporaryDirectory() as td:
            obj = synth.write_object(Path(td) / "period_search_in", cfg, seed=seed)
            with Engine(read_input(Path(td) / "period_search_in"), device=device, form=PS_FORM_MIXED) as eng:
                conw_r, _ = eng.precalc_conw()
                n_t = int(round((eng.info.freq_start - 1 / obj.truth["period_h"]) / eng.info.freq_step)) + 1
                lo, hi = max(1, n_t - half_window), min(int(eng.info.n_max), n_t + half_window - 1)
                full = eng.scan(conw_r, lo, hi)
                tf = eng.timing()
                rl, sl = eng.scan_learned(conw_r, lo, hi, P, **opts)
                r0, s0 = eng.scan_learned(conw_r, lo, hi, P0, **opts)
                rr, sr = eng.scan_refined(conw_r, lo, hi)
            with Engine(read_input(Path(td) / "period_search_in"), device=device, form=PS_FORM_FP64) as e64:
                f64 = e64.scan(conw_r, lo, hi)
                t64 = e64.timing()
                out.append({"seed": seed, "cfg": cfg, "periods": hi - lo + 1, "truth_index": n_t,
                            "best_fp64": lo + int(np.argmin(f64["rms"])), "ms_fp64": t64["kernel_ms"],
                            "best_refined": int(sr["best_index"]), "ms_refined": sr["complete_ms"] + sr["refit_ms"],
                            "refit_refined": int(sr["fits_refit"]),
                            "best_full": lo + int(np.argmin(full["rms"])), "best_learned": int(sl["best_index"]),
                            "best_without_network": int(s0["best_index"]),
                            "evals_full": int(tf["evals"]), "evals_learned": int(sl["evals"]),
                            "evals_without_network": int(s0["evals"]),
                            "ms_full": tf["kernel_ms"],
                            "ms_learned": sl["screen_ms"] + sl["complete_ms"] + sl["refit_ms"],
                            "ms_without_network": s0["screen_ms"] + s0["complete_ms"] + s0["refit_ms"],
                            "completed_learned": int(sl["fits_completed"]),
                            "completed_without_network": int(s0["fits_completed"]),
                            "refit_learned": int(sl["fits_refit"]), "fits": int(sl["fits_total"])})
    return out


def gain_summary(gain: list) -> dict:
    """Totals of evaluate_gain records: how often each scan's best period
    differs from the full FP64 scan's, and time ratios of the scans."""
    ms = {k: sum(g[k] for g in gain) for k in ("ms_full", "ms_learned", "ms_without_network", "ms_fp64", "ms_refined")}
    ef, el, e0 = (sum(g[k] for g in gain) for k in ("evals_full", "evals_learned", "evals_without_network"))
    return {"objects": len(gain),
            "differs_from_fp64": {k: sum(g["best_" + k] != g["best_fp64"] for g in gain)
                                  for k in ("full", "refined", "learned", "without_network")},
            "evals_ratio_full_over_learned": ef / el, "evals_ratio_full_over_without_network": ef / e0,
            "time_ratio_fp64_over": {k: ms["ms_fp64"] / ms["ms_" + k]
                                     for k in ("full", "refined", "learned", "without_network")}}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--train-seeds", type=int, default=16)
    ap.add_argument("--val-seeds", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--eval-seeds", type=int, default=5)
    ap.add_argument("--dump", default="", help="save raw validation trajectories (object, period, pole, record)")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--eval-only", default="", help="evaluate the committed weights only; write the figures here")
    ap.add_argument("--eval-configs", default="c0,c1")
    ap.add_argument("--half-window", type=int, default=100)
    args = ap.parse_args()
    from . import build

    build.build()
    if args.eval_only:
        P, _ = load_default()
        gain = []
        for cfg in args.eval_configs.split(","):
            gain += evaluate_gain(P, zero_predictor(), range(900, 900 + args.eval_seeds), cfg=cfg,
                                  half_window=args.half_window, device=args.device)
        res = {"half_window": args.half_window, "cascade": CASCADE, "summary": gain_summary(gain), "gain": gain}
        Path(args.eval_only).write_text(json.dumps(res, indent=1))
        print(json.dumps(res["summary"]))
        return
    t0 = time.time()
    xtr, ytr, _, _, _ = build_training_set(range(100, 100 + args.train_seeds), device=args.device)
    raw = [] if args.dump else None
    xva, yva, fva, gva, _ = build_training_set(range(500, 500 + args.val_seeds), device=args.device, dump=raw)
    if args.dump:
        np.save(args.dump, np.concatenate(raw))
    t1 = time.time()
    P, hist = train(xtr, ytr, epochs=args.epochs, device=args.device)
    t2 = time.time()
    P0 = zero_predictor()
    pva = predict(P, xva, args.device)
    gain = []
    for cfg in ("c0", "c1"):
        gain += evaluate_gain(P, P0, range(900, 900 + args.eval_seeds), cfg=cfg, device=args.device)
    meta = {"train_samples": int(len(ytr)), "val_samples": int(len(yva)), "epochs": args.epochs,
            "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
            "val_rmse_log": float(np.sqrt(np.mean((pva - yva) ** 2))),
            "val_rmse_log_without_network": float(np.sqrt(np.mean(yva ** 2))),
            "pole_rank_agreement": pole_rank_agreement(P, xva, yva, fva, gva, args.device),
            "pole_rank_agreement_without_network": pole_rank_agreement(P0, xva, yva, fva, gva, args.device),
            "cascade": CASCADE, "collect_s": t1 - t0, "train_s": t2 - t1, "gain": gain}
    if gain:
        meta["gain_summary"] = gain_summary(gain)
    np.save(args.out, P)
    Path(args.out).with_suffix(".json").write_text(json.dumps(meta, indent=1))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
