"""Benchmark: LM period fits/s on one GB300 (per GPU under torchrun).

Workload: the batched scan of one synthetic asteroid with 8 dense
relative lightcurves (3 h, 60 points each, 0.02 mag) and 500 sparse
calibrated points over 8 years (Ndata = 980), trial periods 2-50 h with the
reference's step rule (~40k periods x 10 initial poles), Laplace series
L = M = 6 on the 288-facet grid, 50 LM iterations per fit.  A step is one
contiguous chunk of the period scan (all 10 poles of each period), fitted by
one launch of the persistent fit kernel; successive steps take chunks spread
over the whole 2-50 h range.  Seeded synthetic data (no external dataset).

value      fits/s of the chosen form (--form, default mixed: FP32 facet stage,
           shape contraction and alpha/beta on the tensor cores, FP64 phase,
           chi^2, solve) with the object resident in HBM, from CUDA events
           around the fit kernel on its own stream (sum over steps); the plain
           FP64 form is timed on the same chunks (plain_fp64); on a window of
           --validation-window periods around the true period every scan
           type -- full FP64, full mixed, refined (mixed scan plus FP64 refit
           of the minimum region) and the learned early-stop cascade -- is
           timed and its best period compared with the full FP64 scan's
           (validation.scans, fits/s = the window's fits over the scan's
           kernel time);
e2e        the same through the C ABI with host buffers: ps_prepare (host ->
           device copy of the tables), ps_scan (rows back to the host) and
           ps_destroy per step, wall clock;
roofline   algorithmic FLOP of the fits (2 N F C + 60 N F + N m(m+1) + 9 F C
           per evaluation, 2 m^3 per solve) per launch over the launch time,
           against the FP32 (mixed) or FP64 FMA ceiling measured live on the
           device; for the mixed form also the two contractions' shares:
           the shape contraction (2 N F C, FP16 high/low MMAs) against the
           measured dense BF16 figure (the FP16 rate) and the alpha/beta
           accumulation (N m(m+1), TF32 high/low MMAs) against half of it
           (the TF32 rate);
cpu_baseline  the CPU oracle (a restatement of the reference's FP64 path)
           on all host cores, one fit per thread, on a bounded sample.

`--impl reference` times that CPU implementation alone as the reference arm.
Between timed steps a 256 MiB buffer is rewritten to flush the 126 MB L2.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LM period fits/s on 1 GB300: chosen form vs plain FP64, same best P, χ² in tol"
WORKLOAD = "c1: 8 dense relative LCs + 500 sparse points (Ndata 980), scan 2-50 h, L=M=6, 288 facets, 10 poles, 50 LM iterations"
PROFILES = {False: ROOT / "profiles" / "fit_kernel_fp64_c1.md", True: ROOT / "profiles" / "fit_kernel_mixed_c1.md"}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--form", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip timing the plain FP64 form")
    ap.add_argument("--simt-compare", action="store_true",
                    help="also time the mixed form with its contractions on the SIMT pipes")
    ap.add_argument("--validation-window", type=int, default=300,
                    help="periods of the window around the true period on which every scan type is compared")
    ap.add_argument("--multi-object", type=int, default=0,
                    help="also time K small objects (Ndata logU[100, 2000]) packed into one launch against one "
                         "launch per object")
    ap.add_argument("--periods-per-step", type=int, default=0,
                    help="trial periods per step (0: one per fit slot of the device, i.e. ten fits per slot)")
    ap.add_argument("--cpu-sample-fits", type=int, default=0, help="fits in the CPU baseline sample (0: 2 per core)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--full-scan", action="store_true",
                    help="also run the whole scan of the workload as one refined scan (rank 0) and report its "
                         "time and best period (full_scan)")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(tmpdir: Path):
    from periodsearch_gb300 import read_input, synth

    path = tmpdir / "period_search_in"
    obj = synth.write_object(path, "c1")
    return path, read_input(path), obj


def flops_per_eval(ndata, nfac, ncoef, mfit):
    return 2.0 * ndata * nfac * ncoef + 60.0 * ndata * nfac + ndata * mfit * (mfit + 1) + 9.0 * nfac * ncoef


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self._t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = max(smax, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(path: Path, periods, sample_fits: int):
    """The CPU oracle on all host cores: one fit per thread (ctypes releases
    the GIL), a bounded sample of fits of the same scan."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding
    from concurrent.futures import ThreadPoolExecutor

    oracle_binding.build_oracle()
    cores = os.cpu_count() or 1
    n = sample_fits or 2 * cores
    probs = [oracle_binding.OracleProblem(path) for _ in range(cores)]
    cw = probs[0].info()["conw_r"]
    for p in probs:
        p.setup(cw)
    jobs = [(int(periods[i % len(periods)]), 1 + i % 10) for i in range(n)]
    lock = threading.Lock()
    free = list(range(cores))

    def one(job):
        with lock:
            k = free.pop()
        try:
            p = probs[k]
            return p.fit(p.freq(job[0]), job[1])
        finally:
            with lock:
                free.append(k)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(one, jobs))
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "fits/s", "cores": cores, "kind": "port",
            "sample": f"{n} fits (period indices of the timed chunks x poles 1-10) of the c1 scan, {cores} threads, "
                      f"{dt:.1f} s wall"}


def run_reference_arm(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as td:
        path, data, _ = make_workload(Path(td))
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_binding

        probe = oracle_binding.OracleProblem(path)
        n_max = probe.info()["n_max"]
        cores = os.cpu_count() or 1
        periods = [1 + (k * 7919) % n_max for k in range(4 * cores)]
        for _ in range(args.warmup):
            cpu_baseline(path, periods, cores)
        vals = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            vals.append(cpu_baseline(path, periods, cores))
        dt = time.perf_counter() - t0
        fits = cores * args.steps
        v = fits / dt
        cb = dict(vals[-1])
        cb["value"] = v
        cb["sample"] = f"{args.steps} steps of {cores} fits (one per core) of the c1 scan, oracle port of the reference FP64 path"
        line = {"metric": METRIC, "value": v, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, c1)",
                "config": {"workload": WORKLOAD, "form": "cpu fp64 (reference algorithm)"}, "impl": "reference",
                "cpu_baseline": cb, "e2e": {"value": v, "unit": "fits/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line))


def multi_object(K: int, form: int, local: int, units_per_object: int = 8) -> dict:
    """Packed launch of K objects (sparse calibrated data, Ndata log-uniform
    in [100, 2000], seeded) against one launch per object, on the same
    random (object, period, pole) units."""
    import numpy as np

    from periodsearch_gb300 import Engine, Pack, read_input, synth

    rng = np.random.default_rng(2024)
    engines = []
    with tempfile.TemporaryDirectory() as td:
        for k in range(K):
            nd = int(round(math.exp(rng.uniform(math.log(100), math.log(2000)))))
            cfg = synth.SynthConfig(name=f"mo{k}", n_sparse=nd, sparse_block=1000)
            path = Path(td) / f"o{k}"
            synth.write_object(path, cfg, seed=7000 + k)
            engines.append(Engine(read_input(path), device=local, form=form))
    try:
        conw = [e.precalc_conw()[0] for e in engines]
        obj, per, pole = [], [], []
        for o, e in enumerate(engines):
            for p in rng.choice(int(e.info.n_max), size=units_per_object, replace=False) + 1:
                obj += [o] * 10
                per += [int(p)] * 10
                pole += list(range(1, 11))
        obj, per, pole = np.array(obj), np.array(per), np.array(pole)
        seq_ms = 0.0
        for o, e in enumerate(engines):
            sel = obj == o
            e.fit_batch(conw[o], per[sel], pole[sel])
            seq_ms += e.timing()["kernel_ms"]
        with Pack(engines, form=form) as pk:
            pk.fit(conw, obj, per, pole)   # warm-up
            pk.fit(conw, obj, per, pole)
            pms = pk.timing()["kernel_ms"]
        nd = [e.info.ndata for e in engines]
        return {"objects": K, "fits": int(len(obj)), "ndata_min": min(nd), "ndata_max": max(nd),
                "packed_fits_per_s": len(obj) / (pms / 1e3), "one_launch_per_object_fits_per_s": len(obj) / (seq_ms / 1e3),
                "speedup": seq_ms / pms}
    finally:
        for e in engines:
            e.close()


def _measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def _profile_traffic(mixed: bool):
    """DRAM bytes per fit from the committed ncu summary of that form, if present."""
    prof = PROFILES[mixed]
    if not prof.exists():
        return None
    for line in prof.read_text().splitlines():
        if line.startswith("dram_bytes_per_fit:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def _time_form(Engine, data, form, local, starts, chunk, warmup, steps, flush, sampler=None, tensor_cores=True):
    """Warm-up and timed steps of one form on the given chunk starts."""
    import torch

    eng = Engine(data, device=local, form=form, tensor_cores=tensor_cores)
    info = eng.info
    conw_r, _ = eng.precalc_conw()
    fe = flops_per_eval(info.ndata, info.nfac, info.ncoef, info.mfit)
    fs = 2.0 * info.mfit ** 3
    for k in range(warmup):
        flush.zero_()
        torch.cuda.synchronize()
        eng.scan(conw_r, starts[k], starts[k] + chunk - 1)
    torch.cuda.synchronize()
    kernel_ms, fits, flops, launches, rows, evals = 0.0, 0, 0.0, 0, [], 0
    if sampler:
        sampler.__enter__()
    try:
        for k in range(warmup, warmup + steps):
            flush.zero_()
            torch.cuda.synchronize()
            r = eng.scan(conw_r, starts[k], starts[k] + chunk - 1)
            t = eng.timing()
            kernel_ms += t["kernel_ms"]
            fits += t["fits"]
            launches += t["launches"]
            flops += t["evals"] * fe + (t["evals"] - t["fits"]) * fs
            evals += t["evals"]
            rows.append(r)
    finally:
        if sampler:
            sampler.__exit__(None, None, None)
    torch.cuda.synchronize()
    return {"engine": eng, "conw_r": conw_r, "kernel_ms": kernel_ms, "fits": fits, "flops": flops, "evals": evals,
            "launches": launches, "rows": rows}


def run_engine_arm(args):
    import ctypes as C

    import numpy as np
    import torch

    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, _abi, build

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    build.build()
    torch.cuda.set_device(local)
    chosen = PS_FORM_MIXED if args.form == "mixed" else PS_FORM_FP64
    L = _abi.lib()
    p64, p32 = C.c_double(), C.c_double()
    _abi.check(L.ps_device_fma_peaks(local, C.byref(p64), C.byref(p32)), "ps_device_fma_peaks")

    with tempfile.TemporaryDirectory() as td:
        path, data, obj = make_workload(Path(td))
        probe = Engine(data, device=local, form=chosen)
        n_max = int(probe.info.n_max)
        info = probe.info
        probe.close()
        # a step: one launch over a whole number of waves of the fit slots
        # (ten poles per period), as inside a long scan
        chunk = args.periods_per_step or int(info.slots)
        total_steps = args.warmup + args.steps
        # chunks spread over the scan, distinct per rank (weak scaling)
        starts = [1 + ((k * world + rank) * 7919) % (n_max - chunk) for k in range(total_steps)]
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

        if world > 1:
            torch.distributed.barrier()
        sampler = ClockSampler(local) if rank == 0 else None
        t0 = time.perf_counter()
        main = _time_form(Engine, data, chosen, local, starts, chunk, args.warmup, args.steps, flush, sampler)
        if world > 1:
            torch.distributed.barrier()
        wall = time.perf_counter() - t0
        # plain FP64 on the same chunks (the comparison the metric asks for)
        plain = None
        if chosen != PS_FORM_FP64 and not args.no_fp64_compare:
            plain = _time_form(Engine, data, PS_FORM_FP64, local, starts, chunk, 1, args.steps, flush)
        simt = None
        if chosen == PS_FORM_MIXED and args.simt_compare:
            simt = _time_form(Engine, data, chosen, local, starts, chunk, 1, args.steps, flush, tensor_cores=False)
            simt["engine"].close()

        # e2e: the whole C-ABI path with host buffers, per step
        e2e_t, e2e_fits, h2d, d2h = 0.0, 0, 0, 0
        for k in range(args.steps):
            n0 = starts[args.warmup + k]
            flush.zero_()
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            e2 = Engine(data, device=local, form=chosen)
            rows = e2.scan(main["conw_r"], n0, n0 + chunk - 1)
            h2d = e2.info.h2d_bytes
            e2.close()
            e2e_t += time.perf_counter() - s0
            e2e_fits += chunk * 10
            d2h = chunk * 10 * C.sizeof(_abi.Fit)
            assert np.isfinite(rows["rms"]).any()

        # validation window around the true period: same best period?
        valid = None
        if plain is not None and rank == 0:
            n_truth = int(round((info.freq_start - 1 / obj.truth["period_h"]) / info.freq_step)) + 1
            half = max(args.validation_window // 2, 1)
            lo, hi = max(1, n_truth - half), min(n_max, n_truth + half - 1)
            wfits = (hi - lo + 1) * 10

            def _timed(fn):
                torch.cuda.synchronize()
                out = fn()
                torch.cuda.synchronize()
                return out

            w_main = _timed(lambda: main["engine"].scan(main["conw_r"], lo, hi))
            t_main = main["engine"].timing()["kernel_ms"]
            w_plain = _timed(lambda: plain["engine"].scan(plain["conw_r"], lo, hi))
            t_plain = plain["engine"].timing()["kernel_ms"]
            rel_w = np.abs(w_main["rms"] - w_plain["rms"]) / w_plain["rms"]
            rel_c = np.concatenate([np.abs(a["rms"] - b["rms"]) / b["rms"] for a, b in zip(main["rows"], plain["rows"])])
            bm, bp = int(np.argmin(w_main["rms"])), int(np.argmin(w_plain["rms"]))
            w_ref, st_ref = main["engine"].scan_refined(main["conw_r"], lo, hi)
            t_ref = st_ref["complete_ms"] + st_ref["refit_ms"]
            scans = {"fp64": {"fits_per_s": wfits / (t_plain / 1e3)},
                     "mixed": {"fits_per_s": wfits / (t_main / 1e3)},
                     "refined": {"fits_per_s": wfits / (t_ref / 1e3), "fp64_refits": int(st_ref["fits_refit"]),
                                 "best_index": int(st_ref["best_index"])}}
            try:
                from periodsearch_gb300 import learned

                _, st_l = main["engine"].scan_learned(main["conw_r"], lo, hi, **learned.CASCADE)
                scans["learned"] = {"fits_per_s": wfits / ((st_l["screen_ms"] + st_l["complete_ms"] + st_l["refit_ms"])
                                                           / 1e3),
                                    "fits_screened_out": int(st_l["fits_screened_out"]),
                                    "best_index": int(st_l["best_index"])}
            except Exception as exc:   # no committed predictor
                scans["learned"] = {"unavailable": str(exc)[:120]}
            bp_all = lo + int(np.argmin(w_plain["rms"]))
            scans["fp64"]["best_index"] = bp_all
            scans["mixed"]["best_index"] = lo + int(np.argmin(w_main["rms"]))
            for v in scans.values():
                if "best_index" in v:
                    v["same_best_period_as_fp64"] = v["best_index"] == bp_all
            valid = {"window": [lo, hi], "truth_period_h": obj.truth["period_h"],
                     "scans": scans,
                     "refined_best_index": int(st_ref["best_index"]),
                     "refined_same_best_period": int(st_ref["best_index"]) == bp_all,
                     "refined_fp64_refits": int(st_ref["fits_refit"]),
                     "best_index_chosen": lo + bm, "best_index_fp64": lo + bp, "same_best_period": bm == bp,
                     "best_period_h_chosen": float(w_main["period_h"][bm]),
                     "best_period_h_fp64": float(w_plain["period_h"][bp]),
                     "chi2_rel_at_best": float(abs(w_main["chi2"][bm] - w_plain["chi2"][bp]) / w_plain["chi2"][bp]),
                     "rms_rel_window_median": float(np.median(rel_w)), "rms_rel_window_max": float(rel_w.max()),
                     "rms_rel_timed_median": float(np.median(rel_c)), "rms_rel_timed_max": float(rel_c.max())}

        # the whole job: every period of the scan, chosen form, then the FP64
        # refit of the minimum region; wall clock through the Python API
        full = None
        if args.full_scan and rank == 0:
            eng = main["engine"]
            torch.cuda.synchronize()
            t_full0 = time.perf_counter()
            rows, st = eng.scan_refined(main["conw_r"], 1, n_max)
            torch.cuda.synchronize()
            t_full = time.perf_counter() - t_full0
            b = int(st["best_index"])
            full = {"periods": n_max, "fits": n_max * 10, "fp64_refits": int(st["fits_refit"]), "seconds": t_full,
                    "fits_per_s": n_max * 10 / t_full, "best_index": b,
                    "best_period_h": float(rows["period_h"][b - 1]), "truth_period_h": obj.truth["period_h"]}

        vals = torch.tensor([main["kernel_ms"] / 1e3, e2e_t, float(main["fits"]), float(e2e_fits)],
                            dtype=torch.float64, device=f"cuda:{local}")
        if world > 1:
            import torch.distributed as dist

            mx = vals[:2].clone()
            dist.all_reduce(mx, op=dist.ReduceOp.MAX)
            sm = vals[2:].clone()
            dist.all_reduce(sm, op=dist.ReduceOp.SUM)
            vals = torch.cat([mx, sm])
        dev_s, e2e_s, fits_all, e2e_fits_all = vals.tolist()

        if rank == 0:
            value = fits_all / dev_s
            launches = main["launches"]
            per_launch_s = (main["kernel_ms"] / 1e3) / max(launches, 1)
            achieved = main["flops"] / max(launches, 1) / per_launch_s / 1e12
            mixed = chosen == PS_FORM_MIXED
            peak = p32.value if mixed else p64.value
            traffic_fit = _profile_traffic(mixed)
            roof = {"bound": "fp32" if mixed else "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if peak else None,
                    "traffic": traffic_fit * chunk * 10 if traffic_fit else None,
                    "peak_source": ("FP32" if mixed else "FP64") + " FMA ceiling measured live on this device by "
                                   "ps_device_fma_peaks (MEASURED_PEAKS.json has no FP32/FP64 SIMT figure)",
                    "kernel": ("fit_kernel<mixed,tensor>" if info.tensor_cores else "fit_kernel<mixed>")
                    if mixed else "fit_kernel<fp64>",
                    "algorithmic_flop_per_launch": main["flops"] / max(launches, 1),
                    "fp64_fma_peak_tflops": p64.value, "fp32_fma_peak_tflops": p32.value}
            if mixed and info.tensor_cores:
                peaks = _measured_peaks()
                f16 = peaks.get("bf16_tflops")
                tf32 = f16 / 2 if f16 else None
                per_s = max(launches, 1) * per_launch_s * 1e12
                shape = main["evals"] * 2.0 * info.ndata * info.nfac * info.ncoef / per_s
                alpha = main["evals"] * info.ndata * info.mfit * (info.mfit + 1) / per_s
                roof["tensor_contractions"] = {
                    "shape": {"achieved": shape, "peak": f16, "unit": "TFLOP/s",
                              "frac": shape / f16 if f16 else None,
                              "peak_source": "measured dense BF16 figure of MEASURED_PEAKS.json (the FP16 rate)",
                              "what": "2 N F C per evaluation, run as FP16 high/low-split MMAs (kind::f16)"},
                    "alpha": {"achieved": alpha, "peak": tf32, "unit": "TFLOP/s",
                              "frac": alpha / tf32 if tf32 else None,
                              "peak_source": "half the measured dense BF16 figure (the TF32 rate)",
                              "what": "N m(m+1) per evaluation, run as TF32 high/low-split MMAs"}}
            fp64 = None
            if plain is not None:
                pv = plain["fits"] / (plain["kernel_ms"] / 1e3)
                pl = plain["launches"]
                pa = plain["flops"] / max(pl, 1) / ((plain["kernel_ms"] / 1e3) / max(pl, 1)) / 1e12
                fp64 = {"value": pv, "unit": "fits/s", "speedup_chosen_over_fp64": value / pv,
                        "roofline": {"bound": "fp64", "achieved": pa, "peak": p64.value, "unit": "TFLOP/s",
                                     "frac": pa / p64.value,
                                     "traffic": (_profile_traffic(False) or 0) * chunk * 10 or None}}
            if simt is not None:
                sv = simt["fits"] / (simt["kernel_ms"] / 1e3)
                roof["mixed_simt_contractions"] = {"value": sv, "unit": "fits/s", "tensor_speedup": value / sv}
            mo = multi_object(args.multi_object, chosen, local) if args.multi_object > 0 else None
            cb = None
            if not args.no_cpu_baseline:
                periods = [n for st in starts[args.warmup:] for n in range(st, st + chunk)]
                cb = cpu_baseline(path, periods, args.cpu_sample_fits)
            if full is not None and cb is not None:
                # the same job on the host cores at the measured CPU rate
                full["cpu_baseline_hours"] = full["fits"] / cb["value"] / 3600
            line = {"metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": main["kernel_ms"] / args.steps, "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
                    "data": "synthetic (seeded generator, c1 shapes; no external dataset)",
                    "config": {"workload": WORKLOAD, "form": args.form, "periods_per_step": chunk,
                               "fits_per_step": chunk * 10, "ndata": info.ndata, "nfac": info.nfac,
                               "ncoef": info.ncoef, "mfit": info.mfit, "n_max": n_max, "conw_r": main["conw_r"],
                               "slots": info.slots, "tensor_cores": bool(info.tensor_cores),
                               "tile_points": info.tile_points, "l2": "flushed between steps (256 MiB rewrite)",
                               "truth": obj.truth},
                    "e2e": {"value": e2e_fits_all / e2e_s, "unit": "fits/s", "h2d_bytes_per_step": h2d,
                            "d2h_bytes_per_step": d2h},
                    "gpu_launches": launches, "roofline": roof, "plain_fp64": fp64, "validation": valid,
                    "multi_object": mo, "full_scan": full,
                    "cpu_baseline": cb, "clocks": sampler.summary() if sampler else None, "wall_s": wall}
            print(json.dumps(line))
        main["engine"].close()
        if plain is not None:
            plain["engine"].close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    args = _args()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_engine_arm(args)


if __name__ == "__main__":
    main()
