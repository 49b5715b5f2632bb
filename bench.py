"""Benchmark: LM period fits/s on one GB300 (per GPU under torchrun).

Workload (c1): one synthetic asteroid with 8 dense relative lightcurves
(3 h, 60 points each, 0.02 mag) and 500 sparse calibrated points over 8
years (Ndata = 980), trial periods 2-50 h with the reference's step rule
(40 000 periods x 10 initial poles), Laplace series L = M = 6 on the
288-facet grid, 50 LM iterations per fit.  Seeded synthetic data (no
external dataset).

A step is one scan of a window of --window consecutive trial periods (x 10
poles; 2000 periods = 20 000 fits by default) around the true period, in the
chosen form (--form):

learned    (default) the learned early-stop cascade (ps_scan_learned): every
           fit screened by 8 mixed-precision LM iterations and the in-kernel
           predictor, periods completed (resumed from their screening state)
           in the order of their predicted rows until none can beat the best
           completed row by the calibrated margin, the minimum region
           refitted in full by the plain FP64 form;
refined    the full mixed-precision scan and the same FP64 refit
           (ps_scan_refined);
mixed      the full mixed-precision scan alone (no refit: its best period
           is not guaranteed to be the FP64 form's);
fp64       the plain FP64 scan.

value      fits of the window per second of device time of the step's
           fit-kernel launches (CUDA events on the engine's stream), the
           object resident in HBM; the plain FP64 scan of the SAME window is
           timed beside it (plain_fp64), and every step's best period is
           compared with the FP64 scan's (validation.same_best_period) and
           its chi^2 there with the FP64 form's;
e2e        the same steps through the C ABI with host buffers: ps_prepare
           (host -> device copy of the tables), the scan (rows back to the
           host) and ps_destroy per step, wall clock;
roofline   the kernel with the largest share of the step's device time:
           algorithmic FLOP of its launches over their time (mixed kernel:
           the dense count 2 N F C + 60 N F + N m(m+1) + 9 F C per
           evaluation and 2 m^3 per solve, against the measured dense BF16
           rate, its contractions running on the tensor cores; FP64 kernel:
           the reference's lit-facet work, flops_fp64, against the FP64 FMA
           ceiling measured live, MEASURED_PEAKS.json having no FP64
           figure); every kernel's share in kernels;
cpu_baseline  the reference's own CPU app (oracle/_ref/ps_ref, built from
           its sources) on all host cores, one process per core, each
           fitting one trial period of the window (10 fits) through the
           reference's resume path.  The same leg runs the CPU oracle (the
           reference's FP64 algorithm) as the checker: the headline's row
           at its best period (validation.vs_oracle_at_best: relative error
           in rms, chi^2 and the fitted period, lambda/beta differences) and
           c2's rows at five periods of its window (c2.vs_oracle).

`--impl reference` times that CPU app alone as the reference arm.  Between
timed steps a 256 MiB buffer is rewritten to flush the 126 MB L2.
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
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LM period fits/s on 1 GB300: chosen form vs plain FP64, same best P, χ² in tol"
WORKLOAD = "c1: 8 dense relative LCs + 500 sparse points (Ndata 980), scan 2-50 h, L=M=6, 288 facets, 10 poles, 50 LM iterations"
PROFILES = {False: ROOT / "profiles" / "fit_kernel_fp64_c1.md", True: ROOT / "profiles" / "fit_kernel_mixed_c1.md"}
REF_BIN = ROOT / "oracle" / "_ref" / "ps_ref"
# the c1 object (periodsearch_gb300.synth, seed 1) as committed by
# tests/golden/make_fixtures.py --only-bench-inputs, with its generating
# parameters: both arms read the same file
WORKLOAD_IN = ROOT / "tests" / "golden" / "c1" / "period_search_in"
WORKLOAD_TRUTH = ROOT / "tests" / "golden" / "c1" / "truth.json"
# The reference app runs its convexity-weight pre-pass (at least 100 fits)
# before any scan while the input's convexity weight is below 10
# (conw_r * escl^2 < 10, period_search_BOINC.cpp:485-489); the timed processes
# start at a weight above that so that they run the scan fits alone.  Every
# fit costs the same at any weight: 51 model evaluations and 50 solves with
# N + 3 rows (stop condition 50).
REF_CONW = 10.5


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--form", default="learned", choices=["learned", "refined", "mixed", "fp64"])
    ap.add_argument("--window", type=int, default=2000, help="trial periods per step (x 10 poles)")
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip the FP64 scan of the window")
    ap.add_argument("--multi-object", type=int, default=512,
                    help="also time K objects of the c3 population (Ndata logU[100, 5000]) packed into one launch "
                         "against one launch per object (512: the many-asteroid configuration)")
    ap.add_argument("--c2", type=int, default=300,
                    help="also time the mixed-precision configuration (c1 data with L = M = 8, 81 coefficients, "
                         "512 facets): a mixed scan of this many periods on the tensor cores, the same on the SIMT "
                         "pipes and the FP64 form on a tenth of them")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--full-scan", action="store_true",
                    help="also run the whole scan of the workload (rank 0) as one refined scan and as one learned "
                         "cascade and report their times and best periods (full_scan)")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def flops_per_eval(ndata, nfac, ncoef, mfit):
    """Dense count of one evaluation: the mixed form's tensor-core
    contraction and branch-free facet stage compute every facet."""
    return 2.0 * ndata * nfac * ncoef + 60.0 * ndata * nfac + ndata * mfit * (mfit + 1) + 9.0 * nfac * ncoef


def flops_fp64(info, evals: int, fits: int, lit: int) -> float:
    """The reference's own work over `evals` FP64 evaluations with `lit`
    lit (point, facet) pairs in all (the engine's count): the two dot
    products of every pair (10), the facet law and its sums on the lit pairs
    (70) and the shape contraction over the lit facets (2 C), as bright.c
    does; the normal equations and the curvature; 2 m^3 per solve."""
    n, f, c, m = info.ndata, info.nfac, info.ncoef, info.mfit
    return ((70.0 + 2.0 * c) * lit + evals * (10.0 * n * f + n * m * (m + 1) + 9.0 * f * c) +
            (evals - fits) * 2.0 * m ** 3)


def window_of(n_max: int, freq_start: float, freq_step: float, truth_h: float, width: int, rank: int = 0):
    """[lo, hi] of `width` periods around the true period (rank r > 0: the
    r-th window after it, so that ranks scan disjoint windows)."""
    n_truth = int(round((freq_start - 1 / truth_h) / freq_step)) + 1
    lo = max(1, min(n_max - width + 1, n_truth - width // 2 + rank * width))
    return lo, lo + width - 1


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


# ---------------------------------------------------------------------------
# The reference's CPU app, one process per core (the CPU baseline and the
# reference arm)
# ---------------------------------------------------------------------------

def _input_for_period(text: str, n: int) -> str:
    """period_search_in whose scan ends at period index n (per_end set so
    that n_max = n; the other tokens of line 1 are kept as written, so the
    frequency grid is the original one) and whose convexity weight skips
    the pre-pass (REF_CONW)."""
    lines = text.split("\n")
    tok = lines[0].split()
    per_start, coef = float(tok[0]), float(tok[1])
    jd, i, n_lc = [], 15, int(lines[14].split()[0])
    for _ in range(n_lc):
        npts = int(lines[i].split()[0])
        jd.extend(float(l.split()[0]) for l in lines[i + 1:i + 1 + npts])
        i += 1 + npts
    step = 0.5 / (max(jd) - min(jd)) / 24 * coef          # period_search_BOINC.cpp:786
    f_end = 1 / per_start - (n - 0.5) * step              # n_max = floor((f_s - f_e) / step) + 1 = n
    lines[0] = " ".join([tok[0], tok[1], repr(1 / f_end), tok[3]]) + "\tperiod_start period_step period_end fixed/free"
    lines[3] = f"{REF_CONW}\tconvexity weight"
    return "\n".join(lines)


def reference_step(text: str, periods: list[int]) -> float:
    """One process of the reference app per period index, all at once, each
    resuming at that period (period_search_state = n - 1,
    period_search_BOINC.cpp:237-251) so that it fits that one period (10
    poles).  Returns the wall time."""
    with tempfile.TemporaryDirectory() as td:
        dirs = []
        for n in periods:
            d = Path(td) / str(n)
            d.mkdir()
            (d / "period_search_in").write_text(_input_for_period(text, n))
            (d / "period_search_state").write_text(str(n - 1))
            dirs.append(d)
        t0 = time.perf_counter()
        procs = [subprocess.Popen([str(REF_BIN)], cwd=d, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
                 for d in dirs]
        rcs = [p.wait() for p in procs]
        dt = time.perf_counter() - t0
        if any(rcs):
            raise RuntimeError(f"reference app failed: exit codes {rcs}")
        for d in dirs:
            if len((d / "period_search_out").read_text().splitlines()) != 1:
                raise RuntimeError("reference app did not write one row")
    return dt


def oracle_step(path: Path, periods: list[int], cores: int) -> float:
    """Fallback when the reference app is not built: the CPU oracle (the
    reference's FP64 algorithm restated), one thread per fit."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding

    oracle_binding.build_oracle()
    probs = [oracle_binding.OracleProblem(path) for _ in range(cores)]
    cw = probs[0].info()["conw_r"]
    for p in probs:
        p.setup(cw)
    jobs = [(n, m) for n in periods for m in range(1, 11)]
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
    return time.perf_counter() - t0


def cpu_rate(path: Path, text: str, periods: list[int], cores: int) -> dict:
    """fits/s of the reference's CPU app (or the oracle port) on the given
    periods (10 fits each)."""
    if REF_BIN.exists():
        dt = reference_step(text, periods)
        kind, how = "reference", "processes of the reference app (oracle/_ref/ps_ref), one per core"
    else:
        dt = oracle_step(path, periods[:cores], cores)
        kind, how = "port", "threads of the CPU oracle (reference app not built)"
    return {"value": 10 * len(periods) / dt, "unit": "fits/s", "cores": cores, "kind": kind,
            "sample": f"{len(periods)} trial periods x 10 poles of the c1 window, {how}, {dt:.1f} s wall",
            "wall_s": dt}


def run_reference_arm(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    # (the input is parsed by the oracle: this arm loads nothing of the engine)
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding

    truth = json.loads(WORKLOAD_TRUTH.read_text())
    path = WORKLOAD_IN
    text = path.read_text()
    ora = oracle_binding.OracleProblem(path)
    inf = ora.info()
    n_max = inf["n_max"]
    f1, f2 = ora.freq(1), ora.freq(2)
    ora.close()
    lo, hi = window_of(n_max, f1, f1 - f2, truth["period_h"], args.window)
    cores = os.cpu_count() or 1

    def periods_of(step):
        return [lo + ((step * cores + i) * 7919) % (hi - lo + 1) for i in range(cores)]

    for s in range(args.warmup):
        cpu_rate(path, text, periods_of(s), cores)
    walls, fits, kind = 0.0, 0, None
    t0 = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        r = cpu_rate(path, text, periods_of(s), cores)
        walls += r["wall_s"]
        fits += 10 * cores
        kind = r["kind"]
    total = time.perf_counter() - t0
    v = fits / walls
    cb = {"value": v, "unit": "fits/s", "cores": cores, "kind": kind,
          "sample": f"{args.steps} steps of {cores} trial periods x 10 poles of the c1 window "
                    f"[{lo}, {hi}], " + ("one reference-app process per core resuming at its period; "
                                         f"convexity weight {REF_CONW} (pre-pass skipped)"
                                         if kind == "reference" else "CPU oracle threads")}
    line = {"metric": METRIC, "value": v, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * walls / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, c1)",
            "config": {"workload": WORKLOAD, "form": "reference CPU app, FP64", "window": [lo, hi]},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": total}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# The engine arm
# ---------------------------------------------------------------------------

def _population_objects(pop: str, K: int, base_seed: int):
    """K objects of a synthetic population, generated by spawned worker
    processes (the parent may already hold the GPU)."""
    import multiprocessing as mp

    from periodsearch_gb300 import synth

    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        return pool.starmap(synth.population_object, [(pop, k, base_seed) for k in range(K)], chunksize=8)


def multi_object(K: int, form: int, local: int, units_per_object: int = 4) -> dict:
    """Many asteroids in one launch: K objects of the c3 population (Ndata
    log-uniform in [100, 5000], half sparse-only and half dense+sparse, scan
    2-20 h, each with its own seed), units_per_object random trial periods x
    10 poles each, fitted by one packed launch against one launch per
    object on the same units."""
    import numpy as np

    from periodsearch_gb300 import Engine, Pack, read_input

    objs = _population_objects("c3", K, 3000)
    rng = np.random.default_rng(2024)
    engines = []
    with tempfile.TemporaryDirectory() as td:
        for k, o in enumerate(objs):
            path = Path(td) / f"o{k}"
            path.write_text(o.text)
            engines.append(Engine(read_input(path), device=local, form=form))
    try:
        conw = [e.info.conw_r0 for e in engines]
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
            got = pk.fit(conw, obj, per, pole)
            pms = pk.timing()["kernel_ms"]
        nd = np.array([e.info.ndata for e in engines])
        dense = sum("\n60 0\n" in o.text for o in objs)     # objects with relative 60-point lightcurves
        return {"population": "c3: Ndata logU[100, 5000], sparse-only and dense+sparse, scan 2-20 h",
                "objects": K, "dense_plus_sparse": int(dense),
                "fits": int(len(obj)), "ndata_min": int(nd.min()), "ndata_max": int(nd.max()),
                "ndata_mean": float(nd.mean()), "packed_fits_per_s": len(obj) / (pms / 1e3),
                "packed_ms": pms, "one_launch_per_object_fits_per_s": len(obj) / (seq_ms / 1e3),
                "speedup": seq_ms / pms, "finite": bool(np.isfinite(got["dev"]).all())}
    finally:
        for e in engines:
            e.close()


def c2_measurement(periods: int, local: int, peaks: dict) -> dict:
    """The mixed-precision configuration c2 (c1's data, Laplace series L = M =
    8 on the 512-facet grid): fits/s of the mixed form with its shape
    contraction on the tensor cores (the wide path), of the same form with
    the SIMT contraction, and of the FP64 form, with the tensor form's
    algorithmic FLOP rate against the measured BF16 peak and its rms error
    against the FP64 form per period."""
    import numpy as np

    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input, synth

    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "period_search_in"
        obj = synth.write_object(path, "c2")
        data = read_input(path)
        text = path.read_text()
    out = {"workload": "c2: c1 data (Ndata 980), L=M=8 (81 coefficients), 512 facets, 50 LM iterations"}
    with Engine(data, device=local, form=PS_FORM_MIXED) as eng:
        info = eng.info
        n_max = int(info.n_max)
        lo, hi = window_of(n_max, info.freq_start, info.freq_step, obj.truth["period_h"], periods)
        conw_r = info.conw_r0
        eng.scan(conw_r, lo, lo + 9)      # warm-up
        rows_tc = eng.scan(conw_r, lo, hi)
        t = eng.timing()
        fe = flops_per_eval(info.ndata, info.nfac, info.ncoef, info.mfit)
        flop = t["evals"] * fe + (t["evals"] - t["fits"]) * 2.0 * info.mfit ** 3
        ach = flop / (t["kernel_ms"] / 1e3) / 1e12
        bf16 = peaks.get("bf16_tflops")
        shape = t["evals"] * 2.0 * info.ndata * info.nfac * info.ncoef / (t["kernel_ms"] / 1e3) / 1e12
        out.update({"tensor_cores": bool(info.tensor_cores), "ncoef": info.ncoef, "nfac": info.nfac,
                    "mfit": info.mfit, "window": [lo, hi], "fits": t["fits"],
                    "mixed_tensor_fits_per_s": t["fits"] / (t["kernel_ms"] / 1e3),
                    "roofline": {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                                 "frac": ach / bf16 if bf16 else None,
                                 "shape_contraction_tflops": shape,
                                 "shape_contraction_frac": shape / bf16 if bf16 else None,
                                 "peak_source": "measured dense BF16 burst of MEASURED_PEAKS.json"}})
    with Engine(data, device=local, form=PS_FORM_MIXED, tensor_cores=False) as eng:
        eng.scan(conw_r, lo, hi)
        t = eng.timing()
        out["mixed_simt_fits_per_s"] = t["fits"] / (t["kernel_ms"] / 1e3)
    n64 = max(1, periods // 10)
    with Engine(data, device=local, form=PS_FORM_FP64) as e64:
        rows64 = e64.scan(conw_r, lo, lo + n64 - 1)
        t = e64.timing()
        out["fp64_fits_per_s"] = t["fits"] / (t["kernel_ms"] / 1e3)
    rel = (rows_tc["rms"][:n64] - rows64["rms"]) / rows64["rms"]
    out.update({"tensor_over_simt": out["mixed_tensor_fits_per_s"] / out["mixed_simt_fits_per_s"],
                "tensor_over_fp64": out["mixed_tensor_fits_per_s"] / out["fp64_fits_per_s"],
                "rms_rel_vs_fp64_median": float(np.median(np.abs(rel))), "rms_rel_vs_fp64_max": float(np.abs(rel).max()),
                "fp64_periods": n64})
    # for the CPU-baseline leg's oracle check: the tensor form's best period
    # and four more spread over the window
    best = lo + int(np.argmin(rows_tc["rms"]))
    periods = sorted({best, *(lo + (hi - lo) * k // 4 for k in range(4))})
    out["_check"] = {"text": text, "conw_r": conw_r, "periods": periods, "best": best, "ndata": info.ndata,
                     "rows": {n: rows_tc[n - lo] for n in periods}}
    return out


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


class Scanner:
    """One scan of [lo, hi] in the chosen form through the engine, with the
    device time and algorithmic FLOP of each kernel's launches."""

    def __init__(self, form: str, eng, eng64, conw_r: float, fe: float, fs: float):
        self.form, self.eng, self.eng64, self.conw_r, self.fe, self.fs = form, eng, eng64, conw_r, fe, fs
        self.info = eng.info

    def __call__(self, lo: int, hi: int):
        from periodsearch_gb300 import learned

        nfits = (hi - lo + 1) * 10
        if self.form == "learned":
            rows, st = self.eng.scan_learned(self.conw_r, lo, hi, **learned.cascade_defaults())
            lit = self.eng.timing()["lit_facets"]
        elif self.form == "refined":
            rows, st = self.eng.scan_refined(self.conw_r, lo, hi)
            lit = self.eng.timing()["lit_facets"]
        else:
            eng = self.eng64 if self.form == "fp64" else self.eng
            rows = eng.scan(self.conw_r, lo, hi)
            t = eng.timing()
            lit = t["lit_facets"]
            key = "refit" if self.form == "fp64" else "complete"
            st = {"fits_total": nfits, "launches": t["launches"], "screen_ms": 0.0, "complete_ms": 0.0,
                  "refit_ms": 0.0, "evals_screen": 0, "evals_complete": 0, "evals_refit": 0, "fits_completed": 0,
                  "fits_refit": 0, "fits_screened_out": 0, "refit_rounds": 0}
            st[f"{key}_ms"] = t["kernel_ms"]
            st[f"evals_{key}"] = t["evals"]
            st["fits_completed" if key == "complete" else "fits_refit"] = nfits
        screen_fits = nfits if st["evals_screen"] else 0
        mixed_ms = st["screen_ms"] + st["complete_ms"]
        mixed_flop = ((st["evals_screen"] + st["evals_complete"]) * self.fe +
                      (st["evals_screen"] - screen_fits + st["evals_complete"] - st["fits_completed"]) * self.fs)
        fp64_flop = flops_fp64(self.info, st["evals_refit"], st["fits_refit"], lit)
        # the FP64 refit launches are the refit rounds; every other launch is the mixed kernel
        mixed_launches = st["launches"] - st["refit_rounds"]
        if self.form in ("mixed", "fp64"):
            mixed_launches = st["launches"] if self.form == "mixed" else 0
        fp64_launches = st["launches"] - mixed_launches
        return rows, {"device_ms": mixed_ms + st["refit_ms"], "fits": nfits, "launches": st["launches"],
                      "mixed_ms": mixed_ms, "mixed_flop": mixed_flop, "mixed_launches": mixed_launches,
                      "mixed_evals": st["evals_screen"] + st["evals_complete"],
                      "fp64_ms": st["refit_ms"], "fp64_flop": fp64_flop, "fp64_launches": fp64_launches,
                      "fp64_evals": st["evals_refit"], "stats": st}


def oracle_rows(path: Path, conw_r: float, periods: list[int], cores: int, ndata: int) -> dict:
    """The CPU oracle's rows at the given period indices (all ten poles of
    each, the best pole kept; chi^2 = rms^2 Ndata as in the output rows), on
    `cores` threads.  The checker of the CPU-baseline leg."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_binding

    oracle_binding.build_oracle()
    jobs = [(n, m) for n in periods for m in range(1, 11)]
    nw = max(1, min(cores, len(jobs)))
    probs = [oracle_binding.OracleProblem(path) for _ in range(nw)]
    for p in probs:
        p.setup(conw_r)
    fits = {}

    def work(w):
        for k in range(w, len(jobs), nw):
            fits[jobs[k]] = probs[w].fit_n(*jobs[k])

    with ThreadPoolExecutor(nw) as ex:
        list(ex.map(work, range(nw)))
    for p in probs:
        p.close()
    out = {}
    for n in periods:
        f = min((fits[(n, m)] for m in range(1, 11)), key=lambda f: f["dev"])
        out[n] = {"rms": f["dev"], "chi2": f["dev"] ** 2 * ndata, "period_h": 24.0 * f["prd"], "lambda_deg": f["la"],
                  "beta_deg": f["be"]}
    return out


def versus_oracle(row, orc: dict) -> dict:
    """Relative errors of an engine row against the oracle's row (rms, chi^2,
    the fitted period) and the pole's angular differences in degrees."""
    dl = abs(float(row["lambda_deg"]) - orc["lambda_deg"]) % 360.0
    return {"rms_rel": abs(float(row["rms"]) - orc["rms"]) / orc["rms"],
            "chi2_rel": abs(float(row["chi2"]) - orc["chi2"]) / orc["chi2"],
            "period_rel": abs(float(row["period_h"]) - orc["period_h"]) / orc["period_h"],
            "lambda_deg_diff": min(dl, 360.0 - dl),
            "beta_deg_diff": abs(float(row["beta_deg"]) - orc["beta_deg"])}


def run_engine_arm(args):
    import numpy as np
    import torch

    import ctypes as C

    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, _abi, build, read_input

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    build.build()
    torch.cuda.set_device(local)
    L = _abi.lib()
    p64, p32 = C.c_double(), C.c_double()
    _abi.check(L.ps_device_fma_peaks(local, C.byref(p64), C.byref(p32)), "ps_device_fma_peaks")
    peaks = _measured_peaks()
    bf16 = peaks.get("bf16_tflops")

    truth = json.loads(WORKLOAD_TRUTH.read_text())
    path = WORKLOAD_IN
    text = path.read_text()
    data = read_input(path)
    eng = Engine(data, device=local, form=PS_FORM_MIXED)
    eng64 = Engine(data, device=local, form=PS_FORM_FP64)
    info = eng.info
    n_max = int(info.n_max)
    conw_r, _ = eng.precalc_conw()
    fe = flops_per_eval(info.ndata, info.nfac, info.ncoef, info.mfit)
    fs = 2.0 * info.mfit ** 3
    scan = Scanner(args.form, eng, eng64, conw_r, fe, fs)
    lo, hi = window_of(n_max, info.freq_start, info.freq_step, truth["period_h"], args.window, rank)
    wfits = (hi - lo + 1) * 10
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        scan(lo, hi)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.__enter__()
    steps, t0 = [], time.perf_counter()
    try:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            rows, t = scan(lo, hi)
            t["wall_s"] = time.perf_counter() - s0
            steps.append((rows, t))
    finally:
        if sampler:
            sampler.__exit__(None, None, None)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t0

    # e2e: the same steps through the C ABI with host buffers
    e2e_t, h2d, d2h = 0.0, 0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        e_m = Engine(data, device=local, form=PS_FORM_MIXED)
        e_64 = Engine(data, device=local, form=PS_FORM_FP64) if args.form in ("fp64",) else None
        Scanner(args.form, e_m, e_64, conw_r, fe, fs)(lo, hi)
        h2d = e_m.info.h2d_bytes + (e_64.info.h2d_bytes if e_64 else 0)
        e_m.close()
        if e_64:
            e_64.close()
        e2e_t += time.perf_counter() - s0
    d2h = (hi - lo + 1) * C.sizeof(_abi.Row)

    dev_s = sum(t["device_ms"] for _, t in steps) / 1e3
    vals = torch.tensor([dev_s, e2e_t, float(wfits * args.steps)], dtype=torch.float64, device=f"cuda:{local}")
    if world > 1:
        import torch.distributed as dist

        mx = vals[:2].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = vals[2:].clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        vals = torch.cat([mx, sm])
    dev_all, e2e_all, fits_all = vals.tolist()

    if rank == 0:
        value = fits_all / dev_all
        best_steps = [lo + int(np.argmin(r["rms"])) for r, _ in steps]
        # ---- validation on the same window ----
        valid, fp64 = {"window": [lo, hi], "truth_period_h": truth["period_h"],
                       "best_index_steps": sorted(set(best_steps))}, None
        if not args.no_fp64_compare:
            r64 = eng64.scan(conw_r, lo, hi)
            t64 = eng64.timing()
            b64 = lo + int(np.argmin(r64["rms"]))
            pv = wfits / (t64["kernel_ms"] / 1e3)
            pflop = flops_fp64(info, t64["evals"], t64["fits"], t64["lit_facets"])
            pa = pflop / (t64["kernel_ms"] / 1e3) / 1e12
            fp64 = {"value": pv, "unit": "fits/s", "window": [lo, hi], "fits": wfits,
                    "seconds": t64["kernel_ms"] / 1e3, "best_index": b64,
                    "speedup_chosen_over_fp64": value / pv,
                    "lit_fraction": t64["lit_facets"] / (t64["evals"] * info.ndata * info.nfac),
                    "roofline": {"bound": "fp64", "achieved": pa, "peak": p64.value, "unit": "TFLOP/s",
                                 "frac": pa / p64.value,
                                 "count": "the reference's lit-facet work (flops_fp64)",
                                 "peak_source": "FP64 FMA ceiling measured live by ps_device_fma_peaks"}}
            rows_c = steps[-1][0]
            bc = best_steps[-1]
            valid.update({
                "best_index_fp64": b64, "same_best_period": all(b == b64 for b in best_steps),
                "best_period_h": float(rows_c["period_h"][bc - lo]),
                "chi2_rel_at_best_vs_fp64_form": float(abs(rows_c["chi2"][bc - lo] - r64["chi2"][b64 - lo]) /
                                                       r64["chi2"][b64 - lo]),
                "rms_at_best": float(rows_c["rms"][bc - lo])})
            # the other forms on the same window
            others = {}
            for f in ("learned", "refined", "mixed"):
                if f == args.form:
                    continue
                rr, tt = Scanner(f, eng, eng64, conw_r, fe, fs)(lo, hi)
                bo = lo + int(np.argmin(rr["rms"]))
                rel = np.abs(rr["rms"] - r64["rms"]) / r64["rms"]
                others[f] = {"fits_per_s": wfits / (tt["device_ms"] / 1e3), "best_index": bo,
                             "same_best_period_as_fp64": bo == b64,
                             "rms_rel_vs_fp64_median": float(np.median(rel)),
                             "rms_rel_vs_fp64_max": float(rel.max())}
                if f != "mixed":
                    others[f]["fp64_refits"] = int(tt["stats"]["fits_refit"])
                    others[f]["refit_rounds"] = int(tt["stats"]["refit_rounds"])
            valid["other_forms"] = others
        # ---- per-kernel shares and the dominant kernel's roofline ----
        mixed_ms = sum(t["mixed_ms"] for _, t in steps)
        fp64_ms = sum(t["fp64_ms"] for _, t in steps)
        mixed_flop = sum(t["mixed_flop"] for _, t in steps)
        fp64_flop = sum(t["fp64_flop"] for _, t in steps)
        mixed_l = sum(t["mixed_launches"] for _, t in steps)
        fp64_l = sum(t["fp64_launches"] for _, t in steps)
        launches = mixed_l + fp64_l
        tot_ms = mixed_ms + fp64_ms
        kname = "fit_kernel<mixed,tensor>" if info.tensor_cores else "fit_kernel<mixed>"
        kernels = {kname: {"launches": mixed_l, "ms": mixed_ms, "share": mixed_ms / tot_ms if tot_ms else 0,
                           "tflops": mixed_flop / (mixed_ms / 1e3) / 1e12 if mixed_ms else None},
                   "fit_kernel<fp64>": {"launches": fp64_l, "ms": fp64_ms,
                                        "share": fp64_ms / tot_ms if tot_ms else 0,
                                        "tflops": fp64_flop / (fp64_ms / 1e3) / 1e12 if fp64_ms else None}}
        if mixed_ms >= fp64_ms:
            ach = mixed_flop / (mixed_ms / 1e3) / 1e12
            tr = _profile_traffic(True)
            roof = {"bound": "tensor", "kernel": kname, "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                    "frac": ach / bf16 if bf16 else None,
                    "traffic": tr * (wfits * args.steps / max(mixed_l, 1)) if tr else None,
                    "peak_source": "measured dense BF16 burst of MEASURED_PEAKS.json (the FP16 MMA rate)",
                    "algorithmic_flop_per_launch": mixed_flop / max(mixed_l, 1),
                    "fp32_simt": {"peak": p32.value, "frac": ach / p32.value,
                                  "peak_source": "FP32 FMA ceiling measured live by ps_device_fma_peaks"}}
        else:
            ach = fp64_flop / (fp64_ms / 1e3) / 1e12
            tr = _profile_traffic(False)
            st_last = steps[-1][1]["stats"]
            per_launch = st_last["fits_refit"] / max(st_last["refit_rounds"], 1)
            roof = {"bound": "fp64", "kernel": "fit_kernel<fp64>", "achieved": ach, "peak": p64.value,
                    "unit": "TFLOP/s", "frac": ach / p64.value,
                    "traffic": tr * per_launch if tr else None,
                    "peak_source": "FP64 FMA ceiling measured live by ps_device_fma_peaks "
                                   "(MEASURED_PEAKS.json has no FP64 figure)",
                    "algorithmic_flop_per_launch": fp64_flop / max(fp64_l, 1)}
        st = steps[-1][1]["stats"]
        cascade = {k: st.get(k) for k in ("fits_total", "fits_screened_out", "fits_completed", "fits_refit",
                                          "refit_rounds", "region_periods", "launches")}
        cascade["device_ms_per_step"] = 1000 * dev_all / args.steps
        cascade["wall_ms_per_step"] = 1000 * statistics.mean(t["wall_s"] for _, t in steps)
        mo = multi_object(args.multi_object, PS_FORM_MIXED, local) if args.multi_object > 0 else None
        c2 = c2_measurement(args.c2, local, peaks) if args.c2 > 0 else None
        full = None
        if args.full_scan:
            from periodsearch_gb300 import learned

            # the whole job: every period of the object, by the refined scan
            # and by the learned cascade (the chosen form)
            full = {"periods": n_max, "fits": n_max * 10, "truth_period_h": truth["period_h"]}
            for key, run in (("refined", lambda: eng.scan_refined(conw_r, 1, n_max)),
                             ("learned", lambda: eng.scan_learned(conw_r, 1, n_max, **learned.cascade_defaults()))):
                torch.cuda.synchronize()
                t_full0 = time.perf_counter()
                rows_f, stf = run()
                torch.cuda.synchronize()
                t_full = time.perf_counter() - t_full0
                b = int(stf["best_index"])
                full[key] = {"seconds": t_full, "fits_per_s": n_max * 10 / t_full, "best_index": b,
                             "best_period_h": float(rows_f["period_h"][b - 1]),
                             "fits_completed": int(stf["fits_completed"]), "fp64_refits": int(stf["fits_refit"])}
            full["same_best_period"] = full["refined"]["best_index"] == full["learned"]["best_index"]
        cb = None
        c2_check = c2.pop("_check", None) if c2 else None
        if not args.no_cpu_baseline and world == 1:
            cores = os.cpu_count() or 1
            cb = cpu_rate(path, text, [lo + (i * 7919) % (hi - lo + 1) for i in range(cores)], cores)
            cb.pop("wall_s", None)
            # the CPU oracle as the checker: the headline's row at its best
            # period, and c2's rows at five periods of its window
            bc = best_steps[-1]
            orc = oracle_rows(path, conw_r, [bc], cores, info.ndata)[bc]
            valid["vs_oracle_at_best"] = {"period_index": bc, "oracle": orc,
                                          **versus_oracle(steps[-1][0][bc - lo], orc)}
            if c2_check:
                with tempfile.TemporaryDirectory() as td:
                    p2 = Path(td) / "period_search_in"
                    p2.write_text(c2_check["text"])
                    o2 = oracle_rows(p2, c2_check["conw_r"], c2_check["periods"], cores, c2_check["ndata"])
                per = [{"period_index": n, **versus_oracle(c2_check["rows"][n], o2[n])} for n in c2_check["periods"]]
                c2["vs_oracle"] = {"periods": per, "best_index": c2_check["best"],
                                   "rms_rel_max": max(x["rms_rel"] for x in per),
                                   "chi2_rel_max": max(x["chi2_rel"] for x in per),
                                   "period_rel_max": max(x["period_rel"] for x in per),
                                   "lambda_deg_diff_max": max(x["lambda_deg_diff"] for x in per),
                                   "beta_deg_diff_max": max(x["beta_deg_diff"] for x in per)}
        line = {"metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * dev_all / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.form == "fp64" else "f16/tf32 tensor + f32 + f64",
                "data": "synthetic (seeded generator, c1 shapes; no external dataset)",
                "config": {"workload": WORKLOAD, "form": args.form, "window": [lo, hi], "fits_per_step": wfits,
                           "ndata": info.ndata, "nfac": info.nfac, "ncoef": info.ncoef, "mfit": info.mfit,
                           "n_max": n_max, "conw_r": conw_r, "slots": info.slots,
                           "tensor_cores": bool(info.tensor_cores), "tile_points": info.tile_points,
                           "l2": "flushed between steps (256 MiB rewrite)", "truth": truth},
                "e2e": {"value": fits_all / e2e_all, "unit": "fits/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "roofline": roof, "kernels": kernels, "cascade": cascade,
                "plain_fp64": fp64, "validation": valid, "multi_object": mo, "c2": c2, "full_scan": full,
                "cpu_baseline": cb, "clocks": sampler.summary() if sampler else None, "wall_s": wall}
        print(json.dumps(line))
    eng.close()
    eng64.close()
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
