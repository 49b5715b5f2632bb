"""Generates the golden fixtures of tests/golden/ from the reference tree.

Run where the reference project is present, after `make -C oracle ref
REF_DIR=<reference root>/period_search` has built the reference CPU app into
oracle/_ref/ps_ref.  Writes:

* period_search_in / period_search_out -- the reference's own committed
  golden input/output pair (period_search/period_search_in and _out);
* golden12.full -- the reference binary's rows 1..12 of that input at %.17g
  (input truncated with per_end so that the scan has 12 periods);
* <case>/period_search_in, <case>/period_search_out, <case>/ref.full -- the
  seeded synthetic cases of periodsearch_gb300.synth and the reference
  binary's output for each (text and %.17g);
* wu_<id>/period_search_in, wu_<id>/period_search_out, wu_<id>/ref.full --
  four of the reference's real work units
  (period_search/input_period_search/period_search_in_<id>: survey
  photometry, all relative, L = M = 3, 288 facets, 2-1000 h), each cut to
  its first 12 trial periods, and the reference binary's output for each;
* c1/period_search_in, c1/truth.json -- the benchmark's workload (the
  seeded c1 object of periodsearch_gb300.synth) and its generating
  parameters, so that the benchmark's CPU arms read the input without the
  engine's library (also written alone by --only-bench-inputs, which needs
  no reference tree);
* unit_arrays.json -- golden arrays of the reference's unit tests
  (period_search_pure_cpu_win/UnitTest_pure_cpu_win/arrangers.cpp and the
  test inputs of InnerFunctionsTests.cpp): trifac vertex triplets, normal
  angles, the Laplace basis, the ellipsoid coefficients and the phase function.

Usage: python tests/golden/make_fixtures.py REFERENCE_ROOT [--only-work-units | --only-unit-arrays]
       python tests/golden/make_fixtures.py --only-bench-inputs
"""
from __future__ import annotations

import json
import math
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from oracle_binding import REF_BIN  # noqa: E402
from periodsearch_gb300 import synth  # noqa: E402

SYNTH_CASES = ["tiny_cal", "tiny_rel", "tiny_mix", "tiny_stop", "c0_12"]
# real work units of the reference: 1, 8, 9 and 19 lightcurves (about 100,
# 260, 640 and 840 points)
WORK_UNITS = ["17979", "4332", "26380", "2543"]


def _truncate_periods(text: str, n_periods: int) -> str:
    """Sets per_end so that the scan has exactly n_periods trial periods."""
    lines = text.split("\n")
    per_start, coef, _, ia = lines[0].split()[:4]
    per_start, coef = float(per_start), float(coef)
    jd = []
    i = 15
    n_lc = int(lines[14].split()[0])
    for _ in range(n_lc):
        npts = int(lines[i].split()[0])
        jd.extend(float(l.split()[0]) for l in lines[i + 1:i + 1 + npts])
        i += 1 + npts
    step = 0.5 / (max(jd) - min(jd)) / 24 * coef
    f_end = 1 / per_start - (n_periods - 0.5) * step
    lines[0] = f"{per_start:g} {coef:g} {1 / f_end:.10f} {ia} period_start period_step period_end fixed/free"
    return "\n".join(lines)


def _run_chunked(binary: Path, text: str, n_total: int, n_chunks: int) -> "list[str]":
    """Rows 1..n_total of a reference binary, computed by n_chunks processes
    over contiguous period ranges: each process gets the same input with
    per_end truncated to its last period and a period_search_state holding
    its first period - 1 (the reference's own resume path); every process
    re-runs the convexity pre-pass on periods 1..10."""
    from concurrent.futures import ThreadPoolExecutor

    bounds = [round(i * n_total / n_chunks) for i in range(n_chunks + 1)]

    def one(k):
        lo, hi = bounds[k] + 1, bounds[k + 1]
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "period_search_in").write_text(_truncate_periods(text, max(hi, 10)))
            if lo > 1:
                (td / "period_search_state").write_text(str(lo - 1))
            subprocess.run([str(binary)], cwd=td, check=True, capture_output=True)
            rows = (td / "period_search_out.full").read_text().splitlines()
            return rows[: hi - lo + 1]

    with ThreadPoolExecutor(n_chunks) as ex:
        parts = list(ex.map(one, range(n_chunks)))
    return [r for p in parts for r in p]


def _run_ref(workdir: Path) -> None:
    subprocess.run([str(REF_BIN)], cwd=workdir, check=True, capture_output=True)
    shutil.move(str(workdir / "period_search_out.full"), str(workdir / "ref.full"))


def _arrays(src: str, func: str) -> dict[str, list[float]]:
    """Initialised arrays declared in the body of function `func`."""
    m = re.search(r"\n\w[\w\s\*]*\b" + func + r"\s*\([^)]*\)\s*\{", src)
    body_start = m.end()
    depth, i = 1, body_start
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    body = src[body_start:i]
    out = {}
    for am in re.finditer(r"(?:double|int)\s+(\w+)\s*\[[^\]]*\]\s*=\s*\{([^}]*)\}", body):
        vals = [v.strip() for v in am.group(2).split(",") if v.strip()]
        out[am.group(1)] = [float(v) for v in vals]
    return out


def unit_arrays(ref_root: Path) -> dict:
    ut = ref_root / "period_search_pure_cpu_win" / "UnitTest_pure_cpu_win"
    src = (ut / "arrangers.cpp").read_text()
    out: dict = {"source": "period_search_pure_cpu_win/UnitTest_pure_cpu_win/arrangers.cpp"}
    a = _arrays(src, "get_ifp")
    out["ifp"] = [[int(a[f"_ifp_{j}"][i]) for j in (1, 2, 3)] for i in range(1, 289)]
    out["at"] = _arrays(src, "get_at")["_at"][1:289]
    out["af"] = _arrays(src, "get_af")["_af"][1:289]
    d = _arrays(src, "get_dsph")
    # _dsph_k[i] = Dsph[i][k] for facets 1..146, coefficients 1..16
    out["dsph_146x16"] = [[d[f"_dsph_{k}"][i] for k in range(1, 17)] for i in range(1, 147)]
    out["cg_first_l3"] = _arrays(src, "get_cg_first")["_cg_first_local"][1:17]
    # TestEllfit inputs (InnerFunctionsTests.cpp:356-421): Lmax = Mmax = 3,
    # calibrated data (escl * 0.8), mean brightness and solar phase angle of
    # the reference object's first lightcurve.
    out["ellfit_inputs"] = {"ave": 0.382008772881355651573898057904, "al0": 0.069555451868686835048549710336,
                            "onlyrel": 0, "lmax": 3, "nrows": 6}
    x1 = _arrays(src, "get_xx1")["__xx1"][1:4]
    x2 = _arrays(src, "get_xx2")["__xx2"][1:4]
    cg = _arrays(src, "get_cg24")["_cg"]
    out["phasec"] = {"xx1": x1, "xx2": x2, "par": cg[20:23], "dphp": _arrays(src, "get_dphp")["__dphp"][1:4],
                     "scale": 1.214621163362573641464337015350}
    # TestBright / TestConv (InnerFunctionsTests.cpp): one observation (the
    # first point of the test object) at the 24 parameters of get_cg24;
    # expected brightness (TestBright's _ymod), derivatives (get_dyda, index
    # 0 = the first parameter), and the convexity row 1 (TestConv's _ymod,
    # get_dyda_after_conv, same indexing, except that index 0 keeps the
    # value the test array held before the call, get_dyda_before_conv's)
    tests = (ut / "InnerFunctionsTests.cpp").read_text()

    def ymod_of(method):
        i = tests.index(f"TEST_METHOD({method})")
        return float(re.search(r"_ymod\s*=\s*([-+0-9.eE]+)\s*;", tests[i:]).group(1))

    out["bright"] = {"cg": cg[1:25], "ee": x1, "ee0": x2, "t": _arrays(src, "get_tim")["_tim"][1], "phi0": 0.0,
                     "ymod": ymod_of("TestBright"), "dyda": _arrays(src, "get_dyda")["__dyda"][0:24],
                     "source": "InnerFunctionsTests.cpp TestBright, arrangers.cpp get_cg24/get_tim/get_xx1/"
                               "get_xx2/get_dyda"}
    # TestCurv: facet areas (get_area) and g Dsph (get_dg, one array per
    # coefficient) of the initial ellipsoid (cg_first_l3), facets and
    # coefficients from index 0
    dg = _arrays(src, "get_dg")
    out["curv"] = {"area": _arrays(src, "get_area")["_area_a"][0:288],
                   "dg": [[dg[f"_dg_{k}"][i] for k in range(16)] for i in range(288)],
                   "source": "InnerFunctionsTests.cpp TestCurv, arrangers.cpp get_area/get_dg"}
    out["conv"] = {"cg": cg[1:25], "nc": 1, "ymod": ymod_of("TestConv"),
                   "dyda": _arrays(src, "get_dyda_after_conv")["__dyda"][0:24],
                   "source": "InnerFunctionsTests.cpp TestConv, arrangers.cpp get_dyda_after_conv"}
    return out


def work_units(ref_root: Path) -> None:
    src = ref_root / "period_search" / "input_period_search"
    for wu in WORK_UNITS:
        d = HERE / f"wu_{wu}"
        d.mkdir(exist_ok=True)
        (d / "period_search_in").write_text(_truncate_periods((src / f"period_search_in_{wu}").read_text(), 12))
        _run_ref(d)
        for junk in ("temp", "period_search_state"):
            (d / junk).unlink(missing_ok=True)


BENCH_CASES = ["c1"]


def bench_inputs() -> None:
    for case in BENCH_CASES:
        d = HERE / case
        d.mkdir(exist_ok=True)
        obj = synth.make_object(case)
        (d / "period_search_in").write_text(obj.text)
        (d / "truth.json").write_text(json.dumps(obj.truth, indent=1) + "\n")


def main(ref_root: Path, only_work_units: bool = False, only_unit_arrays: bool = False) -> None:
    bench_inputs()
    if only_unit_arrays:
        (HERE / "unit_arrays.json").write_text(json.dumps(unit_arrays(ref_root)))
        print("unit arrays written to", HERE)
        return
    if not REF_BIN.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF_DIR={ref_root / 'period_search'}"],
                       check=True)
    work_units(ref_root)
    if only_work_units:
        print("work-unit fixtures written to", HERE)
        return
    gold_in = ref_root / "period_search" / "period_search_in"
    shutil.copy(gold_in, HERE / "period_search_in")
    shutil.copy(ref_root / "period_search" / "period_search_out", HERE / "period_search_out")
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "period_search_in").write_text(_truncate_periods(gold_in.read_text(), 12))
        _run_ref(td)
        shutil.copy(td / "ref.full", HERE / "golden12.full")
    for case in SYNTH_CASES:
        d = HERE / case
        d.mkdir(exist_ok=True)
        if case == "c0_12":
            text = _truncate_periods(synth.make_object("c0").text, 12)
        else:
            text = synth.make_object(case).text
        (d / "period_search_in").write_text(text)
        _run_ref(d)
        for junk in ("temp", "period_search_state"):
            (d / junk).unlink(missing_ok=True)
    (HERE / "unit_arrays.json").write_text(json.dumps(unit_arrays(ref_root)))
    # rows 1..134 (the length of the reference's period_search_out) at full
    # precision, from the base build and, on x86-64, from the reference's own
    # AVX2/FMA build: the cross-build agreement of the reference itself
    import os

    cores = os.cpu_count() or 1
    rows = _run_chunked(REF_BIN, gold_in.read_text(), 134, cores)
    (HERE / "golden134.full").write_text("\n".join(rows) + "\n")
    fma = REF_BIN.parent / "ps_ref_fma"
    if not fma.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref_fma",
                        f"FMA_DIR={ref_root / 'period_search_optimization_avx_fma' / 'period_search'}"], check=False)
    if fma.exists():
        rows = _run_chunked(fma, gold_in.read_text(), 134, cores)
        (HERE / "golden134_fma.full").write_text("\n".join(rows) + "\n")
    print("fixtures written to", HERE)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--only-bench-inputs" in sys.argv:
        bench_inputs()
        sys.exit(0)
    if not args:
        sys.exit("\n".join(__doc__.strip().splitlines()[-2:]))
    main(Path(args[0]), "--only-work-units" in sys.argv, "--only-unit-arrays" in sys.argv)
