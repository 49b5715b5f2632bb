"""The benchmark's reference arm runs on the host cores alone: its JSON line
carries the keys the measurement contract asks for (CPU only)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["unit"] == "fits/s" and line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]


def _bench():
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_module", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fp64_flop_count():
    """The FP64 roofline counts the reference's own work: the dense count's
    contraction and facet law scale with the lit (point, facet) pairs; with
    every pair lit it is the dense formulation's size or more."""
    from types import SimpleNamespace

    b = _bench()
    info = SimpleNamespace(ndata=980, nfac=288, ncoef=49, mfit=55)
    evals, fits = 51, 1
    none = b.flops_fp64(info, evals, fits, 0)
    half = b.flops_fp64(info, evals, fits, evals * 980 * 144)
    full = b.flops_fp64(info, evals, fits, evals * 980 * 288)
    assert none < half < full
    assert full - half == half - none                      # linear in the lit pairs
    dense = evals * b.flops_per_eval(980, 288, 49, 55) + (evals - fits) * 2.0 * 55 ** 3
    assert full >= dense


def test_versus_oracle():
    """Relative errors against the oracle's row, and the pole longitude
    difference taken across the 0/360 degree seam."""
    b = _bench()
    orc = {"rms": 0.1, "chi2": 2.0, "period_h": 5.0, "lambda_deg": 359.5, "beta_deg": 10.0}
    row = {"rms": 0.1001, "chi2": 2.004, "period_h": 5.0, "lambda_deg": 0.5, "beta_deg": 9.0}
    v = b.versus_oracle(row, orc)
    assert abs(v["rms_rel"] - 1e-3) < 1e-12 and abs(v["chi2_rel"] - 2e-3) < 1e-12
    assert v["period_rel"] == 0.0
    assert abs(v["lambda_deg_diff"] - 1.0) < 1e-12 and abs(v["beta_deg_diff"] - 1.0) < 1e-12
