"""FP64 fits spread over a thread-block cluster (evaluate_split): when a
launch has fewer FP64 fits than half (a quarter) of the fit slots, each fit
runs on a cluster of 2 (4) CTAs, every one of which sums over the points in
data order (each its share of the normal matrix), so the fits are
bit-identical to the one-CTA kernel's -- and so to the FP64 form's parity
with the CPU oracle."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIELDS = ("dev", "chisq", "period_h", "lambda_deg", "beta_deg", "dark", "totarea", "niter", "err_code")


def _path(case):
    if case == "golden":
        return GOLDEN / "period_search_in"
    if case == "c1":
        return GOLDEN / "c1" / "period_search_in"
    return GOLDEN / case / "period_search_in"


@pytest.mark.parametrize("case", ["tiny_mix", "golden", "c1"])
def test_split_fits_bit_identical(engine_lib, case):
    from periodsearch_gb300 import Engine, PS_FORM_FP64, read_input

    with Engine(read_input(_path(case)), form=PS_FORM_FP64) as eng:
        conw_r = eng.info.conw_r0
        slots = eng.info.slots
        n_max = int(eng.info.n_max)
        rng = np.random.default_rng(3)
        per = rng.integers(1, n_max + 1, size=slots + 8).astype(np.int64)
        pole = rng.integers(1, 11, size=slots + 8).astype(np.int32)
        whole = eng.fit_batch(conw_r, per, pole)                   # more fits than slots: one CTA per fit
        assert eng.timing()["cluster_size"] == 1
        for k, cs in ((slots // 4, 4), (slots // 2, 2)):
            part = eng.fit_batch(conw_r, per[:k], pole[:k])
            assert eng.timing()["cluster_size"] == cs
            for f in FIELDS:
                np.testing.assert_array_equal(part[f], whole[f][:k], err_msg=f"{case} cs={cs} {f}")


def test_split_fits_match_oracle(engine_lib, oracle):
    """Split fits of a relative-and-calibrated object against the oracle's
    fits within the FP64 policy (1e-6 relative in rms)."""
    from periodsearch_gb300 import Engine, PS_FORM_FP64, read_input

    path = _path("tiny_mix")
    ora = oracle.OracleProblem(path)
    conw_r = ora.info()["conw_r"]
    ora.setup(conw_r)
    with Engine(read_input(path), form=PS_FORM_FP64) as eng:
        per = np.repeat(np.arange(1, 4), 10).astype(np.int64)
        pole = np.tile(np.arange(1, 11), 3).astype(np.int32)
        got = eng.fit_batch(conw_r, per, pole)
        assert eng.timing()["cluster_size"] == 4
    want = np.array([ora.fit_n(int(n), int(m))["dev"] for n, m in zip(per, pole)])
    rel = np.abs(got["dev"] - want) / want
    assert np.mean(rel <= 1e-6) >= 0.85 and rel.max() <= 1e-3, rel


def test_refined_scan_with_split_refits(engine_lib):
    """The refined scan's FP64 refit runs split when its set is small; the
    refitted rows equal the FP64 scan's bit for bit."""
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input

    data = read_input(_path("c1"))
    with Engine(data, form=PS_FORM_MIXED) as eng, Engine(data, form=PS_FORM_FP64) as e64:
        conw_r = eng.info.conw_r0
        lo, hi = 24895, 24934
        rows, st = eng.scan_refined(conw_r, lo, hi, 0.001, 1)
        full = e64.scan(conw_r, lo, hi)
    b = int(st["best_index"]) - lo
    assert st["fits_refit"] >= 30
    assert rows["rms"][b] == full["rms"][b]
    assert int(np.argmin(full["rms"])) == b


def test_lit_facet_count(engine_lib):
    """ps_timing.lit_facets: the FP64 kernels' count of lit (point, facet)
    pairs.  A fraction of all pairs in the FP64 form, the same whether the
    fits run one CTA each or over 4-CTA clusters (three quarter-slot batches
    against their union), and 0 for the mixed form."""
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input

    data = read_input(_path("c1"))
    with Engine(data, form=PS_FORM_FP64) as eng:
        conw_r = eng.info.conw_r0
        q = eng.info.slots // 4
        rng = np.random.default_rng(5)
        per = rng.integers(20000, 26000, size=3 * q).astype(np.int64)
        pole = rng.integers(1, 11, size=3 * q).astype(np.int32)
        eng.fit_batch(conw_r, per, pole)
        t = eng.timing()
        assert t["cluster_size"] == 1
        frac = t["lit_facets"] / (t["evals"] * eng.info.ndata * eng.info.nfac)
        assert 0.2 < frac < 0.8
        parts = 0
        for b in range(3):
            eng.fit_batch(conw_r, per[b * q:(b + 1) * q], pole[b * q:(b + 1) * q])
            tb = eng.timing()
            assert tb["cluster_size"] == 4
            parts += tb["lit_facets"]
        assert parts == t["lit_facets"]
    with Engine(data, form=PS_FORM_MIXED) as eng:
        eng.fit_batch(eng.info.conw_r0, per[:8], pole[:8])
        assert eng.timing()["lit_facets"] == 0
