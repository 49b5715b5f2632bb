"""Parity of the CUDA engine (FP64 form) with the oracle and the reference.

Tolerances of the FP64 form (the drop-in):
* one model evaluation (alpha, beta, chi^2, facet areas): 1e-10 relative to
  the largest entry;
* a scan: the best period index identical; rms and chi^2 within 1e-6
  relative on at least 85 % of the periods and within 1e-3 on all; fitted
  period within 1e-6 relative; pole angles within 0.05 degree on the periods
  inside 1e-6.
Rounding differences (CUDA's libm is within 1-2 ulp of glibc's; FMA
contraction; summation order of parallel reductions) are far below 1e-6, but
the 50-iteration LM fit is sensitive to them: a near-tie in an accept/reject
test sends the fit down another path.  The reference shows the same
sensitivity between its own builds (tests/golden/golden134*.full): its
committed period_search_out differs from the same sources rebuilt here by up
to 1.8e-5 in rms, and its AVX2/FMA build by up to 6e-2.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, SYNTH_CASES, WU_CASES

pytestmark = pytest.mark.gpu

RTOL = 1e-6
CASES = SYNTH_CASES + WU_CASES + ["golden"]


def _path(case):
    return GOLDEN / "period_search_in" if case == "golden" else GOLDEN / case / "period_search_in"


def _ref_rows(case):
    if case == "golden":
        return np.loadtxt(GOLDEN / "golden12.full", ndmin=2)
    return np.loadtxt(GOLDEN / case / "ref.full", ndmin=2)


@pytest.fixture(scope="module")
def engines(engine_lib):
    from periodsearch_gb300 import Engine, read_input

    out = {}
    yield lambda case: out.setdefault(case, Engine(read_input(_path(case))))
    for e in out.values():
        e.close()


@pytest.mark.parametrize("case", CASES)
def test_eval_matches_oracle(engines, oracle, case):
    eng = engines(case)
    ora = oracle.OracleProblem(_path(case))
    conw_r = ora.info()["conw_r"]
    rng = np.random.default_rng(3)
    # perturb the shape coefficients by ~5 % of the log-area range that each
    # basis function spans (the unnormalised P_l^m reach 10^4 at l = 6)
    from periodsearch_gb300 import shape_tables

    inf = ora.info()
    h = eng._data.header
    _, _, dsph = shape_tables(h["nrows"], h["lmax"], h["mmax"])
    span = np.abs(dsph).max(axis=0)
    for n, pole in [(1, 1), (2, 6), (1, 9)]:
        cg = ora.initial_cg(n, pole)
        for jitter in (0.0, 0.05):
            c = cg.copy()
            c[: eng.info.ncoef] += jitter * rng.standard_normal(eng.info.ncoef) / span / np.sqrt(inf["ncoef"])
            a_g, b_g, x_g, ar_g = eng.eval(conw_r, c)
            a_o, b_o, x_o, ar_o = ora.eval(c)
            assert abs(x_g - x_o) <= 1e-10 * abs(x_o)
            assert np.abs(a_g - a_o).max() <= 1e-10 * np.abs(a_o).max()
            assert np.abs(b_g - b_o).max() <= 1e-10 * np.abs(b_o).max()
            assert np.abs(ar_g - ar_o).max() <= 1e-12 * np.abs(ar_o).max()
            assert np.array_equal(a_g, a_g.T)


@pytest.mark.parametrize("case", ["tiny_cal", "tiny_rel", "tiny_mix", "tiny_stop"])
def test_fits_match_oracle(engines, oracle, case):
    eng = engines(case)
    ora = oracle.OracleProblem(_path(case))
    conw_r = ora.info()["conw_r"]
    periods = np.repeat(np.arange(1, 5), 10)
    poles = np.tile(np.arange(1, 11), 4)
    got = eng.fit_batch(conw_r, periods, poles)
    for f, n, m in zip(got, periods, poles):
        o = ora.fit_n(int(n), int(m))
        assert f["dev"] == pytest.approx(o["dev"], rel=RTOL)
        assert f["chisq"] == pytest.approx(o["chisq"], rel=RTOL)
        assert f["period_h"] == pytest.approx(24 * o["prd"], rel=RTOL)
        assert f["lambda_deg"] == pytest.approx(o["la"], abs=1e-3)
        assert f["beta_deg"] == pytest.approx(o["be"], abs=1e-3)
        assert f["totarea"] == pytest.approx(o["totarea"], rel=1e-8)
        assert f["dark"] == pytest.approx(o["dark"], rel=1e-4, abs=1e-9)


FRAC_WITHIN = 0.85   # periods whose rms agrees to RTOL
MAX_REL = 1e-3       # every period


def _check_rows(got, ref):
    """The scan policy of the FP64 form (module docstring)."""
    assert got.shape[0] == ref.shape[0]
    g = np.array([list(r) for r in got])
    rel = np.abs(g[:, 1] - ref[:, 1]) / ref[:, 1]
    close = rel <= RTOL
    n_far = int((~close).sum())
    assert n_far <= max(1, int((1 - FRAC_WITHIN) * len(rel))), (n_far, rel)
    assert rel.max() <= MAX_REL
    assert int(np.argmin(g[:, 1])) == int(np.argmin(ref[:, 1]))
    c = close
    np.testing.assert_allclose(g[c, 0], ref[c, 0], rtol=RTOL)        # period
    np.testing.assert_allclose(g[c, 2], ref[c, 2], rtol=2 * RTOL)    # chi^2
    # the pole is the flattest direction of chi^2: angles agree to 0.05 deg
    # where rms agrees to 1e-6 (the output prints whole degrees)
    np.testing.assert_allclose(g[c, 4], ref[c, 4], atol=0.05)        # lambda
    np.testing.assert_allclose(g[c, 5], ref[c, 5], atol=0.05)        # beta
    # dark-facet % is a property of the poorly constrained shape; the output
    # prints it to 0.1
    np.testing.assert_allclose(g[c, 3], ref[c, 3], rtol=1e-3, atol=1e-3)
    return rel


@pytest.mark.parametrize("case", CASES)
def test_scan_matches_reference_binary(engines, oracle, case):
    eng = engines(case)
    ref = _ref_rows(case)
    if case == "golden":
        conw_r = oracle.OracleProblem(_path(case)).info()["conw_r"]
        got = eng.scan(conw_r, 1, 12)
    else:
        conw_r, new_conw = eng.precalc_conw()
        # row 1 of the reference carries conw_r * escl^2 of its pre-pass
        assert conw_r * eng.info.escl * eng.info.escl == ref[0][3]
        got = eng.scan(conw_r, 1, int(eng.info.n_max))
    _check_rows(got, ref)


def test_golden134_scan_policy(engines, oracle):
    """All 134 rows of the reference's golden scan (N = 500 relative points,
    L = 6, 288 facets) against the reference built from the same sources."""
    eng = engines("golden")
    conw_r, new_conw = eng.precalc_conw()
    assert new_conw == 1 and conw_r == oracle.OracleProblem(_path("golden")).info()["conw_r"]
    got = eng.scan(conw_r, 1, 134)
    rel = _check_rows(got, np.loadtxt(GOLDEN / "golden134.full", ndmin=2))
    print("golden134: within 1e-6 %.3f, max %.2e" % ((rel <= RTOL).mean(), rel.max()))


def test_golden_precalc_conw(engines, oracle):
    eng = engines("golden")
    conw_r, new_conw = eng.precalc_conw()
    assert new_conw == 1
    assert conw_r == oracle.OracleProblem(_path("golden")).info()["conw_r"]
    t = eng.timing()
    assert t["fits"] == 100 and t["evals"] == 100 * 51


def test_run_files_end_to_end_with_resume(engine_lib, tmp_path):
    """The file drop-in: fresh run, then a resumed run from a checkpoint."""
    import shutil

    from periodsearch_gb300 import run_files

    case = "tiny_mix"
    ref = _ref_rows(case)
    shutil.copy(_path(case), tmp_path / "period_search_in")
    run_files(tmp_path / "period_search_in", tmp_path / "period_search_out", tmp_path / "period_search_state",
              checkpoint_rows=5)
    got = np.loadtxt(tmp_path / "period_search_out", ndmin=2)
    np.testing.assert_allclose(got[:, 1], ref[:, 1], rtol=2e-6, atol=1e-6)
    assert (tmp_path / "period_search_state").read_text().strip() == str(len(ref))
    # resume after row 5: keep 5 rows and a state file saying 5
    lines = (tmp_path / "period_search_out").read_text().splitlines(keepends=True)
    (tmp_path / "period_search_out").write_text("".join(lines[:5]))
    (tmp_path / "period_search_state").write_text("5")
    run_files(tmp_path / "period_search_in", tmp_path / "period_search_out", tmp_path / "period_search_state",
              checkpoint_rows=4)
    assert (tmp_path / "period_search_out").read_text().splitlines(keepends=True) == lines


def test_bad_arguments(engines):
    from periodsearch_gb300 import EngineError, _abi

    eng = engines("tiny_cal")
    with pytest.raises(EngineError) as e:
        eng.scan(1.0, 3, 2)
    assert e.value.status == _abi.PS_ERR_ARG
    with pytest.raises(EngineError) as e:
        eng.fit_batch(1.0, [1], [11])
    assert e.value.status == _abi.PS_ERR_ARG
