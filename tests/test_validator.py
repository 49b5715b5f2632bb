"""The replica validator (validator/period_search_validator4.cpp:23-109)
on the reference's own output and on planted differences.  Host logic only:
runs without a GPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

OUT = GOLDEN / "period_search_out"


@pytest.fixture(scope="module")
def val(engine_lib):
    from periodsearch_gb300 import validate

    return validate


def _rows(path):
    from periodsearch_gb300 import ROW_DTYPE

    a = np.loadtxt(path, ndmin=2)
    r = np.zeros(len(a), ROW_DTYPE)
    for k, name in enumerate(ROW_DTYPE.names):
        r[name] = a[:, k]
    return r


def _write(path, rows, newline=True):
    text = "\n".join("%.8f  %.6f  %.6f %4.1f %4.0f %4.0f" % tuple(r) for r in rows)
    path.write_text(text + ("\n" if newline else ""))
    return path


def test_reference_output_validates_against_itself(val):
    rep = val.validate_files(OUT, OUT)
    assert rep["match"] and rep["first_mismatch"] == -1
    # the end-of-file read repeats the last row: 134 rows, 135 entries
    assert rep["entries"] == (135, 135)
    assert all(v == 0 for v in rep["max_dev"].values())


def test_reference_builds_agree(val, tmp_path):
    """The reference's AVX2/FMA build (full-precision capture of the same
    work unit) and the golden output are accepted as replicas."""
    fma = np.loadtxt(GOLDEN / "golden134_fma.full", ndmin=2)
    p = _write(tmp_path / "fma_out", fma)
    rep = val.validate_files(OUT, p)
    assert rep["match"]
    a, b = np.loadtxt(OUT)[:, 1], np.loadtxt(p)[:, 1]     # the written (rounded) values
    rel = np.abs(a - b) / np.abs(a + b) / 2
    assert rep["max_dev"]["rms"] == pytest.approx(rel.max(), rel=1e-5, abs=1e-9)


def test_planted_rms_difference_fails_at_its_row(val, tmp_path):
    ref = np.loadtxt(OUT)
    bad = ref.copy()
    bad[9, 1] *= 2.0            # |(a - 2a) / 3a| / 2 = 1/6 > 0.1
    rep = val.validate_files(OUT, _write(tmp_path / "bad", bad))
    assert not rep["match"] and rep["first_mismatch"] == 9 and rep["mismatch_column"] == "rms"
    assert rep["max_dev"]["rms"] == pytest.approx(1 / 6, rel=1e-5)
    assert rep["argmax_dev"]["rms"] == 9
    ok = ref.copy()
    ok[9, 1] *= 1.4             # 0.4 / 2.4 / 2 = 0.083 <= 0.1
    assert val.validate_files(OUT, _write(tmp_path / "ok", ok))["match"]


def test_chisq_rule_only_rejects_sign_changes(val, tmp_path):
    """|(a - b) / (a + b)| / 2 < 0.5 for any two positive values: the chi^2
    column rejects only a sign change (or zero sum)."""
    ref = np.loadtxt(OUT)
    big = ref.copy()
    big[3, 2] *= 1e6
    assert val.validate_files(OUT, _write(tmp_path / "big", big))["match"]
    neg = ref.copy()
    neg[5, 2] = -neg[5, 2]
    rep = val.validate_files(OUT, _write(tmp_path / "neg", neg))
    assert not rep["match"] and rep["first_mismatch"] == 5 and rep["mismatch_column"] == "chisq"


def test_period_column(val, tmp_path):
    ref = np.loadtxt(OUT)
    bad = ref.copy()
    bad[100, 0] = bad[100, 0] * 3       # 2/4/2 = 0.25 > 0.1
    rep = val.validate_files(OUT, _write(tmp_path / "bad", bad))
    assert rep["first_mismatch"] == 100 and rep["mismatch_column"] == "period"


def test_reader_rules(val, tmp_path):
    ref = np.loadtxt(OUT)
    # no trailing newline: no repeated entry, and the counts then differ
    p = _write(tmp_path / "nonl", ref, newline=False)
    rep = val.validate_files(OUT, p)
    assert rep["entries"] == (135, 134) and not rep["match"] and rep["first_mismatch"] == -1
    # fewer rows
    rep = val.validate_files(OUT, _write(tmp_path / "short", ref[:-1]))
    assert not rep["match"] and rep["entries"] == (135, 134)
    # a NaN rms or a partial entry rejects the file
    text = OUT.read_text().splitlines()
    (tmp_path / "nan").write_text("\n".join(text[:5] + [text[5].replace("0.1", "nan", 1)] + text[6:]) + "\n")
    rep = val.validate_files(OUT, tmp_path / "nan")
    assert rep["parse_error"] == (False, True) and not rep["match"]
    (tmp_path / "part").write_text("\n".join(text[:7] + [" ".join(text[7].split()[:4])] + text[8:]) + "\n")
    assert val.validate_files(tmp_path / "part", OUT)["parse_error"] == (True, False)
    (tmp_path / "empty").write_text("")
    assert val.validate_files(tmp_path / "empty", tmp_path / "empty")["parse_error"] == (True, True)
    from periodsearch_gb300 import EngineError

    with pytest.raises(EngineError):
        val.validate_files(OUT, tmp_path / "missing")


def test_rows_api_and_agreement_report(val):
    a = _rows(OUT)
    b = a.copy()
    b["rms"][40] *= 1.01
    b["rms"][41] *= 0.5     # 0.5 / 1.5 / 2 = 0.167
    rep = val.validate_rows(a, a)
    assert rep["match"] and rep["entries"] == (134, 134)
    rep = val.validate_rows(a, b)
    assert not rep["match"] and rep["first_mismatch"] == 41
    assert not val.validate_rows(a[:0], a[:0])["match"]         # no entries never match
    tol = val.validate_rows(a, b, tol=(0.1, 0.2, 0.5))
    assert tol["match"]
    rpt = val.agreement_report({"golden": a, "other": b})
    pair = rpt["pairs"]["golden|other"]
    assert not pair["validator_match"] and pair["rms_rel_max"] == pytest.approx(1.0)
    assert pair["same_best_index"] == (rpt["best_index"]["golden"] == rpt["best_index"]["other"])


def test_cli(val, tmp_path, capsys):
    assert val.main([str(OUT), str(OUT)]) == 0
    ref = np.loadtxt(OUT)
    ref[0, 1] *= 3
    assert val.main([str(OUT), str(_write(tmp_path / "x", ref))]) == 1
