"""Replica validator and cross-build agreement reports.

The project accepts two replicas of a work unit when their
``period_search_out`` files agree under the rule of
validator/period_search_validator4.cpp:71-109 (period and rms within 0.1,
chi^2 within 0.5 of |(a - b) / (a + b)| / 2 on every entry, same number of
entries).  ``ps_validate_rows`` / ``ps_validate_files`` implement it in the
engine library; this module wraps them and adds an agreement report between
any number of builds (the CPU oracle, the FP64 form, the mixed form, ...):
the validator verdict of every pair, the best period index of each, and the
largest relative rms difference.

    python -m periodsearch_gb300.validate out_a out_b [out_c ...]
"""
from __future__ import annotations

import ctypes as C
import itertools
import json
import sys

import numpy as np

from . import _abi

TOL = (0.1, 0.1, 0.5)
COLUMNS = ("period", "rms", "chisq")


def _report(r: _abi.ValidateReport) -> dict:
    return {"match": bool(r.match), "entries": (r.entries_a, r.entries_b), "first_mismatch": r.first_mismatch,
            "mismatch_column": COLUMNS[r.mismatch_column] if r.mismatch_column >= 0 else None,
            "max_dev": dict(zip(COLUMNS, list(r.max_dev))), "argmax_dev": dict(zip(COLUMNS, list(r.argmax_dev))),
            "parse_error": (bool(r.parse_error_a), bool(r.parse_error_b))}


def _tol(tol):
    return None if tol is None else (C.c_double * 3)(*tol)


def validate_rows(a: np.ndarray, b: np.ndarray, tol=None) -> dict:
    """Validator verdict on two row arrays (ROW_DTYPE, as Engine.scan returns)."""
    from . import ROW_DTYPE

    a = np.ascontiguousarray(a, ROW_DTYPE)
    b = np.ascontiguousarray(b, ROW_DTYPE)
    r = _abi.ValidateReport()
    st = _abi.lib().ps_validate_rows(a.ctypes.data_as(C.POINTER(_abi.Row)), len(a),
                                     b.ctypes.data_as(C.POINTER(_abi.Row)), len(b), _tol(tol), C.byref(r))
    _abi.check(st, "ps_validate_rows")
    return _report(r)


def validate_files(path_a, path_b, tol=None) -> dict:
    """Validator verdict on two period_search_out files, read the way the
    validator reads them."""
    r = _abi.ValidateReport()
    st = _abi.lib().ps_validate_files(str(path_a).encode(), str(path_b).encode(), _tol(tol), C.byref(r))
    _abi.check(st, "ps_validate_files")
    return _report(r)


def agreement_report(builds: dict) -> dict:
    """builds: name -> row array of the same period range.  Returns the
    best period index of every build and, for every pair, the validator
    verdict, whether the best index is the same and the largest and median
    relative rms difference."""
    out = {"best_index": {k: int(np.argmin(v["rms"])) for k, v in builds.items()}, "pairs": {}}
    for (ka, a), (kb, b) in itertools.combinations(builds.items(), 2):
        rel = np.abs(a["rms"] - b["rms"]) / np.abs(b["rms"])
        v = validate_rows(a, b)
        out["pairs"][f"{ka}|{kb}"] = {
            "validator_match": v["match"], "validator_max_dev": v["max_dev"],
            "same_best_index": out["best_index"][ka] == out["best_index"][kb],
            "rms_rel_max": float(rel.max()), "rms_rel_median": float(np.median(rel))}
    return out


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) < 2:
        print(__doc__.strip().splitlines()[-1].strip())
        return 2
    ok = True
    for a, b in itertools.combinations(argv, 2):
        rep = validate_files(a, b)
        ok &= rep["match"]
        print(json.dumps({"a": a, "b": b, **rep}))
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
