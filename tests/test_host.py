"""Host-side logic of the engine, without a GPU: the C ABI exports, the
period_search_in reader, the per-object tables against the oracle, the row
format, the synthetic generator and the error paths."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, SYNTH_CASES


def _declared_functions():
    text = (ROOT / "include" / "ps_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ps_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_lib):
    from periodsearch_gb300 import _abi

    names = _declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(engine_lib, n), n
        assert n in _abi.SIGNATURES, f"{n} has no ctypes signature"
    assert engine_lib.ps_abi_version() == 2


def test_reader_matches_oracle(engine_lib, oracle):
    from periodsearch_gb300 import read_input

    for case in ["", *SYNTH_CASES]:
        path = (GOLDEN / case / "period_search_in") if case else (GOLDEN / "period_search_in")
        d = read_input(path)
        o = oracle.OracleProblem(path).info()
        assert d.ndata == o["ndata"]
        assert int(d.lc_points.sum()) == d.ndata
    g = read_input(GOLDEN / "period_search_in")
    assert g.header["lmax"] == 6 and g.header["nrows"] == 6 and g.header["stop_condition"] == 50
    assert list(g.lc_calibrated) == [0] and list(g.lc_weight) == [1.0]
    assert g.jd[0] == 2450874.015183 and g.sun[0, 0] == 2.305127


@pytest.mark.parametrize("nrows,lmax", [(6, 6), (8, 8), (3, 2), (6, 3)])
def test_shape_tables_match_oracle_bitwise(engine_lib, oracle, nrows, lmax):
    from periodsearch_gb300 import shape_tables

    nor, darea, dsph = shape_tables(nrows, lmax, lmax)
    L = oracle.lib()
    nf, nc = dsph.shape
    onor, oarea, odsph = np.zeros(nf * 3), np.zeros(nf), np.zeros(nf * nc)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    L.pso_shape_export.argtypes = [C.c_int] * 3 + [C.POINTER(C.c_int)] + [C.POINTER(C.c_double)] * 5
    L.pso_shape_export(nrows, lmax, lmax, None, None, None, dp(onor), dp(oarea), dp(odsph))
    assert np.array_equal(nor.ravel(), onor)
    assert np.array_equal(darea, oarea)
    assert np.array_equal(dsph.ravel(), odsph)


def test_row_format_matches_reference_text(engine_lib):
    from periodsearch_gb300 import format_row, ROW_DTYPE

    full = np.loadtxt(GOLDEN / "golden12.full", ndmin=2)
    text = (GOLDEN / "period_search_out").read_text().splitlines(keepends=True)
    for i, vals in enumerate(full):
        r = np.array(tuple(vals), ROW_DTYPE)
        assert format_row(r) == text[i]


def test_synthetic_generator_is_seeded(engine_lib):
    from periodsearch_gb300 import synth

    a = synth.make_object("tiny_mix").text
    b = synth.make_object("tiny_mix").text
    c = synth.make_object("tiny_mix", seed=7).text
    assert a == b and a != c
    assert (GOLDEN / "tiny_mix" / "period_search_in").read_text() == a


def test_reader_errors(engine_lib, tmp_path):
    from periodsearch_gb300 import EngineError, read_input, _abi

    with pytest.raises(EngineError) as e:
        read_input(tmp_path / "missing")
    assert e.value.status == _abi.PS_ERR_IO
    text = (GOLDEN / "tiny_cal" / "period_search_in").read_text().split("\n")
    (tmp_path / "trunc").write_text("\n".join(text[:30]))
    with pytest.raises(EngineError) as e:
        read_input(tmp_path / "trunc")
    assert e.value.status == _abi.PS_ERR_IO
    big = text[:15] + ["1001 1"]
    (tmp_path / "big").write_text("\n".join(big))
    with pytest.raises(EngineError) as e:
        read_input(tmp_path / "big")
    assert e.value.status == _abi.PS_ERR_LIMIT


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_prepare_without_device_fails_loudly(engine_lib):
    from periodsearch_gb300 import Engine, EngineError, read_input, _abi

    with pytest.raises(EngineError) as e:
        Engine(read_input(GOLDEN / "tiny_cal" / "period_search_in"))
    assert e.value.status == _abi.PS_ERR_NO_DEVICE


def test_bench_workload_fixture_is_the_generator_output():
    """The benchmark's committed c1 input is exactly what the seeded
    generator writes (tests/golden/make_fixtures.py --only-bench-inputs)."""
    import json

    from periodsearch_gb300 import synth

    obj = synth.make_object("c1")
    d = GOLDEN / "c1"
    assert (d / "period_search_in").read_text() == obj.text
    assert json.loads((d / "truth.json").read_text()) == obj.truth
