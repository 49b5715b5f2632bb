"""The autotuner measures every kernel configuration the object admits and
keeps the fastest; the FP64 form's results do not depend on the
configuration (sums run in data order whatever the tile size), the mixed
form's stay within its tolerance."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c0(tmp_path_factory):
    from periodsearch_gb300 import read_input, synth

    path = tmp_path_factory.mktemp("tune") / "period_search_in"
    synth.write_object(path, "c0", seed=31)
    return read_input(path)


def test_autotune_fp64_keeps_results(engine_lib, c0):
    from periodsearch_gb300 import Engine, PS_FORM_FP64

    with Engine(c0, form=PS_FORM_FP64) as eng:
        conw_r, _ = eng.precalc_conw()
        before = eng.scan(conw_r, 100, 103)
        rep = eng.autotune(conw_r, sample_iters=3)
        c = rep["candidates"]
        print("fp64 autotune", c, "chosen", rep["chosen"])
        assert len(c) >= 2 and {x["tile_points"] for x in c} >= {16, 32}
        assert c[rep["chosen"]]["fits_per_s"] == max(x["fits_per_s"] for x in c)
        after = eng.scan(conw_r, 100, 103)
    np.testing.assert_array_equal(before, after)


def test_autotune_mixed(engine_lib, c0):
    from periodsearch_gb300 import Engine, PS_FORM_MIXED

    with Engine(c0, form=PS_FORM_MIXED) as eng:
        conw_r, _ = eng.precalc_conw()
        before = eng.scan(conw_r, 100, 111)
        rep = eng.autotune(conw_r)
        c = rep["candidates"]
        print("mixed autotune", c, "chosen", rep["chosen"])
        assert {x["basis"] for x in c} == {"tensor", "shared", "l2"}
        best = c[rep["chosen"]]
        assert best["fits_per_s"] == max(x["fits_per_s"] for x in c)
        assert eng.info.tensor_cores == (best["basis"] == "tensor")
        assert eng.info.tile_points == best["tile_points"]
        after = eng.scan(conw_r, 100, 111)
    rel = np.abs(after["rms"] - before["rms"]) / before["rms"]
    assert rel.max() <= 5e-2 and np.median(rel) <= 5e-3
