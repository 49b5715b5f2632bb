"""The largest per-object sizes of a multi-object run (Ndata 5000: 4000
sparse calibrated points in blocks of 1000 plus one relative lightcurve of
1000 points, the reference's POINTS_MAX): both forms against the oracle per
evaluation, and the mixed form's fits against the FP64 form's."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(tmp_path_factory):
    from periodsearch_gb300 import synth

    cfg = synth.SynthConfig(name="big", n_sparse=4000, n_dense=1, dense_points=1000, sparse_block=1000,
                            n_periods=60)
    path = tmp_path_factory.mktemp("big") / "period_search_in"
    synth.write_object(path, cfg, seed=51)
    return path


def test_large_object_eval(engine_lib, oracle, big):
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input

    ora = oracle.OracleProblem(big)
    assert ora.info()["ndata"] == 5000
    conw_r = ora.info()["conw_r"]
    data = read_input(big)
    for form, tol in ((PS_FORM_FP64, (1e-10, 1e-10, 1e-10)), (PS_FORM_MIXED, (1e-5, 1e-4, 1e-3))):
        with Engine(data, form=form) as eng:
            cg = ora.initial_cg(3, 7)
            a_g, b_g, x_g, _ = eng.eval(conw_r, cg)
            a_o, b_o, x_o, _ = ora.eval(cg)
            assert abs(x_g - x_o) <= tol[0] * abs(x_o)
            assert np.abs(a_g - a_o).max() <= tol[1] * np.abs(a_o).max()
            assert np.abs(b_g - b_o).max() <= tol[2] * np.abs(b_o).max()


def test_large_object_fits(engine_lib, big):
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, read_input

    data = read_input(big)
    per = np.repeat([5, 30], 10)
    pole = np.tile(np.arange(1, 11), 2)
    with Engine(data, form=PS_FORM_FP64) as e64:
        conw_r = e64.info.conw_r0
        ref = e64.fit_batch(conw_r, per, pole)
    with Engine(data, form=PS_FORM_MIXED) as eng:
        assert eng.info.tensor_cores == 1
        got = eng.fit_batch(conw_r, per, pole)
    assert np.isfinite(got["dev"]).all() and (got["err_code"] == 0).all()
    rel = (got["dev"] - ref["dev"]) / ref["dev"]
    assert rel.max() <= 5e-2 and rel.min() >= -15e-2 and np.median(np.abs(rel)) <= 5e-3
