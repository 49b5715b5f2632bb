"""Multi-object packing: fits of several objects (uneven Ndata) in one
persistent launch give the same results as each object's own launch, in
both forms; objects with other shape tables are refused."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _objects(tmp_path, specs):
    from periodsearch_gb300 import read_input, synth

    out = []
    for k, (cfg, seed) in enumerate(specs):
        path = tmp_path / f"obj{k}" / "period_search_in"
        path.parent.mkdir()
        synth.write_object(path, cfg, seed=seed)
        out.append(read_input(path))
    return out


@pytest.mark.parametrize("form_name", ["fp64", "mixed"])
def test_pack_matches_single_object_launches(engine_lib, tmp_path, form_name):
    from periodsearch_gb300 import Engine, Pack, PS_FORM_FP64, PS_FORM_MIXED

    form = PS_FORM_FP64 if form_name == "fp64" else PS_FORM_MIXED
    data = _objects(tmp_path, [("c0", 11), ("c1", 12), ("c0", 13)])
    engines = [Engine(d, form=form) for d in data]
    try:
        conw = [e.precalc_conw()[0] for e in engines]
        rng = np.random.default_rng(5)
        obj, per, pole = [], [], []
        for o, e in enumerate(engines):
            n = rng.choice(int(e.info.n_max), size=6, replace=False) + 1
            for p in n:
                for q in (1, 4, 7, 10):
                    obj.append(o)
                    per.append(int(p))
                    pole.append(q)
        perm = rng.permutation(len(obj))
        obj, per, pole = np.array(obj)[perm], np.array(per)[perm], np.array(pole)[perm]
        with Pack(engines, form=form) as pk:
            got = pk.fit(conw, obj, per, pole)
            t = pk.timing()
        assert t["fits"] == len(obj) and t["launches"] == 1
        for o, e in enumerate(engines):
            sel = obj == o
            ref = e.fit_batch(conw[o], per[sel], pole[sel])
            for k in ("dev", "chisq", "period_h", "lambda_deg", "beta_deg", "dark", "totarea"):
                np.testing.assert_array_equal(got[k][sel], ref[k], err_msg=f"object {o} {k}")
            np.testing.assert_array_equal(got["niter"][sel], ref["niter"])
    finally:
        for e in engines:
            e.close()


def test_pack_refuses_other_shape_tables(engine_lib, tmp_path):
    from periodsearch_gb300 import Engine, EngineError, Pack, PS_FORM_FP64, read_input

    data = _objects(tmp_path, [("c0", 21)])
    a = Engine(data[0], form=PS_FORM_FP64)
    b = Engine(read_input(GOLDEN / "tiny_cal" / "period_search_in"), form=PS_FORM_FP64)
    try:
        with pytest.raises(EngineError):
            Pack([a, b], form=PS_FORM_FP64)
    finally:
        a.close()
        b.close()
