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


def _small_population(tmp_path, seeds_and_sizes):
    """Objects of one small shape (L = 3, 72 facets, 8 LM iterations) that
    the oracle fits in milliseconds, with uneven Ndata: sparse calibrated
    blocks, some with dense relative lightcurves."""
    from periodsearch_gb300 import synth

    paths = []
    for k, (seed, n_sparse, n_dense) in enumerate(seeds_and_sizes):
        cfg = synth.SynthConfig(name=f"p{k}", n_sparse=n_sparse, n_dense=n_dense, dense_points=20, lmax=3, nrows=3,
                                n_periods=14, stop_condition=8, sparse_block=60)
        path = tmp_path / f"pop{k}" / "period_search_in"
        path.parent.mkdir()
        synth.write_object(path, cfg, seed=seed)
        paths.append(path)
    return paths


@pytest.mark.parametrize("form_name", ["fp64", "mixed"])
def test_pack_matches_oracle(engine_lib, oracle, tmp_path, form_name):
    """Packed fits of objects with uneven Ndata (30 to 190 points, sparse-only
    and dense+sparse) against the CPU oracle's fits of the same (object,
    period, pole) units: the FP64 form within the FP64 scan policy (1e-6
    relative on at least 85 % of the fits, 1e-3 on all), the mixed form
    within its scan bounds (at most 5e-2 above and 15e-2 below the oracle's
    rms, median within 5e-3)."""
    from periodsearch_gb300 import Engine, Pack, PS_FORM_FP64, PS_FORM_MIXED, read_input

    form = PS_FORM_FP64 if form_name == "fp64" else PS_FORM_MIXED
    paths = _small_population(tmp_path, [(31, 30, 0), (32, 190, 0), (33, 70, 1), (34, 120, 2), (35, 50, 1)])
    engines = [Engine(read_input(p), form=form) for p in paths]
    try:
        conw = [e.info.conw_r0 for e in engines]
        rng = np.random.default_rng(9)
        obj, per, pole = [], [], []
        for o, e in enumerate(engines):
            for p in rng.choice(int(e.info.n_max), size=3, replace=False) + 1:
                for q in rng.choice(10, size=3, replace=False) + 1:
                    obj.append(o)
                    per.append(int(p))
                    pole.append(int(q))
        obj, per, pole = np.array(obj), np.array(per), np.array(pole)
        with Pack(engines, form=form) as pk:
            got = pk.fit(conw, obj, per, pole)
        want = np.zeros(len(obj))
        for o, path in enumerate(paths):
            ora = oracle.OracleProblem(path)
            assert ora.info()["conw_r"] == conw[o]
            ora.setup(conw[o])
            for i in np.flatnonzero(obj == o):
                want[i] = ora.fit_n(int(per[i]), int(pole[i]))["dev"]
        rel = (got["dev"] - want) / want
        if form == PS_FORM_FP64:
            assert np.mean(np.abs(rel) <= 1e-6) >= 0.85, rel
            assert np.abs(rel).max() <= 1e-3, rel
        else:
            assert rel.max() <= 5e-2 and rel.min() >= -15e-2, rel
            assert np.median(np.abs(rel)) <= 5e-3, rel
    finally:
        for e in engines:
            e.close()
