"""The learned early stop on the GPU: the training kernels' gradient against
the numpy reference, training, the in-kernel predictor, and the learned scan
against the full scan (same best period, fewer evaluations)."""
from __future__ import annotations

import numpy as np
import pytest

import mlp_reference as ref
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _data(seed=0, n=300):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, ref.F)).astype(np.float32)
    y = (np.tanh(x[:, 0]) * 0.5 - 0.3 * x[:, 4] + 0.05 * rng.normal(size=n)).astype(np.float32)
    return x, y


def test_gpu_gradient_matches_reference(engine_lib):
    from periodsearch_gb300 import learned

    x, y = _data()
    P = learned.init_weights(x, y, seed=3)
    loss_g, g_g = learned.grad(P, x, y)
    loss_r, g_r = ref.loss_grad(P, x, y)
    assert abs(loss_g - loss_r) <= 1e-4 * loss_r
    sl = slice(ref.O_W1, ref.O_B3 + 1)
    assert np.abs(g_g[sl] - g_r[sl]).max() <= 1e-4 * np.abs(g_r[sl]).max()


def test_gpu_predict_matches_reference(engine_lib):
    from periodsearch_gb300 import learned

    x, y = _data(1)
    P = learned.init_weights(x, y, seed=5)
    np.testing.assert_allclose(learned.predict(P, x), ref.predict(P, x), rtol=1e-4, atol=1e-5)


def test_gpu_training_reduces_loss(engine_lib):
    from periodsearch_gb300 import learned

    x, y = _data(2, 2048)
    P, hist = learned.train(x, y, epochs=30, batch=256, lr=3e-3, seed=1)
    assert hist[-1] < 0.5 * hist[0]
    pred = learned.predict(P, x)
    assert np.sqrt(np.mean((pred - y) ** 2)) < 0.6 * np.std(y)


def test_in_kernel_predictor_matches_host(engine_lib):
    """The screening kernel's prediction equals the host-side predictor on
    the same features (trajectory records hold the features)."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input

    path = GOLDEN / "c0_12" / "period_search_in"
    with Engine(read_input(path), form=PS_FORM_MIXED) as eng:
        conw_r = eng.info.conw_r0
        traj = learned.trajectories(eng, conw_r, 1, 3)
        x, y, dev4, _ = learned.samples(traj)
        P = learned.init_weights(x, y, seed=7)
        scr = eng.screen(conw_r, 1, 3, P)
        assert (scr["screened"] == 1).all() and (scr["niter"] == 4).all()
        assert len(dev4) == 30
        np.testing.assert_allclose(scr["dev"], dev4, rtol=1e-6)
        pred_host = dev4 * np.exp(learned.predict(P, x))
        np.testing.assert_allclose(scr["pred_dev"], pred_host, rtol=1e-4)
        rows, st = eng.scan_learned(conw_r, 1, 3, P, margin=1e9, region_rel=0.0, region_halfwidth=0,
                                    refit_rel=0.0, refit_halfwidth=0)
        assert st["fits_screened_out"] == 0 and st["fits_completed"] == 30 and st["fits_refit"] == 10
        full = eng.scan(conw_r, 1, 3)
        b = int(st["best_index"]) - 1
        others = [n for n in range(3) if n != b]
        np.testing.assert_array_equal(rows["rms"][others], full["rms"][others])   # mixed form, same fits


def test_learned_cascade_bookkeeping(engine_lib):
    """top_k poles per period at stage 2; region and refit widths count as
    documented; rows never come from a fit that did not run in full."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input

    path = GOLDEN / "c0_12" / "period_search_in"
    with Engine(read_input(path), form=PS_FORM_MIXED) as eng:
        conw_r = eng.info.conw_r0
        P = learned.zero_predictor()
        rows, st = eng.scan_learned(conw_r, 1, 12, P, top_k=2, region_rel=0.0, region_halfwidth=0,
                                    refit_rel=0.0, refit_halfwidth=0)
        assert st["fits_total"] == 120 and st["region_periods"] == 1
        assert st["fits_completed"] == 12 * 2 + 8 and st["fits_screened_out"] == 120 - st["fits_completed"]
        assert st["fits_refit"] == 10
        full = eng.scan(conw_r, 1, 12)
        assert (rows["rms"] >= full["rms"] * (1 - 5e-2)).all()     # a subset of poles: never much better
        assert np.isfinite(rows["rms"]).all()


def test_learned_scan_keeps_best_period(engine_lib, tmp_path):
    """On a synthetic object the learned scan (screen, complete, FP64 refit)
    reports the same best period as the full FP64 scan of the same window,
    with FP64 values there, and runs fewer model evaluations."""
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, learned, read_input, synth

    P, meta = learned.load_default()
    if P is None:
        pytest.skip("no trained predictor committed")
    obj = synth.write_object(tmp_path / "period_search_in", "c0", seed=901)
    data = read_input(tmp_path / "period_search_in")
    with Engine(data, form=PS_FORM_FP64) as full:
        conw_r, _ = full.precalc_conw()
        n_t = int(round((full.info.freq_start - 1 / obj.truth["period_h"]) / full.info.freq_step)) + 1
        lo, hi = max(1, n_t - 24), min(int(full.info.n_max), n_t + 23)
        rows_full = full.scan(conw_r, lo, hi)
        evals_full = full.timing()["evals"]
    with Engine(data, form=PS_FORM_MIXED) as eng:
        rows, st = eng.scan_learned(conw_r, lo, hi, P, **meta["cascade"])
    b_full, b = int(np.argmin(rows_full["rms"])), int(np.argmin(rows["rms"]))
    assert b == b_full
    assert rows["rms"][b] == pytest.approx(rows_full["rms"][b_full], rel=1e-9)
    assert st["evals"] < 0.7 * evals_full
    assert st["fits_screened_out"] > 0.5 * st["fits_total"]


def test_trained_predictor_beats_no_network(engine_lib, tmp_path):
    """On a fresh synthetic object the committed network predicts the final
    rms better than the rms after four iterations (the zero predictor)."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input, synth

    P, _ = learned.load_default()
    if P is None:
        pytest.skip("no trained predictor committed")
    obj = synth.write_object(tmp_path / "period_search_in", "c1", seed=907)
    with Engine(read_input(tmp_path / "period_search_in"), form=PS_FORM_MIXED) as eng:
        conw_r, _ = eng.precalc_conw()
        n_t = int(round((eng.info.freq_start - 1 / obj.truth["period_h"]) / eng.info.freq_step)) + 1
        traj = learned.trajectories(eng, conw_r, max(1, n_t - 15), n_t + 16)
    x, y, _, _ = learned.samples(traj)
    err_net = np.sqrt(np.mean((learned.predict(P, x) - y) ** 2))
    err_zero = np.sqrt(np.mean(y ** 2))
    assert err_net < 0.8 * err_zero, (err_net, err_zero)
