"""The learned early stop on the GPU: the training kernels' gradient against
the numpy reference, training, the in-kernel predictor, resumed fits against
uninterrupted ones, the learned scan against the full scan and against its
replay on recorded trajectories, and what the trained network gains over the
same cascade without it."""
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
    the same features (trajectory records hold the features after the
    screening iterations)."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input

    path = GOLDEN / "c0_12" / "period_search_in"
    with Engine(read_input(path), form=PS_FORM_MIXED) as eng:
        conw_r = eng.info.conw_r0
        for k in (4, 8):
            traj = learned.trajectories(eng, conw_r, 1, 3, k)
            x, y, devk, _ = learned.samples(traj)
            P = learned.init_weights(x, y, seed=7)
            scr = eng.screen(conw_r, 1, 3, P, k)
            assert (scr["screened"] == 1).all() and (scr["niter"] == k).all()
            assert len(devk) == 30
            np.testing.assert_allclose(scr["dev"], devk, rtol=1e-6)
            pred_host = devk * np.exp(learned.predict(P, x))
            np.testing.assert_allclose(scr["pred_dev"], pred_host, rtol=1e-4)


def test_resumed_fits_equal_uninterrupted(engine_lib):
    """Fits stopped after the screening iterations and resumed from their
    saved LM state end exactly as the uninterrupted fits: with a margin that
    completes every period, the learned scan's rows outside the FP64 refit
    are bit-identical to the full mixed scan's."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input

    path = GOLDEN / "c0_12" / "period_search_in"
    with Engine(read_input(path), form=PS_FORM_MIXED) as eng:
        conw_r = eng.info.conw_r0
        P = learned.zero_predictor()
        rows, st = eng.scan_learned(conw_r, 1, 12, P, screen_iters=8, margin=10.0, refit_rel=0.0,
                                    refit_halfwidth=0, fill_refit_waves=0)
        assert st["fits_completed"] == 120 and st["fits_screened_out"] == 0 and st["region_periods"] == 12
        assert st["fits_refit"] == 10 and st["refit_rounds"] == 1
        full = eng.scan(conw_r, 1, 12)
        b = int(st["best_index"]) - 1
        others = [n for n in range(12) if n != b]
        np.testing.assert_array_equal(rows["rms"][others], full["rms"][others])
        np.testing.assert_array_equal(rows["period_h"][others], full["period_h"][others])


def test_learned_scan_follows_its_replay(engine_lib):
    """The learned scan's decisions (which periods are completed, the best
    row) are those that replay_cascade derives from the same fits' recorded
    trajectories, for a network and for the zero predictor."""
    from periodsearch_gb300 import Engine, PS_FORM_MIXED, learned, read_input, synth

    o = synth.make_object("c1", seed=931)
    with Engine(_engine_input(o), form=PS_FORM_MIXED) as eng:
        conw_r = eng.info.conw_r0
        nt = int(round((eng.info.freq_start - 1 / o.truth["period_h"]) / eng.info.freq_step)) + 1
        lo, hi = nt - 30, nt + 29
        traj = learned.trajectories(eng, conw_r, lo, hi, 8)
        x, y, _, _ = learned.samples(traj)
        P, _ = learned.train(x, y, epochs=20, seed=3)
        for W in (P, learned.zero_predictor()):
            rows, st = eng.scan_learned(conw_r, lo, hi, W, screen_iters=8, margin=0.01, batch_periods=6,
                                        refit_rel=0.0, refit_halfwidth=0, fill_refit_waves=0)
            devk = traj[:, 10].astype(np.float64)
            pred = eng.screen(conw_r, lo, hi, W, 8)["pred_dev"]      # the scan's own screening predictions
            np.testing.assert_allclose(pred, devk * np.exp(learned.predict(W, traj[:, :10])), rtol=1e-4)
            done, b = learned.replay_cascade(pred.reshape(60, 10), devk.reshape(60, 10),
                                             traj[:, 11].astype(np.float64).reshape(60, 10), 0.01, 6)
            assert st["region_periods"] == int(done.sum())
            assert st["fits_completed"] == 10 * int(done.sum())
            full_rows = traj[:, 11].astype(np.float64).reshape(60, 10).min(axis=1)
            np.testing.assert_allclose(rows["rms"][done & (np.arange(60) != b)],
                                       full_rows[done & (np.arange(60) != b)], rtol=1e-6)


def _engine_input(obj):
    import tempfile
    from pathlib import Path

    from periodsearch_gb300 import read_input

    td = tempfile.mkdtemp()
    p = Path(td) / "period_search_in"
    p.write_text(obj.text)
    return read_input(p)


def test_trained_network_gain(engine_lib):
    """What the committed network gains over the same cascade without it
    (the rms after the screening iterations taken as the final rms), on 160
    fresh objects of the survey population (Ndata 200-3000, 24-period
    windows, half around the true period; recorded full trajectories, the
    cascade's decisions replayed): its log error in the final rms is under
    half the zero predictor's, and at the network's calibrated margin its
    scan misses the full scan's best period less than half as often."""
    from periodsearch_gb300 import learned

    P, meta = learned.load_default()
    if P is None or "margin_without_network" not in meta:
        pytest.skip("no trained predictor committed")
    objs = learned._population("c5", 160, 70000, processes=8)
    wins, _ = learned.collect_windows(objs, 24, meta["screen_iters"], around_truth=lambda k: k % 2 == 0, seed=5)
    x, y = [], []
    for w in wins:
        a, b, _, _ = learned.samples(w["traj"])
        x.append(a)
        y.append(b)
    x, y = np.concatenate(x), np.concatenate(y)
    err_net = np.sqrt(np.mean((learned.predict(P, x) - y) ** 2))
    err_zero = np.sqrt(np.mean(y ** 2))
    assert err_net < 0.5 * err_zero, (err_net, err_zero)
    m = learned.cascade_defaults()["margin"]
    net = learned.replay_windows(wins, P, m, 15)
    zero = learned.replay_windows(wins, learned.zero_predictor(), m, 15)
    assert net["misses"] < 0.5 * max(zero["misses"], 1), (net, zero)


def test_learned_scan_keeps_best_period(engine_lib, tmp_path):
    """On a synthetic object the learned scan (screen, complete, FP64 refit)
    reports the same best period as the full FP64 scan of the same window,
    with FP64 values there, and runs fewer model evaluations."""
    from periodsearch_gb300 import Engine, PS_FORM_FP64, PS_FORM_MIXED, learned, read_input, synth

    P, meta = learned.load_default()
    if P is None or "margin_without_network" not in meta:
        pytest.skip("no trained predictor committed")
    obj = synth.write_object(tmp_path / "period_search_in", "c1", seed=905)
    data = read_input(tmp_path / "period_search_in")
    with Engine(data, form=PS_FORM_FP64) as full:
        conw_r, _ = full.precalc_conw()
        n_t = int(round((full.info.freq_start - 1 / obj.truth["period_h"]) / full.info.freq_step)) + 1
        lo, hi = n_t - 24, n_t + 23
        rows_full = full.scan(conw_r, lo, hi)
        evals_full = full.timing()["evals"]
    with Engine(data, form=PS_FORM_MIXED) as eng:
        rows, st = eng.scan_learned(conw_r, lo, hi, P, **{**learned.cascade_defaults(), "fill_refit_waves": 0})
    b_full, b = int(np.argmin(rows_full["rms"])), int(np.argmin(rows["rms"]))
    assert b == b_full
    assert rows["rms"][b] == pytest.approx(rows_full["rms"][b_full], rel=1e-9)
    assert st["evals"] < 0.7 * evals_full
    assert st["fits_screened_out"] > 0.3 * st["fits_total"]
