"""GB300 period-search engine: a drop-in for the fit path of Asteroids@home
period_search (IanSteveC/PeriodSearch).

The Python surface mirrors the reference's three host phases
(CUDAPrepare / CUDAPrecalc / CUDAStart of
period_search_cuda/period_search/start_CUDA.h) and its file contract
(period_search_in -> period_search_out):

    prob = read_input("period_search_in")
    with Engine(prob) as eng:
        conw_r, ok = eng.precalc_conw()
        rows = eng.scan(conw_r, 1, eng.info.n_max)
    text = "".join(format_row(r) for r in rows)

Everything runs through libps_gb300.so; there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _abi
from ._abi import EngineError, N_POLES, PS_FORM_FP64, PS_FORM_MIXED

__all__ = ["Engine", "Pack", "InputData", "read_input", "run_files", "format_row", "shape_tables", "ROW_DTYPE",
           "FIT_DTYPE", "EngineError", "PS_FORM_FP64", "PS_FORM_MIXED", "N_POLES"]

ROW_DTYPE = np.dtype([(n, "f8") for n in ("period_h", "rms", "chi2", "dark_or_conw", "lambda_deg", "beta_deg")])
FIT_DTYPE = np.dtype([(n, "f8") for n in ("dev", "dark", "totarea", "period_h", "lambda_deg", "beta_deg", "chisq")]
                     + [("niter", "i4"), ("err_code", "i4"), ("pred_dev", "f8"), ("screened", "i4"),
                        ("reserved", "i4")])
HEADER_FIELDS = [f for f, _ in _abi.Header._fields_]


@dataclass
class InputData:
    """Contents of one period_search_in file (0-based arrays)."""
    header: dict
    lc_points: np.ndarray          # int32 [n_lc]
    lc_calibrated: np.ndarray      # int32 [n_lc], 1 calibrated / 0 relative
    lc_weight: np.ndarray          # float64 [n_lc], -1 = not given
    jd: np.ndarray                 # float64 [ndata]
    brightness: np.ndarray         # float64 [ndata]
    sun: np.ndarray                # float64 [ndata, 3] asteroid->Sun
    earth: np.ndarray              # float64 [ndata, 3] asteroid->Earth
    _keep: list = field(default_factory=list, repr=False)

    @property
    def ndata(self) -> int:
        return int(self.jd.shape[0])

    def to_problem(self) -> _abi.Problem:
        """ps_problem view; the arrays stay referenced by this object."""
        h = _abi.Header()
        for k in HEADER_FIELDS:
            v = self.header[k]
            if k in ("par", "ia_par"):
                getattr(h, k)[:] = list(v)
            else:
                setattr(h, k, v)
        arrs = [np.ascontiguousarray(self.lc_points, np.int32), np.ascontiguousarray(self.lc_calibrated, np.int32),
                np.ascontiguousarray(self.lc_weight, np.float64), np.ascontiguousarray(self.jd, np.float64),
                np.ascontiguousarray(self.brightness, np.float64),
                np.ascontiguousarray(self.sun, np.float64).reshape(-1),
                np.ascontiguousarray(self.earth, np.float64).reshape(-1)]
        self._keep = arrs
        p = _abi.Problem()
        p.hdr = h
        p.n_lc = len(arrs[0])
        p.lc_points = arrs[0].ctypes.data_as(C.POINTER(C.c_int32))
        p.lc_calibrated = arrs[1].ctypes.data_as(C.POINTER(C.c_int32))
        p.lc_weight = arrs[2].ctypes.data_as(C.POINTER(C.c_double))
        p.ndata = len(arrs[3])
        p.jd = arrs[3].ctypes.data_as(C.POINTER(C.c_double))
        p.brightness = arrs[4].ctypes.data_as(C.POINTER(C.c_double))
        p.sun = arrs[5].ctypes.data_as(C.POINTER(C.c_double))
        p.earth = arrs[6].ctypes.data_as(C.POINTER(C.c_double))
        return p

    def nbytes(self) -> int:
        return sum(a.nbytes for a in (self.lc_points, self.lc_calibrated, self.lc_weight, self.jd, self.brightness,
                                      self.sun, self.earth))


class Pack:
    """Several objects fitted by one packed launch (ps_pack_create ..
    ps_pack_destroy).  The engines must share the shape tables and stay open
    while the pack lives."""

    def __init__(self, engines, form: int = PS_FORM_FP64):
        self._L = _abi.lib()
        self._engines = list(engines)
        arr = (C.c_void_p * len(self._engines))(*[e._ctx.value for e in self._engines])
        h = C.c_void_p()
        _abi.check(self._L.ps_pack_create(arr, len(self._engines), form, C.byref(h)), "ps_pack_create")
        self._h = h

    def _call(self, name, conw_r, object_index, period_index, pole, *extra):
        cw = np.ascontiguousarray(conw_r, np.float64)
        ob = np.ascontiguousarray(object_index, np.int32)
        pi = np.ascontiguousarray(period_index, np.int64)
        po = np.ascontiguousarray(pole, np.int32)
        out = np.zeros(len(pi), FIT_DTYPE)
        st = getattr(self._L, name)(self._h, cw.ctypes.data_as(C.POINTER(C.c_double)), len(pi),
                                    ob.ctypes.data_as(C.POINTER(C.c_int32)), pi.ctypes.data_as(C.POINTER(C.c_int64)),
                                    po.ctypes.data_as(C.POINTER(C.c_int32)), *extra,
                                    out.ctypes.data_as(C.POINTER(_abi.Fit)))
        if st != _abi.PS_OK:
            raise EngineError(st, name, self._L.ps_pack_last_error(self._h).decode())
        return out

    def fit(self, conw_r, object_index, period_index, pole) -> np.ndarray:
        return self._call("ps_pack_fit", conw_r, object_index, period_index, pole)

    def screen(self, conw_r, object_index, period_index, pole, weights, screen_iters: int) -> np.ndarray:
        """screen_iters LM iterations of every unit with the in-kernel
        predictor (ps_pack_screen)."""
        w = np.ascontiguousarray(weights, np.float32)
        return self._call("ps_pack_screen", conw_r, object_index, period_index, pole, int(screen_iters),
                          w.ctypes.data_as(C.POINTER(C.c_float)))

    def trajectories(self, conw_r, object_index, period_index, pole, feat_iters: int):
        """Full fits with their trajectory records (ps_pack_trajectories),
        features after feat_iters iterations: returns (fits, records[n][16])."""
        traj = np.zeros((len(period_index), _abi.TRAJ_FLOATS), np.float32)
        fits = self._call("ps_pack_trajectories", conw_r, object_index, period_index, pole, int(feat_iters),
                          traj.ctypes.data_as(C.POINTER(C.c_float)))
        return fits, traj

    def timing(self) -> dict:
        t = _abi.Timing()
        _abi.check(self._L.ps_pack_timing(self._h, C.byref(t)), "ps_pack_timing")
        return {k: getattr(t, k) for k, _ in _abi.Timing._fields_}

    def close(self) -> None:
        if self._h:
            self._L.ps_pack_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_input(path: str) -> InputData:
    """Parses period_search_in with the reference's reading rules."""
    L = _abi.lib()
    h = C.c_void_p()
    _abi.check(L.ps_input_read(str(path).encode(), C.byref(h)), "ps_input_read")
    try:
        p = _abi.Problem()
        _abi.check(L.ps_input_problem(h, C.byref(p)), "ps_input_problem")
        n_lc, nd = p.n_lc, p.ndata
        hdr = {k: (list(getattr(p.hdr, k)) if k in ("par", "ia_par") else getattr(p.hdr, k)) for k in HEADER_FIELDS}
        arr = lambda ptr, n, dt: np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)
        return InputData(header=hdr, lc_points=arr(p.lc_points, n_lc, np.int32),
                         lc_calibrated=arr(p.lc_calibrated, n_lc, np.int32),
                         lc_weight=arr(p.lc_weight, n_lc, np.float64), jd=arr(p.jd, nd, np.float64),
                         brightness=arr(p.brightness, nd, np.float64),
                         sun=arr(p.sun, 3 * nd, np.float64).reshape(nd, 3),
                         earth=arr(p.earth, 3 * nd, np.float64).reshape(nd, 3))
    finally:
        L.ps_input_free(h)


def format_row(row) -> str:
    """One output line in the reference's format."""
    r = _abi.Row(*[float(row[n]) for n in ROW_DTYPE.names])
    buf = C.create_string_buffer(256)
    _abi.lib().ps_format_row(C.byref(r), buf, 256)
    return buf.value.decode()


def shape_tables(nrows: int, lmax: int, mmax: int):
    """(nor[nfac,3], darea[nfac], dsph[nfac,ncoef]) of the trifac grid."""
    L = _abi.lib()
    nf, nc = C.c_int32(), C.c_int32()
    _abi.check(L.ps_shape_tables(nrows, lmax, mmax, C.byref(nf), C.byref(nc), None, None, None), "ps_shape_tables")
    nor = np.zeros((nf.value, 3))
    darea = np.zeros(nf.value)
    dsph = np.zeros((nf.value, nc.value))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    _abi.check(L.ps_shape_tables(nrows, lmax, mmax, None, None, dp(nor), dp(darea), dp(dsph)), "ps_shape_tables")
    return nor, darea, dsph


def run_files(in_path: str, out_path: str, state_path: Optional[str] = None, device: int = 0,
              form: int = PS_FORM_FP64, checkpoint_rows: int = 64) -> None:
    """The BOINC app's job on files (period_search_in -> period_search_out)."""
    opt = _abi.Options(device, form, 0, 0)
    st = _abi.lib().ps_run_files(str(in_path).encode(), str(out_path).encode(),
                                 str(state_path).encode() if state_path else None, C.byref(opt), checkpoint_rows)
    _abi.check(st, "ps_run_files")


class Engine:
    """One object prepared on one GPU (ps_prepare .. ps_destroy)."""

    def __init__(self, data: InputData, device: int = 0, form: int = PS_FORM_FP64, ctas_per_sm: int = 0,
                 tensor_cores: bool = True):
        self._L = _abi.lib()
        self._prob = data.to_problem()
        self._data = data
        opt = _abi.Options(device, form, ctas_per_sm, 0 if tensor_cores else _abi.PS_FLAG_NO_TENSOR)
        ctx = C.c_void_p()
        _abi.check(self._L.ps_prepare(C.byref(self._prob), C.byref(opt), C.byref(ctx)), "ps_prepare")
        self._ctx = ctx
        inf = _abi.Info()
        _abi.check(self._L.ps_get_info(ctx, C.byref(inf)), "ps_get_info", ctx)
        self.info = inf

    def close(self) -> None:
        if self._ctx:
            self._L.ps_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def precalc_conw(self):
        cw, nc = C.c_double(), C.c_int32()
        _abi.check(self._L.ps_precalc_conw(self._ctx, C.byref(cw), C.byref(nc)), "ps_precalc_conw", self._ctx)
        return cw.value, nc.value

    def scan(self, conw_r: float, n_lo: int, n_hi: int) -> np.ndarray:
        out = np.zeros(n_hi - n_lo + 1, ROW_DTYPE)
        st = self._L.ps_scan(self._ctx, conw_r, n_lo, n_hi, out.ctypes.data_as(C.POINTER(_abi.Row)))
        _abi.check(st, "ps_scan", self._ctx)
        return out

    def fit_batch(self, conw_r: float, period_index, pole) -> np.ndarray:
        pi = np.ascontiguousarray(period_index, np.int64)
        po = np.ascontiguousarray(pole, np.int32)
        out = np.zeros(len(pi), FIT_DTYPE)
        st = self._L.ps_fit_batch(self._ctx, conw_r, len(pi), pi.ctypes.data_as(C.POINTER(C.c_int64)),
                                  po.ctypes.data_as(C.POINTER(C.c_int32)), out.ctypes.data_as(C.POINTER(_abi.Fit)))
        _abi.check(st, "ps_fit_batch", self._ctx)
        return out

    def rows_of_periods(self, conw_r: float, period_index) -> np.ndarray:
        """Rows of the given periods (all ten poles each, ps_fit_batch in
        one launch, then the best-of-poles reduction ps_rows_from_fits)."""
        per = np.ascontiguousarray(period_index, np.int64)
        fits = self.fit_batch(conw_r, np.repeat(per, N_POLES), np.tile(np.arange(1, N_POLES + 1), len(per)))
        out = np.zeros(len(per), ROW_DTYPE)
        st = self._L.ps_rows_from_fits(fits.ctypes.data_as(C.POINTER(_abi.Fit)), len(per), self.info.ndata,
                                       out.ctypes.data_as(C.POINTER(_abi.Row)))
        _abi.check(st, "ps_rows_from_fits")
        return out

    def eval(self, conw_r: float, cg):
        cg = np.ascontiguousarray(cg, np.float64)
        mf = self.info.mfit
        alpha = np.zeros((mf, mf))
        beta = np.zeros(mf)
        area = np.zeros(self.info.nfac)
        c2 = C.c_double()
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        st = self._L.ps_eval(self._ctx, conw_r, dp(cg), dp(alpha), dp(beta), C.byref(c2), dp(area))
        _abi.check(st, "ps_eval", self._ctx)
        return alpha, beta, c2.value, area

    def trajectories(self, conw_r: float, n_lo: int, n_hi: int, feat_iters: int | None = None) -> np.ndarray:
        from . import learned

        return learned.trajectories(self, conw_r, n_lo, n_hi, feat_iters)

    def screen(self, conw_r: float, n_lo: int, n_hi: int, weights, screen_iters: int | None = None) -> np.ndarray:
        """The screening pass alone (ps_screen): per fit the rms after the
        screening iterations and the predicted final rms."""
        from . import learned

        k = learned.SCREEN_ITERS if screen_iters is None else int(screen_iters)
        w = np.ascontiguousarray(weights, np.float32)
        out = np.zeros((n_hi - n_lo + 1) * N_POLES, FIT_DTYPE)
        r = self._L.ps_screen(self._ctx, conw_r, n_lo, n_hi, k, w.ctypes.data_as(C.POINTER(C.c_float)),
                              out.ctypes.data_as(C.POINTER(_abi.Fit)))
        _abi.check(r, "ps_screen", self._ctx)
        return out

    def autotune(self, conw_r: float, sample_fits: int = 0, sample_iters: int = 0) -> dict:
        """Times the kernel configurations the object admits (ps_autotune)
        and keeps the fastest; returns the measured candidates."""
        r = _abi.TuneReport()
        _abi.check(self._L.ps_autotune(self._ctx, conw_r, sample_fits, sample_iters, C.byref(r)), "ps_autotune",
                   self._ctx)
        inf = _abi.Info()
        _abi.check(self._L.ps_get_info(self._ctx, C.byref(inf)), "ps_get_info", self._ctx)
        self.info = inf
        names = {0: "l2", 1: "shared", 2: "tensor"}
        cands = [{"basis": names.get(c.basis, c.basis), "tile_points": c.tile_points, "ctas_per_sm": c.ctas_per_sm,
                  "slots": c.slots, "fits_per_s": c.fits_per_s} for c in r.cand[:r.n]]
        return {"candidates": cands, "chosen": r.chosen, "sample_fits": r.sample_fits,
                "sample_iters": r.sample_iters}

    def scan_refined(self, conw_r: float, n_lo: int, n_hi: int, refit_rel: float = 0.01, refit_halfwidth: int = 2):
        """Scan in the engine's form, then refit the minimum region in full
        with the FP64 form (ps_scan_refined); returns the rows and the
        statistics."""
        out = np.zeros(n_hi - n_lo + 1, ROW_DTYPE)
        st = _abi.LearnedStats()
        r = self._L.ps_scan_refined(self._ctx, conw_r, n_lo, n_hi, refit_rel, refit_halfwidth,
                                    out.ctypes.data_as(C.POINTER(_abi.Row)), C.byref(st))
        _abi.check(r, "ps_scan_refined", self._ctx)
        return out, {k: getattr(st, k) for k, _ in _abi.LearnedStats._fields_}

    def scan_learned(self, conw_r: float, n_lo: int, n_hi: int, weights=None, **opts):
        """Period scan with the learned early stop (ps_scan_learned); returns
        the rows and the stage statistics.  Options (ps_learned_opts):
        screen_iters, margin, batch_periods, region_halfwidth, refit_rel,
        refit_halfwidth, fill_refit_waves.  Without weights the committed
        predictor is used, with the screening depth and margin it was
        calibrated for (learned.CASCADE)."""
        from . import learned

        if weights is None:
            weights, _ = learned.load_default()
            if weights is None:
                raise EngineError(_abi.PS_ERR_ARG, "scan_learned", "no trained predictor available")
        o = _abi.LearnedOpts(**learned.cascade_defaults())
        for k, v in opts.items():
            setattr(o, k, v)
        w = np.ascontiguousarray(weights, np.float32)
        out = np.zeros(n_hi - n_lo + 1, ROW_DTYPE)
        st = _abi.LearnedStats()
        r = self._L.ps_scan_learned(self._ctx, conw_r, n_lo, n_hi, w.ctypes.data_as(C.POINTER(C.c_float)),
                                    C.byref(o), out.ctypes.data_as(C.POINTER(_abi.Row)), C.byref(st))
        _abi.check(r, "ps_scan_learned", self._ctx)
        return out, {k: getattr(st, k) for k, _ in _abi.LearnedStats._fields_}

    def timing(self) -> dict:
        t = _abi.Timing()
        _abi.check(self._L.ps_last_timing(self._ctx, C.byref(t)), "ps_last_timing", self._ctx)
        return {k: getattr(t, k) for k, _ in _abi.Timing._fields_}
