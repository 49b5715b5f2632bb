"""ctypes view of the C ABI in include/ps_gb300.h.

The library is built in-tree (periodsearch_gb300/libps_gb300.so).  Loading it
never touches the GPU; every entry point that needs one reports
PS_ERR_NO_DEVICE instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libps_gb300.so"

PS_OK = 0
PS_ERR_ARG = 1
PS_ERR_LIMIT = 2
PS_ERR_SINGULAR = 4
PS_ERR_IO = 5
PS_FLAG_NO_TENSOR = 1
PS_ERR_CUDA = 10
PS_ERR_NO_DEVICE = 11
PS_ERR_TIMEOUT = 12

PS_FORM_FP64 = 0
PS_FORM_MIXED = 1
N_POLES = 10


class Header(C.Structure):
    _fields_ = [
        ("per_start", C.c_double), ("per_step_coef", C.c_double), ("per_end", C.c_double), ("ia_prd", C.c_int32),
        ("jd00", C.c_double), ("phi0_deg", C.c_double), ("conw", C.c_double),
        ("lmax", C.c_int32), ("mmax", C.c_int32), ("nrows", C.c_int32),
        ("par", C.c_double * 3), ("ia_par", C.c_int32 * 3),
        ("cl", C.c_double), ("ia_cl", C.c_int32),
        ("stop_condition", C.c_double), ("n_iter_min", C.c_int32),
        ("alamda_incr", C.c_double), ("alamda_start", C.c_double),
    ]


class Problem(C.Structure):
    _fields_ = [
        ("hdr", Header), ("n_lc", C.c_int32),
        ("lc_points", C.POINTER(C.c_int32)), ("lc_calibrated", C.POINTER(C.c_int32)),
        ("lc_weight", C.POINTER(C.c_double)), ("ndata", C.c_int32),
        ("jd", C.POINTER(C.c_double)), ("brightness", C.POINTER(C.c_double)),
        ("sun", C.POINTER(C.c_double)), ("earth", C.POINTER(C.c_double)),
    ]


class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("form", C.c_int32), ("ctas_per_sm", C.c_int32), ("flags", C.c_int32)]


class Row(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("period_h", "rms", "chi2", "dark_or_conw", "lambda_deg", "beta_deg")]


class Fit(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dev", "dark", "totarea", "period_h", "lambda_deg", "beta_deg", "chisq")] + [
        ("niter", C.c_int32), ("err_code", C.c_int32), ("pred_dev", C.c_double), ("screened", C.c_int32),
        ("reserved", C.c_int32)]


class Info(C.Structure):
    _fields_ = [("ndata", C.c_int32), ("n_lc", C.c_int32), ("ncoef", C.c_int32), ("ma", C.c_int32),
                ("mfit", C.c_int32), ("nfac", C.c_int32), ("n_max", C.c_int64), ("escl", C.c_double),
                ("conw_r0", C.c_double), ("freq_start", C.c_double), ("freq_step", C.c_double),
                ("sm_count", C.c_int32), ("slots", C.c_int32), ("h2d_bytes", C.c_int64),
                ("tensor_cores", C.c_int32), ("tile_points", C.c_int32)]


class LearnedStats(C.Structure):
    _fields_ = [("fits_total", C.c_int64), ("fits_screened_out", C.c_int64), ("fits_completed", C.c_int64),
                ("fits_refit", C.c_int64), ("evals", C.c_int64), ("screen_ms", C.c_double),
                ("complete_ms", C.c_double), ("refit_ms", C.c_double), ("best_index", C.c_int64),
                ("region_periods", C.c_int64), ("evals_screen", C.c_int64), ("evals_complete", C.c_int64),
                ("evals_refit", C.c_int64), ("refit_rounds", C.c_int32), ("launches", C.c_int32)]


class ValidateReport(C.Structure):
    _fields_ = [("match", C.c_int32), ("mismatch_column", C.c_int32), ("entries_a", C.c_int64),
                ("entries_b", C.c_int64), ("first_mismatch", C.c_int64), ("max_dev", C.c_double * 3),
                ("argmax_dev", C.c_int64 * 3), ("parse_error_a", C.c_int32), ("parse_error_b", C.c_int32)]


class State(C.Structure):
    _fields_ = [("lmax", C.c_int32), ("mmax", C.c_int32), ("nrows", C.c_int32), ("n_lc", C.c_int32),
                ("lc_points", C.POINTER(C.c_int32)), ("lc_rel", C.POINTER(C.c_int32)), ("ndata", C.c_int32),
                ("tim", C.POINTER(C.c_double)), ("brightness", C.POINTER(C.c_double)), ("sig", C.POINTER(C.c_double)),
                ("weight", C.POINTER(C.c_double)), ("ee", C.POINTER(C.c_double)), ("ee0", C.POINTER(C.c_double)),
                ("phi0", C.c_double), ("par", C.c_double * 3), ("cl", C.c_double), ("alamda_start", C.c_double),
                ("alamda_incr", C.c_double), ("stop_condition", C.c_double), ("n_iter_min", C.c_int32),
                ("ia", C.POINTER(C.c_int32)), ("cg_first", C.POINTER(C.c_double)), ("escl", C.c_double),
                ("freq_start", C.c_double), ("freq_end", C.c_double), ("freq_step", C.c_double),
                ("conw_r", C.c_double)]


class TuneCandidate(C.Structure):
    _fields_ = [("basis", C.c_int32), ("tile_points", C.c_int32), ("ctas_per_sm", C.c_int32), ("slots", C.c_int32),
                ("fits_per_s", C.c_double)]


TUNE_MAX = 16


class TuneReport(C.Structure):
    _fields_ = [("n", C.c_int32), ("chosen", C.c_int32), ("sample_fits", C.c_int32), ("sample_iters", C.c_int32),
                ("cand", TuneCandidate * TUNE_MAX)]


class LearnedOpts(C.Structure):
    _fields_ = [("screen_iters", C.c_int32), ("margin", C.c_double), ("batch_periods", C.c_int32),
                ("region_halfwidth", C.c_int32), ("refit_rel", C.c_double), ("refit_halfwidth", C.c_int32),
                ("fill_refit_waves", C.c_int32)]


MLP_FEATURES = 10
MLP_FLOATS = 4951
TRAJ_FLOATS = 16


class Timing(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("total_ms", C.c_double), ("fits", C.c_int64), ("evals", C.c_int64),
                ("launches", C.c_int32), ("cluster_size", C.c_int32), ("lit_facets", C.c_int64)]


# Every symbol the header declares, with its ctypes signature.
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_CTX = C.c_void_p
SIGNATURES = {
    "ps_status_string": (C.c_char_p, [C.c_int]),
    "ps_abi_version": (C.c_int32, []),
    "ps_input_read": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "ps_input_problem": (C.c_int, [C.c_void_p, C.POINTER(Problem)]),
    "ps_input_free": (None, [C.c_void_p]),
    "ps_prepare": (C.c_int, [C.POINTER(Problem), C.POINTER(Options), C.POINTER(_CTX)]),
    "ps_get_info": (C.c_int, [_CTX, C.POINTER(Info)]),
    "ps_precalc_conw": (C.c_int, [_CTX, _D, _I32]),
    "ps_scan": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_int64, C.POINTER(Row)]),
    "ps_fit_batch": (C.c_int, [_CTX, C.c_double, C.c_int64, _I64, _I32, C.POINTER(Fit)]),
    "ps_fit_batch_noalloc": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "ps_eval": (C.c_int, [_CTX, C.c_double, _D, _D, _D, _D, _D]),
    "ps_last_timing": (C.c_int, [_CTX, C.POINTER(Timing)]),
    "ps_trajectories": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_int64, C.c_int32, C.POINTER(C.c_float)]),
    "ps_mlp_train": (C.c_int, [C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                               C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "ps_mlp_predict": (C.c_int, [C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                 C.POINTER(C.c_float)]),
    "ps_mlp_grad": (C.c_int, [C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                              C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ps_screen": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_int64, C.c_int32, C.POINTER(C.c_float),
                            C.POINTER(Fit)]),
    "ps_tc_selftest": (C.c_int, [C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                                 C.POINTER(C.c_float)]),
    "ps_tc_selftest_f16": (C.c_int, [C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                                 C.POINTER(C.c_float)]),
    "ps_tc_wait_selftest": (C.c_int, [C.c_int32, C.c_int32]),
    "ps_prepare_state": (C.c_int, [C.POINTER(State), C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "ps_precalc_step": (C.c_int, [_CTX, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "ps_autotune": (C.c_int, [_CTX, C.c_double, C.c_int32, C.c_int32, C.POINTER(TuneReport)]),
    "ps_pack_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "ps_pack_fit": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int32),
                              C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(Fit)]),
    "ps_pack_screen": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_float),
                                 C.POINTER(Fit)]),
    "ps_pack_trajectories": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_float),
                                       C.POINTER(Fit)]),
    "ps_pack_timing": (C.c_int, [C.c_void_p, C.POINTER(Timing)]),
    "ps_pack_last_error": (C.c_char_p, [C.c_void_p]),
    "ps_pack_destroy": (None, [C.c_void_p]),
    "ps_validate_rows": (C.c_int, [C.POINTER(Row), C.c_int64, C.POINTER(Row), C.c_int64, C.POINTER(C.c_double),
                                   C.POINTER(ValidateReport)]),
    "ps_validate_files": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.POINTER(ValidateReport)]),
    "ps_scan_refined": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_int64, C.c_double, C.c_int32,
                                  C.POINTER(Row), C.POINTER(LearnedStats)]),
    "ps_scan_learned": (C.c_int, [_CTX, C.c_double, C.c_int64, C.c_int64, C.POINTER(C.c_float),
                                  C.POINTER(LearnedOpts), C.POINTER(Row), C.POINTER(LearnedStats)]),
    "ps_last_error": (C.c_char_p, [_CTX]),
    "ps_destroy": (None, [_CTX]),
    "ps_device_fma_peaks": (C.c_int, [C.c_int32, _D, _D]),
    "ps_format_row": (C.c_int32, [C.POINTER(Row), C.c_char_p, C.c_size_t]),
    "ps_rows_from_fits": (C.c_int, [C.POINTER(Fit), C.c_int64, C.c_int32, C.POINTER(Row)]),
    "ps_run_files": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(Options), C.c_int32]),
    "ps_shape_tables": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _I32, _I32, _D, _D, _D]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libps_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with periodsearch_gb300.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class EngineError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        msg = lib().ps_status_string(status).decode()
        super().__init__(f"{where}: {msg} (status {status}){': ' + detail if detail else ''}")
        self.status = status


def check(status: int, where: str, ctx=None) -> None:
    if status != PS_OK:
        detail = lib().ps_last_error(ctx).decode() if ctx else ""
        raise EngineError(status, where, detail)
