"""ctypes access to the CPU oracle (oracle/libpsoracle.so).

Test infrastructure: the oracle is the checker for the CUDA engine, never a
path of the product.  Used by the tests, __graft_entry__.smoke() and the CPU
baseline leg of bench.py.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "libpsoracle.so"
REF_BIN = ORACLE_DIR / "_ref" / "ps_ref"

ROW_FIELDS = ("period_h", "rms", "chi2", "dark_or_conw", "lambda_deg", "beta_deg")
ROW_DTYPE = np.dtype([(n, "f8") for n in ROW_FIELDS])


class _Row(C.Structure):
    _fields_ = [(n, C.c_double) for n in ROW_FIELDS]


class _State(C.Structure):
    _fields_ = [("chisq_carry", C.c_double)]


_lib = None


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "libpsoracle.so"], check=True)
    return ORACLE_LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        L = C.CDLL(str(ORACLE_LIB))
        L.pso_problem_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.pso_problem_read.restype = C.c_int
        L.pso_problem_free.argtypes = [C.c_void_p]
        L.pso_problem_setup.argtypes = [C.c_void_p, C.c_double]
        L.pso_precalc_conw.argtypes = [C.c_void_p, C.POINTER(_State), C.POINTER(C.c_int)]
        L.pso_precalc_conw.restype = C.c_double
        L.pso_scan.argtypes = [C.c_void_p, C.POINTER(_State), C.c_double, C.c_int, C.c_int, C.POINTER(_Row)]
        L.pso_problem_info.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 6 + [C.POINTER(C.c_double)] * 2
        L.pso_eval_alpha.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
        L.pso_eval_alpha.restype = C.c_double
        L.pso_fit_one.argtypes = [C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.pso_initial_cg.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.pso_freq.argtypes = [C.c_void_p, C.c_int]
        L.pso_freq.restype = C.c_double
        L.pso_run_file.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int]
        L.pso_run_file.restype = C.c_int
        _lib = L
    return _lib


class OracleProblem:
    """One period_search_in file prepared by the oracle."""

    def __init__(self, path):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.pso_problem_read(str(path).encode(), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle could not read {path}: code {rc}")
        self._h = h
        self.state = _State(0.0)
        self._L.pso_problem_setup(h, self.info()["conw_r"])

    def close(self):
        if self._h:
            self._L.pso_problem_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def info(self) -> dict:
        ints = [C.c_int() for _ in range(6)]
        dbl = [C.c_double() for _ in range(2)]
        self._L.pso_problem_info(self._h, *[C.byref(x) for x in ints], *[C.byref(x) for x in dbl])
        keys = ("ndata", "ncoef", "ma", "mfit", "nfac", "n_max")
        out = {k: v.value for k, v in zip(keys, ints)}
        out["conw_r"], out["escl"] = dbl[0].value, dbl[1].value
        return out

    def precalc_conw(self):
        nc = C.c_int()
        cw = self._L.pso_precalc_conw(self._h, C.byref(self.state), C.byref(nc))
        return cw, nc.value

    def setup(self, conw_r: float):
        self._L.pso_problem_setup(self._h, conw_r)

    def scan(self, conw_r: float, n_lo: int, n_hi: int) -> np.ndarray:
        out = np.zeros(n_hi - n_lo + 1, ROW_DTYPE)
        self._L.pso_scan(self._h, C.byref(self.state), conw_r, n_lo, n_hi, out.ctypes.data_as(C.POINTER(_Row)))
        return out

    def eval(self, cg):
        """mrqcof at cg (0-based, ma values) -> (alpha, beta, chisq, area)."""
        inf = self.info()
        mf, nf = inf["mfit"], inf["nfac"]
        cg = np.ascontiguousarray(cg, np.float64)
        alpha = np.zeros((mf, mf))
        beta = np.zeros(mf)
        area = np.zeros(nf)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        c2 = self._L.pso_eval_alpha(self._h, dp(cg), dp(alpha), dp(beta), dp(area))
        return alpha, beta, c2, area

    def initial_cg(self, n: int, pole: int) -> np.ndarray:
        out = np.zeros(self.info()["ma"])
        self._L.pso_initial_cg(self._h, n, pole, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def freq(self, n: int) -> float:
        return self._L.pso_freq(self._h, n)

    def fit_n(self, n: int, pole: int) -> dict:
        """Fit of period index n from pole (1..10)."""
        v = self.fit(self.freq(n), pole)
        keys = ("dev", "dark", "totarea", "prd", "la", "be", "chisq")
        return dict(zip(keys, v))

    def fit(self, freq: float, pole: int) -> np.ndarray:
        out = np.zeros(7)
        self._L.pso_fit_one(self._h, freq, pole, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out


def run_reference_binary(workdir: Path) -> tuple[str, np.ndarray]:
    """Runs the reference app built by `make -C oracle ref` in workdir
    (which holds period_search_in); returns the text and the %.17g rows."""
    subprocess.run([str(REF_BIN)], cwd=workdir, check=True, capture_output=True)
    text = (workdir / "period_search_out").read_text()
    full = np.loadtxt(workdir / "period_search_out.full", ndmin=2)
    return text, full
