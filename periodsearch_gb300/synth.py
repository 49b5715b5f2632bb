"""Seeded synthetic photometry in the period_search_in format.

The workloads of the benchmark and of the parity tests are generated here:

* truth shape: a Gaussian image exp(sum a_lm Y_lm) with orthonormal real
  spherical harmonics, a_00 = 0 and a_lm ~ N(0, (0.15/(l+1))^2);
* pole lambda ~ U[0, 360), sin(beta) ~ U[-1, 1]; period P ~ U[4, 12] h;
* Lommel-Seeliger + Lambert scattering with Lambert weight c = 0.1 and the
  exponential-linear phase function a = 0.5, d = 0.1, k = -0.5;
* geometry: the asteroid on a circular 2.6 AU orbit inclined by up to 5 deg,
  the Earth on a circular 1 AU orbit; observations near opposition;
* sparse calibrated points at random epochs over 8 years (0.1 mag noise) and
  dense relative lightcurves of 3 h with 60 points (0.02 mag noise).

Brightness is the reduced intensity of the forward model (no distance
dimming), multiplied by 10^(-0.4 eps) with eps the Gaussian magnitude noise.
The forward model uses the engine's own facet tables (shape_tables) on a
finer grid than the fits use.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from math import factorial

import numpy as np

YEAR = 365.25


@dataclass
class SynthConfig:
    name: str = "c0"
    seed: int = 1
    lmax_truth: int = 6
    n_sparse: int = 200
    n_dense: int = 0
    dense_points: int = 60
    dense_hours: float = 3.0
    sigma_sparse: float = 0.1
    sigma_dense: float = 0.02
    years: float = 8.0
    # fit settings written into the header
    lmax: int = 6
    nrows: int = 6
    per_start: float = 0.0     # 0: 0.9 * truth period
    per_end: float = 0.0       # 0: 1.1 * truth period
    n_periods: int = 600       # target number of trial periods (sets per_step_coef)
    conw: float = 0.1
    stop_condition: float = 50
    n_iter_min: int = 10
    ia_prd: int = 1
    ia_par: tuple = (1, 1, 1)
    cl_start: float = 0.1
    ia_cl: int = 0
    weights: dict = field(default_factory=dict)   # lightcurve number (1-based) -> weight
    sparse_block: int = 1000   # calibrated points per lightcurve block


# The benchmark and test workloads, by name.
CONFIGS = {
    # single object, 200 sparse calibrated points, scan +-10 % around truth
    "c0": SynthConfig(name="c0"),
    # 8 dense relative lightcurves + 500 sparse points, scan 2-50 h
    "c1": SynthConfig(name="c1", n_sparse=500, n_dense=8, per_start=2.0, per_end=50.0, n_periods=40000),
    # c1 data with lmax = mmax = 8 and nrows = 8
    "c2": SynthConfig(name="c2", n_sparse=500, n_dense=8, per_start=2.0, per_end=50.0, n_periods=40000,
                      lmax_truth=8, lmax=8, nrows=8),
    # small cases that the oracle fits in milliseconds
    "tiny_cal": SynthConfig(name="tiny_cal", n_sparse=40, lmax=2, nrows=3, n_periods=14, stop_condition=8),
    "tiny_rel": SynthConfig(name="tiny_rel", n_sparse=0, n_dense=2, dense_points=20, lmax=3, nrows=3,
                            n_periods=14, stop_condition=8),
    "tiny_mix": SynthConfig(name="tiny_mix", n_sparse=30, n_dense=2, dense_points=15, lmax=3, nrows=3,
                            n_periods=13, stop_condition=10, ia_cl=1, weights={1: 0.5, 3: 2.0}, sparse_block=12),
    "tiny_stop": SynthConfig(name="tiny_stop", n_sparse=36, n_dense=1, dense_points=12, lmax=2, nrows=3,
                             n_periods=12, stop_condition=0.01, n_iter_min=4, ia_par=(1, 0, 1)),
}


def population_config(rng: np.random.Generator, name: str, ndata_lo: int, ndata_hi: int, per_start: float,
                      per_end: float, n_periods: int) -> SynthConfig:
    """One object of a seeded population of work units: Ndata log-uniform
    in [ndata_lo, ndata_hi]; half the objects sparse calibrated data only,
    half with 1-8 dense relative lightcurves (3 h, 60 points) plus sparse
    points (at least 100), as in a survey's mix of work units."""
    nd = int(round(math.exp(rng.uniform(math.log(ndata_lo), math.log(ndata_hi)))))
    n_dense = 0
    if rng.uniform() < 0.5:
        n_dense = int(min(8, max(1, (nd - 100) // 60), rng.integers(1, 9)))
        if nd - 60 * n_dense < 100:
            n_dense = 0
    return SynthConfig(name=name, n_sparse=nd - 60 * n_dense, n_dense=n_dense, per_start=per_start,
                       per_end=per_end, n_periods=n_periods, sparse_block=1000)


# The multi-object populations: many asteroids with uneven Ndata, each with
# its own seed (population_config(rng, ...) with rng seeded per object).
POPULATIONS = {
    # many asteroids in one launch: Ndata logU[100, 5000], scan 2-20 h
    "c3": dict(ndata_lo=100, ndata_hi=5000, per_start=2.0, per_end=20.0, n_periods=20000),
    # the learned early stop's evaluation set: Ndata 200-3000, scan 2-100 h
    "c5": dict(ndata_lo=200, ndata_hi=3000, per_start=2.0, per_end=100.0, n_periods=60000),
}


def population_object(pop: str, k: int, base_seed: int) -> SynthObject:
    """Object k of population `pop` (seed base_seed + k for both its
    configuration and its data)."""
    rng = np.random.default_rng(base_seed + k)
    cfg = population_config(rng, f"{pop}_{k}", **POPULATIONS[pop])
    return make_object(cfg, seed=base_seed + k)


def _ylm_norm(l: int, m: int) -> float:
    n = math.sqrt((2 * l + 1) / (4 * math.pi) * factorial(l - m) / factorial(l + m))
    return n * (math.sqrt(2.0) if m > 0 else 1.0)


def truth_coefficients(rng: np.random.Generator, lmax: int) -> np.ndarray:
    """Coefficients of exp(sum a_lm Y_lm) in the engine's basis order
    (m = 0..lmax, l = m..lmax, cos then sin), orthonormal Y_lm folded in."""
    cg = []
    for m in range(lmax + 1):
        for l in range(m, lmax + 1):
            sd = 0.15 / (l + 1)
            a_c = 0.0 if l == 0 else rng.normal(0.0, sd)
            cg.append(a_c * _ylm_norm(l, m))
            if m:
                cg.append(rng.normal(0.0, sd) * _ylm_norm(l, m))
    return np.array(cg)


def _rot_matrix(beta_from_pole: float, lam: float) -> np.ndarray:
    cb, sb, cl, sl = math.cos(beta_from_pole), math.sin(beta_from_pole), math.cos(lam), math.sin(lam)
    return np.array([[cb * cl, cb * sl, -sb], [-sl, cl, 0.0], [sb * cl, sb * sl, cb]])


def forward_model(t, ee, ee0, nor, area, pole_lam, pole_beta, omega, phi0=0.0, cl=0.1, cls=1.0,
                  phase=(0.5, 0.1, -0.5)) -> np.ndarray:
    """Reduced brightness of a convex body with facet normals nor and areas
    area, Lommel-Seeliger + Lambert scattering and the exponential-linear
    phase function; t in days, ee/ee0 unit vectors to Earth / Sun."""
    B = _rot_matrix(math.radians(90.0 - pole_beta), math.radians(pole_lam))
    f = np.fmod(omega * t + phi0, 2 * math.pi)
    cf, sf = np.cos(f), np.sin(f)
    out = np.empty(len(t))
    for i in range(len(t)):
        Fm = np.array([[cf[i], sf[i], 0.0], [-sf[i], cf[i], 0.0], [0.0, 0.0, 1.0]])
        T = Fm @ B
        e, e0 = T @ ee[i], T @ ee0[i]
        mu, mu0 = nor @ e, nor @ e0
        lit = (mu > 1e-8) & (mu0 > 1e-8)
        s = np.where(lit, mu * mu0 * (cl + cls / np.where(lit, mu + mu0, 1.0)), 0.0)
        br = float(np.sum(area * s))
        alpha = math.acos(float(np.clip(ee[i] @ ee0[i], -1, 1)))
        out[i] = br * (1 + phase[0] * math.exp(-alpha / phase[1]) + phase[2] * alpha)
    return out


def _positions(t, incl, node, theta_a, theta_e):
    ta = 2 * math.pi * t / (YEAR * 2.6 ** 1.5) + theta_a
    te = 2 * math.pi * t / YEAR + theta_e
    # asteroid: circle of radius 2.6 in a plane inclined by incl about the node line
    x, y = 2.6 * np.cos(ta), 2.6 * np.sin(ta)
    cn, sn, ci, si = math.cos(node), math.sin(node), math.cos(incl), math.sin(incl)
    ra = np.stack([cn * x - sn * ci * y, sn * x + cn * ci * y, si * y], axis=1)
    re = np.stack([np.cos(te), np.sin(te), np.zeros_like(te)], axis=1)
    return ra, re


def _observable(ra, re):
    # Sun-Earth-asteroid elongation above 100 degrees (night sky near opposition)
    to_ast = ra - re
    cosel = np.sum(to_ast * (-re), axis=1) / (np.linalg.norm(to_ast, axis=1) * np.linalg.norm(re, axis=1))
    return cosel < math.cos(math.radians(100))


@dataclass
class SynthObject:
    text: str                 # period_search_in
    truth: dict
    ndata: int


def make_object(cfg: SynthConfig | str, seed: int | None = None) -> SynthObject:
    if isinstance(cfg, str):
        cfg = CONFIGS[cfg]
    from . import shape_tables

    rng = np.random.default_rng(cfg.seed if seed is None else seed)
    lam = rng.uniform(0, 360)
    beta = math.degrees(math.asin(rng.uniform(-1, 1)))
    period = rng.uniform(4, 12)
    omega = 2 * math.pi * 24 / period
    cg = truth_coefficients(rng, cfg.lmax_truth)
    nrows_truth = max(cfg.nrows + 2, 8)
    nor, darea, dsph = shape_tables(nrows_truth, cfg.lmax_truth, cfg.lmax_truth)
    area = darea * np.exp(dsph @ cg)

    incl = math.radians(rng.uniform(-5, 5))
    node, theta_a, theta_e = rng.uniform(0, 2 * math.pi, 3)
    jd_start = 2455000.5
    span = cfg.years * YEAR

    def epochs(n, rng):
        out = []
        while len(out) < n:
            t = rng.uniform(0, span, 4 * n + 16)
            ra, re = _positions(t, incl, node, theta_a, theta_e)
            out.extend(t[_observable(ra, re)].tolist())
        return np.sort(np.array(out[:n]))

    blocks = []  # (times, calibrated, sigma)
    if cfg.n_dense:
        starts = epochs(cfg.n_dense, rng)
        for s0 in starts:
            tt = s0 + np.linspace(0, cfg.dense_hours / 24, cfg.dense_points)
            blocks.append((tt, 0, cfg.sigma_dense))
    if cfg.n_sparse:
        ts = epochs(cfg.n_sparse, rng)
        for i in range(0, len(ts), cfg.sparse_block):
            blocks.append((ts[i:i + cfg.sparse_block], 1, cfg.sigma_sparse))

    all_t = np.concatenate([b[0] for b in blocks])
    jd0 = math.floor(jd_start + all_t.min())
    lines = []
    n_periods = cfg.n_periods
    p0 = cfg.per_start or 0.9 * period
    p1 = cfg.per_end or 1.1 * period
    span_days = all_t.max() - all_t.min()
    # trial periods = (1/p0 - 1/p1) / (0.5 / span / 24 * coef)
    coef = (1 / p0 - 1 / p1) * span_days * 48 / max(n_periods - 0.5, 1)
    lines.append(f"{p0:.6f} {coef:.6f} {p1:.6f} {cfg.ia_prd}\tperiod_start period_step period_end fixed/free")
    lines.append("0.0\tinitial epoch")
    lines.append("0.0\tinitial rotation angle")
    lines.append(f"{cfg.conw}\tconvexity weight")
    lines.append(f"{cfg.lmax} {cfg.lmax}\tdegree and order of spherical harmonics")
    lines.append(f"{cfg.nrows}\tnumber of rows")
    lines.append(f"0.5\t{cfg.ia_par[0]}\tscattering parameters")
    lines.append(f"0.1\t{cfg.ia_par[1]}")
    lines.append(f"-0.5\t{cfg.ia_par[2]}")
    lines.append(f"{cfg.cl_start}\t{cfg.ia_cl}\tLS coeff")
    lines.append(f"{cfg.stop_condition}\titeration stop condition")
    lines.append(f"{cfg.n_iter_min}\tminimum number of iterations")
    lines.append("5\tAlamda multiplicative factor")
    lines.append("0.1\tAlamda initial value")
    lines.append(str(len(blocks)))
    ndata = 0
    for tt, calibrated, sigma in blocks:
        ra, re = _positions(tt, incl, node, theta_a, theta_e)
        e_sun = -ra
        e_earth = re - ra
        ee = e_earth / np.linalg.norm(e_earth, axis=1)[:, None]
        ee0 = e_sun / np.linalg.norm(e_sun, axis=1)[:, None]
        jd = jd_start + tt
        br = forward_model(jd - jd0, ee, ee0, nor, area, lam, beta, omega)
        br = br * 10 ** (-0.4 * rng.normal(0.0, sigma, len(tt)))
        lines.append(f"{len(tt)} {calibrated}")
        for i in range(len(tt)):
            lines.append(f"{jd[i]:.6f} {br[i]:.9e} {e_sun[i, 0]:.9e} {e_sun[i, 1]:.9e} {e_sun[i, 2]:.9e} "
                         f"{e_earth[i, 0]:.9e} {e_earth[i, 1]:.9e} {e_earth[i, 2]:.9e}")
        ndata += len(tt)
    # The reference reads "lightcurve weight" pairs until end of file and
    # reuses the last pair at the end; an input always carries at least one.
    for lc, w in sorted((cfg.weights or {1: 1}).items()):
        lines.append(f"{lc} {w}")
    truth = {"period_h": period, "lambda_deg": lam, "beta_deg": beta, "seed": cfg.seed if seed is None else seed,
             "n_periods_target": n_periods}
    return SynthObject(text="\n".join(lines) + "\n", truth=truth, ndata=ndata)


def write_object(path, cfg: SynthConfig | str, seed: int | None = None) -> SynthObject:
    obj = make_object(cfg, seed)
    with open(path, "w") as f:
        f.write(obj.text)
    return obj
