"""ORACLE - test infrastructure only; never part of the product path.

CPU restatement of the reference's fitting path: ``fit`` and ``fit_multik``
(``src/python/fit.py:124-194``, ``:197-397``) and the models of
``src/python/fit_models.py``.  Only ``tests/`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker / the timed CPU
baseline.

The reference fits through lmfit (``Model.fit`` with its default method
'leastsq'; lmfit is unpinned in the reference's ``pyproject.toml:35``) and
returns a pandas DataFrame.  Neither lmfit nor pandas is installed here, so:

* the optimiser itself is the real one: lmfit's 'leastsq' calls
  ``scipy.optimize.leastsq`` (MINPACK lmdif), and so does this oracle, with the
  options lmfit passes (xtol = ftol = gtol = 1e-7, forward-difference
  Jacobian);
* lmfit's wrapper around it is restated from its documented behaviour (lmfit
  1.x): starting values clipped into [min, max]; bounded parameters mapped to
  internal ones by the MINUIT transformations; residual ``(model - data) *
  weights``; ValueError when a residual is not finite (nan_policy 'raise');
  evaluation limit 2000 * (nvary + 1); success = MINPACK info in 1..4;
  covariance inv(R^T R) from MINPACK's last factorisation, taken to external
  parameters through the derivative of the mapping and scaled by
  chi^2 / (ndata - nvary); stderr = its diagonal's square root (0 for fixed
  parameters, None without a covariance).

Parity against lmfit's own outputs is therefore unpinned; the MINPACK core is
pinned by the known-answer tests in ``tests/test_fit.py`` (among them the
published minima of MINPACK's test set), the reference having no test or
golden output for fitting.
"""

from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import numpy as np
from scipy.optimize import leastsq

EPSILON = np.finfo(float).eps

# ---------------------------------------------------------------------------
# models: fit_models.py and fit.py, in their operation order
# ---------------------------------------------------------------------------


def _gexp_isf(x, A, Gamma, beta):  # fit_models.py:515-549
    return A * np.exp(-((x * Gamma) ** beta))


def _dexp_isf(x, A, Gamma1, beta1, Gamma2, beta2, alpha):  # fit_models.py:615-659
    return A * (alpha * np.exp(-((x * Gamma1) ** beta1)) + (1 - alpha) * np.exp(-((x * Gamma2) ** beta2)))


def _fs_isf(x, A, Gamma, sigma):  # fit_models.py:690-735
    return A * (1 + sigma**2 * Gamma * x) ** (-1 / sigma**2)


def _gexp_sf(x, A, B, Gamma, beta):  # fit_models.py:774-808
    return A * (1 - _gexp_isf(x, 1.0, Gamma, beta)) + B


def _dexp_sf(x, A, B, Gamma1, beta1, Gamma2, beta2, alpha):  # fit_models.py:890-936
    return A * (1 - _dexp_isf(x, 1.0, Gamma1, beta1, Gamma2, beta2, alpha)) + B


def _fs_sf(x, A, B, Gamma, sigma):  # fit_models.py:971-1017
    return A * (1 - _fs_isf(x, 1.0, Gamma, sigma)) + B


def _simple_exp(dt, tau, amplitude):  # fit.py:67-74
    return amplitude * np.exp(-dt / tau)


def _simple_sf(dt, A, B, tau):  # fit.py:84-88
    return A * (1 - _simple_exp(dt, tau, 1.0)) + B


INF = np.inf
# name -> (function, parameter names, hints {name: (value, min, max, vary)})
MODELS: Dict[str, tuple] = {
    "generic_exponential_isf_model": (_gexp_isf, ["A", "Gamma", "beta"],
                                      {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                       "beta": (1.0, EPSILON, INF, True)}),
    "simple_exponential_isf_model": (_gexp_isf, ["A", "Gamma", "beta"],
                                     {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                      "beta": (1.0, -INF, INF, False)}),
    "stretched_exponential_isf_model": (_gexp_isf, ["A", "Gamma", "beta"],
                                        {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                         "beta": (1.0, EPSILON, 1.0, True)}),
    "compressed_exponential_isf_model": (_gexp_isf, ["A", "Gamma", "beta"],
                                         {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                          "beta": (1.0, 1.0, INF, True)}),
    "double_exponential_isf_model": (_dexp_isf, ["A", "Gamma1", "beta1", "Gamma2", "beta2", "alpha"],
                                     {"A": (1.0, EPSILON, INF, True), "Gamma1": (1.0, EPSILON, INF, True),
                                      "beta1": (1.0, EPSILON, INF, True), "Gamma2": (1.0, EPSILON, INF, True),
                                      "beta2": (1.0, EPSILON, INF, True), "alpha": (1.0, 0.0, 1.0, True)}),
    "flory_schulz_isf_model": (_fs_isf, ["A", "Gamma", "sigma"],
                               {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                "sigma": (1.0, EPSILON, 1.0, True)}),
    "exponential_distribution_isf_model": (_fs_isf, ["A", "Gamma", "sigma"],
                                           {"A": (1.0, EPSILON, INF, True), "Gamma": (1.0, EPSILON, INF, True),
                                            "sigma": (1.0, -INF, INF, False)}),
    "generic_exponential_model": (_gexp_sf, ["A", "B", "Gamma", "beta"],
                                  {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                   "Gamma": (1.0, EPSILON, INF, True), "beta": (1.0, EPSILON, INF, True)}),
    "simple_exponential_model": (_gexp_sf, ["A", "B", "Gamma", "beta"],
                                 {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                  "Gamma": (1.0, EPSILON, INF, True), "beta": (1.0, -INF, INF, False)}),
    "stretched_exponential_model": (_gexp_sf, ["A", "B", "Gamma", "beta"],
                                    {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                     "Gamma": (1.0, EPSILON, INF, True), "beta": (1.0, EPSILON, 1.0, True)}),
    "compressed_exponential_model": (_gexp_sf, ["A", "B", "Gamma", "beta"],
                                     {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                      "Gamma": (1.0, EPSILON, INF, True), "beta": (1.0, 1.0, INF, True)}),
    "double_exponential_model": (_dexp_sf, ["A", "B", "Gamma1", "beta1", "Gamma2", "beta2", "alpha"],
                                 {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                  "Gamma1": (1.0, EPSILON, INF, True), "beta1": (1.0, EPSILON, INF, True),
                                  "Gamma2": (1.0, EPSILON, INF, True), "beta2": (1.0, EPSILON, INF, True),
                                  "alpha": (1.0, 0.0, 1.0, True)}),
    "flory_schulz_model": (_fs_sf, ["A", "B", "Gamma", "sigma"],
                           {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                            "Gamma": (1.0, EPSILON, INF, True), "sigma": (1.0, EPSILON, 1.0, True)}),
    "exponential_distribution_model": (_fs_sf, ["A", "B", "Gamma", "sigma"],
                                       {"A": (1.0, EPSILON, INF, True), "B": (0.0, -INF, INF, True),
                                        "Gamma": (1.0, EPSILON, INF, True), "sigma": (1.0, -INF, INF, False)}),
    # fit.py:77-81 (tau in [0, inf), amplitude in [0, 2]) and :91-95 (A, B, tau in [0, inf))
    "simple_exp_model": (_simple_exp, ["tau", "amplitude"],
                         {"tau": (None, 0.0, INF, True), "amplitude": (None, 0.0, 2.0, True)}),
    "simple_structure_function": (_simple_sf, ["A", "B", "tau"],
                                  {"A": (1.0, 0.0, INF, True), "B": (0.0, 0.0, INF, True),
                                   "tau": (1.0, 0.0, INF, True)}),
}


def make_params(name: str) -> Dict[str, dict]:
    """The model's parameters from its hints: {name: {value, min, max, vary}}."""
    _, names, hints = MODELS[name]
    out = {}
    for p in names:
        v, lo, hi, vary = hints[p]
        out[p] = {"value": v, "min": lo, "max": hi, "vary": vary}
    return out


# ---------------------------------------------------------------------------
# lmfit's bounded-parameter mappings (MINUIT transformations)
# ---------------------------------------------------------------------------


def _kind(lo: float, hi: float) -> int:
    return (0 if lo == -INF else 1) + (0 if hi == INF else 2)


def to_internal(v: float, lo: float, hi: float) -> float:
    k = _kind(lo, hi)
    if k == 0:
        return v
    if k == 1:
        return np.sqrt((v - lo + 1.0) ** 2 - 1)
    if k == 2:
        return np.sqrt((hi - v + 1.0) ** 2 - 1)
    return np.arcsin(2 * (v - lo) / (hi - lo) - 1)


def from_internal(u: float, lo: float, hi: float) -> float:
    k = _kind(lo, hi)
    if k == 0:
        return u
    if k == 1:
        return lo - 1.0 + np.sqrt(u * u + 1)
    if k == 2:
        return hi + 1 - np.sqrt(u * u + 1)
    return lo + (np.sin(u) + 1) * (hi - lo) / 2.0


def scale_gradient(u: float, lo: float, hi: float) -> float:
    k = _kind(lo, hi)
    if k == 0:
        return 1.0
    if k == 1:
        return u / np.sqrt(u * u + 1.0)
    if k == 2:
        return -u / np.sqrt(u * u + 1.0)
    return np.cos(u) * (hi - lo) / 2.0


class FitFailed(ValueError):
    """lmfit's nan_policy='raise' error."""


def lm_fit(func, names: Sequence[str], params: Dict[str, dict], x: np.ndarray, y: np.ndarray,
           weights: Optional[np.ndarray] = None, max_nfev: Optional[int] = None) -> dict:
    """One lmfit ``Model.fit(y, params, x=x, weights=weights)`` with method 'leastsq'.

    Returns {values, stderr, success, ier, nfev, chisqr, redchi, residual}.
    """
    y = np.asarray(y, dtype=np.float64)
    if not np.all(np.isfinite(y)):
        raise FitFailed("The input contains nan values")
    vals, lo, hi, vary = {}, {}, {}, {}
    for p in names:
        d = params[p]
        lmin = -INF if d.get("min") is None else float(d["min"])
        lmax = INF if d.get("max") is None else float(d["max"])
        if lmin > lmax:
            lmin, lmax = lmax, lmin
        if np.isclose(lmin, lmax, atol=1e-13, rtol=1e-13):
            raise ValueError(f"Parameter '{p}' has min == max")
        v = float(d["value"])
        if v > lmax:
            v = lmax
        if v < lmin:
            v = lmin
        vals[p], lo[p], hi[p], vary[p] = v, lmin, lmax, bool(d.get("vary", True))
    var = [p for p in names if vary[p]]
    nv = len(var)
    limit = 2000 * (nv + 1) if max_nfev is None else int(max_nfev)
    state = {"nfev": 0}

    def external(u):
        e = dict(vals)
        for i, p in enumerate(var):
            e[p] = from_internal(u[i], lo[p], hi[p])
        return e

    class _Abort(Exception):
        pass

    def resid(u):
        state["nfev"] += 1
        if state["nfev"] > limit:
            raise _Abort()
        e = external(u)
        r = func(x, *[e[p] for p in names]) - y
        if weights is not None:
            r = r * weights
        r = np.asarray(r, dtype=np.float64).ravel()
        if not np.all(np.isfinite(r)):
            raise FitFailed("The model function generated NaN values and the fit aborted!")
        return r

    u0 = np.array([to_internal(vals[p], lo[p], hi[p]) for p in var], dtype=np.float64)
    aborted = False
    try:
        best, _, info, _, ier = leastsq(resid, u0, full_output=1, xtol=1e-7, ftol=1e-7, gtol=1e-7,
                                        maxfev=2 * limit)
    except _Abort:
        aborted = True
    if aborted:
        return {"values": {p: np.nan for p in names}, "stderr": {p: None for p in names}, "success": False,
                "ier": -1, "nfev": limit, "chisqr": np.nan, "redchi": np.nan, "residual": None, "aborted": True}
    fvec = info["fvec"]
    chisqr = float((fvec ** 2).sum())
    ndata = len(fvec)
    nfree = ndata - nv
    redchi = chisqr / max(1, nfree)
    e = external(best)
    grad = np.array([scale_gradient(best[i], lo[p], hi[p]) for i, p in enumerate(var)])
    ipvt = np.asarray(info["ipvt"]) - 1 if np.min(info["ipvt"]) >= 1 else np.asarray(info["ipvt"])
    fjac = np.transpose(np.transpose(info["fjac"]) / np.take(grad, ipvt))
    rvec = np.dot(np.triu(np.transpose(fjac)[:nv, :]), np.take(np.eye(nv), ipvt, 0))
    try:
        covar = np.linalg.inv(np.dot(np.transpose(rvec), rvec))
    except (np.linalg.LinAlgError, ValueError):
        covar = None
    stderr = {p: None for p in names}
    if covar is not None:
        covar = covar * redchi  # lmfit's result.covar (varying parameters, in order)
        for p in names:
            stderr[p] = 0.0
        for i, p in enumerate(var):
            stderr[p] = float(np.sqrt(covar[i, i]))
    return {"values": e, "stderr": stderr, "success": ier in (1, 2, 3, 4), "ier": int(ier),
            "nfev": int(info["nfev"]), "chisqr": chisqr, "redchi": redchi, "residual": fvec, "aborted": False,
            "covar": covar, "var_names": var}


def fit_multik(func, names: Sequence[str], params: Dict[str, dict], tau: np.ndarray, data: np.ndarray, ref: int,
               err: Optional[np.ndarray] = None, use_err: bool = False, weights: Optional[np.ndarray] = None,
               fixed_params: Optional[Dict[str, Sequence[float]]] = None,
               fixed_params_min: Optional[Dict[str, Sequence[float]]] = None,
               fixed_params_max: Optional[Dict[str, Sequence[float]]] = None) -> dict:
    """The reference's fit_multik sweep (fit.py:282-397): fit ``ref``, then
    ref-1 .. 0 and ref .. K-1, each warm-started from the previous result.

    Returns {param: array, f"{param}_stderr": array, "success": bool array}.
    """
    import copy

    K = data.shape[0]
    mp = copy.deepcopy(params)
    if fixed_params:
        for p, pv in fixed_params.items():
            mp[p]["vary"] = False
            mp[p]["value"] = pv[ref]
    if fixed_params_min:
        for p, pv in fixed_params_min.items():
            mp[p]["min"] = pv[ref]
    if fixed_params_max:
        for p, pv in fixed_params_max.items():
            mp[p]["max"] = pv[ref]
    res = {p: np.zeros(K) for p in names}
    res.update({f"{p}_stderr": np.zeros(K) for p in names})
    res["success"] = np.zeros(K, dtype=bool)
    w = {"weights": weights}

    def store(idx, r):
        for p in names:
            res[p][idx] = r["values"][p]
            res[f"{p}_stderr"][idx] = np.nan if r["stderr"][p] is None else r["stderr"][p]
        res["success"][idx] = r["success"]

    r = lm_fit(func, names, mp, tau, data[ref], weights=w["weights"])
    store(ref, r)

    def sweep(indices):
        for p in names:
            mp[p]["value"] = res[p][ref]
        for idx in indices:
            if np.isnan(data[idx, 0]):
                for p in names:
                    res[p][idx] = np.nan
                    res[f"{p}_stderr"][idx] = np.nan
                continue
            if use_err and err is not None:
                w["weights"] = 1.0 / err[idx]
            if fixed_params:
                for p, pv in fixed_params.items():
                    mp[p]["value"] = pv[idx]
            if fixed_params_min:
                for p, pv in fixed_params_min.items():
                    mp[p]["min"] = pv[idx]
            if fixed_params_max:
                for p, pv in fixed_params_max.items():
                    mp[p]["max"] = pv[idx]
            r = lm_fit(func, names, mp, tau, data[idx], weights=w["weights"])
            store(idx, r)
            for p in names:
                mp[p]["value"] = r["values"][p]

    sweep(reversed(range(ref)))
    sweep(range(ref, K))
    return res
