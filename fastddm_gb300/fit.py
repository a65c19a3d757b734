r"""Fits of the azimuthal average (or the intermediate scattering function) on
the GPU.

Same interface as the reference's ``src/python/fit.py``: ``fit`` fits one
curve, ``fit_multik`` fits every wavevector of an ``AzimuthalAverage`` or
``IntermediateScatteringFunction``, starting at ``ref`` and sweeping towards
lower and then higher k, each fit starting from the previous result
(``fit.py:282-395``).  The fits are lmfit's 'leastsq' (MINPACK lmdif on
lmfit's bounded-parameter mapping) run on the device, one warp per sweep
(``csrc/fit_lm.cuh``); the sweep towards lower k and the one towards higher k
run concurrently, as they only share the fit at ``ref``.

Differences from the reference, where its dependencies are absent here:
``fit_multik`` returns a :class:`FitTable` (columns as the reference's pandas
DataFrame; ``to_pandas()`` converts when pandas is installed); parameter
expressions (``expr``, ``fixed_params_expr``), methods other than 'leastsq'
and ``nan_policy`` other than 'raise' raise ``NotImplementedError``.

``fit_multik(..., warm_start=...)`` also offers two orders the reference does
not have: ``"ref"`` starts every k from the fit at ``ref`` (all k in parallel),
``"none"`` starts every k from the given initial values.  The default,
``"chain"``, is the reference's sweep.
"""

from __future__ import annotations

import copy
import warnings
from typing import Any, Dict, List, Optional, Sequence, Tuple, Union

import numpy as np

from ._fitting import (NAN_MESSAGE, ST_NONFINITE, FitSpec, Model, ModelResult, Parameter, Parameters, check_bounds,
                       lsq_options, run_fits)
from .azimuthalaverage import AzimuthalAverage
from .intermediatescatteringfunction import IntermediateScatteringFunction


def _simple_exp(dt: Union[np.ndarray, float, int], tau: float, amplitude: float) -> Union[np.ndarray, float]:
    """amplitude * exp(-dt / tau) (fit.py:67-74)"""
    return amplitude * np.exp(-dt / tau)


simple_exp_model = Model(_simple_exp, 6)
simple_exp_model.set_param_hint("tau", min=0.0, max=np.inf)
simple_exp_model.set_param_hint("amplitude", min=0.0, max=2.0)


def _simple_image_structure_function(dt: np.ndarray, A: float, B: float, tau: float) -> np.ndarray:
    """A (1 - exp(-dt / tau)) + B (fit.py:84-88)"""
    return A * (1 - _simple_exp(dt, tau, 1.0)) + B


simple_structure_function = Model(_simple_image_structure_function, 7)
simple_structure_function.set_param_hint("A", min=0.0, max=np.inf, value=1.0)
simple_structure_function.set_param_hint("B", min=0.0, max=np.inf, value=0.0)
simple_structure_function.set_param_hint("tau", min=0.0, max=np.inf, value=1.0)


def _simple_structure_function_parameter_helper(xdata: np.ndarray, ydata: np.ndarray) -> Parameters:
    """Starting values for A, B and tau (fit.py:98-121): B from a quadratic fit of the
    first 5 points, A from the last point, tau where the curve crosses half its span."""
    n = 5
    poly = np.polynomial.Polynomial.fit(xdata[:n], ydata[:n], deg=2)
    B = max(poly.coef[0], 0.0)
    A = max(ydata[-1] - B, 0.0)
    if A > 0.0:
        tau = xdata[np.argmin(np.abs((ydata - B) / A - 0.5))]
    else:
        tau = 1.0
    params = Parameters()
    for name, val in {"A": A, "B": B, "tau": tau}.items():
        params.add(name, min=0.0, max=np.inf, value=val)
    return params


def fit(model: Model, xdata: np.ndarray, ydata: np.ndarray, params: Optional[Union[Parameters, Parameter]] = None,
        estimate_simple_parameters: bool = False, verbose: bool = False, **fitargs: Any) -> ModelResult:
    """Fit ``model`` to ``ydata`` at ``xdata`` on the GPU (fit.py:124-194).

    ``fitargs`` go to :meth:`Model.fit` (``weights``, ``fit_kws``, ``max_nfev``, ``gpu_id``...).
    """
    from .fit_models import from_lmfit

    model = from_lmfit(model)
    model_params = model.make_params()
    fitargs[model.independent_vars[0]] = xdata
    if estimate_simple_parameters:
        simple = _simple_structure_function_parameter_helper(xdata, ydata)
        if verbose:
            print(":: updating given parameters with simple estimates .. ")
        model_params.update({k: p for k, p in simple.items() if k in model.param_names})
    if params is not None:
        model_params.update(params)
        if verbose:
            print(":: Model parameters:")
            model_params.pretty_print()
    result = model.fit(ydata, params=model_params, **fitargs)
    if verbose:
        print(":: Fit report:")
        print(result.fit_report())
    return result


class FitTable:
    """Column table of fit_multik results: one row per k; columns are the
    parameters, their standard errors ``<p>_stderr``, ``success`` and ``k``
    (the reference returns the same columns as a pandas DataFrame)."""

    def __init__(self, columns: Dict[str, np.ndarray], device_ms: float = 0.0, launches: int = 0):
        self._cols = dict(columns)
        self.device_ms = device_ms  # time of the fit launches on the device
        self.launches = launches

    @property
    def columns(self) -> List[str]:
        return list(self._cols)

    def __getitem__(self, name: str) -> np.ndarray:
        return self._cols[name]

    def __contains__(self, name: str) -> bool:
        return name in self._cols

    def __len__(self) -> int:
        return len(next(iter(self._cols.values())))

    def keys(self):
        return self._cols.keys()

    def items(self):
        return self._cols.items()

    def to_dict(self) -> Dict[str, np.ndarray]:
        return dict(self._cols)

    def to_records(self) -> np.ndarray:
        return np.rec.fromarrays(list(self._cols.values()), names=list(self._cols))

    def to_pandas(self):
        import pandas as pd  # optional

        return pd.DataFrame(self._cols)

    def __repr__(self) -> str:
        return f"FitTable({len(self)} rows; columns {self.columns})"


def _copy(d):
    return copy.deepcopy(d) if d is not None else None


class _Sweep:
    """The device problems of one fit_multik call (rows, warm starts, launches) and what
    turns their results into the reference's table."""


def _sweep(data, model: Model, ref: int, ref_params, use_err, fixed_params, fixed_params_min, fixed_params_max,
           fixed_params_expr, warm_start: str, fitargs: Dict[str, Any]) -> _Sweep:
    if fixed_params_expr:
        raise NotImplementedError("fixed_params_expr: parameter expressions are not supported by the device fits")
    if warm_start not in ("chain", "ref", "none"):
        raise ValueError("warm_start must be 'chain', 'ref' or 'none'")
    from .fit_models import from_lmfit

    model = from_lmfit(model)
    model_params = model.make_params()
    ref_params = _copy(ref_params)
    fixed_params, fixed_params_min, fixed_params_max = (_copy(fixed_params), _copy(fixed_params_min),
                                                         _copy(fixed_params_max))
    names = model.param_names
    tau = np.asarray(data.tau, dtype=np.float64)
    Y = np.asarray(data.data, dtype=np.float64)
    K = len(data.k)
    if ref_params is not None:
        model_params.update(ref_params)  # lmfit Parameters are converted
    for p in names:
        if p in fitargs:
            model_params[p].value = fitargs.pop(p)
    for d in (fixed_params, fixed_params_min, fixed_params_max):
        for p, pv in (d or {}).items():
            if p not in model_params:
                raise KeyError(p)
            if len(pv) != K:
                raise ValueError(f"'{p}': {len(pv)} values for {K} wavevectors")
    if fixed_params:
        for p in fixed_params:
            model_params[p].vary = False
    method = fitargs.pop("method", "leastsq")
    nan_policy = fitargs.pop("nan_policy", None)
    iter_cb = fitargs.pop("iter_cb", None)
    model.check_fit_args(method, nan_policy, iter_cb)
    scale_covar = fitargs.pop("scale_covar", True)
    calc_covar = fitargs.pop("calc_covar", True)
    options = lsq_options(fitargs.pop("fit_kws", None), fitargs.pop("max_nfev", None))
    fitargs.pop("verbose", None)
    user_w = fitargs.pop("weights", None)
    fitargs.pop(model.independent_vars[0], None)
    for n in fitargs:
        warnings.warn(f"The keyword argument {n} does not match any arguments of the model function. "
                      "It will be ignored.", UserWarning)

    # weight rows: the user's weights (shared by every k), then 1 / err per k
    rows = []
    w_user = -1
    if user_w is not None:
        w_user = 0
        rows.append(np.broadcast_to(np.asarray(user_w, dtype=np.float64), tau.shape))
    err_base = -1
    if use_err and data.err is not None:
        err_base = len(rows)
        with np.errstate(divide="ignore"):
            rows.extend(1.0 / np.asarray(data.err, dtype=np.float64))
    W = np.stack(rows) if rows else None

    # starting values and bounds of every k (fit.py:311-329, :362-377)
    base = FitSpec(model, model_params)
    init = np.tile(base.init, (K, 1))
    lo = np.tile(base.lo, (K, 1))
    hi = np.tile(base.hi, (K, 1))
    col = {n: j for j, n in enumerate(names)}
    for p, pv in (fixed_params or {}).items():
        init[:, col[p]] = np.asarray(pv, dtype=np.float64)
    for p, pv in (fixed_params_min or {}).items():
        lo[:, col[p]] = np.asarray(pv, dtype=np.float64)
    for p, pv in (fixed_params_max or {}).items():
        hi[:, col[p]] = np.asarray(pv, dtype=np.float64)
    if np.any(np.isnan(init)):
        raise ValueError("a parameter has value NaN")
    lo, hi = check_bounds(lo, hi, names)

    # the fits in the reference's order: ref, then ref-1 .. 0, then ref .. K-1; rows whose first
    # value is NaN are skipped (fit.py:356)
    valid = ~np.isnan(Y[:, 0])
    down = [i for i in range(ref - 1, -1, -1) if valid[i]]
    upk = [i for i in range(ref, K) if valid[i]]
    wrow = (err_base + np.arange(K)) if err_base >= 0 else np.full(K, w_user)
    if warm_start == "none":
        ks = np.array(down + upk, dtype=np.int64)
        wr = wrow[ks]
        pred = np.full(ks.size, -1)
        stages = [[[i] for i in range(ks.size)]]
    else:
        ks = np.array([ref] + down + upk, dtype=np.int64)
        wr = np.concatenate([[w_user], wrow[ks[1:]]])  # the fit at ref takes the weights given (fit.py:337)
        nd, nu = len(down), len(upk)
        pred = np.empty(ks.size, dtype=np.int64)
        pred[0] = -1
        if warm_start == "chain":  # each fit starts from the previous one of its sweep, the first from ref
            pred[1:] = np.arange(ks.size - 1)
            if nd:
                pred[1] = 0
            if nu:
                pred[nd + 1] = 0
            stages = [[[0]], [c for c in (list(range(1, nd + 1)), list(range(nd + 1, nd + nu + 1))) if c]]
        else:
            pred[1:] = 0
            stages = [[[0]], [[i] for i in range(1, ks.size)]]
        stages = [st for st in stages if st]
    bad = ~np.all(np.isfinite(Y[ks]), axis=1)
    if np.any(bad):  # lmfit refuses data with NaN (nan_policy 'raise') at the first such fit
        raise ValueError("The input contains nan values")
    problems = np.stack([ks, wr, pred, np.full(ks.size, base.vary), np.zeros(ks.size, np.int64),
                         np.full(ks.size, tau.size)], axis=1).astype(np.int32)
    sw = _Sweep()
    sw.model, sw.names, sw.K, sw.tau, sw.Y, sw.W = model, names, K, tau, Y, W
    sw.problems, sw.stages, sw.init, sw.lo, sw.hi = problems, stages, init[ks], lo[ks], hi[ks]
    sw.ks, sw.wr, sw.pred, sw.base, sw.model_params = ks, wr, pred, base, model_params
    sw.k = np.asarray(data.k)
    sw.options, sw.scale_covar, sw.calc_covar = options, scale_covar, calc_covar
    sw.init_k, sw.lo_k, sw.hi_k = init, lo, hi
    return sw


def _sweep_results(sw: _Sweep, out: Dict[str, Any], return_model_results: bool):
    """The reference's table (and ModelResults) from the library's outputs for this sweep's problems."""
    model, names, K, tau, Y, W = sw.model, sw.names, sw.K, sw.tau, sw.Y, sw.W
    ks, wr, pred, base, model_params = sw.ks, sw.wr, sw.pred, sw.base, sw.model_params
    init, lo, hi = sw.init_k, sw.lo_k, sw.hi_k
    scale_covar, calc_covar = sw.scale_covar, sw.calc_covar
    # each k's result is its last fit (the refit at ref replaces the first fit there)
    final = np.full(K, -1)
    final[ks] = np.arange(ks.size)
    vals = out["values"][:, : len(names)]
    errs = out["stderr"][:, : len(names)].copy()
    nfree = np.maximum(1, Y.shape[1] - out["nvary"])
    if not calc_covar:
        errs[:] = np.nan
    errs[errs < 0] = np.nan  # no covariance: None in lmfit, NaN in the table
    if not scale_covar:
        redchi = out["chisqr"] / nfree
        varying = np.array([(base.vary >> j) & 1 for j in range(len(names))], dtype=bool)
        with np.errstate(invalid="ignore", divide="ignore"):
            errs[:, varying] /= np.sqrt(redchi)[:, None]
    results: Dict[str, np.ndarray] = {}
    have = final >= 0
    for j, p in enumerate(names):
        results[p] = np.full(K, np.nan)
        results[p][have] = vals[final[have], j]
    for j, p in enumerate(names):
        results[f"{p}_stderr"] = np.full(K, np.nan)
        results[f"{p}_stderr"][have] = errs[final[have], j]
    ok = (out["info"] >= 1) & (out["info"] <= 4) & (out["status"] == 0)
    results["success"] = np.zeros(K, dtype=bool)
    results["success"][have] = ok[final[have]]
    results["k"] = sw.k
    model_results: Optional[List[Optional[ModelResult]]] = None
    if return_model_results:
        model_results = [None] * K
        for k in np.flatnonzero(have):
            pi = int(final[k])
            start = copy.deepcopy(model_params)
            for j, n in enumerate(names):
                v = init[k, j]
                if pred[pi] >= 0 and (base.vary >> j) & 1:  # started from the previous fit, clipped
                    v = min(max(float(out["values"][pred[pi]][j]), lo[k, j]), hi[k, j])
                start[n].value = float(v)
                start[n].min, start[n].max = float(lo[k, j]), float(hi[k, j])
            w = None if wr[pi] < 0 else W[wr[pi]]
            model_results[k] = ModelResult(model, start, Y[k], tau, w, out, pi, scale_covar, calc_covar)
    return FitTable(results, out["device_ms"], out["launches"]), model_results


def fit_multik(data: Union[AzimuthalAverage, IntermediateScatteringFunction], model: Model, ref: int,
               ref_params: Optional[Parameters] = None, return_model_results: Optional[bool] = False,
               use_err: Optional[bool] = False, fixed_params: Optional[Dict[str, Sequence[float]]] = None,
               fixed_params_min: Optional[Dict[str, Sequence[float]]] = None,
               fixed_params_max: Optional[Dict[str, Sequence[float]]] = None,
               fixed_params_expr: Optional[Dict[str, Sequence[str]]] = None, *, warm_start: str = "chain",
               gpu_id: int = 0, **fitargs: Any) -> Tuple[FitTable, Optional[List[Optional[ModelResult]]]]:
    """Fit ``model`` to every k of ``data`` on the GPU (fit.py:197-397).

    Parameters as the reference: the fit at ``ref`` starts from the model's
    values (updated by ``ref_params`` and parameter values given as keyword
    arguments); the sweeps ref-1 .. 0 and ref .. K-1 start each fit from the
    previous one; ``use_err`` weights each k by 1 / ``data.err[k]``;
    ``fixed_params*`` give per-k values and bounds.  Rows whose first value is
    NaN are skipped (NaN results).  ``warm_start``: "chain" (the reference's
    sweep), "ref" or "none" (see the module docstring).
    """
    sw = _sweep(data, model, ref, ref_params, use_err, fixed_params, fixed_params_min, fixed_params_max,
                fixed_params_expr, warm_start, dict(fitargs))
    out = run_fits(sw.model, sw.tau[None, :], sw.Y, sw.W, sw.problems, sw.stages, sw.init, sw.lo, sw.hi,
                   sw.options, gpu_id, covariance=bool(return_model_results) and sw.calc_covar)
    if np.any(out["status"] == ST_NONFINITE):
        raise ValueError(NAN_MESSAGE)
    return _sweep_results(sw, out, bool(return_model_results))


def fit_multik_batch(jobs: Sequence[Dict[str, Any]], model: Model, *, warm_start: str = "chain", gpu_id: int = 0,
                     return_model_results: bool = False, **common: Any
                     ) -> List[Tuple[FitTable, Optional[List[Optional[ModelResult]]]]]:
    """``fit_multik`` of many datasets in one pair of device launches.

    Each job is a dict with ``data`` and ``ref`` and any other argument of
    :func:`fit_multik` for that dataset (``ref_params``, ``use_err``,
    ``fixed_params``..., parameter values such as ``A=``); ``common`` holds
    arguments shared by every job (``fit_kws``, ``max_nfev``, ``weights``...).
    Datasets may differ in their number of k and of lags.  Every fit gives
    what it gives in a ``fit_multik`` call of its own; all sweeps run
    concurrently, the fits at the jobs' ``ref`` first.  The jobs must vary the
    same number of parameters.  Returns one (table, model results) per job.
    """
    if not jobs:
        return []
    sweeps = []
    for job in jobs:
        kw = dict(common)
        kw.update({k: v for k, v in job.items() if k not in ("data", "ref")})
        args = [kw.pop(n, None) for n in ("ref_params", "use_err", "fixed_params", "fixed_params_min",
                                           "fixed_params_max", "fixed_params_expr")]
        args[1] = bool(args[1])
        sweeps.append(_sweep(job["data"], model, job["ref"], *args, warm_start, kw))
    options = sweeps[0].options
    if any(not np.array_equal(sw.options, options) for sw in sweeps):
        raise ValueError("the jobs of one batch share fit_kws and max_nfev")
    nv = {int(sw.base.vary) for sw in sweeps}
    if len({bin(v).count("1") for v in nv}) != 1:
        raise ValueError("the jobs of one batch must vary the same number of parameters")
    m = max(sw.tau.size for sw in sweeps)

    def pad(a):
        out = np.zeros((a.shape[0], m))
        out[:, : a.shape[1]] = a
        return out

    X = np.stack([np.pad(sw.tau, (0, m - sw.tau.size)) for sw in sweeps])
    Ys, Ws, probs, inits, los, his = [], [], [], [], [], []
    nstage = max(len(sw.stages) for sw in sweeps)
    stages: List[List[List[int]]] = [[] for _ in range(nstage)]
    yoff = woff = poff = 0
    offsets = []
    for i, sw in enumerate(sweeps):
        pr = sw.problems.astype(np.int64).copy()
        pr[:, 0] += yoff
        pr[:, 1] = np.where(pr[:, 1] >= 0, pr[:, 1] + woff, -1)
        pr[:, 2] = np.where(pr[:, 2] >= 0, pr[:, 2] + poff, -1)
        pr[:, 4] = i
        probs.append(pr)
        Ys.append(pad(sw.Y))
        if sw.W is not None:
            Ws.append(pad(sw.W))
        inits.append(sw.init)
        los.append(sw.lo)
        his.append(sw.hi)
        # a sweep with one launch (warm_start "none") runs with the others' second launch
        first = nstage - len(sw.stages)
        for s, chains in enumerate(sw.stages):
            stages[first + s].extend([[p + poff for p in c] for c in chains])
        offsets.append(poff)
        yoff += sw.Y.shape[0]
        woff += 0 if sw.W is None else sw.W.shape[0]
        poff += pr.shape[0]
    W = np.concatenate(Ws) if Ws else None
    out = run_fits(sweeps[0].model, X, np.concatenate(Ys), W, np.concatenate(probs).astype(np.int32),
                   [st for st in stages if st], np.concatenate(inits), np.concatenate(los), np.concatenate(his),
                   options, gpu_id, covariance=return_model_results)
    results = []
    for i, (sw, off) in enumerate(zip(sweeps, offsets)):
        n = sw.problems.shape[0]
        part = {k: (v[off:off + n] if isinstance(v, np.ndarray) else v) for k, v in out.items()}
        if np.any(part["status"] == ST_NONFINITE):
            raise ValueError(f"job {i}: " + NAN_MESSAGE)
        results.append(_sweep_results(sw, part, return_model_results))
    return results
