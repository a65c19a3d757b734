"""Parameters, models and fit results for the device fits.

The reference fits through lmfit (``src/python/fit.py``, ``fit_models.py``);
lmfit is not a dependency here.  This module supplies the part of lmfit's
interface those files use (``Parameter``, ``Parameters``, ``Model`` with
``set_param_hint`` / ``make_params`` / ``eval`` / ``fit``, ``ModelResult``),
with the same names, argument meanings and errors, and runs every fit on the
GPU (``fddm_b200_fit_lm``, one warp per chain of fits; ``csrc/fit_lm.cuh``).
Only lmfit's default method, 'leastsq' (MINPACK lmdif), is provided.
"""

from __future__ import annotations

import copy
import ctypes
import math
import warnings
from typing import Any, Dict, Iterable, List, Optional, Sequence

import numpy as np

from . import _lib

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

INF = float("inf")

# lmdif options (host array passed to the library): ftol, xtol, gtol, epsfcn, factor, max_nfev
_LSQ_DEFAULTS = {"ftol": 1e-7, "xtol": 1e-7, "gtol": 1e-7, "epsfcn": 0.0, "factor": 100.0}
_FIT_KWS = set(_LSQ_DEFAULTS) | {"maxfev"}
# result status codes of the library
ST_OK, ST_NONFINITE, ST_ABORTED, ST_INVALID = 0, 1, 2, 3
NAN_MESSAGE = ("The model function generated NaN values and the fit aborted! Please check your model function "
               "and/or set boundaries on parameters where applicable.")


class Parameter:
    """One fit parameter: value, bounds, whether it varies, and after a fit its standard error."""

    def __init__(self, name: str, value: Optional[float] = None, vary: bool = True, min: Optional[float] = -INF,
                 max: Optional[float] = INF, expr: Optional[str] = None, brute_step=None, user_data=None):
        self.name = name
        self.value = value
        self.vary = bool(vary)
        self.min = -INF if min is None else min
        self.max = INF if max is None else max
        self.expr = expr
        self.brute_step = brute_step
        self.user_data = user_data
        self.stderr: Optional[float] = None
        self.correl = None
        self.init_value = value

    def set(self, value=None, vary=None, min=None, max=None, expr=None, brute_step=None):
        if value is not None:
            self.value = value
        if vary is not None:
            self.vary = bool(vary)
        if min is not None:
            self.min = min
        if max is not None:
            self.max = max
        if expr is not None:
            self.expr = expr
        if brute_step is not None:
            self.brute_step = brute_step

    def __repr__(self) -> str:
        s = [f"value={self.value!r}"]
        s.append("(fixed)" if not self.vary else f"+/- {self.stderr:.3g}" if self.stderr is not None else "")
        s.append(f"bounds=[{self.min}:{self.max}]")
        return f"<Parameter '{self.name}', " + ", ".join(x for x in s if x) + ">"


class Parameters(dict):
    """Ordered name -> Parameter mapping (lmfit.Parameters)."""

    def add(self, name, value=None, vary=True, min=-INF, max=INF, expr=None, brute_step=None):
        if isinstance(name, Parameter):
            self[name.name] = copy.copy(name)
        else:
            self[name] = Parameter(name, value=value, vary=vary, min=min, max=max, expr=expr, brute_step=brute_step)

    def add_many(self, *parlist):
        for p in parlist:
            if isinstance(p, Parameter):
                self.add(p)
            else:
                self.add(*p)

    def __setitem__(self, key, par):
        if not isinstance(par, Parameter):
            raise ValueError(f"'{par}' is not a Parameter")
        par.name = key
        super().__setitem__(key, par)

    def update(self, other=(), **kw):
        """Add or replace parameters; lmfit Parameter objects (anything with value, vary,
        min, max and expr) are converted."""
        if isinstance(other, Parameter) or hasattr(other, "vary") and hasattr(other, "name"):
            other = {other.name: other}
        items = other.items() if hasattr(other, "items") else other
        for k, p in list(items) + list(kw.items()):
            self[k] = as_parameter(k, p)
        return self

    def valuesdict(self) -> Dict[str, float]:
        return {k: p.value for k, p in self.items()}

    def copy(self) -> "Parameters":
        return copy.deepcopy(self)

    def __deepcopy__(self, memo):
        out = Parameters()
        for k, p in self.items():
            out[k] = copy.deepcopy(p, memo)
        return out

    def pretty_print(self) -> None:
        print(f"{'Name':<10}{'Value':>14}{'Min':>12}{'Max':>12}{'Stderr':>12}{'Vary':>6}")
        for k, p in self.items():
            se = "None" if p.stderr is None else f"{p.stderr:.5g}"
            print(f"{k:<10}{p.value!s:>14.12}{p.min!s:>12.8}{p.max!s:>12.8}{se:>12}{p.vary!s:>6}")


def as_parameter(name: str, p) -> Parameter:
    """A copy of ``p`` as a Parameter (``p`` may be an lmfit Parameter)."""
    if isinstance(p, Parameter):
        return copy.copy(p)
    q = Parameter(name, value=getattr(p, "value", None), vary=getattr(p, "vary", True),
                  min=getattr(p, "min", -INF), max=getattr(p, "max", INF), expr=getattr(p, "expr", None))
    q.stderr = getattr(p, "stderr", None)
    return q


def _start_value(p: Parameter) -> float:
    v = -INF if p.value is None else float(p.value)
    if math.isnan(v):
        raise ValueError(f"Parameter '{p.name}' has value NaN")
    return v


class FitSpec:
    """One curve to fit: parameter values, bounds and vary flags in the model's parameter order."""

    __slots__ = ("init", "lo", "hi", "vary")

    def __init__(self, model: "Model", params: Parameters):
        names = model.param_names
        missing = [n for n in names if n not in params]
        if missing:
            raise ValueError(f"missing parameter(s) {missing} for model '{model.name}'")
        for n, p in params.items():
            if p.expr is not None and n in names:
                raise NotImplementedError("parameter expressions (expr) are not supported by the device fits")
        self.init = np.array([_start_value(params[n]) for n in names], dtype=np.float64)
        lo = np.array([-INF if params[n].min is None else float(params[n].min) for n in names], dtype=np.float64)
        hi = np.array([INF if params[n].max is None else float(params[n].max) for n in names], dtype=np.float64)
        self.lo, self.hi = check_bounds(lo, hi, names)
        self.vary = sum(1 << i for i, n in enumerate(names) if params[n].vary)
        if self.vary == 0:
            raise ValueError("no parameter varies")


def lsq_options(fit_kws: Optional[dict], max_nfev: Optional[int]) -> np.ndarray:
    """lmdif options array for the library (lmfit's leastsq defaults, overridden by fit_kws)."""
    kw = dict(_LSQ_DEFAULTS)
    for k, v in (fit_kws or {}).items():
        if k not in _FIT_KWS:
            raise NotImplementedError(f"fit_kws '{k}' is not supported by the device fits")
        if k != "maxfev":
            kw[k] = float(v)
    limit = max_nfev if max_nfev is not None else (fit_kws or {}).get("maxfev")
    return np.array([kw["ftol"], kw["xtol"], kw["gtol"], kw["epsfcn"], kw["factor"],
                     0.0 if limit is None else float(limit)], dtype=np.float64)


def _device(gpu_id: int):
    if torch is None or not torch.cuda.is_available():
        raise RuntimeError("the device fits need a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", gpu_id)


def check_bounds(lo: np.ndarray, hi: np.ndarray, names: Sequence[str]):
    """lmfit's bound rules on arrays of bounds: swapped when reversed, min == max refused."""
    lo, hi = np.minimum(lo, hi), np.maximum(lo, hi)
    with np.errstate(invalid="ignore"):
        same = np.isclose(lo, hi, rtol=1e-13, atol=1e-13)
    if np.any(same):
        j = int(np.argwhere(same)[0][-1])
        raise ValueError(f"Parameter '{names[j]}' has min == max")
    return lo, hi


def run_fits(model: "Model", X: np.ndarray, Y: np.ndarray, W: Optional[np.ndarray], problems: np.ndarray,
             stages: Sequence[Sequence[Sequence[int]]], init: np.ndarray, lo: np.ndarray, hi: np.ndarray,
             options: np.ndarray, gpu_id: int = 0, residual: bool = False,
             covariance: bool = False) -> Dict[str, np.ndarray]:
    """Run the fits on the device.

    X, Y, W: rows of abscissae, data and weights (W may be None), as wide as
    the longest problem; problems: int32 (P, 6) rows (y row, weight row or -1,
    pred or -1, vary mask, x row, number of points); stages: launches in order,
    each a list of chains (lists of problem indices); init, lo, hi: (P, nparams)
    starting values and bounds.  The result holds the library's outputs and
    ``device_ms``, the time of the launches on the device.
    """
    lib = _lib.load()
    dev = _device(gpu_id)
    P = int(problems.shape[0])
    npar = lib.fddm_b200_fit_model_nparams(model.device_id)
    nvs = {bin(int(mk)).count("1") for mk in np.unique(problems[:, 3])}
    if len(nvs) != 1:
        raise ValueError("all fits of one call must vary the same number of parameters")
    nvary = nvs.pop()
    X = np.atleast_2d(X)
    m = int(X.shape[1])
    small = int(problems[:, 5].min())
    if small < nvary:
        raise TypeError(f"Improper input: func (m={small}) must be >= n={nvary}")
    f64 = dict(dtype=torch.float64, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)

    def up(a, kind):
        return torch.as_tensor(np.array(a, dtype=np.float64 if kind is f64 else np.int32, order="C"), **kind)

    dx, dy = up(X, f64), up(Y, f64)
    dw = None if W is None else up(W, f64)
    dprob, dinit, dlo, dhi = up(problems, i32), up(init, f64), up(lo, f64), up(hi, f64)
    vals = torch.empty((P, npar), **f64)
    se = torch.empty((P, npar), **f64)
    chisqr = torch.empty(P, **f64)
    nfev = torch.empty(P, **i32)
    info = torch.empty(P, **i32)
    status = torch.empty(P, **i32)
    res = torch.empty((P, m), **f64) if residual else None
    cov = torch.empty((P, npar, npar), **f64) if covariance else None
    most = max(len(s) for s in stages)
    nbytes = ctypes.c_uint64(0)
    _lib.check(lib.fddm_b200_fit_workspace_bytes(model.device_id, m, most, ctypes.byref(nbytes)))
    ws = torch.empty(max(1, nbytes.value // 8), **f64)
    opts = np.ascontiguousarray(options, dtype=np.float64)
    chain_tabs = []
    for chains in stages:
        offs = np.zeros(len(chains) + 1, dtype=np.int32)
        offs[1:] = np.cumsum([len(c) for c in chains])
        flat = np.fromiter((p for c in chains for p in c), dtype=np.int32, count=int(offs[-1]))
        chain_tabs.append((up(offs, i32), up(flat, i32), len(chains)))
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for doff, dlist, nch in chain_tabs:
            _lib.check(lib.fddm_b200_fit_lm(
                model.device_id, m, dx.data_ptr(), dx.shape[1], dx.shape[0], dy.data_ptr(), dy.shape[1], dy.shape[0],
                None if dw is None else dw.data_ptr(), 0 if dw is None else dw.shape[1],
                0 if dw is None else dw.shape[0],
                dprob.data_ptr(), P, doff.data_ptr(), dlist.data_ptr(), nch, nvary,
                dinit.data_ptr(), dlo.data_ptr(), dhi.data_ptr(), opts.ctypes.data,
                vals.data_ptr(), se.data_ptr(), chisqr.data_ptr(), nfev.data_ptr(), info.data_ptr(),
                status.data_ptr(), None if res is None else res.data_ptr(), None if cov is None else cov.data_ptr(),
                ws.data_ptr(), ws.numel() * 8,
                stream.cuda_stream))
        t1.record(stream)
        stream.synchronize()
    out = {"values": vals.cpu().numpy(), "stderr": se.cpu().numpy(), "chisqr": chisqr.cpu().numpy(),
           "nfev": nfev.cpu().numpy(), "info": info.cpu().numpy(), "status": status.cpu().numpy(),
           "nvary": nvary, "device_ms": t0.elapsed_time(t1), "launches": len(chain_tabs)}
    if res is not None:
        out["residual"] = res.cpu().numpy()
    if cov is not None:
        out["covar"] = cov.cpu().numpy()
    if np.any(out["status"] == ST_INVALID):
        raise RuntimeError("fit problems named rows or predecessors that do not exist")
    return out


class ModelResult:
    """Result of one fit (lmfit.model.ModelResult)."""

    def __init__(self, model: "Model", params: Parameters, data: np.ndarray, x: np.ndarray,
                 weights: Optional[np.ndarray], out: Dict[str, np.ndarray], k: int, scale_covar: bool = True,
                 calc_covar: bool = True):
        names = model.param_names
        self.model = model
        self.method = "leastsq"
        self.data = data
        self.weights = weights
        self.userkws = {model.independent_vars[0]: x}
        self.init_params = copy.deepcopy(params)
        self.init_values = {n: params[n].value for n in names}
        st = int(out["status"][k])
        self.ier = int(out["info"][k])
        self.aborted = st == ST_ABORTED
        self.success = (1 <= self.ier <= 4) and st == ST_OK
        self.nfev = int(out["nfev"][k])
        self.ndata = int(data.shape[0])
        self.nvarys = int(out["nvary"])
        self.nfree = self.ndata - self.nvarys
        self.chisqr = float(out["chisqr"][k])
        self.redchi = self.chisqr / max(1, self.nfree)
        with np.errstate(divide="ignore", invalid="ignore"):
            neg2ll = self.ndata * np.log(self.chisqr / self.ndata)
        self.aic = float(neg2ll + 2 * self.nvarys)
        self.bic = float(neg2ll + np.log(self.ndata) * self.nvarys)
        self.message = {1: "Fit succeeded.", 2: "Fit succeeded.", 3: "Fit succeeded.",
                        4: "Fit succeeded. Could not estimate error-bars?"}.get(
            self.ier, "Fit aborted." if self.aborted else "Tolerance seems to be too small.")
        self.params = copy.deepcopy(params)
        self.var_names = [n for n in names if params[n].vary]
        errs = out["stderr"][k]
        # the library's standard errors: -1 without a covariance (None here), NaN where it is not finite
        self.errorbars = bool(calc_covar and all(errs[i] > 0.0 for i, n in enumerate(names) if params[n].vary))
        for i, n in enumerate(names):
            p = self.params[n]
            p.value = float(out["values"][k][i])
            s = float(errs[i])
            if not calc_covar or s < 0.0:
                p.stderr = None
            elif scale_covar or not self.params[n].vary or not math.isfinite(s):
                p.stderr = s
            else:
                p.stderr = s / math.sqrt(self.redchi) if self.redchi > 0 else s
        self.best_values = {n: self.params[n].value for n in names}
        # lmfit's covar: the varying parameters' covariance in var_names order (None without one)
        self.covar = None
        if "covar" in out and calc_covar:
            idx = [i for i, n in enumerate(names) if params[n].vary]
            c = out["covar"][k][np.ix_(idx, idx)]
            if np.all(np.isfinite(c)) and all(self.params[n].stderr is not None for n in self.var_names):
                if not scale_covar and self.redchi > 0:
                    c = c / self.redchi
                self.covar = c
                for a, na in enumerate(self.var_names):
                    pa = self.params[na]
                    pa.correl = {nb: float(c[a, b] / np.sqrt(c[a, a] * c[b, b]))
                                 for b, nb in enumerate(self.var_names) if b != a}
        self.residual = out["residual"][k] if "residual" in out else None

    @property
    def best_fit(self) -> np.ndarray:
        return self.model.eval(self.params, **self.userkws)

    @property
    def init_fit(self) -> np.ndarray:
        return self.model.eval(self.init_params, **self.userkws)

    def eval(self, params=None, **kwargs) -> np.ndarray:
        kw = dict(self.userkws)
        kw.update(kwargs)
        return self.model.eval(self.params if params is None else params, **kw)

    def fit_report(self) -> str:
        lines = ["[[Model]]", f"    {self.model!r}", "[[Fit Statistics]]",
                 "    # fitting method   = leastsq", f"    # function evals   = {self.nfev}",
                 f"    # data points      = {self.ndata}", f"    # variables        = {self.nvarys}",
                 f"    chi-square         = {self.chisqr:.8g}", f"    reduced chi-square = {self.redchi:.8g}",
                 f"    Akaike info crit   = {self.aic:.8g}", f"    Bayesian info crit = {self.bic:.8g}",
                 "[[Variables]]"]
        for n, p in self.params.items():
            if not p.vary:
                lines.append(f"    {n}: {p.value:.8g} (fixed)")
            elif p.stderr is not None:
                rel = f" ({abs(p.stderr / p.value) * 100:.2f}%)" if p.value else ""
                lines.append(f"    {n}: {p.value:.8g} +/- {p.stderr:.8g}{rel} (init = {self.init_values[n]:.8g})")
            else:
                lines.append(f"    {n}: {p.value:.8g} +/- None (init = {self.init_values[n]:.8g})")
        return "\n".join(lines)


class Model:
    """A fit model: the function of the reference (evaluated with numpy by ``eval``)
    and the id of its device evaluation (fitted by ``fit``)."""

    def __init__(self, func, device_id: int, name: Optional[str] = None):
        import inspect

        args = list(inspect.signature(func).parameters)
        self.func = func
        self.device_id = int(device_id)
        self.independent_vars = [args[0]]
        self.param_names = args[1:]
        self.param_hints: Dict[str, Dict[str, Any]] = {}
        self.name = name or func.__name__.lstrip("_")

    def __repr__(self) -> str:
        return f"<fastddm_gb300.Model: {self.name}>"

    def copy(self) -> "Model":
        return copy.deepcopy(self)

    def set_param_hint(self, name: str, **kwargs) -> None:
        if name not in self.param_names:
            raise ValueError(f"'{name}' is not a parameter of model '{self.name}'")
        allowed = {"value", "vary", "min", "max", "expr"}
        bad = set(kwargs) - allowed
        if bad:
            raise ValueError(f"unknown parameter hint(s) {sorted(bad)}")
        self.param_hints.setdefault(name, {}).update(kwargs)

    def make_params(self, **kwargs) -> Parameters:
        params = Parameters()
        for n in self.param_names:
            h = self.param_hints.get(n, {})
            params.add(n, value=h.get("value"), vary=h.get("vary", True), min=h.get("min", -INF),
                       max=h.get("max", INF), expr=h.get("expr"))
        for n, v in kwargs.items():
            if n not in params:
                raise ValueError(f"'{n}' is not a parameter of model '{self.name}'")
            if isinstance(v, dict):
                params[n].set(**v)
            else:
                params[n].value = v
        return params

    def eval(self, params: Optional[Parameters] = None, **kwargs) -> np.ndarray:
        vals = {} if params is None else {n: p.value for n, p in params.items()}
        for n in self.param_names:
            if n in kwargs:
                vals[n] = kwargs[n]
        xname = self.independent_vars[0]
        if xname not in kwargs:
            raise ValueError(f"missing independent variable '{xname}'")
        return self.func(np.asarray(kwargs[xname], dtype=np.float64), *[vals[n] for n in self.param_names])

    # -- fitting -----------------------------------------------------------
    def check_fit_args(self, method: str, nan_policy: Optional[str], iter_cb) -> None:
        if method != "leastsq":
            raise NotImplementedError(f"method '{method}': the device fits provide lmfit's default 'leastsq' only")
        if nan_policy not in (None, "raise"):
            raise NotImplementedError("nan_policy other than 'raise' is not supported by the device fits")
        if iter_cb is not None:
            raise NotImplementedError("iter_cb is not supported by the device fits")

    def split_kwargs(self, params: Parameters, kwargs: dict):
        """lmfit's keyword rules: the independent variable, parameter values by name, the rest ignored."""
        xname = self.independent_vars[0]
        if xname not in kwargs:
            raise ValueError(f"missing independent variable '{xname}'")
        x = np.asarray(kwargs.pop(xname), dtype=np.float64)
        for n in self.param_names:
            if n in kwargs:
                params[n].value = kwargs.pop(n)
        for n in kwargs:
            warnings.warn(f"The keyword argument {n} does not match any arguments of the model function. "
                          "It will be ignored.", UserWarning)
        return x

    def fit(self, data, params: Optional[Parameters] = None, weights=None, method: str = "leastsq", iter_cb=None,
            scale_covar: bool = True, verbose: bool = False, fit_kws: Optional[dict] = None,
            nan_policy: Optional[str] = None, calc_covar: bool = True, max_nfev: Optional[int] = None,
            gpu_id: int = 0, **kwargs) -> ModelResult:
        """Fit ``data`` on the GPU (lmfit ``Model.fit`` with method 'leastsq')."""
        self.check_fit_args(method, nan_policy, iter_cb)
        params = self.make_params() if params is None else copy.deepcopy(params)
        for n in self.param_names:
            if n not in params:
                h = self.param_hints.get(n, {})
                params.add(n, value=h.get("value"), vary=h.get("vary", True), min=h.get("min", -INF),
                           max=h.get("max", INF))
        x = self.split_kwargs(params, dict(kwargs))
        y = np.asarray(data, dtype=np.float64).ravel()
        if y.shape != x.shape:
            raise ValueError(f"data ({y.shape}) and {self.independent_vars[0]} ({x.shape}) differ in shape")
        if not np.all(np.isfinite(y)):
            raise ValueError("The input contains nan values")
        W = None
        if weights is not None:
            W = np.broadcast_to(np.asarray(weights, dtype=np.float64), y.shape)[None, :]
        spec = FitSpec(self, params)
        problems = np.array([[0, 0 if W is not None else -1, -1, spec.vary, 0, y.size]], dtype=np.int32)
        out = run_fits(self, x[None, :], y[None, :], W, problems, [[[0]]], spec.init[None], spec.lo[None], spec.hi[None],
                       lsq_options(fit_kws, max_nfev), gpu_id, residual=True, covariance=calc_covar)
        if int(out["status"][0]) == ST_NONFINITE:
            raise ValueError(NAN_MESSAGE)
        r = ModelResult(self, params, y, x, None if W is None else W[0], out, 0, scale_covar, calc_covar)
        if verbose:
            print(r.fit_report())
        return r
