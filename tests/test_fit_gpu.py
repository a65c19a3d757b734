"""Device fits against the oracle (lmfit's 'leastsq' restated around scipy's MINPACK).

Tolerances.  The device runs MINPACK's algorithm with lmfit's settings, but
its sums over the data run in a different order and CUDA's exp / pow differ
from glibc's in the last bit; MINPACK amplifies such differences through the
forward-difference Jacobian (step 1.5e-8 |x|), so the two runs take slightly
different paths to the same minimum.  On curves started within a factor of
about two of the solution the fitted parameters agree to 1e-5 of their scale
(the amplitude for B) or a tenth of their standard error, whichever is
larger (MINPACK's xtol test stops a poorly determined parameter early, at a
point that depends on the path), chi^2 to 1e-9 relative or 0.05 of a
reduced chi-square unit (a one-standard-error change of any parameter moves
chi^2 by about one such unit; where xtol stops a run in a flat valley the
two runs' chi^2 differ by less than that), standard errors to
5e-2 relative (they come from the last Jacobian, which MINPACK evaluates at
the iterate before the final step, so a run that stops one step apart reads
a slightly different one; started at the solution, where both runs read the
same Jacobian, they agree to 1e-4), and the success flags exactly.
"""

import numpy as np
import pytest

import fit_oracle as fo

pytestmark = pytest.mark.gpu

PAR_TOL = 1e-5   # of the parameter's scale, or
SE_FRAC = 0.1    # of its standard error, whichever is larger
CHI_TOL = 1e-9   # relative, or
CHI_RED = 0.05   # of a reduced chi-square unit, whichever is larger
SE_TOL = 5e-2

# model name -> (true parameters, starting values)
CASES = {
    "generic_exponential_isf_model": ({"A": 1.7, "Gamma": 0.8, "beta": 0.85}, {"A": 1.2, "Gamma": 1.3, "beta": 1.0}),
    "simple_exponential_isf_model": ({"A": 1.7, "Gamma": 0.8, "beta": 1.0}, {"A": 1.2, "Gamma": 1.3}),
    "stretched_exponential_isf_model": ({"A": 1.7, "Gamma": 0.8, "beta": 0.7}, {"A": 1.2, "Gamma": 1.3, "beta": 1.0}),
    "compressed_exponential_isf_model": ({"A": 1.7, "Gamma": 0.8, "beta": 1.4}, {"A": 1.2, "Gamma": 1.3, "beta": 1.0}),
    "double_exponential_isf_model": ({"A": 1.5, "Gamma1": 20.0, "beta1": 1.0, "Gamma2": 0.2, "beta2": 0.9,
                                      "alpha": 0.4},
                                     {"A": 1.2, "Gamma1": 12.0, "beta1": 1.0, "Gamma2": 0.3, "beta2": 1.0,
                                      "alpha": 0.5}),
    "flory_schulz_isf_model": ({"A": 1.7, "Gamma": 0.8, "sigma": 0.6}, {"A": 1.2, "Gamma": 1.3, "sigma": 0.9}),
    "exponential_distribution_isf_model": ({"A": 1.7, "Gamma": 0.8, "sigma": 1.0}, {"A": 1.2, "Gamma": 1.3}),
    "generic_exponential_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "beta": 0.85},
                                  {"A": 600.0, "B": 10.0, "Gamma": 1.3, "beta": 1.0}),
    "simple_exponential_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "beta": 1.0},
                                 {"A": 600.0, "B": 10.0, "Gamma": 1.3}),
    "stretched_exponential_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "beta": 0.7},
                                    {"A": 600.0, "B": 10.0, "Gamma": 1.3, "beta": 0.95}),
    "compressed_exponential_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "beta": 1.4},
                                     {"A": 600.0, "B": 10.0, "Gamma": 1.3, "beta": 1.1}),
    "double_exponential_model": ({"A": 900.0, "B": 25.0, "Gamma1": 20.0, "beta1": 1.0, "Gamma2": 0.2, "beta2": 0.9,
                                  "alpha": 0.4},
                                 {"A": 700.0, "B": 10.0, "Gamma1": 12.0, "beta1": 1.0, "Gamma2": 0.3, "beta2": 1.0,
                                  "alpha": 0.5}),
    "flory_schulz_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "sigma": 0.6},
                           {"A": 600.0, "B": 10.0, "Gamma": 1.3, "sigma": 0.9}),
    "exponential_distribution_model": ({"A": 900.0, "B": 25.0, "Gamma": 0.8, "sigma": 1.0},
                                       {"A": 600.0, "B": 10.0, "Gamma": 1.3}),
    "simple_exp_model": ({"tau": 1.3, "amplitude": 0.9}, {"tau": 0.8, "amplitude": 0.6}),
    "simple_structure_function": ({"A": 900.0, "B": 25.0, "tau": 1.3}, {"A": 600.0, "B": 10.0, "tau": 0.8}),
}


def _model(name):
    from fastddm_gb300 import fit as gfit
    from fastddm_gb300 import fit_models

    return getattr(gfit, name) if name in ("simple_exp_model", "simple_structure_function") else \
        getattr(fit_models, name)


def _curve(name, seed, m=150, noise=0.01):
    func, names, _ = fo.MODELS[name]
    truth, _ = CASES[name]
    x = np.logspace(-2, 2, m)
    y = func(x, *[truth[n] for n in names])
    rng = np.random.default_rng(seed)
    return x, y * (1 + noise * rng.standard_normal(m))


def _scale(name, p, vals):
    """B is compared on the scale of the amplitude"""
    return abs(vals["A"]) if p == "B" else max(abs(vals[p]), 1e-12)


def _compare(name, dev, ora, names):
    assert dev.success == ora["success"]
    for p in names:
        d, o = dev.params[p].value, ora["values"][p]
        ds, os_ = dev.params[p].stderr, ora["stderr"][p]
        tol = PAR_TOL * _scale(name, p, ora["values"])
        if os_ is not None and np.isfinite(os_):
            tol = max(tol, SE_FRAC * os_)
        assert abs(d - o) <= tol, (name, p, d, o, os_)
        if os_ is None:
            assert ds is None
        elif np.isnan(os_):  # e.g. a parameter exactly on its bound: lmfit's inv() gives NaN
            assert ds is not None and np.isnan(ds), (name, p, ds)
        elif os_ > 0:
            assert abs(ds / os_ - 1) < SE_TOL, (name, p, ds, os_)
        else:
            assert ds == 0.0
    tol = max(CHI_TOL * ora["chisqr"], CHI_RED * ora["redchi"])
    assert abs(dev.chisqr - ora["chisqr"]) <= tol, (name, dev.chisqr, ora["chisqr"], tol)


@pytest.mark.parametrize("name", sorted(CASES))
def test_model_fit_matches_the_oracle(name):
    model = _model(name)
    func, names, _ = fo.MODELS[name]
    _, start = CASES[name]
    for seed in range(3):
        x, y = _curve(name, seed)
        w = 1.0 / (0.01 * np.abs(y) + 1e-3)
        xname = model.independent_vars[0]
        params = model.make_params(**start)
        dev = model.fit(y, params=params, weights=w, **{xname: x})
        op = fo.make_params(name)
        for k, v in start.items():
            op[k]["value"] = v
        ora = fo.lm_fit(func, names, op, x, y, weights=w)
        _compare(name, dev, ora, names)
        # residual and best fit as lmfit reports them
        np.testing.assert_allclose(dev.residual, (dev.best_fit - y) * w, rtol=1e-9, atol=1e-9 * np.abs(w * y).max())


@pytest.mark.parametrize("name", ["simple_exponential_model", "stretched_exponential_isf_model",
                                  "double_exponential_model", "flory_schulz_model"])
def test_standard_errors_at_the_solution(name):
    """Started at the oracle's solution both runs factor the same Jacobian: lmfit's covariance
    (inv(R^T R) through the bound mappings, times chi^2 / nfree) agrees closely."""
    model = _model(name)
    func, names, _ = fo.MODELS[name]
    _, start = CASES[name]
    x, y = _curve(name, 11)
    op = fo.make_params(name)
    for k, v in start.items():
        op[k]["value"] = v
    first = fo.lm_fit(func, names, op, x, y)
    for k in names:
        op[k]["value"] = first["values"][k]
    ora = fo.lm_fit(func, names, op, x, y)
    params = model.make_params(**{k: first["values"][k] for k in names})
    dev = model.fit(y, params=params, **{model.independent_vars[0]: x})
    for p in names:
        os_, ds = ora["stderr"][p], dev.params[p].stderr
        if os_ is not None and np.isfinite(os_) and os_ > 0:
            assert abs(ds / os_ - 1) < 1e-4, (name, p, ds, os_)
    # lmfit's covar and correlations: entries relative to sqrt(c_ii c_jj)
    if ora["covar"] is not None and np.all(np.isfinite(ora["covar"])):
        assert dev.var_names == ora["var_names"]
        d = np.sqrt(np.outer(np.diag(ora["covar"]), np.diag(ora["covar"])))
        assert np.max(np.abs(dev.covar - ora["covar"]) / d) < 1e-4, name
        a, b = dev.var_names[0], dev.var_names[1]
        assert abs(dev.params[a].correl[b] - ora["covar"][0, 1] / d[0, 1]) < 1e-4


def test_fit_with_estimated_simple_parameters():
    from fastddm_gb300 import fit as gfit

    x, y = _curve("simple_structure_function", 7)
    r = gfit.fit(gfit.simple_structure_function, x, y, estimate_simple_parameters=True)
    p = gfit._simple_structure_function_parameter_helper(x, y)
    op = fo.make_params("simple_structure_function")
    for k in ("A", "B", "tau"):
        op[k]["value"] = p[k].value
    func, names, _ = fo.MODELS["simple_structure_function"]
    _compare("simple_structure_function", r, fo.lm_fit(func, names, op, x, y), names)


class AA:
    def __init__(self, data, err, k, tau):
        self.data, self.err, self.k, self.tau = data, err, k, tau


def _aa(K=64, m=100, seed=0, nan_rows=()):
    rng = np.random.default_rng(seed)
    tau = np.logspace(-2, 2, m)
    k = np.linspace(0.2, 3.0, K)
    A = 1000.0 * np.exp(-k)
    B = 20.0 + 0 * k
    G = 0.5 * k ** 2
    data = A[:, None] * (1 - np.exp(-G[:, None] * tau[None, :])) + B[:, None]
    err = 0.01 * data + 1.0
    data = data + err * rng.standard_normal(data.shape)
    for r in nan_rows:
        data[r, :] = np.nan
    return AA(data, err, k, tau), (A, B, G)


@pytest.mark.parametrize("use_err", [False, True])
def test_fit_multik_chain_matches_the_oracle(use_err):
    from fastddm_gb300 import fit as gfit
    from fastddm_gb300 import fit_models

    aa, (A, B, G) = _aa(nan_rows=(5, 40))
    ref = 20
    fmin = {"B": np.full(len(aa.k), 0.0)}
    table, mres = gfit.fit_multik(aa, fit_models.simple_exponential_model, ref, A=A[ref], B=B[ref],
                                  Gamma=1.3 * G[ref], use_err=use_err, fixed_params_min=fmin,
                                  return_model_results=True)
    params = fo.make_params("simple_exponential_model")
    params["A"]["value"], params["B"]["value"], params["Gamma"]["value"] = A[ref], B[ref], 1.3 * G[ref]
    names = ["A", "B", "Gamma", "beta"]
    want = fo.fit_multik(fo.MODELS["simple_exponential_model"][0], names, params, aa.tau, aa.data, ref,
                         err=aa.err, use_err=use_err, fixed_params_min=fmin)
    np.testing.assert_array_equal(table["success"], want["success"])
    ok = ~np.isnan(want["A"])
    assert np.array_equal(ok, ~np.isnan(table["A"]))
    for p in names:
        scale = np.abs(want["A"][ok]) if p == "B" else np.maximum(np.abs(want[p][ok]), 1e-12)
        tol = np.maximum(PAR_TOL * scale, SE_FRAC * np.nan_to_num(want[f"{p}_stderr"][ok]))
        assert np.all(np.abs(table[p][ok] - want[p][ok]) <= tol), p
        se, wse = table[f"{p}_stderr"][ok], want[f"{p}_stderr"][ok]
        pos = wse > 0
        assert np.all(np.abs(se[pos] / wse[pos] - 1) < SE_TOL), p
    assert mres[5] is None and mres[ref].success


def test_fit_multik_fixed_params_and_orders():
    from fastddm_gb300 import fit as gfit
    from fastddm_gb300 import fit_models

    aa, (A, B, G) = _aa(K=96, seed=2)
    chain, _ = gfit.fit_multik(aa, fit_models.simple_exponential_model, 30, A=A[30], Gamma=G[30],
                               fixed_params={"B": B}, use_err=True)
    np.testing.assert_array_equal(chain["B"], B)
    assert np.all(chain["B_stderr"] == 0.0) and np.all(chain["success"])
    for order in ("ref", "none"):
        other, _ = gfit.fit_multik(aa, fit_models.simple_exponential_model, 30, A=A[30], Gamma=G[30],
                                   fixed_params={"B": B}, use_err=True, warm_start=order)
        # a well-posed curve has one minimum, whatever the start
        np.testing.assert_allclose(other["Gamma"], chain["Gamma"], rtol=1e-4)
        np.testing.assert_allclose(other["A"], chain["A"], rtol=1e-4)


def test_non_finite_residual_raises_like_lmfit():
    from fastddm_gb300 import fit_models

    x, y = _curve("simple_exponential_model", 0)
    w = np.ones_like(y)
    w[7] = np.inf
    m = fit_models.simple_exponential_model
    with pytest.raises(ValueError, match="NaN values"):
        m.fit(y, params=m.make_params(**CASES["simple_exponential_model"][1]), weights=w, x=x)


def test_evaluation_limit_stops_the_fit():
    from fastddm_gb300 import fit_models

    x, y = _curve("generic_exponential_model", 1)
    m = fit_models.generic_exponential_model
    r = m.fit(y, params=m.make_params(**CASES["generic_exponential_model"][1]), x=x, max_nfev=12)
    assert not r.success and r.aborted and r.nfev == 13


def test_fit_multik_batch_matches_single_calls():
    """Three datasets of different sizes in one batch (six sweeps, a CTA each, as in single calls):
    bit-identical to fit_multik on each; 320 datasets (640 sweeps: more than four per SM, a warp
    each): within tolerance."""
    from fastddm_gb300 import fit as gfit
    from fastddm_gb300 import fit_models

    m = fit_models.simple_exponential_model
    sets = [_aa(K=K, m=mm, seed=s) for K, mm, s in ((30, 80, 1), (48, 120, 2), (20, 60, 3))]
    jobs = [dict(data=a, ref=len(a.k) // 3, A=A[len(a.k) // 3], B=B[len(a.k) // 3], Gamma=G[len(a.k) // 3],
                 use_err=True) for a, (A, B, G) in sets]
    batch = gfit.fit_multik_batch(jobs, m)
    for job, (tb, _) in zip(jobs, batch):
        kw = {k: v for k, v in job.items() if k not in ("data", "ref")}
        ta, _ = gfit.fit_multik(job["data"], m, job["ref"], **kw)
        for col in ta.columns:
            np.testing.assert_array_equal(tb[col], ta[col], err_msg=col)
    many = [_aa(K=24, m=50 + (s % 7) * 10, seed=100 + s) for s in range(320)]
    jobs = [dict(data=a, ref=8, A=A[8], B=B[8], Gamma=G[8], use_err=True) for a, (A, B, G) in many]
    batch = gfit.fit_multik_batch(jobs, m)
    for job, (tb, _) in zip(jobs[:10], batch[:10]):
        kw = {k: v for k, v in job.items() if k not in ("data", "ref")}
        ta, _ = gfit.fit_multik(job["data"], m, job["ref"], **kw)
        np.testing.assert_array_equal(tb["success"], ta["success"])
        for p in ("A", "Gamma"):
            tol = np.maximum(PAR_TOL * np.abs(ta[p]), SE_FRAC * ta[f"{p}_stderr"])
            assert np.all(np.abs(tb[p] - ta[p]) <= tol), p


def test_fit_on_a_side_stream_equals_the_default_stream():
    """The fit launches on the caller's current stream (a non-zero stream handle crosses the C ABI)."""
    import torch

    from fastddm_gb300 import fit_models

    m = fit_models.simple_exponential_model
    x, y = _curve("simple_exponential_model", 3)
    p = m.make_params(**CASES["simple_exponential_model"][1])
    ref = m.fit(y, params=p, x=x)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        got = m.fit(y, params=p, x=x)
    for n in m.param_names:
        assert got.params[n].value == ref.params[n].value
    assert got.chisqr == ref.chisqr and got.nfev == ref.nfev


def test_pipeline_ddm_azimuthal_average_fit():
    """DDM of a drift-free Brownian scene, its azimuthal average, the polyfit noise estimate and the
    reference's sweep (set up as fit.py's docstring does) against the oracle's sweep on the same
    average: parameters within tolerance on every k the oracle determines well, success flags equal."""
    import copy

    import fastddm_gb300 as fddm
    from fastddm_gb300 import fit as gfit
    from fastddm_gb300 import fit_models, noise_est
    from fastddm_gb300.synthetic import Scene, make_stack

    # D = 0.05 px^2/frame and k up to 1.5: Gamma = D k^2 up to ~0.1/frame, resolved by lags 1..255
    imgs = make_stack(Scene(256, 128, 128, 300, 2.0, 2000.0, 0.05, 500.0, 0.0, "uint16", 3))
    lags = np.arange(1, 256)
    sf = fddm.ddm(imgs, lags, mode="fft")
    aa = fddm.azimuthal_average(sf, bins=32, range=(0.0, 1.5))
    a = copy.copy(aa)
    data = a._data.copy()
    data[~np.all(np.isfinite(a.err) & (a.err > 0), axis=1), 0] = np.nan  # the one-pixel k = 0 bin
    a._data = data
    B, _ = noise_est.estimate_camera_noise(a, mode="polyfit")
    valid = np.flatnonzero(~np.isnan(a.data[:, 0]))
    ref = int(valid[len(valid) // 4])
    A0 = 2.0 * a.var[ref] - B[ref]
    G0 = 1.0 / a.tau[int(np.argmin(np.abs((a.data[ref] - B[ref]) / A0 - 0.5)))]
    table, _ = gfit.fit_multik(a, fit_models.simple_exponential_model, ref, A=A0, B=B[ref], Gamma=G0,
                               use_err=True)
    params = fo.make_params("simple_exponential_model")
    params["A"]["value"], params["B"]["value"], params["Gamma"]["value"] = A0, B[ref], G0
    want = fo.fit_multik(fo.MODELS["simple_exponential_model"][0], ["A", "B", "Gamma", "beta"], params, a.tau,
                         a.data, ref, err=a.err, use_err=True)
    np.testing.assert_array_equal(table["success"], want["success"])
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.maximum(want["A_stderr"] / np.abs(want["A"]), want["Gamma_stderr"] / np.abs(want["Gamma"]))
    wd = ~np.isnan(want["A"]) & want["success"] & np.isfinite(rel) & (rel < 0.1)
    assert wd.sum() >= 8  # enough well-determined k for the comparison to mean something
    for n in ("A", "B", "Gamma"):
        scale = np.abs(want["A"][wd]) if n == "B" else np.abs(want[n][wd])
        tol = np.maximum(PAR_TOL * scale, SE_FRAC * want[f"{n}_stderr"][wd])
        assert np.all(np.abs(table[n][wd] - want[n][wd]) <= tol), n
