"""Fitting row on the CPU: the oracle's MINPACK core against known answers, the
bounded-parameter mappings, the lmfit-style parameter / model interface, and
fit_multik's construction of the device problems (chains, warm starts,
weights, per-k bounds), driven through a fake device that runs every problem
with the oracle in launch order."""

import numpy as np
import pytest

import fit_oracle as fo
from fastddm_gb300 import _fitting, fit_models
from fastddm_gb300 import fit as gfit

EPS = np.finfo(float).eps


# -- the oracle's optimiser is MINPACK: known answers ------------------------
def test_oracle_rosenbrock_known_answer():
    """Rosenbrock as least squares (f1 = 10 (b - a^2), f2 = 1 - a): minimum at (1, 1), chi^2 = 0."""

    def rosen(x, a, b):
        return np.array([10.0 * (b - a * a), 1.0 - a])

    par = {"a": {"value": -1.2, "min": -np.inf, "max": np.inf}, "b": {"value": 1.0, "min": -np.inf, "max": np.inf}}
    r = fo.lm_fit(rosen, ["a", "b"], par, np.zeros(2), np.zeros(2))
    assert r["success"]
    assert abs(r["values"]["a"] - 1.0) < 1e-8 and abs(r["values"]["b"] - 1.0) < 1e-8
    assert r["chisqr"] < 1e-20


def test_oracle_linear_least_squares_known_answer():
    rng = np.random.default_rng(3)
    x = np.linspace(0, 5, 40)
    y = 1.5 - 0.7 * x + 0.05 * rng.standard_normal(x.size)
    par = {"c0": {"value": 0.0}, "c1": {"value": 0.0}}
    r = fo.lm_fit(lambda x, c0, c1: c0 + c1 * x, ["c0", "c1"], par, x, y)
    c1, c0 = np.polyfit(x, y, 1)
    # the forward-difference Jacobian and xtol = 1e-7 bound the agreement
    assert abs(r["values"]["c0"] - c0) < 1e-7 and abs(r["values"]["c1"] - c1) < 1e-7
    # stderr = sqrt(diag(inv(V^T V)) * chi^2 / (n - 2)), the textbook formula
    V = np.stack([np.ones_like(x), x], 1)
    cov = np.linalg.inv(V.T @ V) * r["chisqr"] / (x.size - 2)
    assert abs(r["stderr"]["c0"] / np.sqrt(cov[0, 0]) - 1) < 1e-6
    assert abs(r["stderr"]["c1"] / np.sqrt(cov[1, 1]) - 1) < 1e-6


@pytest.mark.parametrize("case", ["bard", "kowalik_osborne", "meyer", "beale"])
def test_oracle_moré_garbow_hillstrom_known_answers(case):
    """Problems of the MINPACK test set (Moré, Garbow and Hillstrom, ACM TOMS 7, 1981) from their
    standard starting points: the minimum sums of squares they publish."""
    if case == "bard":
        y = np.array([0.14, 0.18, 0.22, 0.25, 0.29, 0.32, 0.35, 0.39, 0.37, 0.58, 0.73, 0.96, 1.34, 2.10, 4.39])
        u = np.arange(1, 16)
        v, w = 16 - u, np.minimum(u, 16 - u)
        func, names, start, want = (lambda x, a, b, c: a + u / (b * v + c * w)), list("abc"), (1, 1, 1), 8.21487e-3
    elif case == "kowalik_osborne":
        y = np.array([0.1957, 0.1947, 0.1735, 0.1600, 0.0844, 0.0627, 0.0456, 0.0342, 0.0323, 0.0235, 0.0246])
        u = np.array([4.0, 2.0, 1.0, 0.5, 0.25, 0.167, 0.125, 0.1, 0.0833, 0.0714, 0.0625])
        func = lambda x, a, b, c, d: a * (u ** 2 + u * b) / (u ** 2 + u * c + d)
        names, start, want = list("abcd"), (0.25, 0.39, 0.415, 0.39), 3.07505e-4
    elif case == "meyer":
        y = np.array([34780, 28610, 23650, 19630, 16370, 13720, 11540, 9744, 8261, 7030, 6005, 5147, 4427, 3820,
                      3307, 2872], float)
        t = 45.0 + 5.0 * np.arange(1, 17)
        func, names, start, want = (lambda x, a, b, c: a * np.exp(b / (t + c))), list("abc"), (0.02, 4000, 250), 87.9458
    else:  # beale: minimum 0 at (3, 0.5)
        y = np.array([1.5, 2.25, 2.625])
        func = lambda x, a, b: np.array([a * (1 - b), a * (1 - b * b), a * (1 - b ** 3)])
        names, start, want = list("ab"), (1.0, 1.0), 0.0
    par = {n: {"value": float(v)} for n, v in zip(names, start)}
    r = fo.lm_fit(func, names, par, np.zeros(y.size), y)
    assert r["success"]
    if want == 0.0:
        assert r["chisqr"] < 1e-20 and abs(r["values"]["a"] - 3.0) < 1e-8 and abs(r["values"]["b"] - 0.5) < 1e-8
    else:
        assert abs(r["chisqr"] / want - 1) < 1e-5, r["chisqr"]


def test_oracle_bound_is_respected():
    """A parameter whose unconstrained optimum lies below its lower bound ends on the bound."""
    x = np.linspace(0, 4, 30)
    y = -0.5 + 2.0 * x
    par = {"c0": {"value": 1.0, "min": 0.0, "max": np.inf}, "c1": {"value": 1.0}}
    r = fo.lm_fit(lambda x, c0, c1: c0 + c1 * x, ["c0", "c1"], par, x, y)
    assert 0.0 <= r["values"]["c0"] < 1e-3


@pytest.mark.parametrize("lo,hi", [(-np.inf, np.inf), (0.5, np.inf), (-np.inf, 7.0), (0.5, 7.0)])
def test_mappings_round_trip(lo, hi):
    for v in (0.6, 1.0, 3.3, 6.9):
        u = fo.to_internal(v, lo, hi)
        assert abs(fo.from_internal(u, lo, hi) - v) < 1e-12
        # scale_gradient is d(external)/d(internal)
        h = 1e-6
        num = (fo.from_internal(u + h, lo, hi) - fo.from_internal(u - h, lo, hi)) / (2 * h)
        assert abs(fo.scale_gradient(u, lo, hi) - num) < 1e-6 * max(1.0, abs(num))


# -- parameter / model interface ---------------------------------------------
def test_models_match_the_oracle_functions_and_hints():
    x = np.logspace(-2, 2, 50)
    samples = {
        "generic_exponential_isf_model": dict(A=2.0, Gamma=0.7, beta=0.8),
        "double_exponential_isf_model": dict(A=2.0, Gamma1=5.0, beta1=1.0, Gamma2=0.1, beta2=0.9, alpha=0.4),
        "flory_schulz_isf_model": dict(A=2.0, Gamma=0.5, sigma=0.6),
        "generic_exponential_model": dict(A=2.0, B=0.3, Gamma=0.7, beta=1.2),
        "double_exponential_model": dict(A=2.0, B=0.3, Gamma1=5.0, beta1=1.0, Gamma2=0.1, beta2=0.9, alpha=0.4),
        "flory_schulz_model": dict(A=2.0, B=0.3, Gamma=0.5, sigma=0.6),
    }
    for name in fo.MODELS:
        if name in ("simple_exp_model", "simple_structure_function"):
            m = getattr(gfit, name)
        else:
            m = getattr(fit_models, name)
        func, names, hints = fo.MODELS[name]
        assert m.param_names == names, name
        p = m.make_params()
        for n in names:
            v, lo, hi, vary = hints[n]
            assert p[n].value == v and p[n].min == lo and p[n].max == hi and p[n].vary == vary, (name, n)
        base = next((s for k, s in samples.items() if name.startswith(k.replace("_model", "").split("_isf")[0])
                     and ("_isf" in name) == ("_isf" in k)), None)
        vals = {n: (base or {}).get(n, 0.8) for n in names}
        np.testing.assert_array_equal(m.eval(x=x, **vals) if m.independent_vars == ["x"] else
                                      m.eval(dt=x, **vals), func(x, *[vals[n] for n in names]))


def test_parameter_interface():
    m = fit_models.simple_exponential_model.copy()
    with pytest.raises(ValueError):
        m.set_param_hint("C", value=1.0)
    with pytest.raises(ValueError):
        m.set_param_hint("A", bogus=1.0)
    m.set_param_hint("A", value=5.0, max=10.0)
    p = m.make_params(Gamma=2.0)
    assert p["A"].value == 5.0 and p["A"].max == 10.0 and p["A"].min == EPS and p["Gamma"].value == 2.0
    q = p.copy()
    q["A"].value = 1.0
    assert p["A"].value == 5.0
    p.update(q)
    assert p["A"].value == 1.0 and p["A"] is not q["A"]
    assert list(p.valuesdict()) == ["A", "B", "Gamma", "beta"]
    p["A"].min = 2.0
    p["A"].max = 2.0
    with pytest.raises(ValueError, match="min == max"):
        _fitting.FitSpec(m, p)
    p["A"].max = 3.0
    p["B"].expr = "A / 2"
    with pytest.raises(NotImplementedError):
        _fitting.FitSpec(m, p)
    with pytest.raises(NotImplementedError):
        _fitting.lsq_options({"diag": 1.0}, None)
    np.testing.assert_array_equal(_fitting.lsq_options(None, None), [1e-7, 1e-7, 1e-7, 0.0, 100.0, 0.0])


def test_start_values_are_clipped_and_vary_mask():
    m = fit_models.stretched_exponential_model
    p = m.make_params(beta=3.0)
    s = _fitting.FitSpec(m, p)
    assert s.vary == 0b1111 and s.init[3] == 3.0 and s.hi[3] == 1.0  # clipped on the device, as lmfit does
    p = fit_models.simple_exponential_model.make_params()
    assert _fitting.FitSpec(fit_models.simple_exponential_model, p).vary == 0b0111


# -- fit_multik's problems, run through the oracle ---------------------------
class FakeDevice:
    """Runs the problems of run_fits with the oracle, chain by chain in launch order,
    honouring the warm starts (pred) the way the kernel does."""

    def __init__(self, model_name):
        self.func, self.names, _ = fo.MODELS[model_name]
        self.launches = []

    def __call__(self, model, x, Y, W, problems, stages, init, lo, hi, options, gpu_id=0, residual=False,
                 covariance=False):
        P = len(init)
        npar = len(self.names)
        vals = np.full((P, npar), np.nan)
        se = np.full((P, npar), np.nan)
        out = {"values": vals, "stderr": se, "chisqr": np.zeros(P), "nfev": np.zeros(P, np.int32),
               "info": np.zeros(P, np.int32), "status": np.zeros(P, np.int32),
               "nvary": bin(int(problems[0][3])).count("1"), "device_ms": 0.0, "launches": len(stages)}
        self.problems = np.array(problems)
        done = set()
        for chains in stages:
            self.launches.append([list(c) for c in chains])
            for chain in chains:
                for pi in chain:
                    row, wrow, pred, vary, xrow, npts = (int(v) for v in problems[pi])
                    assert pred < 0 or pred in done  # a warm start only reads a finished fit
                    par = {}
                    for i, n in enumerate(self.names):
                        v = init[pi][i]
                        if (vary >> i) & 1 and pred >= 0:
                            v = vals[pred][i]
                        par[n] = {"value": v, "min": lo[pi][i], "max": hi[pi][i], "vary": bool((vary >> i) & 1)}
                    r = fo.lm_fit(self.func, self.names, par, x[xrow, :npts], Y[row, :npts],
                                  None if wrow < 0 else W[wrow, :npts])
                    vals[pi] = [r["values"][n] for n in self.names]
                    se[pi] = [-1.0 if r["stderr"][n] is None else r["stderr"][n] for n in self.names]
                    out["chisqr"][pi] = r["chisqr"]
                    out["info"][pi] = r["ier"]
                    done.add(pi)
        return out


class AA:
    """An azimuthal average: data (K, m), err, k, tau."""

    def __init__(self, data, err, k, tau):
        self.data, self.err, self.k, self.tau = data, err, k, tau


def synthetic_aa(K=24, m=60, seed=0, nan_rows=()):
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
def test_fit_multik_chain_matches_the_reference_loop(monkeypatch, use_err):
    aa, (A, B, G) = synthetic_aa(nan_rows=(3,))
    ref = 10
    fake = FakeDevice("simple_exponential_model")
    monkeypatch.setattr(gfit, "run_fits", fake)
    model = fit_models.simple_exponential_model
    fixed_min = {"B": np.full(len(aa.k), 5.0)}
    table, mres = gfit.fit_multik(aa, model, ref, A=A[ref], B=B[ref], Gamma=G[ref] * 1.3, use_err=use_err,
                                  fixed_params_min=fixed_min, return_model_results=True)
    # launches: the fit at ref, then the two sweeps side by side
    assert len(fake.launches) == 2 and fake.launches[0] == [[0]] and len(fake.launches[1]) == 2
    params = fo.make_params("simple_exponential_model")
    params["A"]["value"], params["B"]["value"], params["Gamma"]["value"] = A[ref], B[ref], G[ref] * 1.3
    want = fo.fit_multik(fo.MODELS["simple_exponential_model"][0], ["A", "B", "Gamma", "beta"], params, aa.tau,
                         aa.data, ref, err=aa.err, use_err=use_err, fixed_params_min=fixed_min)
    for col in ("A", "B", "Gamma", "beta", "A_stderr", "Gamma_stderr", "success"):
        np.testing.assert_array_equal(table[col], want[col], err_msg=col)
    np.testing.assert_array_equal(table["k"], aa.k)
    assert np.isnan(table["A"][3]) and mres[3] is None and not table["success"][3]
    assert mres[ref].success and mres[ref].params["Gamma"].value == table["Gamma"][ref]
    # the row after the NaN row starts from the fit before it
    assert mres[2].init_values["Gamma"] == table["Gamma"][4]


def test_fit_multik_fixed_params_and_other_orders(monkeypatch):
    aa, (A, B, G) = synthetic_aa(K=12, seed=1)
    fixed = {"B": B}
    for order in ("ref", "none"):
        fake = FakeDevice("simple_exponential_model")
        monkeypatch.setattr(gfit, "run_fits", fake)
        table, _ = gfit.fit_multik(aa, fit_models.simple_exponential_model, 5, A=A[5], Gamma=G[5],
                                   fixed_params=fixed, warm_start=order)
        np.testing.assert_array_equal(table["B"], B)
        assert np.all(table["B_stderr"] == 0.0) and np.all(table["success"])
        np.testing.assert_allclose(table["Gamma"], G, rtol=0.05)
        if order == "ref":  # every k starts from the fit at ref, in one launch
            assert fake.launches[0] == [[0]] and all(len(c) == 1 for c in fake.launches[1])
        else:
            assert len(fake.launches) == 1 and len(fake.launches[0]) == 12


def test_fit_multik_errors(monkeypatch):
    aa, _ = synthetic_aa(K=6)
    monkeypatch.setattr(gfit, "run_fits", FakeDevice("simple_exponential_model"))
    m = fit_models.simple_exponential_model
    with pytest.raises(NotImplementedError):
        gfit.fit_multik(aa, m, 2, fixed_params_expr={"B": ["A"] * 6})
    with pytest.raises(NotImplementedError):
        gfit.fit_multik(aa, m, 2, method="nelder")
    with pytest.raises(ValueError, match="values for"):
        gfit.fit_multik(aa, m, 2, fixed_params={"B": [1.0, 2.0]})
    aa.data[2, 5] = np.nan  # lmfit refuses data with NaN (nan_policy 'raise')
    with pytest.raises(ValueError, match="nan"):
        gfit.fit_multik(aa, m, 2)


def test_simple_parameter_helper():
    x = np.logspace(-2, 2, 80)
    y = 50.0 * (1 - np.exp(-x / 2.0)) + 3.0
    p = gfit._simple_structure_function_parameter_helper(x, y)
    assert abs(p["B"].value - 3.0) < 0.5 and abs(p["A"].value - 50.0) < 1.0
    assert 1.0 < p["tau"].value < 2.0


def test_lmfit_models_and_parameters_are_converted(monkeypatch):
    """A reference user's lmfit objects (duck-typed here: lmfit is not installed) drive the device fits."""

    class LmParam:
        def __init__(self, name, value, vary=True, min=-np.inf, max=np.inf, expr=None):
            self.name, self.value, self.vary, self.min, self.max, self.expr = name, value, vary, min, max, expr
            self.stderr = None

    class LmModel:  # what lmfit.Model(_generic_exponential) with set_param_hint calls holds
        def __init__(self, func):
            self.func = func
            self.param_hints = {}

    m = LmModel(fit_models._generic_exponential)
    m.param_hints = {"A": {"value": 1.0, "min": EPS, "max": np.inf}, "B": {"value": 0.0},
                     "Gamma": {"value": 1.0, "min": EPS, "max": np.inf}, "beta": {"value": 1.0, "vary": False}}
    dm = fit_models.from_lmfit(m)
    assert dm.device_id == fit_models.GENERIC_EXP_SF and dm.param_names == ["A", "B", "Gamma", "beta"]
    p = dm.make_params()
    assert p["beta"].vary is False and p["A"].min == EPS
    p.update({"A": LmParam("A", 7.0, min=1.0)})
    assert isinstance(p["A"], _fitting.Parameter) and p["A"].value == 7.0 and p["A"].min == 1.0
    with pytest.raises(NotImplementedError):
        fit_models.from_lmfit(LmModel(lambda x, a: a * x))
    aa, (A, B, G) = synthetic_aa(K=8, seed=4)
    monkeypatch.setattr(gfit, "run_fits", FakeDevice("simple_exponential_model"))
    ref_params = {"A": LmParam("A", A[3], min=EPS), "B": LmParam("B", B[3]), "Gamma": LmParam("Gamma", G[3], min=EPS)}
    table, _ = gfit.fit_multik(aa, m, 3, ref_params=ref_params)
    np.testing.assert_allclose(table["Gamma"], G, rtol=0.05)


def test_fit_multik_batch_gives_each_job_its_own_result(monkeypatch):
    """Datasets of different sizes (k and lags) in one batch: each table equals its own fit_multik."""
    a1, (A1, B1, G1) = synthetic_aa(K=10, m=40, seed=5, nan_rows=(2,))
    a2, (A2, B2, G2) = synthetic_aa(K=14, m=60, seed=6)
    m = fit_models.simple_exponential_model
    fake = FakeDevice("simple_exponential_model")
    monkeypatch.setattr(gfit, "run_fits", fake)
    jobs = [dict(data=a1, ref=4, A=A1[4], B=B1[4], Gamma=G1[4], use_err=True),
            dict(data=a2, ref=9, A=A2[9], B=B2[9], Gamma=G2[9], fixed_params_min={"B": np.zeros(14)})]
    batch = gfit.fit_multik_batch(jobs, m)
    assert len(fake.launches) == 2 and len(fake.launches[0]) == 2 and len(fake.launches[1]) == 4
    alone = [gfit.fit_multik(a1, m, 4, A=A1[4], B=B1[4], Gamma=G1[4], use_err=True)[0],
             gfit.fit_multik(a2, m, 9, A=A2[9], B=B2[9], Gamma=G2[9], fixed_params_min={"B": np.zeros(14)})[0]]
    for (tb, _), ta in zip(batch, alone):
        for col in ta.columns:
            np.testing.assert_array_equal(tb[col], ta[col], err_msg=col)
    with pytest.raises(ValueError, match="same number"):
        gfit.fit_multik_batch([dict(data=a1, ref=4), dict(data=a2, ref=9, fixed_params={"B": B2})], m)


def test_fit_abi_refuses_bad_arguments_without_device_work(built_lib):
    """Argument checks of fddm_b200_fit_lm that return before any device work (CPU)."""
    import ctypes

    lib = built_lib
    u64 = ctypes.c_uint64
    nb = u64(0)
    assert lib.fddm_b200_fit_model_nparams(3) == 4 and lib.fddm_b200_fit_model_nparams(99) == 0
    assert lib.fddm_b200_fit_workspace_bytes(99, 10, 1, ctypes.byref(nb)) == 1
    opts = np.array([1e-7, 1e-7, 1e-7, 0.0, 100.0, 0.0])
    args = dict(m=10, nx=1, ny=1, nw=0, nprob=1, nch=1, nvary=3)

    def call(model=3, opts=opts, **kw):
        a = dict(args, **kw)
        dummy = ctypes.c_void_p(16)  # never dereferenced: every case fails its checks first
        return lib.fddm_b200_fit_lm(model, a["m"], dummy, a["m"], a["nx"], dummy, a["m"], a["ny"], None, 0, a["nw"],
                                    dummy, a["nprob"], dummy, dummy, a["nch"], a["nvary"], dummy, dummy, dummy,
                                    opts.ctypes.data, dummy, dummy, dummy, dummy, dummy, dummy, None, None,
                                    dummy, 1 << 20, None)

    assert call(model=99) == 1                 # unknown model
    assert call(nvary=5) == 1                  # more varying parameters than the model has
    assert call(m=2) == 1                      # fewer points than varying parameters
    big = opts.copy()
    big[5] = 1e7
    assert call(opts=big) == 4                 # max_nfev above the limit
    assert "max_nfev" in lib.fddm_b200_last_error().decode()


def test_fit_multik_host_options(monkeypatch):
    """calc_covar, scale_covar, a user weights array shared by every k, and lmfit's warning for
    keyword arguments that are not the model's."""
    aa, (A, B, G) = synthetic_aa(K=8, seed=7)
    m = fit_models.simple_exponential_model
    fake = FakeDevice("simple_exponential_model")
    monkeypatch.setattr(gfit, "run_fits", fake)
    base, _ = gfit.fit_multik(aa, m, 3, A=A[3], B=B[3], Gamma=G[3])
    nocov, _ = gfit.fit_multik(aa, m, 3, A=A[3], B=B[3], Gamma=G[3], calc_covar=False)
    assert np.all(np.isnan(nocov["A_stderr"])) and np.array_equal(nocov["A"], base["A"])
    unscaled, mres = gfit.fit_multik(aa, m, 3, A=A[3], B=B[3], Gamma=G[3], scale_covar=False,
                                     return_model_results=True)
    red = np.array([r.redchi for r in mres])
    np.testing.assert_allclose(unscaled["Gamma_stderr"], base["Gamma_stderr"] / np.sqrt(red), rtol=1e-12)
    assert np.all(unscaled["beta_stderr"] == 0.0)  # fixed: 0, not divided
    w = 1.0 / (1.0 + np.arange(aa.tau.size))
    with pytest.warns(UserWarning, match="does not match"):
        weighted, _ = gfit.fit_multik(aa, m, 3, A=A[3], B=B[3], Gamma=G[3], weights=w, bogus=1)
    assert np.all(fake.problems[:, 1] == 0)  # every fit, the first at ref included, reads the weights row
    assert not np.array_equal(weighted["Gamma"], base["Gamma"])
    with pytest.raises(ValueError, match="warm_start"):
        gfit.fit_multik(aa, m, 3, warm_start="sideways")
