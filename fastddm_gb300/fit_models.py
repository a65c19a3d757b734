r"""Relaxation models for fitting the azimuthal average of the image structure
function and the intermediate scattering function.

Same names, functions, parameters and parameter hints as the reference's
``src/python/fit_models.py``.  Each model is a :class:`Model` whose ``fit``
runs on the GPU (``fddm_b200_fit_lm``); ``eval`` evaluates the function with
numpy.  Parameter hints use ``EPSILON`` (machine epsilon) as the lower bound of
strictly positive parameters.

Intermediate scattering function models ``f(x)``:

* ``generic_exponential_isf_model``     A exp(-(Gamma x)^beta), beta in (0, inf)
* ``simple_exponential_isf_model``      beta fixed at 1
* ``stretched_exponential_isf_model``   beta in (0, 1]
* ``compressed_exponential_isf_model``  beta in [1, inf)
* ``double_exponential_isf_model``      A (alpha e1 + (1 - alpha) e2), alpha in [0, 1]
* ``flory_schulz_isf_model``            A (1 + sigma^2 Gamma x)^(-1/sigma^2), sigma in (0, 1]
* ``exponential_distribution_isf_model``  sigma fixed at 1

Structure function models ``D(x) = A (1 - f(x)) + B`` with the same names
without ``_isf``; ``B`` (noise) is unbounded.
"""

from typing import Union

import numpy as np

from ._fitting import Model

EPSILON = np.finfo(float).eps

# device evaluation ids (include/fddm_b200.h)
GENERIC_EXP_ISF, DOUBLE_EXP_ISF, FLORY_SCHULZ_ISF = 0, 1, 2
GENERIC_EXP_SF, DOUBLE_EXP_SF, FLORY_SCHULZ_SF = 3, 4, 5
SIMPLE_EXP, SIMPLE_SF = 6, 7


# -- intermediate scattering function models (fit_models.py:515-766) --------
def _generic_exponential_isf(x: Union[np.ndarray, float], A: float, Gamma: float, beta: float):
    r"""A \exp(-(\Gamma x)^\beta)"""
    return A * np.exp(-((x * Gamma) ** beta))


def _double_exponential_isf(x, A: float, Gamma1: float, beta1: float, Gamma2: float, beta2: float, alpha: float):
    r"""A (\alpha \exp(-(\Gamma_1 x)^{\beta_1}) + (1 - \alpha) \exp(-(\Gamma_2 x)^{\beta_2}))"""
    return A * (alpha * np.exp(-((x * Gamma1) ** beta1)) + (1 - alpha) * np.exp(-((x * Gamma2) ** beta2)))


def _flory_schulz_isf(x, A: float, Gamma: float, sigma: float):
    r"""A (1 + \sigma^2 \Gamma x)^{-1/\sigma^2}"""
    return A * (1 + sigma**2 * Gamma * x) ** (-1 / sigma**2)


# -- structure function models (fit_models.py:774-1055) ---------------------
def _generic_exponential(x, A: float, B: float, Gamma: float, beta: float):
    r"""A (1 - \exp(-(\Gamma x)^\beta)) + B"""
    return A * (1 - _generic_exponential_isf(x, 1.0, Gamma, beta)) + B


def _double_exponential(x, A: float, B: float, Gamma1: float, beta1: float, Gamma2: float, beta2: float,
                        alpha: float):
    r"""A (1 - \alpha e_1 - (1 - \alpha) e_2) + B"""
    return A * (1 - _double_exponential_isf(x, 1.0, Gamma1, beta1, Gamma2, beta2, alpha)) + B


def _flory_schulz(x, A: float, B: float, Gamma: float, sigma: float):
    r"""A (1 - (1 + \sigma^2 \Gamma x)^{-1/\sigma^2}) + B"""
    return A * (1 - _flory_schulz_isf(x, 1.0, Gamma, sigma)) + B


def _model(func, device_id: int, hints: dict) -> Model:
    m = Model(func, device_id)
    for name, h in hints.items():
        m.set_param_hint(name, **h)
    return m


_POS = dict(value=1.0, min=EPSILON, max=np.inf)
_NOISE = dict(value=0.0, min=-np.inf, max=np.inf)

generic_exponential_isf_model = _model(_generic_exponential_isf, GENERIC_EXP_ISF,
                                       {"A": _POS, "Gamma": _POS, "beta": _POS})
simple_exponential_isf_model = _model(_generic_exponential_isf, GENERIC_EXP_ISF,
                                      {"A": _POS, "Gamma": _POS, "beta": dict(value=1.0, vary=False)})
stretched_exponential_isf_model = _model(_generic_exponential_isf, GENERIC_EXP_ISF,
                                         {"A": _POS, "Gamma": _POS, "beta": dict(value=1.0, min=EPSILON, max=1.0)})
compressed_exponential_isf_model = _model(_generic_exponential_isf, GENERIC_EXP_ISF,
                                          {"A": _POS, "Gamma": _POS, "beta": dict(value=1.0, min=1.0, max=np.inf)})
double_exponential_isf_model = _model(_double_exponential_isf, DOUBLE_EXP_ISF,
                                      {"A": _POS, "Gamma1": _POS, "beta1": _POS, "Gamma2": _POS, "beta2": _POS,
                                       "alpha": dict(value=1.0, min=0.0, max=1.0)})
flory_schulz_isf_model = _model(_flory_schulz_isf, FLORY_SCHULZ_ISF,
                                {"A": _POS, "Gamma": _POS, "sigma": dict(value=1.0, min=EPSILON, max=1.0)})
exponential_distribution_isf_model = _model(_flory_schulz_isf, FLORY_SCHULZ_ISF,
                                            {"A": _POS, "Gamma": _POS, "sigma": dict(value=1.0, vary=False)})

generic_exponential_model = _model(_generic_exponential, GENERIC_EXP_SF,
                                   {"A": _POS, "B": _NOISE, "Gamma": _POS, "beta": _POS})
simple_exponential_model = _model(_generic_exponential, GENERIC_EXP_SF,
                                  {"A": _POS, "B": _NOISE, "Gamma": _POS, "beta": dict(value=1.0, vary=False)})
stretched_exponential_model = _model(_generic_exponential, GENERIC_EXP_SF,
                                     {"A": _POS, "B": _NOISE, "Gamma": _POS,
                                      "beta": dict(value=1.0, min=EPSILON, max=1.0)})
compressed_exponential_model = _model(_generic_exponential, GENERIC_EXP_SF,
                                      {"A": _POS, "B": _NOISE, "Gamma": _POS,
                                       "beta": dict(value=1.0, min=1.0, max=np.inf)})
double_exponential_model = _model(_double_exponential, DOUBLE_EXP_SF,
                                  {"A": _POS, "B": _NOISE, "Gamma1": _POS, "beta1": _POS, "Gamma2": _POS,
                                   "beta2": _POS, "alpha": dict(value=1.0, min=0.0, max=1.0)})
flory_schulz_model = _model(_flory_schulz, FLORY_SCHULZ_SF,
                            {"A": _POS, "B": _NOISE, "Gamma": _POS, "sigma": dict(value=1.0, min=EPSILON, max=1.0)})
exponential_distribution_model = _model(_flory_schulz, FLORY_SCHULZ_SF,
                                        {"A": _POS, "B": _NOISE, "Gamma": _POS, "sigma": dict(value=1.0, vary=False)})


# the device evaluation of each model function of the reference, by the function's name
_DEVICE_IDS = {
    "_generic_exponential_isf": GENERIC_EXP_ISF, "_double_exponential_isf": DOUBLE_EXP_ISF,
    "_flory_schulz_isf": FLORY_SCHULZ_ISF, "_generic_exponential": GENERIC_EXP_SF,
    "_double_exponential": DOUBLE_EXP_SF, "_flory_schulz": FLORY_SCHULZ_SF, "_simple_exp": SIMPLE_EXP,
    "_simple_image_structure_function": SIMPLE_SF,
}


def from_lmfit(model) -> Model:
    """The device model for an lmfit ``Model`` built on one of the reference's
    functions (``fit_models.py``, ``fit.py``), with its parameter hints.

    Raises ``NotImplementedError`` for any other function: only these models
    have a device evaluation.
    """
    if isinstance(model, Model):
        return model
    func = getattr(model, "func", None)
    name = getattr(func, "__name__", None)
    if name not in _DEVICE_IDS:
        raise NotImplementedError(f"no device evaluation for the model function {name!r}")
    m = Model(func, _DEVICE_IDS[name])
    for pname, hint in (getattr(model, "param_hints", None) or {}).items():
        if pname in m.param_names:
            m.set_param_hint(pname, **{k: v for k, v in hint.items() if k in ("value", "vary", "min", "max", "expr")})
    return m
