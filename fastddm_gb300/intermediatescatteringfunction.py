"""Intermediate scattering function estimated from the azimuthal average:
``IntermediateScatteringFunction`` and ``azavg2isf_estimate`` with the
interface and results of the reference's
``src/python/intermediatescatteringfunction.py`` (container ``:75-211``,
estimate ``:733-885``).

f(k, tau) = 1 - (D(k, tau) - B(k)) / A(k), with the noise B from
``estimate_camera_noise`` (or given) and the plateau A + B from twice the
variance or power spectrum (or given); the uncertainty propagates those of
D, B and A + B.  The arithmetic is elementwise over (k, tau) in the
reference's operation order, so the results are identical to the
reference's loop over k.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from ._config import DTYPE
from .azimuthalaverage import AzimuthalAverage
from .noise_est import estimate_camera_noise


@dataclass
class IntermediateScatteringFunction:
    """Intermediate scattering function container (same fields as the reference)."""

    _data: np.ndarray
    _err: Optional[np.ndarray]
    k: np.ndarray
    tau: np.ndarray
    bin_edges: np.ndarray

    @property
    def data(self) -> np.ndarray:
        return self._data

    @property
    def err(self) -> Optional[np.ndarray]:
        return self._err

    @property
    def shape(self) -> Tuple[int, int]:
        return self.data.shape

    def save(self, fname: str = "analysis_blob") -> None:
        """Write the object to ``fname`` (``.isf.ddm`` appended if missing) in the reference's format."""
        from ._io import save_isf

        save_isf(self, fname)


def _custom(values, errors, dim_k: int, what: str):
    if values is not None and len(values) != dim_k:
        raise RuntimeError(f"Custom {what} array dimension not compatible with given azimuthal average.\n"
                           f"Size of {what} should be {dim_k}.")
    if errors is None:
        errors = values
    if errors is not None and len(errors) != dim_k:
        raise RuntimeError(f"Custom {what}_err array dimension not compatible with given azimuthal average.\n"
                           f"Size of {what}_err should be {dim_k}.")
    return values, errors


def azavg2isf_estimate(az_avg: AzimuthalAverage, noise_est: str = "polyfit", plateau_est: str = "var",
                       noise: Optional[np.ndarray] = None, noise_err: Optional[np.ndarray] = None,
                       plateau: Optional[np.ndarray] = None, plateau_err: Optional[np.ndarray] = None,
                       **kwargs) -> IntermediateScatteringFunction:
    """AzimuthalAverage -> IntermediateScatteringFunction (``intermediatescatteringfunction.py:733-885``)."""
    dim_k, dim_t = az_avg.shape
    if noise_est == "custom":
        noise, noise_err = _custom(noise, noise_err, dim_k, "noise")
    else:
        noise, noise_err = estimate_camera_noise(az_avg, mode=noise_est, **kwargs)
    noise = noise.astype(DTYPE)
    noise_err = noise_err.astype(DTYPE)
    if plateau_est == "custom":
        plateau, plateau_err = _custom(plateau, plateau_err, dim_k, "plateau")
    elif plateau_est == "var":
        plateau = 2 * az_avg.var
        plateau_err = 2 * az_avg.var if az_avg.var_err is None else 2 * az_avg.var_err
    elif plateau_est == "power_spec":
        plateau = 2 * az_avg.power_spec
        plateau_err = 2 * az_avg.power_spec if az_avg.power_spec_err is None else 2 * az_avg.power_spec_err
    else:
        raise RuntimeError(f"Unsupported plateau_est mode {plateau_est}. "
                           f"Possible values are {['custom', 'power_spec', 'var']}")
    plateau = plateau.astype(DTYPE)
    plateau_err = plateau_err.astype(DTYPE)

    apb = plateau[:, None]          # A + B
    b = noise[:, None]              # B
    a = apb - b                     # A
    s_apb = plateau_err[:, None]
    s_b = noise_err[:, None]
    y = az_avg.data.astype(DTYPE)
    s_y = y if az_avg.err is None else az_avg.err.astype(DTYPE)
    data = 1 - (y - b) / a
    sigma2 = ((y - b) / a ** 2 * s_apb) ** 2
    sigma2 += ((apb - y) / a ** 2 * s_b) ** 2
    sigma2 += (s_y / a) ** 2
    err = np.sqrt(sigma2)
    return IntermediateScatteringFunction(data, err, az_avg.k.astype(DTYPE), az_avg.tau.astype(DTYPE),
                                          az_avg.bin_edges.astype(DTYPE))
