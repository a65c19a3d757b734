"""Container of the image structure function, interface of the reference's
``ImageStructureFunction`` (``src/python/imagestructurefunction.py:71-406``).

``_data`` has shape ``(len(lags) + 2, ny, nx // 2 + 1)``: the structure
function per lag, then the average power spectrum, then the variance, each
y-fftshifted (half plane in x).  When produced by ``core='b200'`` the object
also keeps the device copy of ``_data`` (``_device_data``), so that
``azimuthal_average`` can run on it without another host-to-device copy.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional, Tuple

import numpy as np


def _reconstruct_full_spectrum(halfplane: np.ndarray, shape: Tuple[int, int]) -> np.ndarray:
    """Full (Hermitian-symmetric) x-fftshifted plane from the half plane.

    The half plane is the rfft layout in x (columns 0..nx//2) with y already
    shifted.  Columns nx//2+1.. of the full plane are the mirrored columns
    1..nx//2-1 (even nx) or 1..nx//2 (odd nx); mirroring in y pairs row r with
    row (ny - r) of the unshifted plane, which in the shifted layout means rows
    1.. (even ny; row 0 mirrors onto itself) or rows 0.. (odd ny).
    Same result as ``src/python/imagestructurefunction.py:887-944``.
    """
    height, width = shape
    dim_y, dim_x = halfplane.shape
    full = np.zeros(shape, dtype=halfplane.dtype)
    full[:, :dim_x] = halfplane
    x_end = dim_x - 1 if width % 2 == 0 else dim_x
    y_start = 1 if height % 2 == 0 else 0
    full[y_start:height, dim_x:] = halfplane[y_start:height, 1:x_end][::-1, ::-1]
    if height % 2 == 0:
        full[0, dim_x:] = halfplane[0, 1:x_end][::-1]
    return np.fft.fftshift(full, axes=-1)


@dataclass
class ImageStructureFunction:
    """Image structure function container (same fields as the reference)."""

    _data: np.ndarray
    _kx: np.ndarray
    _ky: np.ndarray
    _width: int
    _height: int
    _tau: np.ndarray
    _pixel_size: float = 1.0
    _delta_t: float = 1.0
    _device_data: Optional[Any] = field(default=None, repr=False, compare=False)

    @property
    def data(self) -> np.ndarray:
        """The structure function, ``(lag, ky, kx)``."""
        return self._data[:-2]

    @property
    def kx(self) -> np.ndarray:
        return self._kx

    @property
    def ky(self) -> np.ndarray:
        return self._ky

    @property
    def width(self) -> int:
        return self._width

    @property
    def height(self) -> int:
        return self._height

    @property
    def tau(self) -> np.ndarray:
        return self._tau

    @property
    def power_spec(self) -> np.ndarray:
        """Average power spectrum of the frames."""
        return self._data[-2]

    @property
    def var(self) -> np.ndarray:
        """Variance over time of the Fourier-transformed frames."""
        return self._data[-1]

    @property
    def shape(self) -> Tuple[int, int, int]:
        return self.data.shape

    @property
    def pixel_size(self) -> float:
        return self._pixel_size

    @pixel_size.setter
    def pixel_size(self, pixel_size: float) -> None:
        self._kx *= self._pixel_size / pixel_size
        self._ky *= self._pixel_size / pixel_size
        self._pixel_size = pixel_size

    @property
    def delta_t(self) -> float:
        return self._delta_t

    @delta_t.setter
    def delta_t(self, delta_t: float) -> None:
        self._tau *= delta_t / self._delta_t
        self._delta_t = delta_t

    def __len__(self) -> int:
        return len(self.data)

    def save(self, fname: str = "analysis_blob", from_device: bool = False) -> None:
        """Write the object to ``fname`` (``.sf.ddm`` appended if missing) in the
        reference's file format (``imagestructurefunction.py:279-293``);
        ``from_device`` streams the device copy of ``_data`` instead of the host array."""
        from ._io import save_sf

        save_sf(self, fname, from_device)

    def set_frame_rate(self, frame_rate: float) -> None:
        self.delta_t = 1 / frame_rate

    def full_shape(self) -> Tuple[int, int, int]:
        dim_t, dim_y = self.shape[:-1]
        return dim_t, dim_y, self._width

    def full_slice(self, idx: int) -> np.ndarray:
        if 0 <= idx < len(self.data):
            return _reconstruct_full_spectrum(self._data[idx], (self.height, self.width))
        raise IndexError(f"Index out of range. Choose an index between 0 and {len(self.data)}.")

    def full_power_spec(self) -> np.ndarray:
        return _reconstruct_full_spectrum(self._data[-2], (self.height, self.width))

    def full_var(self) -> np.ndarray:
        return _reconstruct_full_spectrum(self._data[-1], (self.height, self.width))

    def full_kx(self) -> np.ndarray:
        full = np.zeros_like(self.kx, shape=(self.width,))
        n = len(self.kx)
        full[:n] = self.kx
        full[n:] = -self.kx[1:-1][::-1] if self.width % 2 == 0 else -self.kx[1:][::-1]
        return np.fft.fftshift(full)

    def full_ky(self) -> np.ndarray:
        return self.ky
