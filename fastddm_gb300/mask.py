"""Masks for the azimuthal average, same as ``src/python/mask.py:29-64`` of the reference."""

from __future__ import annotations

from typing import Optional, Tuple

import numpy as np


def central_cross_mask(shape: Tuple[int, int], kx: Optional[np.ndarray] = None,
                       ky: Optional[np.ndarray] = None) -> np.ndarray:
    """Boolean mask that excludes the kx = 0 column and the ky = 0 row.

    Without ``kx``/``ky`` the half-plane layout is assumed: column 0 and row
    ``shape[0] // 2`` are the axes.
    """
    mask = np.full(shape, True)
    if kx is None or ky is None:
        mask[:, 0] = False
        mask[shape[0] // 2] = False
        return mask
    gx, gy = np.meshgrid(kx, ky)
    mask[(gx == 0.0) | (gy == 0.0)] = False
    return mask
