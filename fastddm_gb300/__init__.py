"""fastddm_gb300: GB300-native (sm_103a) image-structure-function core for FastDDM.

A drop-in ``core='b200'`` for ``fastddm.ddm(img_seq, lags, mode='fft'|'diff',
window=...)`` and a device implementation of ``azimuthal_average``.  The
numerical work runs in hand-written CUDA kernels (``csrc/``) behind the C ABI
declared in ``include/fddm_b200.h``; PyTorch only supplies device memory and
streams.
"""

from ._config import DTYPE, IS_SINGLE_PRECISION
from ._ddm import ddm, _backend
from ._ddm_b200 import DdmPlan, ddm_device, ddm_diff_b200, ddm_fft_b200
from ._fftopt import next_fast_len
from .azimuthalaverage import AzimuthalAverage, azimuthal_average, azimuthal_average_array
from .imagestructurefunction import ImageStructureFunction
from ._io import AAReader, ISFReader, SFReader, ddm_save, load
from .intermediatescatteringfunction import IntermediateScatteringFunction, azavg2isf_estimate
from .noise_est import estimate_camera_noise
from . import lags, mask, utils, window

__version__ = "0.1.0"


def _load_tuning_table() -> None:
    """Measured launch shapes of the temporal kernels (``tuning_table.json``), when the library is built."""
    from . import _build, autotune

    # only an up-to-date library: loading a stale one would keep it in the process across a rebuild
    if _build.LIB_PATH.exists() and not _build.is_stale():
        try:
            autotune.load_table()
        except (OSError, RuntimeError, ValueError, KeyError, AttributeError):  # no table: the occupancy model
            pass


_load_tuning_table()
