"""Build-time facts of the GB300 package (the reference generates its counterpart,
``src/python/_config.py.in:10-16``, from CMake options)."""

import numpy as np

IS_SINGLE_PRECISION = False  # results are always float64, like the reference's default build
DTYPE = np.float64
ARCH = "sm_103a"
