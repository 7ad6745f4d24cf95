"""GB300-native PSTD solve with openPSTD's kernel API.

The configuration classes (``config``) import without a GPU.  The solver
(``kernel.PSTDKernel``) loads the in-tree CUDA library ``libpstd_gb300.so``
and raises if it is missing: there is no CPU fallback.
"""
from .config import (PSTDSettings, DomainConf, DomainConfEdge, PSTDConfiguration,  # noqa: F401
                     RK_COEFFICIENTS)

__version__ = "0.1.0"
