"""GB300 engine for CompFinance's Monte Carlo valuation and AAD-risk path.

The engine is the C-ABI shared library ``libcfgpu.so`` (CUDA kernels for sm_103a plus a
host C++ runtime).  This package binds it with ctypes under the reference's own names
(``main.h``: value, AADriskOne, AADriskAggregate, AADriskMulti, dupireCalib,
dupireSuperbucket; ``store.h``: putBlackScholes, putDupire, putEuropean, putBarrier,
putEuropeans).  There is no CPU fallback: without the library every call raises.
"""
from .api import Engine, NumericalParam, CfError, library_path  # noqa: F401

__all__ = ["Engine", "NumericalParam", "CfError", "library_path"]
