"""GB300 (sm_103a) implementation of euc's triangle pipeline.

The CUDA library (libeuc_gb300.so) is loaded lazily by `euc_gb300.capi`; the
pure-Python modules (abi, scenes) work without a GPU.
"""
from . import abi  # noqa: F401
