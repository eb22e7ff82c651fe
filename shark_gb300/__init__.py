"""GB300-native per-step Godunov update (gas + N dust species) for the SHARK driver.

The compute path is the sm_103a CUDA library ``libshark_gpu.so`` behind the C ABI in
``include/shark_gpu.h``; :mod:`shark_gb300.solver` binds it with ctypes and
:mod:`shark_gb300.setups` builds the run configurations and initial states of the in-scope
problems.  Build with :func:`shark_gb300.build.build`.
"""
from .config import SharkConfig, default_config  # noqa: F401
from . import setups  # noqa: F401


def Shark(cfg):
    """Open a device-resident run (see :class:`shark_gb300.solver.Shark`)."""
    from .solver import Shark as _Shark
    return _Shark(cfg)
