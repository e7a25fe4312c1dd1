"""pyalign_gb300: pyalign's batched alignment solve on one GB300 (sm_103a).

``pyalign_gb300.algorithm`` is a drop-in for pyalign's native ``algorithm`` module.  To run
an installed pyalign (0.4.x) on the GPU, call :func:`install` before importing pyalign::

    import pyalign_gb300
    pyalign_gb300.install()
    import pyalign          # pyalign.solve now drives the GB300 kernels

The C ABI underneath is declared in include/pyalign_gb300.h.
"""

import importlib.machinery
import sys
import types

from . import algorithm

__all__ = ["algorithm", "install"]


def install():
    """Register ``algorithm`` as ``pyalign.algorithm.native.algorithm``.

    pyalign/cpu.py:21-47 imports the first of pyalign.algorithm.{native, intel_avx2,
    apple_m1, generic}.algorithm that exists; registering ``native`` makes it pick the
    GPU module.  Must run before ``import pyalign``.
    """
    if "pyalign.solve" in sys.modules:
        raise RuntimeError("call pyalign_gb300.install() before importing pyalign")
    pkg = types.ModuleType("pyalign.algorithm.native")
    pkg.__path__ = []
    pkg.__spec__ = importlib.machinery.ModuleSpec("pyalign.algorithm.native", None, is_package=True)
    algorithm.__spec__ = importlib.machinery.ModuleSpec("pyalign.algorithm.native.algorithm", None)
    pkg.algorithm = algorithm
    sys.modules["pyalign.algorithm.native"] = pkg
    sys.modules["pyalign.algorithm.native.algorithm"] = algorithm
    return algorithm
