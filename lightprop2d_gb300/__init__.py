"""GB300-native (sm_103a) backend for lightprop2d's angular-spectrum propagation.

Drop-in surface (lightprop2d/__init__.py:7-8): ``Beam2D``, the unit constants
``nm, um, mm, cm, m`` and every generator of ``profiles``.  ``backend`` holds
the tensor-level wrappers of the C ABI (include/lightprop2d_gb300.h).
"""
from .beam2d import Beam2D, nm, um, mm, cm, m  # noqa: F401
from .profiles import *  # noqa: F401,F403
from .profiles import __all__ as _profiles_all

__all__ = ("Beam2D", "nm", "um", "mm", "cm", "m") + tuple(_profiles_all)
__version__ = "0.1.0"
