"""GB300-native drop-in for PtyLab's per-position ptychography reconstruction loop.

Engines (ePIE, mPIE, qNewton) and Operators (object2detector /
detector2object) keep PtyLab's call surface; the work runs in libptyg.so, a
library of hand-written sm_103a CUDA kernels behind a C ABI (include/ptyg.h).
"""

__version__ = "0.1.0"

from . import Engines, Operators  # noqa: E402,F401
from .ExperimentalData import ExperimentalData  # noqa: E402,F401
from .Monitor import DummyMonitor  # noqa: E402,F401
from .Params import Params  # noqa: E402,F401
from .Reconstruction import Reconstruction  # noqa: E402,F401
