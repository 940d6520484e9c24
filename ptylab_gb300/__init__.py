"""GB300-native drop-in for PtyLab's per-position ptychography reconstruction loop.

Engines (ePIE, mPIE, qNewton) and Operators (object2detector /
detector2object) keep PtyLab's call surface; the work runs in libptyg.so, a
library of hand-written sm_103a CUDA kernels behind a C ABI (include/ptyg.h).
"""

__version__ = "0.1.0"

from . import Engines, Operators  # noqa: E402,F401
from .CalibrationFPM import IlluminationCalibration  # noqa: E402,F401
from .ExperimentalData import ExperimentalData  # noqa: E402,F401
from .Monitor import DummyMonitor  # noqa: E402,F401
from .Params import Params  # noqa: E402,F401
from .Reconstruction import Reconstruction  # noqa: E402,F401


def easyInitialize(filename, engine=None, operationMode="CPM", dummyMonitor=False):
    """PtyLab's standard set-up (PtyLab/__init__.py:11-58): load the
    measurement file, build Params and a Reconstruction with its initial
    guesses and the engine; FPM also returns an IlluminationCalibration and
    sets the 'NA' position order and probeBoundary.  The monitor is a
    DummyMonitor either way (no plotting window here)."""
    if engine is None:
        engine = Engines.ePIE
    if operationMode not in ("CPM", "FPM"):
        raise NotImplementedError()
    experimentalData = ExperimentalData(filename, operationMode)
    monitor = DummyMonitor()
    params = Params()
    reconstruction = Reconstruction(experimentalData, params)
    reconstruction.initializeObjectProbe()
    if operationMode == "CPM":
        eng = engine(reconstruction, experimentalData, params, monitor)
        return experimentalData, reconstruction, params, monitor, eng
    calib = IlluminationCalibration(reconstruction, experimentalData)
    eng = engine(reconstruction, experimentalData, params, monitor)
    params.positionOrder = "NA"
    params.probeBoundary = True
    return experimentalData, reconstruction, params, monitor, eng, calib
