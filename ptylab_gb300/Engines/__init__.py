"""GB300 engines with PtyLab's constructor and attribute surface
(``Engines.ePIE/mPIE/qNewton/mqNewton/e3PIE(reconstruction, experimentalData, params, monitor)``)."""

from .BaseEngine import BaseEngine
from .batch import reconstruct_batch
from .e3PIE import e3PIE
from .ePIE import ePIE
from .mPIE import mPIE
from .mqNewton import mqNewton
from .qNewton import qNewton

__all__ = ["BaseEngine", "e3PIE", "ePIE", "mPIE", "mqNewton", "qNewton", "reconstruct_batch"]
