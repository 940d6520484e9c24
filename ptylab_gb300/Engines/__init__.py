"""GB300 engines with PtyLab's constructor and attribute surface
(``Engines.ePIE/mPIE/qNewton/mqNewton/e3PIE(reconstruction, experimentalData, params, monitor)``),
plus e3qNewton, a quasi-Newton gradient engine for multislice scans."""

from .BaseEngine import BaseEngine
from .batch import reconstruct_batch
from .e3PIE import e3PIE
from .e3qNewton import e3qNewton
from .ePIE import ePIE
from .mPIE import mPIE
from .mqNewton import mqNewton
from .qNewton import qNewton

__all__ = ["BaseEngine", "e3PIE", "e3qNewton", "ePIE", "mPIE", "mqNewton", "qNewton", "reconstruct_batch"]
