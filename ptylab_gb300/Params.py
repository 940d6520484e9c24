"""Reconstruction switches, mirroring PtyLab's ``Params`` (PtyLab/Params/Params.py:31-231).

Same attribute names and defaults, so engine code and user scripts written for
PtyLab read the same flags.  ``gpuSwitch`` checks this package's own CUDA
library and ``torch.cuda`` instead of CuPy (Params.py:10-28, 207-231).
"""

from __future__ import annotations

import logging

import numpy as np

logger = logging.getLogger("GPU")


def _check_gpu_availability(verbose=False):
    """True when libptyg loads and device 0 is an sm_103a GPU."""
    from . import _native

    ok = _native.available(0)
    if verbose:
        logger.info("GB300 kernels available" if ok else "GB300 kernels unavailable")
    return ok


class Params(object):
    def __init__(self):
        self.positionCorrectionSwitch_radius = 1
        self.objectTVfreq = 5
        self.objectTVregSwitch = False
        self.objectTVregStepSize = 1e-3
        self.weigh_probe_updates_by_intensity = False
        self.logger = logging.getLogger("Params")
        self.dump_obj = False
        self.fftshiftSwitch = False
        self.fftshiftFlag = False
        self.FourierMaskSwitch = False
        self.CPSCswitch = False
        self.CPSCupsamplingFactor = None
        self.intensityConstraint = "standard"
        self.propagatorType = "Fraunhofer"
        self.momentumAcceleration = False
        self.adaptiveMomentumAcceleration = False
        self._gpuSwitch = _check_gpu_availability(verbose=False)
        self.saveMemory = False
        self.probeUpdateStart = 1
        self.objectUpdateStart = 1
        self.positionOrder = "random"
        self.orthogonalizationSwitch = False
        self.orthogonalizationFrequency = 10
        self.objectSmoothenessSwitch = False
        self.objectSmoothenessWidth = 2
        self.objectSmoothnessAleph = 1e-2
        self.absObjectSwitch = False
        self.absObjectBeta = 1e-2
        self.objectContrastSwitch = False
        self.probeSmoothenessSwitch = False
        self.probeSmoothnessAleph = 5e-2
        self.probeSmoothenessWidth = 3
        self.probeBoundary = False
        self.absorbingProbeBoundary = False
        self.absorbingProbeBoundaryAleph = 5e-2
        self.probePowerCorrectionSwitch = False
        self.probeSpectralPowerCorrectionSwitch = False
        self.modulusEnforcedProbeSwitch = False
        self.absProbeSwitch = False
        self.absProbeBeta = 1e-2
        self.couplingSwitch = False
        self.couplingAleph = 50e-2
        self.binaryProbeSwitch = False
        self.binaryProbeThreshold = 0.1
        self.binaryProbeAleph = 10e-2
        self.backgroundModeSwitch = False
        self.comStabilizationSwitch = False
        self.PSDestimationSwitch = False
        self.positionCorrectionSwitch = False
        self.adaptiveDenoisingSwitch = False
        self.l2reg = False
        self.l2reg_probe_aleph = 0.01
        self.l2reg_object_aleph = 0.001
        self.TV_autofocus = False
        # the autofocus's and OPR's settings, with PtyLab's defaults
        # (Params.py:127-192): present so scripts that set or read them run;
        # switching either feature on raises NotImplementedError
        self.TV_autofocus_metric = "TV"
        self.TV_autofocus_intensityonly = False
        self.TV_autofocus_stepsize = 5
        self.TV_autofocus_aleph = 0.01
        self.TV_autofocus_roi = [0.4, 0.6]
        self.TV_autofocus_range_dof = 11
        self.TV_autofocus_friction = 0.7
        self.TV_autofocus_what = "object"
        self.TV_autofocus_run_every = 3
        self.TV_autofocus_min_z = None
        self.TV_autofocus_max_z = None
        self.TV_autofocus_nplanes = 11
        self.map_position_to_z_change = False
        self.OPRP = False
        self.OPR_modes = np.array([0])
        self.OPR_subspace = 4
        self.OPR_alpha = 0.05
        self.OPR_tv_freq = 5
        self.OPR_tv = False
        self.OPR_tsvd_type = "gram"
        self.OPR_orthogonalize_modes = True
        self.OPR_fast_orthogonalization = True
        self.OPR_neighbor_constraint = False
        self.SHG_probe = False

    @property
    def propagator(self):
        """Alias for propagatorType."""
        return self.propagatorType

    @propagator.setter
    def propagator(self, value):
        self.propagatorType = value

    @property
    def gpuSwitch(self):
        return self._gpuSwitch

    @gpuSwitch.setter
    def gpuSwitch(self, value: bool):
        if value:
            if _check_gpu_availability():
                self._gpuSwitch = value
            else:
                raise AttributeError(
                    "GB300 kernels (libptyg.so on an sm_103a device) unavailable, cannot set `self.gpuSwitch = True`"
                )
        else:
            self._gpuSwitch = value
