"""Learned warm start: a small encoder-decoder network, trained on the GPU by
this package's own tensor-core kernels, that maps diffraction patterns to
object patches stitched into an initial object for the reconstruction engines."""

from .network import LEVELS, WarmStartNet, layer_specs

__all__ = ["LEVELS", "WarmStartNet", "layer_specs"]
