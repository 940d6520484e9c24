"""Measurement-file loading with PtyLab's function names and behaviour
(PtyLab/io/readHdf5.py:1-125), over this package's own HDF5 reader instead
of PyTables and h5py."""

from __future__ import annotations

import logging
from pathlib import Path

import numpy as np

from . import hdf5

logger = logging.getLogger("readHdf5")

# These extensions can be loaded (readHdf5.py:14)
allowed_extensions = [".h5", ".hdf5", ".mat"]


def scalify(l):
    """Arrays of one element become Python scalars (readHdf5.py:17-27):
    MATLAB and h5py store scalars as [1, 1] or [1] arrays."""
    l = np.asarray(l).squeeze()
    try:
        return l.item()
    except ValueError:
        return l


def loadInputData(filename, requiredFields, optionalFields):
    """Required and optional fields of a measurement file as a dict
    (readHdf5.py:30-94).  Missing optional fields are None; an encoder stored
    as (2, n) is transposed to (n, 2) and centred, as the reference does."""
    filename = Path(filename)
    if not filename.exists():
        raise FileNotFoundError(f"Could not find file {filename}.")
    logger.debug("Loading input data: %s", filename)
    if filename.suffix not in allowed_extensions:
        raise NotImplementedError(
            "%s is not a valid extension. Currently, only these extensions are allowed: %s."
            % (filename.suffix, ["   ".join(allowed_extensions)][0])
        )
    dataset = dict()
    try:
        with hdf5.File(filename, "r") as f:
            for key in requiredFields:
                dataset[key] = scalify(f[key][()])
            for key in optionalFields:
                dataset[key] = scalify(f[key][()]) if key in f else None
    except Exception:
        logger.error("Error reading hdf5 file!")
        raise
    if "encoder" in dataset and dataset["encoder"] is not None:
        enc = np.asarray(dataset["encoder"])
        logger.info("Found encoder with shape %s", enc.shape)
        if enc.ndim == 2 and enc.shape[0] < enc.shape[1]:
            enc = enc.T
            logger.warning("Automatically changing the shape of encoder.")
            enc = enc - enc.mean(axis=0, keepdims=True)
        dataset["encoder"] = enc
    return dataset


def getOrientation(filename):
    """The file's ``orientation`` entry, or None (readHdf5.py:97-107)."""
    orientation = None
    with hdf5.File(filename, "r") as f:
        if "orientation" in f.keys():
            raw_value = np.array(f["orientation"][()]).ravel()[0]
            orientation = scalify(raw_value)
    return orientation


def checkDataFields(filename, requiredFields):
    """KeyError when a required field is missing (readHdf5.py:110-125)."""
    with hdf5.File(filename, "r") as f:
        fileFields = list(f.keys())
    for k in requiredFields:
        if k not in fileFields:
            raise KeyError("hdf5 file misses key %s" % k)
    return None
