"""PtyLab's measurement and result files (PtyLab/io/readHdf5.py), read and
written by this package's own HDF5 implementation (``hdf5``)."""
