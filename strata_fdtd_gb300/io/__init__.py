"""Result files (io/ of rjwalters/strata-fdtd).  ``legacy`` writes and reads
the raw-binary and JSON formats; the HDF5 writer and reader need h5py,
which this build does not use, and raise when constructed."""
from . import legacy  # noqa: F401


class _NeedsHDF5:
    def __init__(self, *args, **kwargs):
        raise NotImplementedError(
            f"{type(self).__name__} writes HDF5 through h5py, which is not available here; "
            "io.legacy.export_simulation writes the same results as binary and JSON files")


class HDF5ResultWriter(_NeedsHDF5):
    """Not available: HDF5 output (io/hdf5.py:24-240) needs h5py."""


class HDF5ResultReader(_NeedsHDF5):
    """Not available: HDF5 input (io/hdf5.py:243-) needs h5py."""


OutputHDF5Writer, OutputHDF5Reader = HDF5ResultWriter, HDF5ResultReader
__all__ = ["legacy", "HDF5ResultWriter", "HDF5ResultReader", "OutputHDF5Writer",
           "OutputHDF5Reader"]
