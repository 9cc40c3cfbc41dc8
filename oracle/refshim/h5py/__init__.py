"""Empty h5py stand-in (the reference's HDF5 reader/writer are never called)."""


class File:  # pragma: no cover - never used
    def __init__(self, *args, **kwargs):
        raise RuntimeError("h5py is not available in this environment")
