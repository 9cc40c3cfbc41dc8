"""Empty MDAnalysis stand-in: importing the reference's PDB/PSF/DCD parsers
must succeed, but they are never called by the fixture scripts."""


class Universe:  # pragma: no cover - never used
    def __init__(self, *args, **kwargs):
        raise RuntimeError("MDAnalysis is not available in this environment")
