def guess_atom_type(name):  # pragma: no cover - never used
    raise RuntimeError("MDAnalysis is not available in this environment")
