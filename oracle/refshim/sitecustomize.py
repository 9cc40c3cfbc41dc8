"""numpy 2 removed ``np.round_``, which the reference's ``unwrap_vec`` calls
(mdpy/utils/pbc.py:42); alias it back so the reference runs unmodified."""
import numpy as _np

if not hasattr(_np, "round_"):
    _np.round_ = _np.round
