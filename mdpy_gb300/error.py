"""Exception classes with the names mdpy raises on the hot path
(mdpy/error.py), plus the mapping from the C ABI's status codes.

A user catching ``mdpy.error.NonBoundedError`` and friends can catch the same
names here.  ``DeviceError`` is new: it carries a CUDA failure reported by
``libmdg``.
"""


class EnvironmentVariableError(Exception):
    pass


class UnitDimensionDismatchedError(Exception):
    pass


class GeomtryDimError(Exception):
    pass


class ArrayDimError(Exception):
    pass


class ParticleConflictError(Exception):
    pass


class ConstraintConflictError(Exception):
    pass


class ModifyJoinedTopologyError(Exception):
    pass


class NonBoundedError(Exception):
    pass


class PBCPoorDefinedError(Exception):
    pass


class CellListPoorDefinedError(Exception):
    pass


class ParameterPoorDefinedError(Exception):
    pass


class DumperPoorDefinedError(Exception):
    pass


class FileFormatError(Exception):
    pass


class ParticleLossError(Exception):
    pass


class DeviceError(RuntimeError):
    """A CUDA or library failure inside libmdg (allocation, launch, cuFFT)."""


class FixedPointOverflowError(ArithmeticError):
    """A force or energy left the int64 fixed-point range (|F| >= 2^31 in
    internal units); the step that produced it is not trustworthy."""


class DeviceTimeoutError(RuntimeError):
    """A bounded device-side wait gave up (the work item never completed)."""


# status codes of include/mdg.h -> exception class
_STATUS = {
    1: ValueError,            # MDG_ERR_INVALID
    2: DeviceError,           # MDG_ERR_CUDA
    3: MemoryError,           # MDG_ERR_NOMEM
    4: PBCPoorDefinedError,   # MDG_ERR_BOX
    5: CellListPoorDefinedError,  # MDG_ERR_CUTOFF
    6: ParticleLossError,     # MDG_ERR_PARTICLE_LOSS
    7: FixedPointOverflowError,   # MDG_ERR_OVERFLOW
    8: DeviceError,           # MDG_ERR_CUFFT
    9: DeviceTimeoutError,    # MDG_ERR_TIMEOUT
    10: ValueError,           # MDG_ERR_CAPACITY
    11: NonBoundedError,      # MDG_ERR_STATE
}


def status_to_exception(code: int, message: str) -> Exception:
    cls = _STATUS.get(code, RuntimeError)
    return cls("libmdg status %d: %s" % (code, message))
