"""Error types mirroring ``GeostatError`` (crates/geostat-core/src/error.rs:14-39).

The C ABI returns the same numeric codes (include/geostat_gb300.h, GS_ERR_*);
``raise_for`` maps a code and the library's last message to the matching
exception.  All subclass ``ValueError`` because the reference's Python
binding raises ``ValueError`` for every ``GeostatError``
(crates/geostat-python/src/lib.rs:46-48).
"""


class GeostatError(ValueError):
    code = 0


class InsufficientData(GeostatError):
    code = 1


class DimensionMismatch(GeostatError):
    code = 2


class SingularSystem(GeostatError):
    code = 3


class InvalidParameter(GeostatError):
    code = 4


class NoNeighbors(GeostatError):
    code = 5


class DuplicatePoints(GeostatError):
    code = 6


class CudaError(RuntimeError):
    """A CUDA runtime failure inside the library (no reference counterpart)."""
    code = 100


class OutOfDeviceMemory(RuntimeError):
    """A request needs more device memory than the library may use."""
    code = 101


class IoError(OSError):
    """File input/output (the geostat CLI's I/O errors)."""
    code = 102


class Cancelled(RuntimeError):
    """A serving request cancelled before it started (no reference counterpart)."""
    code = 103


_BY_CODE = {c.code: c for c in (InsufficientData, DimensionMismatch, SingularSystem,
                                InvalidParameter, NoNeighbors, DuplicatePoints, CudaError,
                                OutOfDeviceMemory, IoError, Cancelled)}


def raise_for(code: int, message: str):
    if code == 0:
        return
    raise _BY_CODE.get(code, RuntimeError)(message)
