"""Exception types mirroring the .NET ones the reference throws, and the
mapping from C-ABI status codes to them."""
from __future__ import annotations

from . import _native


class ArgumentException(ValueError):
    def __init__(self, message: str = "", param_name: str | None = None):
        super().__init__(message)
        self.ParamName = param_name


class ArgumentNullException(ArgumentException):
    def __init__(self, param_name: str):
        super().__init__(f"Value cannot be null. (Parameter '{param_name}')", param_name)


class ArgumentOutOfRangeException(ArgumentException):
    def __init__(self, param_name: str):
        super().__init__(f"Specified argument was out of the range of valid values. (Parameter '{param_name}')",
                         param_name)


class IndexOutOfRangeException(IndexError):
    pass


class InvalidOperationException(RuntimeError):
    pass


class DeviceOutOfMemoryError(MemoryError):
    """Device memory for the factor or its workspaces could not be reserved."""


class DeviceWaitTimeoutError(RuntimeError):
    """A bounded device wait expired; the context is still usable."""


class RefinementNotConvergedError(InvalidOperationException):
    """Iterative refinement did not reach its tolerance."""


def raise_for_status(status: int, message) -> None:
    if status == _native.OK:
        return
    if isinstance(message, bytes):
        message = message.decode(errors="replace")
    if status in (_native.BAD_ARG, _native.PATTERN_MISMATCH):
        raise ArgumentException(message)
    if status == _native.NOT_SPD:
        raise InvalidOperationException(message)
    if status == _native.OOM:
        raise DeviceOutOfMemoryError(message)
    if status == _native.TIMEOUT:
        raise DeviceWaitTimeoutError(message)
    if status == _native.NO_CONVERGENCE:
        raise RefinementNotConvergedError(message)
    if status == _native.TOO_DENSE:
        raise InvalidOperationException(message)
    if status == _native.OUT_OF_RANGE:
        err = ArgumentOutOfRangeException("")
        err.args = (message,)
        raise err
    if status == _native.NOT_IN_PATTERN:
        raise InvalidOperationException(message)
    raise InvalidOperationException(f"native call failed with status {status}: {message}")
