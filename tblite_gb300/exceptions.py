"""Exception types of the Python surface (same names as python/tblite/exceptions.py)."""


class TBLiteRuntimeError(RuntimeError):
    """Raised when the engine reports an error."""


class TBLiteTypeError(TypeError):
    """Raised on wrong argument types."""


class TBLiteValueError(ValueError):
    """Raised on invalid argument values."""
