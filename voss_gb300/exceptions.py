"""Exceptions (the reference's bindings/python/voss/exceptions.py and
primes.py:22-27)."""


class VossError(RuntimeError):
    """Base exception for all voss errors."""


class VossInvalidNError(VossError):
    """Raised when N is below the allowed minimum."""


class VossInvalidArgError(VossError):
    """Raised when an argument is invalid."""
