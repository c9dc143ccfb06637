"""Tolerance configuration of the tolerant comparisons (approx_float).

Mirrors the reference's ``ApproxConfig`` and its module-level
``real_space_tolerance`` / ``reciprocal_space_tolerance`` accessors
(wrap/_approx.cpp:7-40; src/approx_config.hpp:17-72).  A grid copies the
reciprocal-space tolerance and the digit count into its device tables when
it is built (``brx_geometry.float_tolerance`` and ``digit``); changing the
global configuration afterwards affects grids built later, as the reference's
global config does for objects that read it at construction.
"""
from __future__ import annotations


class ApproxConfig:
    """(digits, real-space tolerance, reciprocal-space tolerance)."""

    def __init__(self, digits=1000, real_space_tolerance=1e-10, reciprocal_space_tolerance=1e-10):
        self.digits = digits
        self.real_space_tolerance = real_space_tolerance
        self.reciprocal_space_tolerance = reciprocal_space_tolerance

    @property
    def digits(self):
        return self._digits

    @digits.setter
    def digits(self, v):
        v = int(v)
        if v < 1:
            raise ValueError("digits must be positive")
        self._digits = v

    @property
    def real_space_tolerance(self):
        return self._direct

    @real_space_tolerance.setter
    def real_space_tolerance(self, v):
        self._direct = _tolerance(v)

    @property
    def reciprocal_space_tolerance(self):
        return self._reciprocal

    @reciprocal_space_tolerance.setter
    def reciprocal_space_tolerance(self, v):
        self._reciprocal = _tolerance(v)

    def __repr__(self):
        return (f"ApproxConfig(digits={self.digits}, real_space_tolerance={self.real_space_tolerance}, "
                f"reciprocal_space_tolerance={self.reciprocal_space_tolerance})")


def _tolerance(v):
    v = float(v)
    if not v >= 0:
        raise ValueError("a tolerance must be non-negative")
    return v


# the reference's global configuration: digit 1000, 1e-12 in both spaces
# (src/approx_config.hpp:17)
config = ApproxConfig(1000, 1e-12, 1e-12)


def real_space_tolerance(tol=None):
    """The global real-space tolerance; with an argument, set it."""
    if tol is None:
        return config.real_space_tolerance
    config.real_space_tolerance = tol


def reciprocal_space_tolerance(tol=None):
    """The global reciprocal-space tolerance; with an argument, set it."""
    if tol is None:
        return config.reciprocal_space_tolerance
    config.reciprocal_space_tolerance = tol
