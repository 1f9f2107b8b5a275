"""Minimal stand-in for ``astropy`` so reference test modules import.

Only ``astropy.units.deg`` (as radians) and ``astropy.units.mm`` (as 1.0) are
needed by the reference's conservative/multilinear known-answer tests.
"""

from . import units  # noqa: F401
