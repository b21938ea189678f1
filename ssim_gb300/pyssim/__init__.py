"""Mirror of the reference's Python package ``pyssim`` (pyssim/fem/__init__.py)."""
from . import fem

__all__ = ["fem"]
