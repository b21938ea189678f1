"""Mirror of the reference's compiled module ``libssim`` (bindings/src/main.cpp:5-12): ``libssim.fem``
holds the time-step classes and ``unit_box``, all backed by the GB300 library."""
from . import fem

__all__ = ["fem"]
