"""turbotops_gb300 — the GB300 front end of turbotops' Vietoris–Rips persistence.

    >>> import numpy as np, turbotops_gb300 as tg
    >>> dgms, info = tg.persistence(points, maxdim=2)        # turbo_tops.persistence drop-in

Device stages one by one: ``turbotops_gb300.ops`` (torch tensors); the C-ABI
itself: ``turbotops_gb300.capi`` and include/turbotops_gb300.h.
"""
from .api import canonical, format_diagram, persistence

__all__ = ["persistence", "canonical", "format_diagram", "__version__"]
__version__ = "0.1.0"
