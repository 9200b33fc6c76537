"""Dose-grid container; re-exported from ``phantom`` (``conehead/dosegrid.py``)."""
from .phantom import DoseGrid

__all__ = ["DoseGrid"]
