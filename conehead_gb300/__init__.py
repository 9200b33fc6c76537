"""GB300-native collapsed-cone dose engine with conehead's calculate() API."""
from .source import Source
from .block import Block
from .phantom import SimplePhantom, GridPhantom, DoseGrid

__all__ = ["Source", "Block", "SimplePhantom", "GridPhantom", "DoseGrid"]
