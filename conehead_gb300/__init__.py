"""GB300-native collapsed-cone dose engine with conehead's calculate() API.

Host model objects (Source, Block, phantoms) mirror the reference's
attribute contract; the dose path itself runs only on the GPU through the
CUDA library built by ``conehead_gb300.build``.
"""
from .source import Source
from .block import Block
from .phantom import SimplePhantom, GridPhantom, DoseGrid
from .conehead import Conehead

__all__ = ["Source", "Block", "SimplePhantom", "GridPhantom", "DoseGrid", "Conehead"]
