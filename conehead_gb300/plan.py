"""RT Plan beams as (Source, Block) pairs for the dose engine.

The reference reads only the block map from a plan (conehead/block.py:87-215)
and leaves the gantry and collimator to the caller (example.py:12-19).  This
helper reads both from control point 0 of every static beam, so a whole plan
goes to ``Conehead.calculate_batch`` in one call.  The isocentre position is
not applied: the reference's sources always aim at the origin of the
phantom's coordinates.
"""
import numpy as np

from .block import Block
from .dicom import read
from .source import Source


def plan_beams(plan, model="varian_clinac_6MV"):
    """[(Source, Block)] for each beam of ``plan`` (a Dataset or a file path)."""
    if not hasattr(plan, "BeamSequence"):
        plan = read(plan, force=True)
    out = []
    for i, beam in enumerate(plan.BeamSequence):
        cp = beam.ControlPointSequence[0]
        sad = beam.get("SourceAxisDistance") if hasattr(beam, "get") else getattr(beam, "SourceAxisDistance", None)
        src = Source(model) if sad is None else Source(model, sad=np.float32(float(sad) / 10))
        src.gantry = float(getattr(cp, "GantryAngle", 0.0) or 0.0) % 360
        src.collimator = float(getattr(cp, "BeamLimitingDeviceAngle", 0.0) or 0.0) % 360
        out.append((src, Block.from_plan(plan, beam=i)))
    return out
