"""Minimal DICOM reader for RT Plan files (no pydicom).

The reference reads plans with ``pydicom.dcmread(path, force=True)``
(example.py:11) and walks them by keyword in ``Block._set_from_plan``
(conehead/block.py:87-215).  pydicom is not a dependency here, so this
module parses the file itself and returns a ``Dataset`` with the same
keyword access (``plan.BeamSequence[0].ControlPointSequence[0]...``), which
both this package's ``Block`` and the reference's accept.

Supported encodings: with or without the 128-byte preamble and ``DICM``
marker; file meta group in explicit VR little endian; data set in implicit
VR little endian (what the reference's fixture uses), explicit VR little
endian, deflated explicit VR little endian, or explicit VR big endian.
Sequences and items of defined and undefined length are both read.

Value decoding follows the DICOM value representations: ``DS`` becomes
``float`` (one value) or a list of floats (backslash-separated values), the
way pydicom's ``DSfloat`` values behave in NumPy; ``IS`` becomes ``int`` or
a list of ints; text VRs become ``str`` with padding stripped; binary
numeric VRs are unpacked; everything else stays ``bytes``.  An empty numeric
value reads as ``None``.

In implicit VR files the VR of an element comes from the data dictionary
below, which covers the RT Plan attributes the dose path and its callers
use.  Elements not in it keep their raw bytes (VR ``UN``), except that an
element of undefined length is read as a sequence, as the standard requires.
"""
import os
import struct
import zlib

IMPLICIT_LE = "1.2.840.10008.1.2"
EXPLICIT_LE = "1.2.840.10008.1.2.1"
DEFLATED_LE = "1.2.840.10008.1.2.1.99"
EXPLICIT_BE = "1.2.840.10008.1.2.2"

UNDEFINED = 0xFFFFFFFF
ITEM = 0xFFFEE000
ITEM_END = 0xFFFEE00D
SEQ_END = 0xFFFEE0DD

# VRs with a 2-byte reserved field and a 4-byte length in explicit VR
_LONG_VRS = {"OB", "OD", "OF", "OL", "OV", "OW", "SQ", "SV", "UC", "UN", "UR", "UT", "UV"}
_ALL_VRS = _LONG_VRS | {"AE", "AS", "AT", "CS", "DA", "DS", "DT", "FL", "FD", "IS", "LO",
                        "LT", "PN", "SH", "SL", "SS", "ST", "TM", "UI", "UL", "US"}
_TEXT_VRS = {"AE", "AS", "CS", "DA", "DT", "LO", "LT", "PN", "SH", "ST", "TM", "UC", "UI",
             "UR", "UT"}
_BINARY = {"US": "H", "SS": "h", "UL": "I", "SL": "i", "FL": "f", "FD": "d", "UV": "Q",
           "SV": "q"}

# tag -> (VR, keyword).  RT Plan module attributes plus the common
# identification attributes of the file.
DICTIONARY = {
    0x00020010: ("UI", "TransferSyntaxUID"),
    0x00080005: ("CS", "SpecificCharacterSet"),
    0x00080012: ("DA", "InstanceCreationDate"),
    0x00080013: ("TM", "InstanceCreationTime"),
    0x00080016: ("UI", "SOPClassUID"),
    0x00080018: ("UI", "SOPInstanceUID"),
    0x00080020: ("DA", "StudyDate"),
    0x00080030: ("TM", "StudyTime"),
    0x00080060: ("CS", "Modality"),
    0x00080070: ("LO", "Manufacturer"),
    0x00081040: ("LO", "InstitutionalDepartmentName"),
    0x00081150: ("UI", "ReferencedSOPClassUID"),
    0x00081155: ("UI", "ReferencedSOPInstanceUID"),
    0x00100010: ("PN", "PatientName"),
    0x00100020: ("LO", "PatientID"),
    0x00185100: ("CS", "PatientPosition"),
    0x0020000D: ("UI", "StudyInstanceUID"),
    0x0020000E: ("UI", "SeriesInstanceUID"),
    0x00200052: ("UI", "FrameOfReferenceUID"),
    0x300A0002: ("SH", "RTPlanLabel"),
    0x300A0003: ("LO", "RTPlanName"),
    0x300A0004: ("ST", "RTPlanDescription"),
    0x300A000C: ("CS", "RTPlanGeometry"),
    0x300A0070: ("SQ", "FractionGroupSequence"),
    0x300A0071: ("IS", "FractionGroupNumber"),
    0x300A0078: ("IS", "NumberOfFractionsPlanned"),
    0x300A0080: ("IS", "NumberOfBeams"),
    0x300A0082: ("DS", "BeamDoseSpecificationPoint"),
    0x300A0084: ("DS", "BeamDose"),
    0x300A0086: ("DS", "BeamMeterset"),
    0x300A00A0: ("IS", "NumberOfBrachyApplicationSetups"),
    0x300A00B0: ("SQ", "BeamSequence"),
    0x300A00B2: ("SH", "TreatmentMachineName"),
    0x300A00B3: ("CS", "PrimaryDosimeterUnit"),
    0x300A00B4: ("DS", "SourceAxisDistance"),
    0x300A00B6: ("SQ", "BeamLimitingDeviceSequence"),
    0x300A00B8: ("CS", "RTBeamLimitingDeviceType"),
    0x300A00BA: ("DS", "SourceToBeamLimitingDeviceDistance"),
    0x300A00BC: ("IS", "NumberOfLeafJawPairs"),
    0x300A00BE: ("DS", "LeafPositionBoundaries"),
    0x300A00C0: ("IS", "BeamNumber"),
    0x300A00C2: ("LO", "BeamName"),
    0x300A00C3: ("ST", "BeamDescription"),
    0x300A00C4: ("CS", "BeamType"),
    0x300A00C6: ("CS", "RadiationType"),
    0x300A00CE: ("CS", "TreatmentDeliveryType"),
    0x300A00D0: ("IS", "NumberOfWedges"),
    0x300A00E0: ("IS", "NumberOfCompensators"),
    0x300A00ED: ("IS", "NumberOfBoli"),
    0x300A00F0: ("IS", "NumberOfBlocks"),
    0x300A010E: ("DS", "FinalCumulativeMetersetWeight"),
    0x300A0110: ("IS", "NumberOfControlPoints"),
    0x300A0111: ("SQ", "ControlPointSequence"),
    0x300A0112: ("IS", "ControlPointIndex"),
    0x300A0114: ("DS", "NominalBeamEnergy"),
    0x300A011A: ("SQ", "BeamLimitingDevicePositionSequence"),
    0x300A011C: ("DS", "LeafJawPositions"),
    0x300A011E: ("DS", "GantryAngle"),
    0x300A011F: ("CS", "GantryRotationDirection"),
    0x300A0120: ("DS", "BeamLimitingDeviceAngle"),
    0x300A0121: ("CS", "BeamLimitingDeviceRotationDirection"),
    0x300A0122: ("DS", "PatientSupportAngle"),
    0x300A0123: ("CS", "PatientSupportRotationDirection"),
    0x300A0125: ("DS", "TableTopEccentricAngle"),
    0x300A0126: ("CS", "TableTopEccentricRotationDirection"),
    0x300A0128: ("DS", "TableTopVerticalPosition"),
    0x300A0129: ("DS", "TableTopLongitudinalPosition"),
    0x300A012A: ("DS", "TableTopLateralPosition"),
    0x300A012C: ("DS", "IsocenterPosition"),
    0x300A012E: ("DS", "SurfaceEntryPoint"),
    0x300A0130: ("DS", "SourceToSurfaceDistance"),
    0x300A0134: ("DS", "CumulativeMetersetWeight"),
    0x300A0180: ("SQ", "PatientSetupSequence"),
    0x300A0182: ("IS", "PatientSetupNumber"),
    0x300A01B0: ("CS", "SetupTechnique"),
    0x300C0004: ("SQ", "ReferencedBeamSequence"),
    0x300C0006: ("IS", "ReferencedBeamNumber"),
    0x300C0060: ("SQ", "ReferencedStructureSetSequence"),
    0x300C006A: ("IS", "ReferencedPatientSetupNumber"),
    0x300E0002: ("CS", "ApprovalStatus"),
}
_KEYWORDS = {kw: tag for tag, (_, kw) in DICTIONARY.items()}


class DicomError(ValueError):
    """The bytes are not a DICOM data set this reader understands."""


class Element:
    __slots__ = ("tag", "VR", "value")

    def __init__(self, tag, vr, value):
        self.tag, self.VR, self.value = tag, vr, value

    @property
    def keyword(self):
        return DICTIONARY.get(self.tag, (None, ""))[1]

    def __repr__(self):
        return f"({self.tag >> 16:04X},{self.tag & 0xFFFF:04X}) {self.VR} {self.keyword}: {self.value!r}"


class Dataset:
    """Ordered elements with keyword attribute access, like a pydicom Dataset."""

    def __init__(self):
        self._elements = {}

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        tag = _KEYWORDS.get(name)
        if tag is None or tag not in self._elements:
            raise AttributeError(f"Dataset has no attribute '{name}'")
        return self._elements[tag].value

    def __contains__(self, key):
        tag = _KEYWORDS.get(key) if isinstance(key, str) else key
        return tag in self._elements

    def __getitem__(self, tag):
        return self._elements[tag]

    def __iter__(self):
        return iter(self._elements.values())

    def __len__(self):
        return len(self._elements)

    def get(self, name, default=None):
        try:
            return getattr(self, name)
        except AttributeError:
            return default

    def add(self, elem):
        self._elements[elem.tag] = elem

    def __repr__(self):
        return "\n".join(repr(e) for e in self)


class _Reader:
    def __init__(self, buf, explicit, little):
        self.buf = buf
        self.explicit = explicit
        self.end = "<" if little else ">"

    def _u16(self, off):
        return struct.unpack_from(self.end + "H", self.buf, off)[0]

    def _u32(self, off):
        return struct.unpack_from(self.end + "I", self.buf, off)[0]

    def _need(self, off, n):
        if off + n > len(self.buf):
            raise DicomError(f"truncated data set: {n} bytes wanted at offset {off}, {len(self.buf)} present")

    def header(self, off):
        """(tag, VR or None, length, offset of the value)."""
        self._need(off, 8)
        tag = (self._u16(off) << 16) | self._u16(off + 2)
        if (tag >> 16) == 0xFFFE:                      # items and delimiters carry no VR
            return tag, None, self._u32(off + 4), off + 8
        if not self.explicit:
            return tag, DICTIONARY.get(tag, ("UN", ""))[0], self._u32(off + 4), off + 8
        vr = self.buf[off + 4:off + 6].decode("ascii", "replace")
        if vr not in _ALL_VRS:
            raise DicomError(f"unknown VR {vr!r} at offset {off}")
        if vr in _LONG_VRS:
            self._need(off, 12)
            return tag, vr, self._u32(off + 8), off + 12
        return tag, vr, self._u16(off + 6), off + 8

    def dataset(self, off, stop, item=False):
        """Read elements from ``off`` up to ``stop`` (or an item delimiter)."""
        ds = Dataset()
        while off < stop:
            tag, vr, length, off = self.header(off)
            if tag == ITEM_END:
                if not item:
                    raise DicomError("item delimiter outside an item")
                return ds, off
            if tag in (ITEM, SEQ_END):
                raise DicomError(f"unexpected item tag {tag:08X} in a data set")
            if vr == "SQ" or length == UNDEFINED:
                seq, off = self.sequence(off, length, vr)
                ds.add(Element(tag, "SQ", seq))
                continue
            self._need(off, length)
            ds.add(Element(tag, vr, self.value(vr, self.buf[off:off + length])))
            off += length
        if item:
            raise DicomError("item of undefined length ends without a delimiter")
        return ds, off

    def sequence(self, off, length, vr):
        items = []
        stop = len(self.buf) if length == UNDEFINED else off + length
        reader = self
        if vr == "UN" and length == UNDEFINED and self.explicit:
            reader = _Reader(self.buf, False, self.end == "<")   # PS3.5 6.2.2: UN SQ is implicit VR
        while off < stop:
            tag, _, ilen, off = reader.header(off)
            if tag == SEQ_END:
                return items, off
            if tag != ITEM:
                raise DicomError(f"expected an item in a sequence, got tag {tag:08X}")
            if ilen == UNDEFINED:
                ds, off = reader.dataset(off, len(self.buf), item=True)
            else:
                reader._need(off, ilen)
                ds, _ = reader.dataset(off, off + ilen)
                off += ilen
            items.append(ds)
        if length == UNDEFINED:
            raise DicomError("sequence of undefined length ends without a delimiter")
        return items, off

    def value(self, vr, raw):
        if vr in ("DS", "IS"):
            parts = [p.strip(" \x00") for p in raw.decode("ascii", "replace").split("\\")]
            conv = float if vr == "DS" else int
            vals = [conv(p) if p else None for p in parts]
            if len(vals) == 1:
                return vals[0]
            return vals
        if vr in _TEXT_VRS or vr == "PN":
            text = raw.decode("latin-1").rstrip(" \x00")
            if vr in ("LT", "ST", "UT"):
                return text
            parts = text.split("\\")
            return parts[0] if len(parts) == 1 else parts
        if vr in _BINARY:
            code = _BINARY[vr]
            n = len(raw) // struct.calcsize(code)
            vals = list(struct.unpack(self.end + code * n, raw[:n * struct.calcsize(code)]))
            return vals[0] if n == 1 else vals
        if vr == "AT":
            n = len(raw) // 4
            vals = [(self._tag_at(raw, 4 * i)) for i in range(n)]
            return vals[0] if n == 1 else vals
        return bytes(raw)

    def _tag_at(self, raw, off):
        g, e = struct.unpack_from(self.end + "HH", raw, off)
        return (g << 16) | e


def _looks_explicit(buf, off):
    """Heuristic for files without a meta header: a VR follows the tag."""
    if off + 6 > len(buf):
        return False
    vr = buf[off + 4:off + 6]
    return vr.isalpha() and vr.isupper() and vr.decode("ascii") in _ALL_VRS


def read(source, force=True):
    """Read a DICOM file (path, bytes or binary file object) into a Dataset.

    ``force`` accepts files without the preamble and ``DICM`` marker, as
    ``pydicom.dcmread(..., force=True)`` does; with ``force=False`` such a
    file raises ``DicomError``.
    """
    if isinstance(source, (bytes, bytearray, memoryview)):
        buf = bytes(source)
    elif hasattr(source, "read"):
        buf = source.read()
    else:
        with open(os.fspath(source), "rb") as f:
            buf = f.read()
    off = 0
    if len(buf) >= 132 and buf[128:132] == b"DICM":
        off = 132
    elif buf[:4] == b"DICM":
        off = 4
    elif not force:
        raise DicomError("no DICM marker (pass force=True to read a bare data set)")
    meta = Dataset()
    if off + 2 <= len(buf) and struct.unpack_from("<H", buf, off)[0] == 0x0002:
        r = _Reader(buf, True, True)
        while off + 2 <= len(buf) and struct.unpack_from("<H", buf, off)[0] == 0x0002:
            tag, vr, length, voff = r.header(off)
            r._need(voff, length)
            meta.add(Element(tag, vr, r.value(vr, buf[voff:voff + length])))
            off = voff + length
    syntax = meta.get("TransferSyntaxUID")
    if syntax is None:
        explicit, little = _looks_explicit(buf, off), True
    elif syntax == IMPLICIT_LE:
        explicit, little = False, True
    elif syntax == EXPLICIT_LE:
        explicit, little = True, True
    elif syntax == EXPLICIT_BE:
        explicit, little = True, False
    elif syntax == DEFLATED_LE:
        buf = buf[:off] + zlib.decompress(buf[off:], -15)
        explicit, little = True, True
    else:
        raise DicomError(f"transfer syntax {syntax} is not supported (compressed pixel data?)")
    ds, _ = _Reader(buf, explicit, little).dataset(off, len(buf))
    ds.file_meta = meta
    return ds


def dcmread(fp, force=False):
    """``pydicom.dcmread`` stand-in for RT Plan files."""
    return read(fp, force=force)
