"""RT Plan reading and the jaw + MLC block map, on the CPU.

* The pydicom-free reader is pinned on the reference's plan fixture
  (RP.3DCRT.dcm, implicit VR little endian without a preamble), copied
  under tests/golden/: device types, jaw and leaf positions, leaf
  boundaries, angles.  The same data set re-encoded by a small writer in
  this file (explicit VR little and big endian, deflated, with preamble and
  file meta, defined-length sequences) must read back identically.
* ``MLCField`` maps equal those of the reference's own
  ``Block._set_from_plan`` (conehead/block.py:87-215), run on the fixture
  and on seeded synthetic plans: the SHA-256 of every full 4000 x 4000 map
  and the map inside its nonzero box are stored in tests/golden/plans.npz
  by tests/golden/make_golden.py.
* The leaf table handed to the device kernel describes the same map, cell
  for cell (a pure-Python evaluation of the ``ch_mlc`` rules).
"""
import hashlib
import os
import struct
import sys
import zlib

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from make_golden import _plan_ns, synthetic_plans  # noqa: E402

FIXTURE = os.path.join(GOLDEN, "RP.3DCRT.dcm")


@pytest.fixture(scope="module")
def plans():
    z = np.load(os.path.join(GOLDEN, "plans.npz"))
    return z


@pytest.fixture(scope="module")
def fixture_plan():
    from conehead_gb300 import dicom
    return dicom.read(FIXTURE, force=True)


# --------------------------------------------------------------- reader --
def test_reader_pins_the_fixture(fixture_plan):
    ds = fixture_plan
    assert ds.Modality == "RTPLAN" and ds.RTPlanLabel == "MLC"
    assert ds.SOPClassUID == "1.2.840.10008.5.1.4.1.1.481.5"
    assert len(ds.BeamSequence) == 1
    beam = ds.BeamSequence[0]
    assert beam.BeamType == "STATIC" and beam.RadiationType == "PHOTON"
    assert beam.SourceAxisDistance == 1000.0 and beam.NumberOfControlPoints == 2
    devs = [d.RTBeamLimitingDeviceType for d in beam.BeamLimitingDeviceSequence]
    assert devs == ["ASYMX", "ASYMY", "MLCX"]
    mlc = beam.BeamLimitingDeviceSequence[2]
    assert mlc.NumberOfLeafJawPairs == 60
    b = np.array(mlc.LeafPositionBoundaries)
    assert len(b) == 61 and b[0] == -200.0 and b[-1] == 200.0
    assert np.all(np.diff(b)[10:50] == 5.0) and np.all(np.diff(b)[:10] == 10.0)
    cp = beam.ControlPointSequence[0]
    pos = {d.RTBeamLimitingDeviceType: d.LeafJawPositions for d in cp.BeamLimitingDevicePositionSequence}
    assert pos["ASYMX"] == [-34.0, 33.0] and pos["ASYMY"] == [-41.0, 42.0]
    ends = np.array(pos["MLCX"])
    assert len(ends) == 120
    assert ends[21] == -14.0 and ends[22] == -17.3 and ends[38] == -13.7
    assert ends[81] == 25.5 and ends[98] == 20.1 and ends[0] == -105.0 and ends[119] == -105.0
    assert cp.GantryAngle == 0.0 and cp.BeamLimitingDeviceAngle == 0.0
    assert cp.IsocenterPosition == [-1.7, 21.1, 12.2] and cp.NominalBeamEnergy == 6.0
    assert beam.ControlPointSequence[1].CumulativeMetersetWeight == 1.0


# a small encoder, enough to re-encode the fixture in other transfer syntaxes
def _encode(ds, explicit, little):
    from conehead_gb300 import dicom
    e = "<" if little else ">"
    out = bytearray()
    for el in ds:
        g, n = el.tag >> 16, el.tag & 0xFFFF
        vr = el.VR
        if vr == "SQ":
            body = bytearray()
            for item in el.value:
                ib = _encode(item, explicit, little)
                body += struct.pack(e + "HHI", 0xFFFE, 0xE000, len(ib)) + ib
            val = bytes(body)
        else:
            v = el.value
            if vr in ("DS", "IS"):
                vals = v if isinstance(v, list) else [v]
                txt = "\\".join("" if x is None else repr(x) if vr == "DS" else str(x) for x in vals)
            elif isinstance(v, list):
                txt = "\\".join(v)
            elif isinstance(v, bytes):
                txt = None
            else:
                txt = v
            val = v if txt is None else txt.encode("latin-1")
            if len(val) % 2:
                val += b"\x00" if vr == "UI" else b" "
        if not explicit:
            out += struct.pack(e + "HHI", g, n, len(val))
        elif vr in dicom._LONG_VRS:
            out += struct.pack(e + "HH", g, n) + vr.encode() + b"\x00\x00" + struct.pack(e + "I", len(val))
        else:
            out += struct.pack(e + "HH", g, n) + vr.encode() + struct.pack(e + "H", len(val))
        out += val
    return bytes(out)


def _file(ds, syntax):
    from conehead_gb300 import dicom
    little = syntax != dicom.EXPLICIT_BE
    body = _encode(ds, syntax != dicom.IMPLICIT_LE, little)
    if syntax == dicom.DEFLATED_LE:
        c = zlib.compressobj(9, zlib.DEFLATED, -15)
        body = c.compress(body) + c.flush()
    uid = syntax.encode() + (b"\x00" if len(syntax) % 2 else b"")
    meta = struct.pack("<HH", 2, 0x10) + b"UI" + struct.pack("<H", len(uid)) + uid
    return b"\x00" * 128 + b"DICM" + meta + body


def _same(a, b):
    assert [e.tag for e in a] == [e.tag for e in b]
    for x, y in zip(a, b):
        if x.VR == "SQ":
            assert len(x.value) == len(y.value)
            for p, q in zip(x.value, y.value):
                _same(p, q)
        elif x.tag in __import__("conehead_gb300.dicom", fromlist=["DICTIONARY"]).DICTIONARY:
            assert x.value == y.value, x


@pytest.mark.parametrize("syntax", ["1.2.840.10008.1.2", "1.2.840.10008.1.2.1", "1.2.840.10008.1.2.1.99",
                                    "1.2.840.10008.1.2.2"])
def test_reader_round_trips_transfer_syntaxes(fixture_plan, syntax):
    from conehead_gb300 import dicom
    back = dicom.read(_file(fixture_plan, syntax), force=False)
    assert back.file_meta.TransferSyntaxUID == syntax
    _same(fixture_plan, back)
    # and the same block table
    from conehead_gb300.block import MLCField
    a, b = MLCField.from_plan(fixture_plan), MLCField.from_plan(back)
    assert a.window == b.window and np.array_equal(a.a_end, b.a_end) and np.array_equal(a.b_start, b.b_start)


def test_reader_refuses_bare_data_without_force_and_truncation():
    from conehead_gb300 import dicom
    raw = open(FIXTURE, "rb").read()
    with pytest.raises(dicom.DicomError):
        dicom.read(raw, force=False)
    with pytest.raises(dicom.DicomError):
        dicom.read(raw[:-40], force=True)
    # reading from a file object works too
    with open(FIXTURE, "rb") as f:
        assert dicom.dcmread(f, force=True).BeamSequence[0].BeamType == "STATIC"


# ------------------------------------------------------------ block maps --
def _cases(fixture_plan):
    out = {"fixture": fixture_plan}
    for name, d in synthetic_plans().items():
        out[name] = _plan_ns(d)
    return out


def test_mlc_maps_equal_reference(plans, fixture_plan):
    from conehead_gb300.block import Block
    for name, plan in _cases(fixture_plan).items():
        if f"{name}/raises" in plans.files:
            with pytest.raises(ValueError):
                Block(plan=plan)
            continue
        blk = Block(plan=plan)
        assert blk.device_mlc() is not None           # map not built yet
        v = blk.block_values
        assert blk.device_mlc() is None               # now the engine reads the map
        assert v.dtype == np.float32 and v.shape == tuple(plans[f"{name}/shape"])
        assert hashlib.sha256(v.tobytes()).digest() == plans[f"{name}/sha256"].tobytes(), name
        r0, r1, c0, c1 = plans[f"{name}/bbox"]
        assert np.array_equal(v[r0:r1, c0:c1], plans[f"{name}/crop"]), name


def test_mlc_window_covers_every_open_cell(plans, fixture_plan):
    from conehead_gb300.block import MLCField
    for name, plan in _cases(fixture_plan).items():
        if f"{name}/raises" in plans.files:
            continue
        m = MLCField.from_plan(plan)
        r0, r1, c0, c1 = m.window
        br0, br1, bc0, bc1 = plans[f"{name}/bbox"]
        assert r0 <= br0 and br1 <= r1 and c0 <= bc0 and bc1 <= c1, name
        # a sub-window evaluation equals the slice of the full map
        sub = m.values(r0 + 7, r1 - 3, c0 + 11, c1 - 5)
        full = m.values()
        assert np.array_equal(sub, full[r0 + 7:r1 - 3, c0 + 11:c1 - 5])


def _ch_mlc_cell(m, r, c):
    """Cell value by the rules documented for ch_mlc (the device kernel's rules)."""
    if not (m.open_r0 <= r < m.open_r1 and m.open_c0 <= c < m.open_c1):
        return np.float32(0)
    pair = [n for n in range(m.n_pairs) if m.row0[n] <= r < m.row0[n] + m.rows[n]]
    if not pair:
        return np.float32(1)
    n = pair[0]
    i, w = r - m.row0[n], m.rows[n]

    def profile(k):
        v = np.float32(1)
        for row, x in ((0, 0.2), (1, 0.5), (2, 0.75), (w - 1, 0.2), (w - 2, 0.5), (w - 3, 0.75)):
            if k == row:
                v = np.float32(x)
        return v

    def leaf(p, ramp):
        return np.float32(np.float32(1) - np.float32(np.float64(p) * ramp))

    if m.b_start[n] <= c < m.map_cols - 1:
        j = c - m.b_start[n]
        return leaf(profile(w - 1 - i), m.tip[14 - j] if j < 15 else 1.0)
    if c < m.a_end[n]:
        k = c - (m.a_end[n] - 15)
        return leaf(profile(i), m.tip[k] if k >= 0 else 1.0)
    return np.float32(1)


def test_ch_mlc_table_describes_the_same_map(fixture_plan):
    from conehead_gb300.block import MLCField
    rng = np.random.default_rng(4)
    for name, plan in _cases(fixture_plan).items():
        m = MLCField.from_plan(plan)
        if m.rows != 4000:
            continue
        s = m.struct()
        full = m.values()
        r0, r1, c0, c1 = m.window
        # every leaf-end neighbourhood and edge row, plus random cells
        cells = [(rng.integers(0, 4000), rng.integers(0, 4000)) for _ in range(300)]
        for n in range(0, s.n_pairs, 3):
            r = s.row0[n] + rng.integers(0, s.rows[n])
            for c in list(range(s.a_end[n] - 17, s.a_end[n] + 2)) + list(range(s.b_start[n] - 2, s.b_start[n] + 17)):
                cells.append((r, c))
            for rr in (s.row0[n], s.row0[n] + 1, s.row0[n] + 2, s.row0[n] + s.rows[n] - 1):
                cells.append((rr, (c0 + c1) // 2))
        for r, c in cells:
            if 0 <= r < 4000 and 0 <= c < 4000:
                assert _ch_mlc_cell(s, int(r), int(c)) == full[r, c], (name, r, c)
    assert s.tip[0] == 1.0 and s.tip[14] == 0.0


def test_linspace_tip_ramp_is_numpys():
    from conehead_gb300.block import MLCField
    assert np.array_equal(MLCField.tip_ramp(), np.linspace(1.0, 0.0, 15))


def test_plan_errors_mirror_the_reference(fixture_plan):
    import types
    from conehead_gb300.block import Block, MLCField
    ns = types.SimpleNamespace
    arc = ns(BeamSequence=[ns(BeamType="DYNAMIC", BeamLimitingDeviceSequence=[], ControlPointSequence=[])])
    with pytest.raises(NotImplementedError, match="STATIC"):
        Block(plan=arc)
    bnd = np.arange(-200, 201, 10.0)
    ends = np.r_[np.full(40, -10.0), np.full(40, 10.0)]
    MLCField(bnd, ends, [-50, 50], [-50, 50])                     # fine
    with pytest.raises(ValueError, match="3"):
        MLCField(np.r_[-200.0, -199.8, np.arange(-190, 201, 10.0)], np.r_[np.full(41, -10.0), np.full(41, 10.0)],
                 [-50, 50], [-50, 50])                             # a 0.2 mm leaf
    with pytest.raises(ValueError, match="tip"):
        MLCField(bnd, np.r_[np.full(40, -199.0), np.full(40, 10.0)], [-50, 50], [-50, 50])
    with pytest.raises(ValueError, match="tip"):
        MLCField(bnd, np.r_[np.full(40, -10.0), np.full(40, 199.0)], [-50, 50], [-50, 50])
    with pytest.raises(ValueError, match="leaf positions"):
        MLCField(bnd, np.full(60, 0.0), [-50, 50], [-50, 50])
    no_mlc = ns(BeamSequence=[ns(BeamType="STATIC", BeamLimitingDeviceSequence=[],
                                 ControlPointSequence=[ns(BeamLimitingDevicePositionSequence=[])])])
    with pytest.raises(ValueError, match="lacks"):
        Block(plan=no_mlc)


def test_block_from_plan_picks_one_beam(fixture_plan):
    from conehead_gb300.block import Block
    d = synthetic_plans()["two_beams"]
    plan = _plan_ns(d)
    last = Block(plan=plan).mlc
    first = Block.from_plan(plan, beam=0).mlc
    # the reference's walk over all beams keeps beam 0's X jaw, which beam 1
    # lacks, and takes beam 1's leaves and Y jaw
    assert last.window[2:] == first.window[2:] and last.window[:2] != first.window[:2]
    assert not np.array_equal(first.a_end, last.a_end)
    with pytest.raises(ValueError, match="jaw_x"):
        Block.from_plan(plan, beam=1)               # beam 1 alone has no X jaw


def test_plan_beams_reads_angles(fixture_plan):
    from conehead_gb300.plan import plan_beams
    beams = plan_beams(FIXTURE)
    assert len(beams) == 1
    src, blk = beams[0]
    assert src.gantry == 0.0 and src.collimator == 0.0 and float(src.sad) == 100.0
    assert blk.device_mlc() is not None and blk.mlc.window == (1590, 2420, 1660, 2330)
