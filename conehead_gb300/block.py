"""Jaw/MLC transmission map in the isocentre plane.

Same contract as ``conehead/block.py:7-85``: ``block_values`` is a float32
transmission map sampled every 0.1 mm over [-20, 20) cm in both beam
directions (4000 x 4000).  Row index follows the beam x axis, column index
the beam z axis.  The dose kernels look a point (x, z) up as
``block_values[floor(100 x) + 1999, floor(100 z) + 1999]`` with the
reference's quirks (see ``transmission``).

``set_square`` reproduces the reference's integer truncation exactly.
``set_rect`` is an extension for asymmetric jaw fields (x1, x2, z1, z2 in cm
at the isocentre plane) built with the same truncation rule; the reference
only offers square fields and DICOM plans.

``Block(plan=...)`` takes an RT Plan data set (this package's
``dicom.read`` or a pydicom one) and builds the jaw + MLCX map of
``conehead/block.py:87-215`` -- the last beam of the plan, as the reference
does; ``Block.from_plan(plan, beam=i)`` picks one beam.  The leaf table
(``MLCField``) is kept, and the 64 MB host map is only built when
``block_values`` is read: the dose engine rasterises the jaw opening of the
map on the GPU from the table instead.
"""
import numpy as np

MAP_COLS = 4000          # columns of a plan map (leaf travel), conehead/block.py:186
TIP_CELLS = 15           # leaf-end ramp length, conehead/block.py:155


def _slice_stop(v, n):
    """End of ``a[:v]`` on an axis of length n (negative v counts from the end)."""
    return slice(None, v).indices(n)[1]


def _slice_start(v, n):
    """Start of ``a[v:]`` on an axis of length n."""
    return slice(v, None).indices(n)[0]


def _profile(w):
    """Tongue-and-groove factor of each row of a leaf w rows high.

    Rows 0, 1, 2 get 0.2, 0.5, 0.75, then rows w-1, w-2, w-3 get 0.2, 0.5,
    0.75; on leaves narrower than 6 rows the later writes win
    (conehead/block.py:148-154).
    """
    p = np.ones(w, dtype=np.float32)
    for row, v in ((0, 0.20), (1, 0.50), (2, 0.75), (w - 1, 0.20), (w - 2, 0.50), (w - 3, 0.75)):
        p[row] = v
    return p


class MLCField:
    """Jaws and MLCX leaves of one static beam in 0.1 mm map cells.

    Built from the DICOM numbers with the reference's rounding
    (conehead/block.py:95-134): leaf boundaries as float32, leaf ends and jaw
    positions as float64, each ``floor(10 * mm)``.  The map is ``rows`` x
    4000; leaf pair n covers rows ``row0[n] .. row0[n] + rows_of[n]``, its
    bank-A leaf columns ``[0, a_end[n])`` and its bank-B leaf columns
    ``[b_start[n], 3999)``; ``window`` is the jaw opening (rows, columns)
    with numpy's slice rules applied to the jaw indices exactly as the
    reference slices with them.
    """

    def __init__(self, boundaries_mm, leaf_ends_mm, jaw_x_mm, jaw_y_mm):
        bnd = np.floor(np.array(boundaries_mm, dtype=np.float32) * 10)
        ends = np.floor(np.array(leaf_ends_mm, dtype=np.float64) * 10)
        jx = np.floor(np.array(jaw_x_mm, dtype=np.float64) * 10)
        jy = np.floor(np.array(jaw_y_mm, dtype=np.float64) * 10)
        n_pairs = len(bnd) - 1
        if n_pairs < 1:
            raise ValueError("MLC needs at least two leaf boundaries")
        half = int(len(ends) / 2)
        ends_a, ends_b = ends[:half], ends[half:]
        if len(ends_a) < n_pairs or len(ends_b) < n_pairs:
            raise ValueError(f"{len(ends)} leaf positions for {n_pairs} leaf pairs")
        self.boundaries, self.ends, self.jaw_x, self.jaw_y = bnd, ends, jx, jy
        self.rows = int(np.abs(bnd[0] - bnd[-1]))
        self.row0 = np.array([int(bnd[n] + np.abs(bnd[0])) for n in range(n_pairs)], dtype=np.int64)
        self.rows_of = np.array([int(np.abs(bnd[n + 1] - bnd[n])) for n in range(n_pairs)], dtype=np.int64)
        self.a_end = np.array([int(2000 + int(e)) for e in ends_a[:n_pairs]], dtype=np.int64)
        self.b_start = np.array([int(2000 + int(e)) for e in ends_b[:n_pairs]], dtype=np.int64)
        self._check()
        c0 = _slice_stop(int(2000 + jx[0]), MAP_COLS)
        c1 = _slice_start(int(2000 + jx[1]), MAP_COLS)
        r0 = _slice_stop(int(self.rows / 2 + jy[0]), self.rows)
        r1 = _slice_start(int(self.rows / 2 + jy[1]), self.rows)
        self.window = (r0, max(r0, r1), c0, max(c0, c1))

    def _check(self):
        """Leaf tables the reference cannot build raise here too.

        The reference fails on leaves under 3 rows (IndexError), leaf lengths
        under the 15-cell tip and leaves outside the map (numpy broadcast
        errors).  Overlapping or unordered leaf rows, which it would paint
        over each other, are refused as well.
        """
        prev = 0
        for n in range(len(self.row0)):
            r0, w = int(self.row0[n]), int(self.rows_of[n])
            if w < 3:
                raise ValueError(f"leaf pair {n} is {w} cells wide; the leaf profile needs 3")
            if r0 < prev or r0 + w > self.rows:
                raise ValueError(f"leaf pair {n} rows [{r0}, {r0 + w}) overlap another pair or leave the "
                                 f"{self.rows}-row map")
            if not TIP_CELLS <= self.a_end[n] <= MAP_COLS:
                raise ValueError(f"bank A leaf {n} ends at cell {self.a_end[n]}: outside the map or "
                                 f"shorter than its {TIP_CELLS}-cell tip")
            if not 0 <= self.b_start[n] <= MAP_COLS - 1 - TIP_CELLS:
                raise ValueError(f"bank B leaf {n} ends at cell {self.b_start[n]}: outside the map or "
                                 f"shorter than its {TIP_CELLS}-cell tip")
            prev = r0 + w

    # ------------------------------------------------------------ sources --
    @classmethod
    def from_plan(cls, plan, beam=None):
        """Leaf table of one beam of an RT Plan data set.

        ``beam=None`` follows ``Block._set_from_plan``: every beam must be
        STATIC and each device keeps the value of the last beam that has it
        (so the last beam wins).  An integer picks that beam alone.
        """
        beams = list(plan.BeamSequence)
        chosen = beams if beam is None else [beams[beam]]
        found = {}
        for bm in chosen:
            if bm.BeamType != "STATIC":
                raise NotImplementedError("Only beams with type 'STATIC' are currently implemented.")
            for dev in bm.BeamLimitingDeviceSequence:
                if dev.RTBeamLimitingDeviceType == "MLCX":
                    found["boundaries"] = np.array(dev.LeafPositionBoundaries, dtype=np.float32)
            for dev in bm.ControlPointSequence[0].BeamLimitingDevicePositionSequence:
                kind = dev.RTBeamLimitingDeviceType
                if kind in ("X", "ASYMX"):
                    found["jaw_x"] = np.array(dev.LeafJawPositions)
                if kind in ("Y", "ASYMY"):
                    found["jaw_y"] = np.array(dev.LeafJawPositions)
                elif kind == "MLCX":
                    found["ends"] = np.array(dev.LeafJawPositions)
        missing = [k for k in ("boundaries", "ends", "jaw_x", "jaw_y") if k not in found]
        if missing:
            raise ValueError("plan beam lacks " + ", ".join(missing) +
                             " (needs an MLCX device and X/ASYMX and Y/ASYMY jaws)")
        return cls(found["boundaries"], found["ends"], found["jaw_x"], found["jaw_y"])

    # -------------------------------------------------------------- values --
    @staticmethod
    def tip_ramp():
        return np.linspace(1.0, 0.0, TIP_CELLS)

    def values(self, r0=0, r1=None, c0=0, c1=MAP_COLS):
        """Map cells [r0, r1) x [c0, c1) on the host (float32), zero outside the map.

        Leaf cells are ``1 - float32(profile * ramp)`` with the product taken
        in float64, as numpy computes ``area[:, -15:] *= linspace(...)`` on a
        float32 array followed by ``1 - area``.
        """
        r1 = self.rows if r1 is None else r1
        out = np.zeros((max(r1 - r0, 0), max(c1 - c0, 0)), dtype=np.float32)
        wr0, wr1, wc0, wc1 = self.window
        lo_r, hi_r, lo_c, hi_c = max(r0, wr0), min(r1, wr1), max(c0, wc0), min(c1, wc1)
        if lo_r >= hi_r or lo_c >= hi_c:
            return out
        view = out[lo_r - r0:hi_r - r0, lo_c - c0:hi_c - c0]
        view[:] = 1.0
        cols = np.arange(lo_c, hi_c)
        ramp = self.tip_ramp()
        for n in range(len(self.row0)):
            p0, w = int(self.row0[n]), int(self.rows_of[n])
            a, b = max(p0, lo_r), min(p0 + w, hi_r)
            if a >= b:
                continue
            prof = _profile(w)
            rows = np.arange(a, b) - p0
            # bank A: columns [0, a_end), ramp over its last 15 columns
            ra = np.ones(len(cols))
            k = cols - (self.a_end[n] - TIP_CELLS)
            ra[k >= 0] = ramp[k[k >= 0].clip(max=TIP_CELLS - 1)]
            leaf_a = np.float32(1) - (prof[rows, None].astype(np.float64) * ra[None, :]).astype(np.float32)
            in_a = cols < self.a_end[n]
            # bank B: columns [b_start, 3999), rows and ramp reversed
            rb = np.ones(len(cols))
            j = cols - self.b_start[n]
            tip_b = (j >= 0) & (j < TIP_CELLS)
            rb[tip_b] = ramp[TIP_CELLS - 1 - j[tip_b]]
            leaf_b = np.float32(1) - (prof[w - 1 - rows, None].astype(np.float64) * rb[None, :]).astype(np.float32)
            in_b = (cols >= self.b_start[n]) & (cols < MAP_COLS - 1)
            block = view[a - lo_r:b - lo_r]
            block[:, in_a] = leaf_a[:, in_a]
            block[:, in_b] = leaf_b[:, in_b]
        return out

    def struct(self):
        """The ``ch_mlc`` table of the C ABI."""
        from . import _native as N
        if len(self.row0) > N.CH_MAX_LEAF_PAIRS:
            raise ValueError(f"at most {N.CH_MAX_LEAF_PAIRS} leaf pairs")
        m = N.MLC()
        m.n_pairs = len(self.row0)
        m.map_rows, m.map_cols = self.rows, MAP_COLS
        m.open_r0, m.open_r1, m.open_c0, m.open_c1 = self.window
        for n in range(m.n_pairs):
            m.row0[n], m.rows[n] = int(self.row0[n]), int(self.rows_of[n])
            m.a_end[n], m.b_start[n] = int(self.a_end[n]), int(self.b_start[n])
        for k, v in enumerate(self.tip_ramp()):
            m.tip[k] = float(v)
        return m


class Block:
    def __init__(self, rotation=np.array([0, 0, 0], dtype=np.float32), plan=None):
        self.rotation = rotation
        self.mlc = None
        self._values = None
        self._rects = []
        if plan is not None:
            self._set_mlc(MLCField.from_plan(plan))
            return
        self.xmin = np.float32(-20)
        self.xmax = np.float32(20)
        self.xnum = np.int32(4000)
        self.xres = self.xnum / (self.xmax - self.xmin)
        self.ymin = np.float32(-20)
        self.ymax = np.float32(20)
        self.ynum = np.int32(4000)
        self.yres = self.ynum / (self.ymax - self.ymin)
        self._rects = []        # jaw openings (row and column slices) not yet painted into a map

    @classmethod
    def from_plan(cls, plan, beam=None, rotation=np.array([0, 0, 0], dtype=np.float32)):
        """Block of one beam of a plan (``beam=None``: the reference's rule)."""
        blk = cls(rotation)
        blk._set_mlc(MLCField.from_plan(plan, beam))
        return blk

    def _set_mlc(self, mlc):
        # the reference builds a RegularGridInterpolator over 4000 x rows
        # points for the map, which scipy refuses unless the leaf bank spans
        # 400 mm (conehead/block.py:199-215)
        if mlc.rows != MAP_COLS:
            raise ValueError(f"MLC leaf boundaries span {mlc.rows} cells; plan maps must span "
                             f"{MAP_COLS} (400 mm) as the reference's map interpolator requires")
        self.mlc = mlc
        self._values = None
        self.xmin, self.xmax, self.xnum = -20, 20, MAP_COLS
        self.ymin, self.ymax, self.ynum = mlc.boundaries[0] / 100, mlc.boundaries[-1] / 100, mlc.rows

    @property
    def block_values(self):
        """The transmission map, built on first read.

        Until then a jaw block is only its list of opened rectangles and a
        plan block its leaf table, and the engine hands those to the GPU
        directly.  Once read, the engine uses this array (which the caller may
        edit) instead.
        """
        if self._values is None:
            if self.mlc is not None:
                self._values = self.mlc.values()
            else:
                v = np.zeros((self.xnum, self.ynum), dtype=np.float32)
                for r0, r1, c0, c1 in self._rects:
                    v[r0:r1, c0:c1] = np.float32(1)
                self._values = v
            self._rects = []
        return self._values

    @block_values.setter
    def block_values(self, value):
        self._values = value
        self.mlc = None
        self._rects = []

    def device_mlc(self):
        """The leaf table when the map has never been materialised, else None."""
        return self.mlc if self._values is None else None

    def device_rect(self):
        """(r0, r1, c0, c1): the open cells when the map was never materialised
        and is one rectangle of ones (one opening, or openings nested in the
        largest); (0, 0, 0, 0) when nothing is open; None otherwise."""
        if self._values is not None or self.mlc is not None:
            return None
        n_r, n_c = int(self.xnum), int(self.ynum)
        boxes = []
        for r0, r1, c0, c1 in self._rects:
            a, b, _ = slice(r0, r1).indices(n_r)
            c, d, _ = slice(c0, c1).indices(n_c)
            if a < b and c < d:
                boxes.append((a, b, c, d))
        if not boxes:
            return (0, 0, 0, 0)
        big = max(boxes, key=lambda q: (q[1] - q[0]) * (q[3] - q[2]))
        if all(big[0] <= q[0] and q[1] <= big[1] and big[2] <= q[2] and q[3] <= big[3] for q in boxes):
            return big
        return None

    def transmission(self, position):
        """Transmission at an isocentre-plane point (cm), reference rules.

        The point is converted to 0.1 mm cells with ``floor(100 p) + 2000``;
        a cell index outside [0, 3999] gives 0, otherwise the map is read at
        ``index - 1`` (so index 0 wraps to the last row/column).
        """
        cell = np.floor(np.asarray(position, dtype=np.float32) * np.float32(100))
        cell = cell + np.float32(2000)
        for c in cell:
            if c < 0 or c > 3999:
                return np.float32(0)
        return self.block_values[int(cell[0]) - 1, int(cell[1]) - 1]

    def _open(self, x1, x2, y1, y2):
        if self._values is None:
            self._rects.append((x1, x2, y1, y2))
        else:
            self._values[x1:x2, y1:y2] = np.float32(1)

    def set_square(self, length):
        """Open a centred square of side ``length`` cm."""
        half = length / 2
        lo_x = int((self.xnum / 2) - half * self.xres)
        hi_x = int((self.xnum / 2) + half * self.xres)
        lo_y = int((self.ynum / 2) - half * self.yres)
        hi_y = int((self.ynum / 2) + half * self.yres)
        self._open(lo_x, hi_x, lo_y, hi_y)

    def set_rect(self, x1, x2, z1, z2):
        """Open the jaw rectangle [x1, x2] x [z1, z2] cm (x1 < x2, z1 < z2).

        Cell limits use the same ``int(n/2 + pos * res)`` truncation that
        ``set_square`` applies, so ``set_rect(-a/2, a/2, -a/2, a/2)`` equals
        ``set_square(a)``.
        """
        if not (x1 < x2 and z1 < z2):
            raise ValueError("set_rect needs x1 < x2 and z1 < z2")
        lo_x = int((self.xnum / 2) + x1 * self.xres)
        hi_x = int((self.xnum / 2) + x2 * self.xres)
        lo_y = int((self.ynum / 2) + z1 * self.yres)
        hi_y = int((self.ynum / 2) + z2 * self.yres)
        self._open(max(lo_x, 0), min(hi_x, int(self.xnum)),
                   max(lo_y, 0), min(hi_y, int(self.ynum)))
