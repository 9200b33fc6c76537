"""CPU-side checks of the C ABI library (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import REPO
from conehead_gb300 import _native as N
from conehead_gb300.build import build


@pytest.fixture(scope="module")
def library():
    path = build()
    assert os.path.exists(path)
    return ctypes.CDLL(path)


def declared_symbols():
    names = set()
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(ch_\w+)\s*\(", text, re.M))
    return names


def test_header_declares_the_api():
    names = declared_symbols()
    for n in ("ch_plan_create", "ch_dose", "ch_dose_batch", "ch_dose_scatter", "ch_dda_trace"):
        assert n in names


def test_library_exports_every_declared_symbol(library):
    for name in declared_symbols():
        assert hasattr(library, name), name


def test_binding_covers_every_declared_symbol():
    assert declared_symbols() == set(N.SIGNATURES)


def test_status_strings(library):
    L = N.lib()
    assert L.ch_status_string(0) == b"ok"
    assert L.ch_status_string(5) == b"ray parallel to the blocking plane"
    assert L.ch_version() >= 1


def test_struct_sizes_match_header_layout():
    # ch_settings: 11 doubles + 2 ints + 3 x 32 floats
    assert ctypes.sizeof(N.Settings) == 11 * 8 + 2 * 4 + 3 * 32 * 4 + 8   # options + padding to 8
    assert ctypes.sizeof(N.Grid) == 36
    assert N.Beam.block.offset == 3 * 8 + 3 * 8 + 9 * 8 + 8 + 2 * 4


def test_block_crop_keeps_every_nonzero():
    import numpy as np
    from conehead_gb300 import Block
    b = Block()
    b.set_rect(-3.0, 5.0, -1.0, 2.5)
    crop, r0, c0 = N.block_crop(b.block_values)
    full = np.zeros_like(b.block_values)
    full[r0:r0 + crop.shape[0], c0:c0 + crop.shape[1]] = crop
    assert np.array_equal(full, b.block_values)
    assert crop.shape == (800, 350)


def test_mlc_table_validation_runs_on_the_host():
    """ch_block_from_mlc refuses bad leaf tables before touching the GPU."""
    import ctypes
    from conehead_gb300 import _native as N
    from conehead_gb300.block import MLCField
    import numpy as np
    L = N.lib()
    good = MLCField(np.arange(-200, 201, 10.0), np.r_[np.full(40, -10.0), np.full(40, 10.0)], [-50, 50], [-50, 50])

    def status(mutate):
        m = good.struct()
        mutate(m)
        return L.ch_block_from_mlc(ctypes.byref(m), ctypes.c_void_p(0x1000), 4, 4, 0, 0, None)

    def narrow(m):
        m.rows[3] = 2

    def overlap(m):
        m.row0[5] -= 1

    def short_a(m):
        m.a_end[0] = 14

    def short_b(m):
        m.b_start[0] = 3985

    def too_many(m):
        m.n_pairs = N.CH_MAX_LEAF_PAIRS + 1

    def jaw_outside(m):
        m.open_r1 = m.map_rows + 1

    def tip_nan(m):
        m.tip[3] = float("nan")

    for mutate, word in ((narrow, "3 rows"), (overlap, "overlap"), (short_a, "bank A"), (short_b, "bank B"),
                         (too_many, "n_pairs"), (jaw_outside, "jaw"), (tip_nan, "tip")):
        assert status(mutate) == 1
        assert word in L.ch_last_error().decode(), mutate.__name__
    m = good.struct()
    assert L.ch_block_from_mlc(ctypes.byref(m), None, 4, 4, 0, 0, None) == 1
    assert L.ch_block_from_mlc(ctypes.byref(m), ctypes.c_void_p(0x1000), 0, 4, 0, 0, None) == 1
    assert ctypes.sizeof(N.MLC) == 8 * 4 + 4 * 4 * N.CH_MAX_LEAF_PAIRS + 8 * N.CH_MLC_TIP_CELLS
