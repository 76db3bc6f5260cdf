"""CPU checks of the C-ABI library: it loads, exports every entry point declared in
include/gsevt.h, its struct sizes match the Python binding, and argument validation
answers without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from gsevt import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gsevt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gsevt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = _declared()
    assert len(names) >= 19
    for n in names:
        assert hasattr(L, n), n
    assert sorted(_lib.EXPORTED) == names


def test_abi_struct_sizes_match():
    sizes = _lib.check_abi()
    assert sizes[0] == 192  # gsevt_view


def test_workspace_sizing_and_offsets():
    L = _lib.Layout()
    L.num_views, L.num_maps, L.num_pairs = 2, 1, 1
    L.num_vg, L.num_scan_blocks, L.preprocess_blocks = 1000, 8, 4
    L.total_tiles, L.total_pixels, L.channels, L.sort_bits = 24, 6144, 1, 37
    L.key_capacity, L.loss_blocks = 100000, 3
    small = _lib.lib().gsevt_workspace_bytes(C.byref(L))
    L.key_capacity = 200000
    big = _lib.lib().gsevt_workspace_bytes(C.byref(L))
    assert big >= small + 100000 * 16  # two key and two value buffers of 4 bytes
    off = _lib.workspace_offsets(L)
    assert off["status"] == 0 and off["recC"] is None and off["gradC"] is None
    # recA / recB are the two 16-byte halves of one 32-byte record per slot
    assert off["recB"] == off["recA"] + 16
    seen = [v for k, v in off.items() if v is not None and k != "recB"]
    assert seen == sorted(seen) and all(v % 256 == 0 for v in seen)
    # the sort-count region also holds the cooperative sort's digit-major table:
    # 256 digits x 160 block columns plus 256 row totals, 32-bit each
    assert off["sort_counter"] - off["sort_hist"] >= (160 + 1) * 256 * 4


def test_argument_validation_without_gpu():
    L = _lib.lib()
    assert L.gsevt_preprocess_fwd(None, None) == -1
    f = _lib.Frame()
    f.L.num_views = 0
    assert L.gsevt_bin_and_sort(C.byref(f), 0, None) == -1
    assert L.gsevt_events_accumulate(10, None, None, None, 64, 48, None, 9, 3, None, None, None, None) == -1
    assert L.gsevt_events_accumulate(0, None, None, None, 64, 48, None, 8, 1, C.c_void_p(16), C.c_void_p(16),
                                     None, None) == -1  # even kernel size
    # a camera with fx = 0 is rejected before anything is enqueued (the fake pointers are
    # never touched)
    cam = (C.c_double * 9)(0.0, 300.0, 32.0, 24.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    assert L.gsevt_events_accumulate(0, None, None, None, 64, 48, cam, 9, 1, C.c_void_p(16), C.c_void_p(16),
                                     None, None) == -1
    assert L.gsevt_pack_map(10, None, None, None, None, None, None, 16, 1.0, None, None) == -1
    assert L.gsevt_chain_view_grad(None, None, 0.0, None, None, None, None) == -1


def test_status_names():
    assert _lib.status_names(0) == "none"
    assert _lib.status_names(_lib.STATUS_KEY_OVERFLOW | _lib.STATUS_LAYOUT) == (
        "key capacity overflow, layout provides too few super-tiles")
    assert _lib.status_names(_lib.STATUS_SORT_TIMEOUT) == "bounded device wait ran out"
    assert "unknown flags 0x40" in _lib.status_names(0x40 | _lib.STATUS_NONFINITE)


def test_tuning_table_round_trip(tmp_path):
    """The autotuner's table: shape keys, record / save / load / lookup, and the layout's
    tuning struct in the binding."""
    from gsevt import tuner
    L = _lib.Layout()
    L.num_views, L.num_maps, L.num_vg, L.total_pixels = 2, 1, 1_000_000, 614400
    key = tuner.shape_key(L)
    assert key == "v2-m1-g1000000-p614400"
    trials = [(dict(tuner.DEFAULTS), 0.64), (dict(tuner.DEFAULTS, blend_staging=2), 0.62)]
    path = str(tmp_path / "table.json")
    table = tuner.record({}, L, trials[1][0], 0.62, trials, workload="w", device="d")
    tuner.save_table(table, path)
    loaded = tuner.load_table(path)
    assert loaded[key]["default_ms"] == 0.64
    assert tuner.lookup(L, loaded) == dict(tuner.DEFAULTS, blend_staging=2)
    L.num_vg += 1
    assert tuner.lookup(L, loaded) is None
    assert tuner.load_table(str(tmp_path / "missing.json")) == {}
    L.tuning.blend_staging = 2
    assert bytes(L)[-32:-28] == (2).to_bytes(4, "little")  # the struct's first tuning field
