"""CPU tests of map / event / trajectory I/O (gsevt.io)."""
import math
import os

import numpy as np
import pytest

from gsevt import io as gio
from gsevt import pose as gpose


def test_ply_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(0)
    n = 50
    xyz = rng.normal(size=(n, 3)).astype(np.float32)
    feats = rng.normal(size=(n, 16, 3)).astype(np.float32)
    op = rng.normal(size=(n, 1)).astype(np.float32)
    sc = rng.normal(-4, 0.5, size=(n, 3)).astype(np.float32)
    rot = rng.normal(size=(n, 4)).astype(np.float32)
    p = str(tmp_path / "map.ply")
    gio.save_ply(p, xyz, feats, op, sc, rot)
    raw = gio.load_ply(p)
    for k, v in (("xyz", xyz), ("features", feats), ("opacity", op), ("scaling", sc), ("rotation", rot)):
        assert np.array_equal(raw[k], v), k
    # channel-major f_rest layout: f_rest_{c * 15 + k} is coefficient k + 1 of channel c
    hdr = open(p, "rb").read().split(b"end_header\n")[0].decode()
    assert "property float f_rest_44" in hdr and "property float f_rest_45" not in hdr
    m = gio.activate(raw)
    np.testing.assert_allclose(np.linalg.norm(m["rot"], axis=1), 1.0, atol=1e-6)
    np.testing.assert_allclose(m["opacity"], 1 / (1 + np.exp(-op[:, 0])), rtol=1e-6)
    np.testing.assert_allclose(m["scale"], np.exp(sc), rtol=1e-6)


def test_ascii_ply(tmp_path):
    p = str(tmp_path / "a.ply")
    names = ["x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity", "scale_0", "scale_1", "scale_2",
             "rot_0", "rot_1", "rot_2", "rot_3"]
    with open(p, "w") as f:
        f.write("ply\nformat ascii 1.0\nelement vertex 2\n")
        f.write("".join("property float %s\n" % n for n in names) + "end_header\n")
        f.write(" ".join(str(float(i)) for i in range(14)) + "\n")
        f.write(" ".join(str(float(i + 1)) for i in range(14)) + "\n")
    raw = gio.load_ply(p, sh_degree=0)
    assert raw["xyz"].tolist() == [[0, 1, 2], [1, 2, 3]]
    assert raw["features"].shape == (2, 1, 3) and raw["rotation"][1].tolist() == [11, 12, 13, 14]


def test_events_txt_windows(tmp_path):
    rng = np.random.default_rng(1)
    n = 1050
    ts = np.sort(rng.integers(0, 10 ** 6, n))
    x, y, pol = rng.integers(0, 640, n), rng.integers(0, 480, n), rng.integers(0, 2, n)
    p = str(tmp_path / "events.txt")
    with open(p, "w") as f:
        for i in range(n):
            f.write("%d %d %d %d\n" % (ts[i], x[i], y[i], pol[i]))
    wins = gio.load_events_txt(p, 100)
    assert len(wins) == 10  # leftover 50 events dropped
    assert np.array_equal(wins[3].x, x[300:400]) and np.array_equal(wins[3].y, y[300:400])
    assert np.array_equal(wins[3].polarity, pol[300:400]) and wins[3].size() == 100
    assert abs(wins[0].duration() - (ts[99] - ts[0]) / 1e6) < 1e-12
    assert len(gio.load_events_txt(p, 100, array_nums=4)) == 4
    late = gio.load_events_txt(p, 100, start_time=int(ts[500]))
    assert late[0].ts[0] >= ts[500]


def test_tum_writer(tmp_path):
    R = gpose.exp_so3([0.3, -0.2, 0.5])
    t = np.array([1.0, 2.0, 3.0])
    p = str(tmp_path / "traj.txt")
    gio.write_tum(p, [(0.5, R, t)])
    f = [float(v) for v in open(p).read().split()]
    assert f[:4] == [0.5, 1.0, 2.0, 3.0]
    qx, qy, qz, qw = f[4:]
    # rebuild R from the quaternion
    Rq = np.array([[1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)],
                   [2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)],
                   [2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)]])
    np.testing.assert_allclose(Rq, R, atol=1e-12)
    for Rm in (gpose.exp_so3([math.pi - 1e-3, 0.1, 0.0]), gpose.exp_so3([0.0, math.pi * 0.999, 0.0])):
        q = gio.rotation_to_quaternion_xyzw(Rm)
        assert abs(np.linalg.norm(q) - 1) < 1e-12


def test_tum_writer_formats_numbers_as_the_reference(tmp_path):
    """utils/tracker.py:264-265 formats the float32 translation and the quaternion with an
    f-string of numpy scalars; the writer does the same, so a float32 translation keeps
    exactly the float32 value."""
    R = gpose.exp_so3([0.1, 0.2, -0.3]).astype(np.float32)
    t = np.array([0.1, -0.2, 0.3], np.float32)
    p = str(tmp_path / "traj32.txt")
    gio.write_tum(p, [(1.25, R, t)])
    fields = open(p).read().split()
    assert fields[:4] == ["1.25", f"{t[0]}", f"{t[1]}", f"{t[2]}"]
    assert [np.float32(float(v)) for v in fields[1:4]] == list(t)


def test_event_overlay_known_answer():
    """utils/visualizer.py: events scaled by 255 / max |E|, positive -> red, negative ->
    blue (BGR image), truncated; render difference scaled the same way, grey (d + 255) / 2
    truncated; 0.6 events + 0.4 render rounded half to even (cv2.addWeighted)."""
    E = np.array([[1.0, -0.5, 0.0]], np.float32)
    D = np.array([[0.5, -1.0, 0.0]], np.float32)
    img = gio.event_overlay(E, D)
    assert img.dtype == np.uint8 and img.shape == (1, 3, 3)
    # events: (B, G, R) = (0, 0, 255), (127, 0, 0), (0, 0, 0); render grey 191, 0, 127
    np.testing.assert_array_equal(img[0, 0], [76, 76, 229])   # 0.4*191 = 76.4; 0.6*255 + 76.4
    np.testing.assert_array_equal(img[0, 1], [76, 0, 0])      # 0.6*127 = 76.2
    np.testing.assert_array_equal(img[0, 2], [51, 51, 51])    # 0.4*127 = 50.8
    # no events at all: an event image of zeros (the reference would divide by zero)
    z = gio.event_overlay(np.zeros((2, 2), np.float32), D[:, :2].repeat(2, 0))
    assert z.shape == (2, 2, 3)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    bgr = rng.integers(0, 256, size=(17, 23, 3), dtype=np.uint8)
    p = str(tmp_path / "x.png")
    gio.write_png(p, bgr)
    raw = open(p, "rb").read()
    assert raw[:8] == b"\x89PNG\r\n\x1a\n" and raw[12:16] == b"IHDR"
    rgb = gio.read_png_rgb(p)
    np.testing.assert_array_equal(rgb, bgr[..., ::-1])


def _parse_lines_python(text):
    """Plain per-line restatement of the events.txt format for the parser tests."""
    out = []
    for line in text.decode().split("\n"):
        tok = line.split()
        if tok:
            ts, x, y, p = (int(t) for t in tok)
            out.append((ts, x, y, 1 if p != 0 else 0))
    return out


def test_native_event_parser_matches_line_parse():
    """gsevt_parse_events_txt (host threads, no GPU) against a per-line parse: spaces and
    tabs, CRLF line ends, blank lines, a last line without a newline, and a buffer large
    enough for several threads, whose result does not depend on the thread count."""
    rng = np.random.default_rng(3)
    n = 120_000
    ts = np.cumsum(rng.integers(0, 50, n)) + 10 ** 12
    x, y, p = rng.integers(0, 1280, n), rng.integers(0, 720, n), rng.integers(-1, 2, n)
    seps = [" ", "\t", "  "]
    lines = []
    for i in range(n):
        s = rng.integers(0, 3)
        lines.append(seps[s].join(str(int(v)) for v in (ts[i], x[i], y[i], p[i])) + ("\r" if i % 7 == 0 else ""))
        if i % 1000 == 0:
            lines.append("   ")
    text = "\n".join(lines).encode()  # no newline after the last line
    assert len(text) > (1 << 20)
    ref = np.array(_parse_lines_python(text), np.int64)
    for threads in (1, 3, 8):
        got = gio.parse_events_txt(text, threads=threads)
        assert got[0].shape[0] == n
        assert np.array_equal(got[0], ref[:, 0]) and np.array_equal(got[1], ref[:, 1])
        assert np.array_equal(got[2], ref[:, 2]) and np.array_equal(got[3], ref[:, 3])
        assert got[1].dtype == np.uint16 and got[3].dtype == np.uint8


def test_native_event_parser_rejects_malformed_lines():
    import ctypes as C
    from gsevt import _lib
    good = b"1 2 3 1\n4 5 6 0\n"
    for bad in (b"7 8 9\n", b"7 8 9 1 5\n", b"7 x 9 1\n", b"7 70000 9 1\n", b"7 -1 9 1\n"):
        with pytest.raises(ValueError, match="after 2 events"):
            gio.parse_events_txt(good + bad + good)
    # an output capacity below the line count is refused before parsing
    ts = np.empty(1, np.int64)
    xy = np.empty(1, np.uint16)
    pol = np.empty(1, np.uint8)
    cnt = C.c_size_t(5)
    st = _lib.lib().gsevt_parse_events_txt(good, len(good), ts.ctypes.data, xy.ctypes.data, xy.ctypes.data,
                                           pol.ctypes.data, 1, C.byref(cnt), 0)
    assert st == _lib.GSEVT_ERR_TOO_LARGE and cnt.value == 0
    assert gio.parse_events_txt(b"")[0].shape == (0,)
