"""Map, event and trajectory I/O for real sequences.

- `load_ply` / `save_ply`: the 3D Gaussian Splatting PLY layout read by the reference's
  GaussianModel.load_ply (gaussian_splatting/scene/gaussian_model.py:238-327): x y z,
  optional normals, f_dc_0..2, f_rest_0..(3 (deg+1)^2 - 4) (channel-major), opacity (logit),
  scale_* (log), rot_* (w, x, y, z, unnormalised).  A small binary/ascii PLY reader in
  numpy replaces the plyfile dependency.
- `load_events_txt`: "ts x y polarity" integer lines chunked into windows of
  max_events_per_frame events, leftover events dropped (utils/event_camera/event.py:11-39).
- `write_tum`: "timestamp tx ty tz qx qy qz qw" lines (utils/tracker.py:258-265).
- `event_overlay` / `write_png`: the per-frame tracking image of utils/tracker.py:267-270
  (utils/visualizer.py:7-44): the signed event frame in red (positive) and blue
  (negative) over the signed normalised render difference in grey, 60 / 40, written as a
  PNG.  The video and GIF assembly of utils/tracker.py:281-285 needs an encoder (cv2,
  PIL) and is not provided.
"""
import struct
import zlib

import numpy as np

from .events import EventArray

_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def _read_vertex_table(path):
    with open(path, "rb") as f:
        if f.readline().strip() != b"ply":
            raise ValueError("%s is not a PLY file" % path)
        fmt, count, props, in_vertex = None, 0, [], False
        while True:
            line = f.readline()
            if not line:
                raise ValueError("%s: PLY header has no end_header" % path)
            tok = line.decode("ascii", "replace").split()
            if not tok:
                continue
            if tok[0] == "format":
                fmt = tok[1]
            elif tok[0] == "element":
                in_vertex = tok[1] == "vertex"
                if in_vertex:
                    count = int(tok[2])
            elif tok[0] == "property" and in_vertex:
                if tok[1] == "list":
                    raise ValueError("%s: list properties in the vertex element are not supported" % path)
                props.append((tok[2], _PLY_TYPES[tok[1]]))
            elif tok[0] == "end_header":
                break
        if fmt == "ascii":
            data = np.loadtxt(f, max_rows=count, ndmin=2)
            return {name: data[:, i] for i, (name, _) in enumerate(props)}
        endian = "<" if fmt == "binary_little_endian" else ">"
        dt = np.dtype([(name, endian + t) for name, t in props])
        rec = np.frombuffer(f.read(dt.itemsize * count), dtype=dt, count=count)
        return {name: rec[name] for name, _ in props}


def load_ply(path, sh_degree=3):
    """Raw (un-activated) parameters as the reference's GaussianModel holds them:
    xyz [N,3], features [N,(deg+1)^2,3], opacity [N,1] (logit), scaling [N,3] (log),
    rotation [N,4] (w,x,y,z, unnormalised)."""
    v = _read_vertex_table(path)
    xyz = np.stack([v["x"], v["y"], v["z"]], axis=1).astype(np.float32)
    n = xyz.shape[0]
    k = (sh_degree + 1) ** 2
    dc = np.stack([v["f_dc_%d" % c] for c in range(3)], axis=1).astype(np.float32)  # [N, 3]
    rest_names = sorted([p for p in v if p.startswith("f_rest_")], key=lambda s: int(s.split("_")[-1]))
    if len(rest_names) != 3 * k - 3:
        raise ValueError("expected %d f_rest_* properties for SH degree %d, found %d"
                         % (3 * k - 3, sh_degree, len(rest_names)))
    if rest_names:
        rest = np.stack([v[p] for p in rest_names], axis=1).astype(np.float32).reshape(n, 3, k - 1)
    else:
        rest = np.zeros((n, 3, 0), np.float32)
    features = np.concatenate([dc[:, None, :], rest.transpose(0, 2, 1)], axis=1)
    scale_names = sorted([p for p in v if p.startswith("scale_")], key=lambda s: int(s.split("_")[-1]))
    rot_names = sorted([p for p in v if p.startswith("rot")], key=lambda s: int(s.split("_")[-1]))
    return dict(xyz=xyz, features=np.ascontiguousarray(features),
                opacity=np.asarray(v["opacity"], np.float32).reshape(n, 1),
                scaling=np.stack([v[p] for p in scale_names], axis=1).astype(np.float32),
                rotation=np.stack([v[p] for p in rot_names], axis=1).astype(np.float32))


def activate(raw):
    """exp(scale), sigmoid(opacity), normalised quaternion (gaussian_model.py:75-95), in the
    synthetic-map dict layout used by the batched tracker (xyz, scale, rot, opacity, sh)."""
    rot = raw["rotation"].astype(np.float64)
    rot /= np.linalg.norm(rot, axis=1, keepdims=True)
    return dict(xyz=raw["xyz"], scale=np.exp(raw["scaling"].astype(np.float64)).astype(np.float32),
                rot=rot.astype(np.float32),
                opacity=(1.0 / (1.0 + np.exp(-raw["opacity"].astype(np.float64)))).reshape(-1).astype(np.float32),
                sh=raw["features"])


def save_ply(path, xyz, features, opacity, scaling, rotation):
    """Write the binary little-endian 3DGS layout (normals written as zeros)."""
    xyz = np.asarray(xyz, np.float32)
    n = xyz.shape[0]
    feats = np.asarray(features, np.float32).reshape(n, -1, 3)
    k = feats.shape[1]
    names = ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
    names += ["f_rest_%d" % i for i in range(3 * (k - 1))]
    names += ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    cols = [xyz, np.zeros((n, 3), np.float32), feats[:, 0, :],
            feats[:, 1:, :].transpose(0, 2, 1).reshape(n, -1), np.asarray(opacity, np.float32).reshape(n, 1),
            np.asarray(scaling, np.float32).reshape(n, 3), np.asarray(rotation, np.float32).reshape(n, 4)]
    table = np.ascontiguousarray(np.concatenate(cols, axis=1), dtype="<f4")
    header = "ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % n
    header += "".join("property float %s\n" % nm for nm in names) + "end_header\n"
    with open(path, "wb") as f:
        f.write(header.encode("ascii"))
        f.write(table.tobytes())


def parse_events_txt(text, threads=0):
    """(ts int64, x uint16, y uint16, polarity uint8) arrays of an events.txt buffer, parsed
    by the library's multi-threaded host parser (gsevt_parse_events_txt)."""
    import ctypes as C
    from . import _lib
    buf = bytes(text)
    cap = buf.count(b"\n") + 1
    ts = np.empty(cap, np.int64)
    x = np.empty(cap, np.uint16)
    y = np.empty(cap, np.uint16)
    pol = np.empty(cap, np.uint8)
    n = C.c_size_t(0)
    st = _lib.lib().gsevt_parse_events_txt(buf, len(buf), ts.ctypes.data, x.ctypes.data, y.ctypes.data,
                                           pol.ctypes.data, cap, C.byref(n), int(threads))
    if st != _lib.GSEVT_OK:
        raise ValueError("events text: %s after %d events" % (_lib.ERRORS.get(st, "error %d" % st), n.value))
    k = n.value
    return ts[:k], x[:k], y[:k], pol[:k]


def load_events_txt(path, max_events_per_frame, array_nums=None, start_time=None):
    """Windows of max_events_per_frame events from "ts x y polarity" lines: events before
    start_time are skipped, the leftover events after the last full window are dropped,
    and at most array_nums windows are returned (utils/event_camera/event.py:11-39)."""
    with open(path, "rb") as f:
        ts, x, y, pol = parse_events_txt(f.read())
    if start_time is not None:
        keep = ts >= start_time
        ts, x, y, pol = ts[keep], x[keep], y[keep], pol[keep]
    m = int(max_events_per_frame)
    nwin = ts.shape[0] // m
    if array_nums is not None:
        nwin = min(nwin, int(array_nums))
    return [EventArray(x[i * m:(i + 1) * m], y[i * m:(i + 1) * m], pol[i * m:(i + 1) * m], ts[i * m:(i + 1) * m])
            for i in range(nwin)]


def rotation_to_quaternion_xyzw(R):
    """Unit quaternion (x, y, z, w) of a rotation matrix (Shepperd's method)."""
    R = np.asarray(R, np.float64)
    tr = np.trace(R)
    if tr > 0:
        s = 2.0 * np.sqrt(tr + 1.0)
        q = [(R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s]
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = 2.0 * np.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k])
        q = [0.0, 0.0, 0.0, (R[k, j] - R[j, k]) / s]
        q[i] = 0.25 * s
        q[j] = (R[j, i] + R[i, j]) / s
        q[k] = (R[k, i] + R[i, k]) / s
    q = np.asarray(q)
    if q[3] < 0:
        q = -q
    return q / np.linalg.norm(q)


def _quaternion_xyzw(R):
    # the reference converts with scipy's Rotation.from_matrix(R).as_quat()
    # (utils/tracker.py:261-262); without scipy, Shepperd's method
    try:
        from scipy.spatial.transform import Rotation
    except ImportError:
        return rotation_to_quaternion_xyzw(R)
    return Rotation.from_matrix(np.asarray(R)).as_quat()


def write_tum(path, trajectory):
    """trajectory: iterable of (timestamp, R (world->camera rotation), t) as the tracker
    returns them; written as the reference does (utils/tracker.py:258-265): translation and
    quaternion (x, y, z, w) of R, t, each number printed as its numpy scalar (so a float32
    translation prints as float32)."""
    with open(path, "w") as f:
        for ts, R, t in trajectory:
            q = _quaternion_xyzw(R)
            t = np.asarray(t).reshape(3)
            f.write(f"{ts} {t[0]} {t[1]} {t[2]} {q[0]} {q[1]} {q[2]} {q[3]}\n")


def _scaled(x):
    # x * (255 / max |x|) in the array's precision (utils/visualizer.py:14-17, 31-34)
    x = np.asarray(x)
    m = max(x.max(), abs(x.min())) if x.size else 0
    if not m > 0:
        return np.zeros_like(x)
    return x * (x.dtype.type(255) / m)


def event_overlay(sign_delta_Ie, sign_delta_Ir):
    """The tracking image of one frame as a BGR uint8 [H, W, 3] array, as the reference
    builds it: get_delta_Ie_img (positive events in the red channel, negative in blue,
    values scaled to 255 by the largest magnitude and truncated), get_delta_Ir_img (grey
    (d + 255) / 2 of the scaled render difference, truncated) and overlay_two_imgs
    (0.6 events + 0.4 render, rounded half to even and saturated, as cv2.addWeighted).
    Inputs: [H, W] (or [1, H, W]) arrays or tensors."""
    def host(a):
        if hasattr(a, "detach"):
            a = a.detach().cpu().numpy()
        a = np.asarray(a)
        return a.reshape(a.shape[-2], a.shape[-1])
    e = _scaled(host(sign_delta_Ie))
    ev = np.zeros(e.shape + (3,), np.uint8)
    ev[..., 2] = np.where(e > 0, e, 0).astype(np.uint8)   # red: positive (BGR order)
    ev[..., 0] = (-np.where(e < 0, e, 0)).astype(np.uint8)  # blue: negative
    r = _scaled(host(sign_delta_Ir))
    grey = ((r + r.dtype.type(255)) / r.dtype.type(2)).astype(np.uint8)
    rd = np.repeat(grey[..., None], 3, axis=2)
    mix = ev.astype(np.float32) * np.float32(0.6) + rd.astype(np.float32) * np.float32(0.4)
    return np.clip(np.rint(mix), 0, 255).astype(np.uint8)


def write_png(path, bgr):
    """Writes a BGR uint8 [H, W, 3] image as an 8-bit RGB PNG (the file cv2.imwrite makes
    of it), with the standard library's zlib."""
    bgr = np.asarray(bgr, np.uint8)
    h, w = bgr.shape[:2]
    rgb = np.ascontiguousarray(bgr[..., ::-1])
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return (struct.pack(">I", len(data)) + tag + data +
                struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF))

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def read_png_rgb(path):
    """Reads back an 8-bit RGB PNG with no row filters (as write_png makes them)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    rows = zlib.decompress(idat)
    stride = 1 + 3 * w
    out = np.frombuffer(rows, np.uint8).reshape(h, stride)
    assert (out[:, 0] == 0).all()
    return out[:, 1:].reshape(h, w, 3).copy()
