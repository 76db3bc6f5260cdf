"""Event windows and the device event frame.

`EventArray` holds one window as arrays (x, y uint16; polarity uint8; ts int64 us), the
role of utils/event_camera/event.py:72-100 (duration() in seconds from microsecond
timestamps, time() = window centre).  `EventFrame` keeps the reference's constructor
and attributes (event.py:103-128: sign_delta_Ie, unsign_delta_Ie as [1, H, W]) and
computes them with gsevt_events_accumulate (count, undistortion, blur, normalisation),
which also returns the nearest-neighbour pyramid of utils/tracker.py:78-91.
"""
import ctypes as C

import numpy as np
import torch

from ._lib import check, lib
from .engine import _ptr, _stream


class EventArray:
    def __init__(self, x, y, polarity, ts):
        self.x = np.ascontiguousarray(x, np.uint16)
        self.y = np.ascontiguousarray(y, np.uint16)
        self.polarity = np.ascontiguousarray(polarity, np.uint8)
        self.ts = np.ascontiguousarray(ts, np.int64)

    def size(self):
        return int(self.x.shape[0])

    def duration(self):
        return float(self.ts[-1] - self.ts[0]) / 1e6 if self.size() > 0 else 0

    def time(self):
        return (self.ts[0] + (self.ts[-1] - self.ts[0]) / 2) / 1e6


def pyramid_sizes(width, height, levels):
    return [(int(width * 0.5 ** l), int(height * 0.5 ** l)) for l in range(levels)]


def camera_params(intrinsic, distortion):
    """(fx, fy, cx, cy, k1, k2, p1, p2, k3) from a 3x3 intrinsic matrix and OpenCV-order
    distortion factors, or None when every distortion factor is zero."""
    if distortion is None:
        return None
    d = np.zeros(5)
    dd = np.asarray(distortion, np.float64).reshape(-1)
    d[:min(5, dd.size)] = dd[:5]
    if not np.any(d):
        return None
    K = np.asarray(intrinsic, np.float64).reshape(3, 3)
    return (K[0, 0], K[1, 1], K[0, 2], K[1, 2], d[0], d[1], d[2], d[3], d[4])


def event_frames(x, y, polarity, width, height, ksize=9, levels=3, device="cuda", camera=None):
    """Device tensors (x, y, polarity) -> (signed levels, unsigned levels), each a list of
    [1, h, w] tensors (level 0 first).  camera: None or (fx, fy, cx, cy, k1, k2, p1, p2, k3)
    to undistort the accumulated frame."""
    n = int(x.shape[0])
    sizes = pyramid_sizes(width, height, levels)
    tot = sum(w * h for w, h in sizes)
    out_s = torch.empty(tot, dtype=torch.float32, device=device)
    out_u = torch.empty(tot, dtype=torch.float32, device=device)
    scratch = torch.empty(int(lib().gsevt_event_scratch_bytes(width, height)), dtype=torch.uint8, device=device)
    cam = None if camera is None else (C.c_double * 9)(*[float(v) for v in camera])
    check(lib().gsevt_events_accumulate(n, _ptr(x) if n else None, _ptr(y) if n else None,
                                        _ptr(polarity) if n else None, width, height, cam, ksize, levels,
                                        _ptr(scratch), _ptr(out_s), _ptr(out_u), _stream()),
          "gsevt_events_accumulate")
    sig, uns, o = [], [], 0
    for w, h in sizes:
        sig.append(out_s[o:o + w * h].view(1, h, w))
        uns.append(out_u[o:o + w * h].view(1, h, w))
        o += w * h
    return sig, uns


class EventFrame:
    """EventFrame(img_width, img_height, intrinsic, distortion_factors, gaussian_kernel_size,
    event_array): the reference's constructor; undistortion is applied when any
    distortion factor is non-zero."""

    def __init__(self, img_width, img_height, intrinsic, distortion_factors, gaussian_kernel_size,
                 event_array, device="cuda", levels=3):
        self.device = device
        self.img_width, self.img_height = int(img_width), int(img_height)
        self.intrinsic, self.distortion_factors = intrinsic, distortion_factors
        self.gaussian_kernel_size = int(gaussian_kernel_size)
        t = lambda a: torch.from_numpy(a).to(device)
        ea = event_array
        self.sign_pyramid, self.unsign_pyramid = event_frames(
            t(ea.x), t(ea.y), t(ea.polarity), self.img_width, self.img_height, self.gaussian_kernel_size,
            levels, device, camera=camera_params(intrinsic, distortion_factors))
        self.sign_delta_Ie = self.sign_pyramid[0]
        self.unsign_delta_Ie = self.unsign_pyramid[0]
