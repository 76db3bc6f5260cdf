"""Depth order of the visible slots at full frame sizes.  Frames of up to 8192 slots per
SM sort in one cooperative launch, larger ones in per-pass onesweep launches; both must
give the stable ascending order of the 32-bit depth keys, ties in slot order, which is
the order the reference's stable (tile | depth) key sort leaves within a tile.  The maps
put every Gaussian on one of a few dozen depth planes, so nearly every key is tied."""
import numpy as np
import pytest
import torch

from gsevt import _lib
from gsevt import pose as gpose
from gsevt import synthetic
from gsevt.engine import GSFrame, MapSpec, ViewSpec

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda")


def _region(frame, name, dtype, count):
    off = _lib.workspace_offsets(frame.L)[name]
    nbytes = count * torch.empty((), dtype=dtype).element_size()
    return frame.workspace[off:off + nbytes].view(dtype)


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


@pytest.mark.parametrize("n,views", [(3000, 1), (1_200_000, 1), (700_000, 2)])
def test_depth_order_is_the_stable_sort_of_the_depth_keys(n, views):
    m = synthetic.make_map(n, 5)
    # identity rotation and zero translation: the camera-space depth is z itself, so
    # z on a 1/16 m grid gives 49 depth values with thousands of exact ties each (and
    # zero low key bytes, whose passes are the identity permutation)
    m["xyz"][:, 2] = (np.round(m["xyz"][:, 2] * 16.0) / 16.0).astype(np.float32)
    cam = synthetic.PinholeCamera(640, 480, 600.0)
    R, t = np.eye(3), np.zeros(3)
    ms = MapSpec(n, xyz=_t(m["xyz"]), opacity=_t(m["opacity"]), scales=_t(m["scale"]), rotations=_t(m["rot"]),
                 shs=_t(m["sh"]))
    # a second view with the same pose repeats every depth key in later slots
    vs = [ViewSpec(cam.width, cam.height, 0, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t),
                   tanfovx=cam.tanfovx, tanfovy=cam.tanfovy) for _ in range(views)]
    fr = GSFrame([ms], vs, channels=1, device=DEV)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    status = _region(fr, "status", torch.int32, 16).cpu().numpy().view(np.uint32)
    assert status[0] == 0  # no overflow, no timed-out wait
    vg = fr.L.num_vg
    binv = _region(fr, "bin", torch.int32, 4 * vg).view(vg, 4).cpu().numpy()
    vis = binv[:, 0] > 0
    nvis = int(status[5])
    assert nvis == int(vis.sum()) and nvis > 0.2 * vg
    slots = np.nonzero(vis)[0].astype(np.uint32)
    keys = binv[vis, 3].view(np.uint32)
    assert len(np.unique(keys)) < 100  # the ties are really there
    order = np.argsort(keys, kind="stable")
    got_k = _region(fr, "dkeys0", torch.int32, nvis).cpu().numpy().view(np.uint32)
    got_v = _region(fr, "dvals0", torch.int32, nvis).cpu().numpy().view(np.uint32)
    assert np.array_equal(got_k, keys[order])
    assert np.array_equal(got_v, slots[order])
