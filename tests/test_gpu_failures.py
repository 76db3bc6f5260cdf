"""Failure paths on the GPU, made to happen without faulting or hanging anything: a
spin limit of one poll (gsevt_layout.spin_limit) makes the sorts' bounded waits (the
cooperative sort's grid barriers, the onesweep passes' look-back) run out.  Each wait
then records GSEVT_STATUS_SORT_TIMEOUT and gives up; the stages that follow the sort do
nothing, every index stays inside its buffer, and the next call with the default limit
computes the normal result."""
import numpy as np
import pytest
import torch

from oracle import oracle
from gsevt import _lib
from gsevt import pose as gpose
from gsevt import synthetic
from gsevt.batched import BatchedTracker, Problem
from gsevt.engine import GSFrame, MapSpec, ViewSpec, pack_map
import helpers

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _ranges(frame, name, count):
    off = _lib.workspace_offsets(frame.L)[name]
    return frame.workspace[off:off + 8 * count].view(torch.int32).view(-1, 2).cpu().numpy().view(np.uint32)


def test_batched_step_whose_waits_run_out():
    """The batched step at 20k Gaussians (one cooperative launch for the depth sort and the
    super-tile binning): with a one-poll limit the barrier waits run out; the status says
    so, the pose state is untouched and every tile and super-tile range stays inside the
    value buffers.  The next step with the default limit equals a fresh tracker's first
    step (same loss bits; pose within FP32 atomic-order noise)."""
    sc = synthetic.Scenario(20000, 0, 320, 240, 300.0, 30000)
    m, cam = sc.map, sc.camera
    pk = pack_map(_t(m["xyz"]), _t(m["opacity"]), _t(m["sh"]), scales=_t(m["scale"]), rotations=_t(m["rot"]))
    rng = np.random.default_rng(3)
    E = rng.normal(size=cam.width * cam.height).astype(np.float32)
    E /= np.linalg.norm(E.astype(np.float64))
    Et = _t(E)

    def tracker():
        p = Problem(0, sc.init_R, sc.init_t, sc.init_lin, sc.init_ang, sc.delta_tau, cam.width, cam.height, cam.fx,
                    cam.fy, Et, opt_vel=True)
        return BatchedTracker([{"packed": pk, "n": 20000}], [p], device=DEV)

    bt = tracker()
    before = bt.states()
    bt.frame.set_spin_limit(1)
    bt.step()
    torch.cuda.synchronize()
    st, _ = bt.check_status()
    assert st & _lib.STATUS_SORT_TIMEOUT, _lib.status_names(st)
    after = bt.states()
    for k in ("R", "t", "lin_vel", "ang_vel", "iter"):
        assert np.array_equal(after[k], before[k]), k
    cap = bt.frame.L.key_capacity
    for name, count in (("ranges", bt.frame.L.total_tiles), ("sranges", bt.frame.L.super_tiles)):
        r = _ranges(bt.frame, name, count)
        assert np.all(r[:, 0] <= r[:, 1]) and np.all(r[:, 1] <= cap), name
    bt.frame.set_spin_limit(0)
    bt.step()
    torch.cuda.synchronize()
    assert bt.check_status()[0] == 0
    ref = tracker()
    ref.step()
    a, b = bt.states(), ref.states()
    assert a["iter"][0] == b["iter"][0] == 1
    assert a["loss"][0] == b["loss"][0]
    np.testing.assert_allclose(a["R"][0], b["R"][0], atol=1e-8)
    np.testing.assert_allclose(a["t"][0], b["t"][0], atol=1e-8)


def test_frame_path_whose_waits_run_out():
    """The drop-in's frame path with a key capacity above the cooperative sort's (2M pairs,
    so the tile sort runs the onesweep passes with their look-back waits): with a one-poll
    limit the status reports the timeout, the tile ranges stay inside the buffers, and
    render() raises rather than return an image; with the default limit the next render is
    bit-exact against the oracle."""
    m, cam = helpers.scene(20000, 320, 240, 300.0, seed=0)
    R, t = helpers.random_pose(11)
    n = m["xyz"].shape[0]
    spec = MapSpec(n, xyz=_t(m["xyz"]), opacity=_t(m["opacity"]), scales=_t(m["scale"]), rotations=_t(m["rot"]),
                   shs=_t(m["sh"]))
    view = ViewSpec(cam.width, cam.height, 0, R=R, t=t, P=cam.proj, campos=gpose.campos(R, t), tanfovx=cam.tanfovx,
                    tanfovy=cam.tanfovy)
    fr = GSFrame([spec], [view], channels=1, key_capacity=2_000_000, device=DEV)
    fr.set_spin_limit(1)
    fr.preprocess()
    fr.bin_and_sort(0)
    fr.blend()
    torch.cuda.synchronize()
    st, _ = fr.status()
    assert st & _lib.STATUS_SORT_TIMEOUT, _lib.status_names(st)
    r = _ranges(fr, "ranges", fr.L.total_tiles)
    assert np.all(r[:, 0] <= r[:, 1]) and np.all(r[:, 1] <= fr.L.key_capacity)
    with pytest.raises(_lib.GsevtError, match="bounded device wait ran out"):
        fr.render(exact_keys=True)
    fr.set_spin_limit(0)
    fr.render(exact_keys=True)
    torch.cuda.synchronize()
    assert fr.status()[0] == 0
    res = oracle.rasterize_view(m["xyz"], helpers.cov6(m), m["sh"], m["opacity"], helpers.view_vector(R, t, cam),
                                cam.width, cam.height, [0.0], nch=1)
    got = fr.pixels(0)[0].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), res["image"][0].view(np.uint32))
