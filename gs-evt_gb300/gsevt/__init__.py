"""gsevt: GB300-native tracking hot path of GS-EVT (Gaussian-splatting event-camera
tracking).  Modules:
  _lib      ctypes binding of libgsevt.so (C ABI in include/gsevt.h)
  engine    rendering frame engine over the C ABI (maps, views, pairs, workspace)
  batched   batched adjoint tracker (one launch sequence for all views, CUDA graph)
  tracker   plain per-view path with the reference's RenderFrame / Tracker API
  renderer  render1 / render2 over the drop-in rasterizer
  camera    Camera with the reference's pose / velocity update API
  events    event windows and the device event frame
  synthetic seeded synthetic maps, cameras, motion and events
  pose      host FP64 SE(3) algebra
The drop-in rasterizer module `diff_gaussian_rasterization` sits beside this package.
"""
__all__ = ["_lib", "engine", "batched", "tracker", "renderer", "camera", "events", "synthetic", "pose"]
