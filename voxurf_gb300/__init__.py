"""voxurf_gb300 — GB300-native (sm_103a) Voxurf per-ray voxel-SDF
volume-rendering step.

Drop-in modules mirroring the reference's JIT extensions:
  render_utils_cuda, total_variation_cuda, adam_upd_cuda
and the host-side mirror of the reference's Python interface for the path:
  grid (DenseGrid, MaskGrid), voxurf_fine / voxurf_coarse (Voxurf models),
  utils (Adam with per-voxel lr).
All compute runs in libvoxurf_gb300.so through a C ABI; there is no CPU path.
"""

__version__ = "0.1.0"
