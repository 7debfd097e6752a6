"""Seeded synthetic scenes, cameras and ray batches.

No dataset is available, so every workload uses generated inputs with the
shapes of the reference's DTU runs: a [-1,1]^3 bbox, 49 cameras on a sphere
of radius 3 looking at the origin, 1600x1200 pinhole images with f = 1.2 W,
OpenCV axes (inverse_y=True, configs/dtu_e2e/fine.py:19), and analytic SDF
grids plus noise.  Rays follow get_rays (lib/voxurf_fine.py:1001-1029, pixel
centres +0.5) and viewdirs = rays_d/|rays_d| (voxurf_fine.py:1064).
"""
from __future__ import annotations

import math

import numpy as np
import torch

BBOX_MIN = (-1.0, -1.0, -1.0)
BBOX_MAX = (1.0, 1.0, 1.0)


def fibonacci_poses(n: int = 49, radius: float = 3.0) -> np.ndarray:
    """[n, 4, 4] camera-to-world matrices (OpenCV: x right, y down, z forward)
    on a Fibonacci lattice of the sphere, each looking at the origin."""
    golden = math.pi * (3.0 - math.sqrt(5.0))
    poses = np.zeros((n, 4, 4), np.float64)
    up = np.array([0.0, 0.0, 1.0])
    for i in range(n):
        z = 1.0 - (2 * i + 1) / n
        r = math.sqrt(max(0.0, 1.0 - z * z))
        phi = golden * i
        pos = radius * np.array([r * math.cos(phi), r * math.sin(phi), z])
        fwd = -pos / np.linalg.norm(pos)
        right = np.cross(fwd, up)
        right /= np.linalg.norm(right)
        down = np.cross(fwd, right)
        poses[i, :3, 0] = right
        poses[i, :3, 1] = down
        poses[i, :3, 2] = fwd
        poses[i, :3, 3] = pos
        poses[i, 3, 3] = 1.0
    return poses


def intrinsics(H: int = 1200, W: int = 1600, focal: float | None = None) -> np.ndarray:
    f = 1.2 * W if focal is None else focal
    return np.array([[f, 0.0, W / 2.0], [0.0, f, H / 2.0], [0.0, 0.0, 1.0]])


def rays_for_pixels(c2w: np.ndarray, K: np.ndarray, px: np.ndarray, py: np.ndarray):
    """Rays through pixel centres (px+0.5, py+0.5) of one camera, OpenCV axes
    (voxurf_fine.py:1010, 1021-1028).  Returns float32 (o, d, viewdir)."""
    i = px.astype(np.float32) + 0.5
    j = py.astype(np.float32) + 0.5
    dirs = np.stack([(i - K[0, 2]) / K[0, 0], (j - K[1, 2]) / K[1, 1], np.ones_like(i)], -1).astype(np.float32)
    R = c2w[:3, :3].astype(np.float32)
    d = (dirs[:, None, :] * R[None]).sum(-1)
    o = np.broadcast_to(c2w[:3, 3].astype(np.float32), d.shape).copy()
    v = d / np.linalg.norm(d, axis=-1, keepdims=True)
    return o, d.astype(np.float32), v.astype(np.float32)


def random_rays(n: int, seed: int = 0, H: int = 1200, W: int = 1600, n_poses: int = 49, radius: float = 3.0):
    """n rays drawn uniformly from all n_poses*H*W pixels (seeded).
    Returns float32 numpy (rays_o, rays_d, viewdirs) each [n, 3]."""
    rng = np.random.default_rng(seed)
    poses = fibonacci_poses(n_poses, radius)
    K = intrinsics(H, W)
    flat = rng.integers(0, n_poses * H * W, size=n)
    cam = flat // (H * W)
    pix = flat % (H * W)
    py, px = pix // W, pix % W
    o = np.empty((n, 3), np.float32)
    d = np.empty((n, 3), np.float32)
    v = np.empty((n, 3), np.float32)
    for c in np.unique(cam):
        sel = cam == c
        o[sel], d[sel], v[sel] = rays_for_pixels(poses[c], K, px[sel], py[sel])
    return o, d, v


def view_rays(pose_index: int, H: int, W: int, n_poses: int = 49, radius: float = 3.0, focal: float | None = None):
    """All H*W rays of one view (row-major), float32 numpy."""
    poses = fibonacci_poses(n_poses, radius)
    K = intrinsics(H, W, focal)
    py, px = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    return rays_for_pixels(poses[pose_index % n_poses], K, px.reshape(-1), py.reshape(-1))


def grid_coords(R: int, bbox_min=BBOX_MIN, bbox_max=BBOX_MAX) -> np.ndarray:
    """[R, R, R, 3] world coordinates of the grid points (align_corners)."""
    axes = [np.linspace(bbox_min[a], bbox_max[a], R) for a in range(3)]
    return np.stack(np.meshgrid(*axes, indexing="ij"), -1)


def sdf_sphere(p, radius=0.5, centre=(0.0, 0.0, 0.0)):
    return np.linalg.norm(p - np.asarray(centre), axis=-1) - radius


def sdf_torus(p, R=0.6, r=0.15):
    q = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - R
    return np.sqrt(q * q + p[..., 2] ** 2) - r


def make_sdf(kind: str, R: int, seed: int = 0, noise: float | None = None, shape: tuple | None = None) -> np.ndarray:
    """float32 [R, R, R] SDF grid.

    kind: 'sphere' (r=0.5, noise 0.01 -- coarse stage scene),
          'sphere_torus' (min(sphere r=0.45, torus R=0.6 r=0.15), noise 0.005;
                          shape = (sphere r, torus R, torus r) overrides the sizes),
          'spheres64' (64 spheres, centres U(-0.8,0.8)^3, radii U(0.05,0.2)).
    """
    rng = np.random.default_rng(seed)
    if kind == "spheres64":
        # union of 64 spheres in float64 torch (all host threads: the 384^3
        # grid has 57M points)
        c = rng.uniform(-0.8, 0.8, size=(64, 3))
        rr = rng.uniform(0.05, 0.2, size=64)
        axes = [torch.linspace(BBOX_MIN[a], BBOX_MAX[a], R, dtype=torch.float64) for a in range(3)]
        st = torch.full((R, R, R), float("inf"), dtype=torch.float64)
        for k in range(64):
            dx = (axes[0] - c[k, 0]) ** 2
            dy = (axes[1] - c[k, 1]) ** 2
            dz = (axes[2] - c[k, 2]) ** 2
            d2 = dx[:, None, None] + dy[None, :, None] + dz[None, None, :]
            torch.minimum(st, d2.sqrt_() - rr[k], out=st)
        s = st.numpy()
        sd = 0.005 if noise is None else noise
        s = s + rng.normal(0.0, sd, size=s.shape)
        return s.astype(np.float32)
    p = grid_coords(R)
    if kind == "sphere":
        s = sdf_sphere(p, 0.5)
        sd = 0.01 if noise is None else noise
    elif kind == "sphere_torus":
        rs, tR, tr = (0.45, 0.6, 0.15) if shape is None else shape
        s = np.minimum(sdf_sphere(p, rs), sdf_torus(p, tR, tr))
        sd = 0.005 if noise is None else noise
    else:
        raise ValueError(kind)
    s = s + rng.normal(0.0, sd, size=s.shape)
    return s.astype(np.float32)


def make_k0(R: int, C: int = 12, seed: int = 1, std: float = 0.1, device="cpu") -> torch.Tensor:
    """float32 [R, R, R, C] feature grid ~ N(0, std) (channel-last)."""
    g = torch.Generator(device=device).manual_seed(seed)
    return torch.randn((R, R, R, C), generator=g, device=device, dtype=torch.float32) * std
