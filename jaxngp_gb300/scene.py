"""Procedural training scenes: Gaussian density blobs (and thin shells) in a unit box, seen by
pinhole cameras on the upper hemisphere, with ground-truth RGBA images rendered on the GPU.

These stand in for the reference's NeRF-synthetic captures (800x800 RGBA views of an object in
[-1, 1]^3, loaded by utils/data.py); the dataset itself is not used.  The data layout matches what
the reference's training step reads (app/nerf/_utils.py:84-170): ``transforms`` [V, 12] (row-major
3x3 camera-to-world rotation, then the camera position) and ``rgbas`` [V*H*W, 4] uint8.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L


@dataclass
class PinholeCamera:
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    near: float = 0.3

    @staticmethod
    def from_fov(width: int, height: int, fov_deg: float, near: float = 0.3) -> "PinholeCamera":
        f = (width / 2) / math.tan(math.radians(fov_deg) / 2)
        return PinholeCamera(width, height, f, f, width / 2, height / 2, near)

    @property
    def n_pixels(self) -> int:
        return self.width * self.height


def look_at(pos: np.ndarray, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """Camera-to-world [3, 4] for a camera at `pos` looking at `target` (camera looks along -z,
    y up, the CG convention of utils/types.py:436-437)."""
    pos = np.asarray(pos, np.float64)
    fwd = np.asarray(target, np.float64) - pos
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, up)
    if np.linalg.norm(right) < 1e-8:
        right = np.cross(fwd, (0.0, 1.0, 0.0))
    right /= np.linalg.norm(right)
    cam_up = np.cross(right, fwd)
    R = np.stack([right, cam_up, -fwd], axis=1)
    return np.concatenate([R, pos[:, None]], axis=1)


def hemisphere_poses(n: int, radius: float, rng: np.random.Generator) -> np.ndarray:
    """n camera-to-world [n, 3, 4] poses at `radius` on the upper hemisphere, aimed at the origin."""
    poses = []
    for k in range(n):
        z = rng.uniform(0.05, 1.0)
        phi = rng.uniform(0, 2 * np.pi)
        r = math.sqrt(1 - z * z)
        poses.append(look_at(radius * np.array([r * math.cos(phi), r * math.sin(phi), z])))
    return np.stack(poses)


def orbit_poses(n: int, radius: float, elevation_deg: float = 25.0) -> np.ndarray:
    """An orbit of n poses around the z axis (like SceneMeta.make_frames_with_orbiting_trajectory,
    utils/types.py:888-921)."""
    el = math.radians(elevation_deg)
    return np.stack([look_at(radius * np.array([math.cos(el) * math.cos(a), math.cos(el) * math.sin(a), math.sin(el)]))
                     for a in np.linspace(0, 2 * np.pi, n, endpoint=False)])


def poses_to_transforms(poses: np.ndarray) -> np.ndarray:
    """[V, 3, 4] -> [V, 12]: rotation rows then translation (app/nerf/_utils.py:107-110)."""
    return np.concatenate([poses[:, :, :3].reshape(-1, 9), poses[:, :, 3]], axis=1).astype(np.float32)


@dataclass
class BlobScene:
    blobs: np.ndarray            # [B, 8]: centre (3), sigma, peak density, rgb (3)
    shells: np.ndarray           # [S, 8]: centre (3), radius, thickness, peak, c0, c1
    bound: float = 1.0

    @staticmethod
    def random(n_blobs: int = 64, n_shells: int = 0, seed: int = 0) -> "BlobScene":
        """Blobs with centres ~U[-0.5,0.5]^3, sigma ~U[0.03,0.15], peak ~U[10,200], RGB ~U[0,1]
        (the 64-blob training scene), plus thin shells with radius ~U[0.1,0.4] and thickness 0.01
        (the harder 512-blob + 8-shell scene)."""
        rng = np.random.default_rng(seed)
        b = np.zeros((n_blobs, 8), np.float32)
        b[:, 0:3] = rng.uniform(-0.5, 0.5, (n_blobs, 3))
        b[:, 3] = rng.uniform(0.03, 0.15, n_blobs)
        b[:, 4] = rng.uniform(10, 200, n_blobs)
        b[:, 5:8] = rng.uniform(0, 1, (n_blobs, 3))
        s = np.zeros((max(n_shells, 1), 8), np.float32)
        s[:n_shells, 0:3] = rng.uniform(-0.4, 0.4, (n_shells, 3))
        s[:n_shells, 3] = rng.uniform(0.1, 0.4, n_shells)
        s[:n_shells, 4] = 0.01
        s[:n_shells, 5] = rng.uniform(50, 200, n_shells)
        s[:n_shells, 6:8] = rng.uniform(0, 1, (n_shells, 2))
        scene = BlobScene(b, s[:n_shells] if n_shells else np.zeros((0, 8), np.float32))
        return scene

    def density(self, x: np.ndarray) -> np.ndarray:
        """Analytic density at points x [N, 3] (float64, CPU)."""
        x = np.asarray(x, np.float64)
        out = np.zeros(x.shape[0])
        for bl in self.blobs:
            r2 = ((x - bl[:3]) ** 2).sum(-1)
            out += bl[4] * np.exp(-r2 / (2 * bl[3] ** 2))
        for sh in self.shells:
            dist = np.abs(np.linalg.norm(x - sh[:3], axis=-1) - sh[3])
            out += np.where(dist <= sh[4], sh[5], 0.0)
        return out


@dataclass
class SceneData:
    """What the training step reads: cameras, poses, RGBA pixels (all views, row-major)."""
    camera: PinholeCamera
    transforms: torch.Tensor     # [V, 12] f32, device
    rgbas: torch.Tensor          # [V*H*W, 4] u8, device
    bound: float
    scene: BlobScene

    @property
    def n_views(self) -> int:
        return self.transforms.shape[0]

    @property
    def n_pixels(self) -> int:
        return self.n_views * self.camera.n_pixels


def make_scene_data(n_blobs: int = 64, n_shells: int = 0, n_views: int = 100, width: int = 800, height: int = 800,
                    fov_deg: float = 40.0, radius: float = 4.0, n_steps: int = 4096, seed: int = 0,
                    device="cuda") -> SceneData:
    """The synthetic training set; by default the 64-blob scene seen from 100 views at 800x800,
    fov 40, radius 4, with targets from 4096-step quadrature."""
    scene = BlobScene.random(n_blobs, n_shells, seed)
    cam = PinholeCamera.from_fov(width, height, fov_deg)
    poses = hemisphere_poses(n_views, radius, np.random.default_rng(seed + 1))
    transforms = torch.from_numpy(poses_to_transforms(poses)).to(device)
    rgbas = render_views(scene, cam, transforms, n_steps)
    return SceneData(cam, transforms, rgbas, scene.bound, scene)


def _render_views(scene, cam, transforms, v0, nv, n_steps):
    dev = transforms.device
    blobs = torch.from_numpy(scene.blobs).to(dev)
    shells = torch.from_numpy(scene.shells if len(scene.shells) else np.zeros((1, 8), np.float32)).to(dev)
    out = torch.empty(nv * cam.n_pixels, 4, dtype=torch.uint8, device=dev)
    d = L.NgpRenderBlobsDescriptor(nv * cam.n_pixels, len(scene.blobs), n_steps, cam.width, cam.height,
                                   transforms.shape[0], v0, len(scene.shells), cam.fx, cam.fy, cam.cx, cam.cy,
                                   scene.bound)
    L.call("ngp_render_blobs", [transforms, blobs, shells, out], d)
    return out


def render_views(scene: BlobScene, cam: PinholeCamera, transforms: torch.Tensor, n_steps: int = 4096) -> torch.Tensor:
    """Ground truth for every view of `transforms`: [V*H*W, 4] uint8."""
    V = transforms.shape[0]
    out = torch.empty(V * cam.n_pixels, 4, dtype=torch.uint8, device=transforms.device)
    per = max(1, (1 << 22) // cam.n_pixels)
    for v0 in range(0, V, per):
        nv = min(per, V - v0)
        out[v0 * cam.n_pixels:(v0 + nv) * cam.n_pixels] = _render_views(scene, cam, transforms, v0, nv, n_steps)
    return out


def psnr_u8(a: torch.Tensor, b: torch.Tensor) -> float:
    """utils/data.py:407-410 on uint8 images."""
    mse = ((a.double() - b.double()) ** 2).mean().item()
    return float(min(max(20 * math.log10(255 / math.sqrt(mse + 1e-15)), 0.0), 100.0))
