"""The synthetic workload's host side, without a GPU: the pinhole camera of the 64-blob scene
(800x800, fov 40: fx = fy = 400 / tan 20 deg = 1098.99, cx = cy = 400), camera poses at radius 4
aimed at the origin (upper hemisphere for training, a 25-degree orbit for rendering, the
camera looking along -z as in utils/types.py:436-437), the [V, 12] transform layout
(app/nerf/_utils.py:107-110), and the blob/shell parameter ranges."""
import math

import numpy as np


def test_camera_intrinsics():
    from jaxngp_gb300.scene import PinholeCamera
    cam = PinholeCamera.from_fov(800, 800, 40.0)
    assert abs(cam.fx - 1098.99) < 5e-3 and cam.fx == cam.fy and (cam.cx, cam.cy) == (400.0, 400.0)
    assert cam.n_pixels == 640000
    hd = PinholeCamera.from_fov(1920, 1080, 40.0)
    assert abs(hd.fx - 960.0 / math.tan(math.radians(20.0))) < 1e-9 and (hd.cx, hd.cy) == (960.0, 540.0)


def test_poses_look_at_the_origin():
    from jaxngp_gb300.scene import hemisphere_poses, orbit_poses, poses_to_transforms
    for poses, upper in [(hemisphere_poses(100, 4.0, np.random.default_rng(1)), True), (orbit_poses(120, 4.0), True)]:
        R, t = poses[:, :, :3], poses[:, :, 3]
        assert np.allclose(np.linalg.norm(t, axis=1), 4.0)
        assert np.allclose(np.einsum("vij,vkj->vik", R, R), np.eye(3)[None], atol=1e-12)   # orthonormal
        assert np.allclose(np.linalg.det(R), 1.0)
        view = -R[:, :, 2]   # the camera looks along its -z axis
        assert np.allclose(view, -t / 4.0, atol=1e-12)
        assert (t[:, 2] > 0).all() == upper
        tr = poses_to_transforms(poses)
        assert tr.shape == (len(poses), 12) and tr.dtype == np.float32
        assert np.allclose(tr[:, :9].reshape(-1, 3, 3), R) and np.allclose(tr[:, 9:], t)
    orbit = orbit_poses(120, 4.0)
    assert np.allclose(orbit[:, 2, 3], 4.0 * math.sin(math.radians(25.0)))


def test_blob_ranges():
    from jaxngp_gb300.scene import BlobScene
    s = BlobScene.random(512, 8, 0)
    b, sh = s.blobs, s.shells
    assert b.shape == (512, 8) and sh.shape == (8, 8)
    assert (np.abs(b[:, :3]) <= 0.5).all() and (b[:, 3] >= 0.03).all() and (b[:, 3] <= 0.15).all()
    assert (b[:, 4] >= 10).all() and (b[:, 4] <= 200).all() and (b[:, 5:] >= 0).all() and (b[:, 5:] <= 1).all()
    assert (sh[:, 3] >= 0.1).all() and (sh[:, 3] <= 0.4).all() and (sh[:, 4] == np.float32(0.01)).all()
    assert BlobScene.random(64, 0, 0).shells.shape == (0, 8)
    # the density is the sum of the blobs' Gaussians: at a blob's centre at least its peak
    c = b[:1, :3].astype(np.float64)
    assert s.density(c)[0] >= b[0, 4] * (1 - 1e-6)
