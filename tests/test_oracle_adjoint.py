"""CPU: the exact integrator adjoint, written out, against FP64 central differences."""
import numpy as np

from oracle import adjoint as A


def test_exact_adjoint_formula_matches_fd64():
    rng = np.random.default_rng(0)
    for case in range(40):
        n = 64
        stop = case % 2 == 1
        sigma = rng.uniform(0, 60 if stop else 4, n)
        dt = np.full(n, 0.02)
        z = 1.0 + np.cumsum(dt)
        rgb = rng.uniform(size=(n, 3))
        bg = rng.uniform(size=3)
        g = rng.normal(size=4)
        _, op, used = A.integrate_forward64(sigma, rgb, dt, z, bg)
        T = 1 - op
        if stop and (T > 1e-4 * 0.5 or used == n):
            continue
        fd = A.ray_fd64(sigma, rgb, dt, z, bg, g)
        an = A.ray_adjoint64(sigma, rgb, dt, z, bg, g)
        for a, b in zip(an, fd):
            assert np.abs(a - b).max() <= 1e-6 * max(1.0, np.abs(b).max()), (case, np.abs(a - b).max())
