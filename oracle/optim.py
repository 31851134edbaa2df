"""CPU restatement of the reference's optimiser.  TEST INFRASTRUCTURE ONLY.

app/nerf/_utils.py:19-77 builds

    optax.chain(
        optax.multi_transform({"network": adam(lr_sch, b1=.9, b2=.99, eps=1e-15, eps_root=1e-15), ...}),
        optax.add_decayed_weights(1e-6, mask={density_mlp, rgb_mlp: True, position_encoder: False}))

with lr_sch = optax.exponential_decay(lr, transition_steps=10_000, decay_rate=1/3, staircase=True,
transition_begin=10_000, end_value=lr/100).  Restated here from optax's published definitions, in
float32 and in optax's order of operations:

    scale_by_adam:           mu = (1-b1) g + b1 mu;   nu = (1-b2) (g*g) + b2 nu
                             mu_hat = mu / (1 - b1^t);   nu_hat = nu / (1 - b2^t)     (t = count + 1)
                             u = mu_hat / (sqrt(nu_hat + eps_root) + eps)
    scale_by_learning_rate:  u = -lr(count) * u                     (the schedule sees the count before the update)
    add_decayed_weights:     u = u + wd * p                         (after the lr scaling, as chained)
    apply_updates:           p = p + u
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def exponential_decay(count: int, init_value: float, transition_steps: int = 10_000, decay_rate: float = 1 / 3,
                      transition_begin: int = 10_000, staircase: bool = True, end_value: float | None = None) -> float:
    """optax.exponential_decay evaluated at `count`, in float32."""
    c = count - transition_begin
    if c <= 0:
        return float(f32(init_value))
    p = c / transition_steps
    if staircase:
        p = math.floor(p)
    v = f32(init_value) * f32(decay_rate) ** f32(p)
    if end_value is not None:
        v = max(v, f32(end_value)) if decay_rate < 1 else min(v, f32(end_value))
    return float(f32(v))


def reference_lr(count: int, lr: float = 1e-2) -> float:
    """The learning rate the reference's schedule gives update number `count` (0-based)."""
    return exponential_decay(count, lr, end_value=lr / 100)


def adam_update(p, g, mu, nu, count: int, lr: float, weight_decay: float = 0.0, b1: float = 0.9, b2: float = 0.99,
                eps: float = 1e-15, eps_root: float = 1e-15):
    """One step of the chain on float32 arrays; returns new (p, mu, nu).  `count` is the number of
    updates made before this one; `lr` the schedule's value at `count`."""
    p, g, mu, nu = (np.asarray(x, np.float32) for x in (p, g, mu, nu))
    b1_, b2_ = f32(b1), f32(b2)
    mu = (f32(1) - b1_) * g + b1_ * mu
    nu = (f32(1) - b2_) * (g * g) + b2_ * nu
    t = count + 1
    bc1 = f32(1) - b1_ ** f32(t)
    bc2 = f32(1) - b2_ ** f32(t)
    mu_hat = mu / bc1
    nu_hat = nu / bc2
    u = mu_hat / (np.sqrt(nu_hat + f32(eps_root)) + f32(eps))
    u = f32(-lr) * u
    if weight_decay:
        u = u + f32(weight_decay) * p
    return (p + u).astype(np.float32), mu.astype(np.float32), nu.astype(np.float32)
