"""The closed form of the fallback march's lookahead chain (chain_t in marching.cu), restated in
float32 and checked against the sequential additions it replaces.

With the constant step c of a bound <= 1 march, t after j occupied steps is fl(...fl(t0 + c) + c...).
While every exact sum stays below t0's next power of two and c/ulp(t0) is not an exact
round-to-even tie, each addition adds the same delta = fl(t0 + c) - t0, so t_j = t0 + j*delta,
every operation exact.  The device takes the closed form only under the guard restated here.  The
GPU tests check the device march against the oracle bit for bit; this test shows the identity
itself, on random and adversarial cases (ties, sums near a power of two, tiny t0)."""
import numpy as np

f32 = np.float32


def sequential(t0, c, n=32):
    out = np.empty(n, np.float32)
    t = f32(t0)
    for j in range(n):
        out[j] = t
        t = f32(t + c)
    return out


def closed_form(t0, c):
    """The device's fast form, or None where its guard sends it to the sequential additions."""
    if not t0 > 0:
        return None
    e = int(np.array([t0], np.float32).view(np.uint32)[0]) & 0x7F800000
    if not ((24 << 23) < e < (253 << 23)):
        return None
    u = np.array([e - (23 << 23)], np.uint32).view(np.float32)[0]
    top = np.array([e + (1 << 23)], np.uint32).view(np.float32)[0]
    x = f32(c / u)
    delta = f32(f32(t0 + c) - t0)
    if f32(x - np.floor(x)) == f32(0.5) or not f32(t0 + f32(f32(32.0) * f32(delta + c))) < top:
        return None
    return np.array([f32(t0 + f32(f32(j) * delta)) for j in range(32)], np.float32)


def test_closed_form_equals_the_sequential_additions():
    rng = np.random.default_rng(0)
    cases = [(f32(np.exp(rng.uniform(np.log(1e-3), np.log(50)))), f32(np.exp(rng.uniform(np.log(1e-5), np.log(0.05)))))
             for _ in range(20000)]
    cases.append((f32(1.0), f32(2 * np.sqrt(3) / 1024)))   # the bound-1 march's step
    for _ in range(500):
        t0 = f32(rng.uniform(1, 2))
        cases.append((t0, f32((rng.integers(1, 30000) + 0.5) * np.spacing(t0))))           # exact ties
        cases.append((f32(np.nextafter(f32(2.0), f32(0)) - f32(rng.integers(0, 2000)) * np.spacing(f32(1.5))),
                      f32(rng.uniform(1e-4, 1e-2))))                                          # just below 2
        cases.append((f32(rng.uniform(1e-30, 1e-20)), f32(rng.uniform(1e-4, 1e-2))))       # c far above t0
    taken = 0
    for t0, c in cases:
        fast = closed_form(t0, c)
        if fast is None:
            continue
        taken += 1
        assert np.array_equal(fast, sequential(t0, c)), (t0, c)
    assert taken > len(cases) // 3
    # the guard refuses the cases where t0 + j*delta differs from the additions: a round-to-even
    # tie and a chain that crosses a power of two
    for t0, c in [(f32(1.5118216276168823), f32(2265.5 * np.spacing(f32(1.5118216276168823)))),
                  (f32(1.999), f32(0.01))]:
        delta = f32(f32(t0 + c) - t0)
        naive = np.array([f32(t0 + f32(j) * delta) for j in range(32)], np.float32)
        assert not np.array_equal(naive, sequential(t0, c))
        assert closed_form(t0, c) is None

