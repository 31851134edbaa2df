"""CPU restatement of the spherical-harmonics direction encoding.  TEST INFRASTRUCTURE ONLY.

models/encoders.py:361-406 (SphericalHarmonicsEncoder, flax) and its CUDA twin
deps/spherical-harmonics-encoding-jax/lib/impl/spherical_harmonics_encoding.cu:22-118 evaluate the
real spherical harmonics of degrees 0..L-1 (L <= 8, L^2 outputs) of a unit direction with the
published closed-form polynomials (the ones tiny-cuda-nn uses).  Restated here in float32 with
the reference's order of operations; every coefficient is computed from its closed form
(e.g. 3 sqrt(35) / (4 sqrt(pi))) and rounded to float32, as the reference's decimal literals are.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32
_S = math.sqrt(math.pi)


def _c(num: float, den: float) -> np.float32:
    return f32(num / (den * _S))


# coefficients: C[name] = closed form / sqrt(pi)
C = {
    "0": _c(1, 2), "1": _c(math.sqrt(3), 2), "4": _c(math.sqrt(15), 2), "6a": _c(3 * math.sqrt(5), 4),
    "6b": _c(math.sqrt(5), 4), "8": _c(math.sqrt(15), 4), "9": _c(math.sqrt(70), 8), "10": _c(math.sqrt(105), 2),
    "11": _c(math.sqrt(42), 8), "12": _c(math.sqrt(7), 4), "14": _c(math.sqrt(105), 4),
    "16": _c(3 * math.sqrt(35), 4), "17": _c(3 * math.sqrt(70), 8), "18": _c(3 * math.sqrt(5), 4),
    "19": _c(3 * math.sqrt(10), 8), "20a": _c(-90, 16), "20b": _c(105, 16), "20c": _c(9, 16),
    "22": _c(3 * math.sqrt(5), 8), "24a": _c(-18 * math.sqrt(35), 16), "24b": _c(3 * math.sqrt(35), 16),
    "25": _c(3 * math.sqrt(154), 32), "26": _c(3 * math.sqrt(385), 4), "27": _c(-math.sqrt(770), 32),
    "28": _c(math.sqrt(1155), 4), "29": _c(math.sqrt(165), 16), "30": _c(math.sqrt(11), 16),
    "32": _c(math.sqrt(1155), 8), "34": _c(3 * math.sqrt(385), 16), "36": _c(math.sqrt(6006), 32),
    "37": _c(3 * math.sqrt(2002), 32), "38": _c(3 * math.sqrt(91), 8), "39": _c(-math.sqrt(2730), 32),
    "40": _c(math.sqrt(2730), 32), "41": _c(math.sqrt(273), 16), "42a": _c(105 * math.sqrt(13), 32),
    "42b": _c(-315 * math.sqrt(13), 32), "42c": _c(231 * math.sqrt(13), 32), "42d": _c(-5 * math.sqrt(13), 32),
    "44": _c(math.sqrt(2730), 64), "46": _c(3 * math.sqrt(91), 32), "48a": _c(15 * math.sqrt(6006), 64),
    "48b": _c(math.sqrt(6006), 64), "49": _c(3 * math.sqrt(715), 64), "50": _c(3 * math.sqrt(10010), 32),
    "51": _c(-3 * math.sqrt(385), 64), "52": _c(3 * math.sqrt(385), 8), "53": _c(-3 * math.sqrt(35), 64),
    "54": _c(3 * math.sqrt(70), 32), "55": _c(math.sqrt(105), 64), "56": _c(math.sqrt(15), 32),
    "58": _c(math.sqrt(70), 64), "60": _c(3 * math.sqrt(385), 32), "62": _c(3 * math.sqrt(10010), 64),
}


def encode(dirs: np.ndarray, degree: int) -> np.ndarray:
    """[n, 3] unit directions -> [n, degree^2] float32 (degree in 1..8)."""
    if not 1 <= degree <= 8:
        raise ValueError("degree must be in 1..8")
    d = np.asarray(dirs, np.float32)
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xy, xz, yz = x * y, x * z, y * z
    x2, y2, z2 = x * x, y * y, z * z
    x4, y4, z4 = x2 * x2, y2 * y2, z2 * z2
    x6, y6, z6 = x4 * x2, y4 * y2, z4 * z2
    k = C
    t = f32
    o = np.empty((d.shape[0], degree * degree), np.float32)
    o[:, 0] = k["0"]
    if degree <= 1:
        return o
    o[:, 1] = -k["1"] * y
    o[:, 2] = k["1"] * z
    o[:, 3] = -k["1"] * x
    if degree <= 2:
        return o
    o[:, 4] = k["4"] * xy
    o[:, 5] = -k["4"] * yz
    o[:, 6] = k["6a"] * z2 - k["6b"]
    o[:, 7] = -k["4"] * xz
    o[:, 8] = k["8"] * x2 - k["8"] * y2
    if degree <= 3:
        return o
    o[:, 9] = k["9"] * y * (t(-3) * x2 + y2)
    o[:, 10] = k["10"] * xy * z
    o[:, 11] = k["11"] * y * (t(1) - t(5) * z2)
    o[:, 12] = k["12"] * z * (t(5) * z2 - t(3))
    o[:, 13] = k["11"] * x * (t(1) - t(5) * z2)
    o[:, 14] = k["14"] * z * (x2 - y2)
    o[:, 15] = k["9"] * x * (-x2 + t(3) * y2)
    if degree <= 4:
        return o
    o[:, 16] = k["16"] * xy * (x2 - y2)
    o[:, 17] = k["17"] * yz * (t(-3) * x2 + y2)
    o[:, 18] = k["18"] * xy * (t(7) * z2 - t(1))
    o[:, 19] = k["19"] * yz * (t(3) - t(7) * z2)
    o[:, 20] = k["20a"] * z2 + k["20b"] * z4 + k["20c"]
    o[:, 21] = k["19"] * xz * (t(3) - t(7) * z2)
    o[:, 22] = k["22"] * (x2 - y2) * (t(7) * z2 - t(1))
    o[:, 23] = k["17"] * xz * (-x2 + t(3) * y2)
    o[:, 24] = k["24a"] * x2 * y2 + k["24b"] * x4 + k["24b"] * y4
    if degree <= 5:
        return o
    o[:, 25] = k["25"] * y * (t(10) * x2 * y2 - t(5) * x4 - y4)
    o[:, 26] = k["26"] * xy * z * (x2 - y2)
    o[:, 27] = k["27"] * y * (t(3) * x2 - y2) * (t(9) * z2 - t(1))
    o[:, 28] = k["28"] * xy * z * (t(3) * z2 - t(1))
    o[:, 29] = k["29"] * y * (t(14) * z2 - t(21) * z4 - t(1))
    o[:, 30] = k["30"] * z * (t(-70) * z2 + t(63) * z4 + t(15))
    o[:, 31] = k["29"] * x * (t(14) * z2 - t(21) * z4 - t(1))
    o[:, 32] = k["32"] * z * (x2 - y2) * (t(3) * z2 - t(1))
    o[:, 33] = k["27"] * x * (x2 - t(3) * y2) * (t(9) * z2 - t(1))
    o[:, 34] = k["34"] * z * (t(-6) * x2 * y2 + x4 + y4)
    o[:, 35] = k["25"] * x * (t(10) * x2 * y2 - x4 - t(5) * y4)
    if degree <= 6:
        return o
    o[:, 36] = k["36"] * xy * (t(-10) * x2 * y2 + t(3) * x4 + t(3) * y4)
    o[:, 37] = k["37"] * yz * (t(10) * x2 * y2 - t(5) * x4 - y4)
    o[:, 38] = k["38"] * xy * (x2 - y2) * (t(11) * z2 - t(1))
    o[:, 39] = k["39"] * yz * (t(3) * x2 - y2) * (t(11) * z2 - t(3))
    o[:, 40] = k["40"] * xy * (t(-18) * z2 + t(33) * z4 + t(1))
    o[:, 41] = k["41"] * yz * (t(30) * z2 - t(33) * z4 - t(5))
    o[:, 42] = k["42a"] * z2 + k["42b"] * z4 + k["42c"] * z6 + k["42d"]
    o[:, 43] = k["41"] * xz * (t(30) * z2 - t(33) * z4 - t(5))
    o[:, 44] = k["44"] * (x2 - y2) * (t(11) * z2 * (t(3) * z2 - t(1)) - t(7) * z2 + t(1))
    o[:, 45] = k["39"] * xz * (x2 - t(3) * y2) * (t(11) * z2 - t(3))
    o[:, 46] = k["46"] * (t(11) * z2 - t(1)) * (t(-6) * x2 * y2 + x4 + y4)
    o[:, 47] = k["37"] * xz * (t(10) * x2 * y2 - x4 - t(5) * y4)
    o[:, 48] = k["48a"] * x2 * y4 - k["48a"] * x4 * y2 + k["48b"] * x6 - k["48b"] * y6
    if degree <= 7:
        return o
    o[:, 49] = k["49"] * y * (t(-21) * x2 * y4 + t(35) * x4 * y2 - t(7) * x6 + y6)
    o[:, 50] = k["50"] * xy * z * (t(-10) * x2 * y2 + t(3) * x4 + t(3) * y4)
    o[:, 51] = k["51"] * y * (t(13) * z2 - t(1)) * (t(-10) * x2 * y2 + t(5) * x4 + y4)
    o[:, 52] = k["52"] * xy * z * (x2 - y2) * (t(13) * z2 - t(3))
    o[:, 53] = k["53"] * y * (t(3) * x2 - y2) * (t(13) * z2 * (t(11) * z2 - t(3)) - t(27) * z2 + t(3))
    o[:, 54] = k["54"] * xy * z * (t(-110) * z2 + t(143) * z4 + t(15))
    o[:, 55] = k["55"] * y * (t(-135) * z2 + t(495) * z4 - t(429) * z6 + t(5))
    o[:, 56] = k["56"] * z * (t(315) * z2 - t(693) * z4 + t(429) * z6 - t(35))
    o[:, 57] = k["55"] * x * (t(-135) * z2 + t(495) * z4 - t(429) * z6 + t(5))
    o[:, 58] = k["58"] * z * (x2 - y2) * (t(143) * z2 * (t(3) * z2 - t(1)) - t(187) * z2 + t(45))
    o[:, 59] = k["53"] * x * (x2 - t(3) * y2) * (t(13) * z2 * (t(11) * z2 - t(3)) - t(27) * z2 + t(3))
    o[:, 60] = k["60"] * z * (t(13) * z2 - t(3)) * (t(-6) * x2 * y2 + x4 + y4)
    o[:, 61] = k["51"] * x * (t(13) * z2 - t(1)) * (t(-10) * x2 * y2 + x4 + t(5) * y4)
    o[:, 62] = k["62"] * z * (t(15) * x2 * y4 - t(15) * x4 * y2 + x6 - y6)
    o[:, 63] = k["49"] * x * (t(-35) * x2 * y4 + t(21) * x4 * y2 - x6 + t(7) * y6)
    return o
