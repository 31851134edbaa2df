"""The spherical-harmonics restatement (oracle/sh.py) against the reference's own encoder
(models/encoders.py:361-406 run on the NumPy stand-in for jax, tests/golden/sh_encodings.npz):
bit-exact for every degree 1..8, directions random and axis-aligned."""
import numpy as np
import pytest

from oracle import sh
from tests.golden_util import load


@pytest.mark.parametrize("degree", range(1, 9))
def test_sh_oracle_matches_reference(degree):
    z = load("sh_encodings")
    out = sh.encode(z["dirs"], degree)
    assert out.shape == (len(z["dirs"]), degree * degree)
    assert np.array_equal(out, z[f"deg{degree}"])


def test_sh_degree_4_is_the_field_encoding():
    """The field's colour MLP reads degrees 0..3 (16 values) of this encoding (oracle.field.sh4)."""
    from oracle import field as Fd
    z = load("sh_encodings")
    assert np.array_equal(sh.encode(z["dirs"], 4), Fd.sh4(z["dirs"]))


def test_sh_rejects_bad_degree():
    with pytest.raises(ValueError):
        sh.encode(np.zeros((2, 3), np.float32), 9)
