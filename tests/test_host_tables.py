"""The host side of the encoder without a GPU: the descriptor jaxngp_gb300.encoders.LevelTable
builds (the per-level scales cast to float32, resolutions, row offsets, the first hashed level,
the table size, the float32 bound and 2*bound) against the oracle's restatement of
encoders.py:77-114, over the training configuration, the 1.447 per-level scale, the proposal's
4-level table and small and 32-level tables."""
import numpy as np
import pytest

from oracle import hashgrid as H

CASES = [
    dict(L=16, T=2 ** 19, N_min=16, N_max=2048),
    dict(L=16, T=2 ** 19, N_min=16, N_max=4096),
    dict(L=16, T=2 ** 19, N_min=16, N_max=2048, per_level_scale=1.447),
    dict(L=4, T=2 ** 16, N_min=16, N_max=128),
    dict(L=8, T=2 ** 12, N_min=16, N_max=512),
    dict(L=4, T=2 ** 14, N_min=4, N_max=16),
    dict(L=1, T=2 ** 12, N_min=4, N_max=256, per_level_scale=1.5),
    dict(L=32, T=2 ** 16, N_min=16, N_max=4096),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
@pytest.mark.parametrize("bound", [1.0, 2.0, 16.0])
def test_descriptor_matches_the_oracle_tables(case, bound):
    from jaxngp_gb300.encoders import LevelTable
    kw = dict(case)
    pls = kw.pop("per_level_scale", None)
    ref = H.LevelTable(kw["L"], kw["T"], 2, kw["N_min"], kw["N_max"], per_level_scale=pls)
    d = LevelTable(kw["L"], kw["T"], 2, kw["N_min"], kw["N_max"], pls).descriptor(1000, bound)
    L = kw["L"]
    assert (d.L, d.F, d.T, d.n_coords) == (L, 2, kw["T"], 1000)
    assert d.first_hash_level == ref.first_hash_level and d.n_params == ref.n_params
    assert [d.scales[i] for i in range(L)] == [float(np.float32(s)) for s in ref.scales]
    assert [d.resolutions[i] for i in range(L)] == list(ref.resolutions)
    assert [d.offsets[i] for i in range(L + 1)] == list(ref.offsets)
    assert d.bound == float(np.float32(bound)) and d.two_bound == float(np.float32(2 * bound))


def test_descriptor_limits():
    from jaxngp_gb300.encoders import LevelTable
    with pytest.raises(ValueError):
        LevelTable(33, 2 ** 12, 2, 16, 512).descriptor(10, 1.0)
    with pytest.raises(NotImplementedError):
        LevelTable(4, 2 ** 12, 4, 16, 512).descriptor(10, 1.0)
