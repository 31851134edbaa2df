"""The field's parameters on the host, without a GPU: the packed weight layout the kernels read
(W0 @0, W1 @2048, W2 @3072, W3 @5120, W4 @9216; 9408 floats, flax's [in, out] row-major), and the
interchange with the reference's parameter tree (models/nerfs.py: position_encoder / density_mlp /
rgb_mlp, Dense_i/kernel; encoders.py:105-114's "latent codes stored on grid vertices" [P, 2]),
against the oracle's tree -- the one the golden field fixture fed to the reference's own
make_nerf_ngp."""
import numpy as np
import torch

from oracle import field as Fd
from oracle import hashgrid as H


def test_packed_layout():
    from jaxngp_gb300 import _lib as L
    from jaxngp_gb300.field import OFFSETS, SHAPES, pack_weights, unpack_weights
    assert OFFSETS == {"W0": 0, "W1": 2048, "W2": 3072, "W3": 5120, "W4": 9216}
    assert sum(a * b for _, (a, b) in SHAPES) == L.MLP_WEIGHTS == 9408
    w = {k: torch.arange(a * b, dtype=torch.float32).reshape(a, b) + 10000 * i for i, (k, (a, b)) in enumerate(SHAPES)}
    flat = pack_weights(w)
    assert flat.shape == (9408,)
    for k, (a, b) in SHAPES:
        assert torch.equal(flat[OFFSETS[k]:OFFSETS[k] + a * b].view(a, b), w[k])   # row-major [in, out]
        assert torch.equal(unpack_weights(flat)[k], w[k])


def test_flax_tree_round_trip():
    from jaxngp_gb300.encoders import PARAM_NAME
    from jaxngp_gb300.field import NGPField
    f = NGPField(1.0, T=2 ** 14, device="cpu", seed=3)
    tab = H.LevelTable(16, 2 ** 14, 2, 16, 2048)
    tree = f.flax_params()
    assert set(tree) == {"position_encoder", "density_mlp", "rgb_mlp"}
    assert PARAM_NAME == "latent codes stored on grid vertices"
    assert tree["position_encoder"][PARAM_NAME].shape == (tab.n_params, 2)
    w = Fd.init_weights(7)
    ref = Fd.to_flax_params(w)
    for mod in ("density_mlp", "rgb_mlp"):
        assert {k: set(v) for k, v in tree[mod].items()} == {k: set(v) for k, v in ref[mod].items()}
        for dense in ref[mod]:
            assert tree[mod][dense]["kernel"].shape == ref[mod][dense]["kernel"].shape
    lat = np.random.default_rng(0).uniform(-1, 1, (tab.n_params, 2)).astype(np.float32)
    f.load_flax_params({"position_encoder": {PARAM_NAME: lat}, **ref})
    back = f.flax_params()
    assert np.array_equal(back["position_encoder"][PARAM_NAME], lat)
    for mod in ("density_mlp", "rgb_mlp"):
        for dense in ref[mod]:
            assert np.array_equal(back[mod][dense]["kernel"], np.asarray(ref[mod][dense]["kernel"], np.float32))
