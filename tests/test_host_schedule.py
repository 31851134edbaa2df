"""The training step's host-side formulas, without a GPU, against the reference's definitions:
the occupancy-grid cascades and the march's step-size portion of a scene bound
(utils/types.py:858-860, :874-886) and the learning-rate schedule (app/nerf/_utils.py:19-27:
optax.exponential_decay from lr, transition_begin and transition_steps 10k, rate 1/3,
staircase, floor lr/100 -- the first drop comes at 20k steps)."""
import pytest


@pytest.mark.parametrize("bound,k", [(0.5, 1), (1.0, 1), (1.5, 2), (2.0, 2), (3.0, 3), (4.0, 3), (16.0, 5), (64.0, 7)])
def test_cascades(bound, k):
    from jaxngp_gb300.trainer import cascades_for
    assert cascades_for(bound) == k


@pytest.mark.parametrize("bound,sp", [(0.5, 0.0), (1.0, 0.0), (1.5, 1 / 256), (3.9, 1 / 256), (4.0, 5e-3),
                                      (15.9, 5e-3), (16.0, 6e-3), (63.0, 6e-3), (64.0, 1 / 128), (100.0, 1 / 128)])
def test_stepsize_portion(bound, sp):
    from jaxngp_gb300.trainer import stepsize_portion_for
    assert stepsize_portion_for(bound) == sp


@pytest.mark.parametrize("count,factor", [(0, 1.0), (9999, 1.0), (10000, 1.0), (19999, 1.0), (20000, 1 / 3),
                                          (29999, 1 / 3), (30000, 1 / 9), (40000, 1 / 27), (50000, 1 / 81),
                                          (60000, 1 / 100), (1_000_000, 1 / 100)])
def test_learning_rate_schedule(count, factor):
    from jaxngp_gb300.trainer import lr_at
    assert lr_at(1e-2, count) == pytest.approx(1e-2 * factor, rel=1e-12)
