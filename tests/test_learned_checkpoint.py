"""Checkpoint and resume of learned-filter training: params, scale and the Adam state
(sgb_lf_get_state / sgb_lf_set_state) saved to one file, and a filter loaded from it that
continues exactly as the uninterrupted one does.

The batches are single rows of 128 samples: one row is one weight-gradient tile, so every
gradient sum has one nonzero term and training is bitwise reproducible, which lets the test
ask for equality rather than a tolerance."""
import numpy as np
import pytest

from sinograms import learned as LF

pytestmark = pytest.mark.gpu


def _batches(n):
    out = []
    for i in range(n):
        rng = np.random.default_rng(500 + i)
        z = rng.standard_normal((1, 128)).astype(np.float32)
        t = (z + 0.3 * rng.standard_normal((1, 128))).astype(np.float32)
        out.append((z, t, 1e-3 * (1.0 - 0.1 * i)))
    return out


def test_resumed_training_equals_uninterrupted_training(cuda, tmp_path):
    steps = _batches(7)
    lf = LF.LearnedFilter(scale=0.9, seed=5)
    for z, t, lr in steps[:4]:
        lf.train_step(z, t, lr)
    path = str(tmp_path / "lf_checkpoint.npz")
    lf.save_checkpoint(path)
    m0, v0, s0 = lf.adam_state()
    assert s0 == 4 and np.any(m0 != 0) and np.any(v0 != 0)
    for z, t, lr in steps[4:]:
        lf.train_step(z, t, lr)

    resumed = LF.LearnedFilter.load_checkpoint(path)
    m1, v1, s1 = resumed.adam_state()
    assert s1 == 4 and np.array_equal(m1, m0) and np.array_equal(v1, v0)
    for z, t, lr in steps[4:]:
        resumed.train_step(z, t, lr)
    assert np.array_equal(resumed.params(), lf.params())
    assert resumed.adam_state()[2] == 7

    # the same params without the Adam state take different steps
    restarted = LF.LearnedFilter.load(path)
    for z, t, lr in steps[4:]:
        restarted.train_step(z, t, lr)
    assert not np.array_equal(restarted.params(), lf.params())


def test_adam_state_of_the_wrong_size_is_refused(cuda):
    lf = LF.LearnedFilter(scale=1.0, seed=0)
    with pytest.raises(ValueError):
        lf.set_adam_state(np.zeros(3), np.zeros(3), 1)
