"""Host-side detection of uneven batches (no GPU)."""
import numpy as np

from lime_gb300 import engine


def test_ragged_detection():
    a, b = np.eye(3), np.eye(5)
    assert engine.is_ragged([a, b])
    assert engine.is_ragged((a, a))
    # the reference's driven form [H0, [H1, f1]] is not an uneven batch
    assert not engine.is_ragged([a, [b, np.cos]])
    # a single Hamiltonian in a list stays the driven solver's form
    assert not engine.is_ragged([a])
    assert not engine.is_ragged(np.stack([a, a]))
