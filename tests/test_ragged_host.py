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


def test_pack_count():
    # the tensor-core paths pack chains of n <= 32 block-diagonally to 64
    assert engine.pack_count(8, 'split') == 8
    assert engine.pack_count(5, 'split') == 12
    assert engine.pack_count(32, 'split') == 2
    assert engine.pack_count(33, 'split') == 1
    assert engine.pack_count(1, 'split') == 64
    assert engine.pack_count(8, 'fp64') == 1


def test_block_diagonal_embedding_and_unpack():
    import torch
    rng = np.random.default_rng(3)
    G, p, n = 2, 3, 4
    blocks = torch.as_tensor(rng.normal(size=(G, p, n, n)) + 1j * rng.normal(size=(G, p, n, n)))
    full = engine._embed(blocks)
    assert full.shape == (G, p * n, p * n)
    for g in range(G):
        for q in range(p):
            for r in range(p):
                blk = full[g, q * n:(q + 1) * n, r * n:(r + 1) * n]
                assert torch.equal(blk, blocks[g, q] if q == r else torch.zeros_like(blk))
    # 5 instances in 2 packed launches of 3: outputs go back per instance
    m, T = 2, 7
    o = torch.as_tensor(rng.normal(size=(G, T, p * m)))
    grp = engine.RaggedGroup(idx=[4, 0, 2, 1, 3], n=n, n_obs=m, pack=p, gen=None, rho=None, e_ops=None)
    out = grp.unpack(o, None, full)
    assert len(out) == 5
    for j, (oj, sj, rj) in enumerate(out):
        g, q = divmod(j, p)
        assert sj is None
        assert torch.equal(oj, o[g, :, q * m:(q + 1) * m])
        assert torch.equal(rj, blocks[g, q])
