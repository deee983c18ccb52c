"""The uneven batch in one grouped persistent launch per GEMM phase
(lime_lindblad_rk4_stream_groups): every schedule gives the same bits as
one launch sequence per size (the tiles do the same arithmetic, only the
place where a finished tile is parked differs), and all agree with the FP64
path; the autotuner measures the schedules and caches its choice."""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _batch(sizes, seed, n_ops=3):
    rng = np.random.default_rng(seed)
    H, C, R, E = [], [], [], []
    for n in sizes:
        h, c = chains.uneven_chain(n, rng, n_ops=n_ops)
        H.append(h)
        C.append(c)
        R.append(chains.ground_dm(n))
        E.append([chains.population_ops(n)[0], chains.population_ops(n)[n - 1]])
    return H, C, R, E


SIZES = [8, 16, 64, 8, 130, 32, 256, 64, 16, 130]


def _run(sched, steps=24, sizes=SIZES, seed=3, prec='split'):
    from lime_gb300 import engine
    H, C, R, E = _batch(sizes, seed)
    return engine.propagate_ragged(H, R, 0.05, steps, C, E, precision=prec, schedule=sched, obs_every=2)


def _same(a, b):
    """(obs, states, rho) lists equal bit for bit (states None on both)."""
    for x, y in zip(a, b):
        assert len(x) == len(y)
        for u, v in zip(x, y):
            assert (u is None and v is None) or torch.equal(u, v)


def test_grouped_launch_matches_streams_bitwise_and_fp64():
    base = {'mode': 'streams', 'order': 1, 'n_ctas': 0, 'pack': True}
    ref = _run(base)
    for sched in ({'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True},
                  {'mode': 'groups', 'order': 0, 'n_ctas': 0, 'pack': True},
                  {'mode': 'groups', 'order': 1, 'n_ctas': 3, 'pack': True}):
        _same(_run(sched), ref)
    o64, _, r64 = _run(None, prec='fp64')
    osp, _, rsp = ref[0], None, ref[2]
    for a, b in zip(osp, o64):
        assert (a - b).abs().max().item() < 1e-6
    for a, b in zip(rsp, r64):
        assert (a - b).abs().max().item() < 1e-6


def test_grouped_launch_unpacked_and_without_dense_operators():
    """Unpacked small chains; a group without dense collapse operators (its
    stage update runs in the elementwise kernel between the grouped
    launches) next to groups with them."""
    from lime_gb300 import engine
    rng = np.random.default_rng(5)
    sizes = [16, 80, 130, 80]
    H, C, R, E = _batch(sizes, 7)
    # chain 1 and 3 (n = 80): diagonal (dephasing) operators only
    for i in (1, 3):
        n = sizes[i]
        C[i] = [np.diag(np.sqrt(rng.uniform(0.005, 0.02, n))).astype(complex) for _ in range(2)]
    outs = []
    for sched in ({'mode': 'streams', 'pack': False}, {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': False},
                  {'mode': 'groups', 'order': 1, 'n_ctas': 2, 'pack': False}):
        outs.append(engine.propagate_ragged(H, R, 0.05, 20, C, E, precision='split', schedule=sched))
    _same(outs[1], outs[0])
    _same(outs[2], outs[0])
    o64, _, _ = engine.propagate_ragged(H, R, 0.05, 20, C, E, precision='fp64')
    for a, b in zip(outs[1][0], o64):
        assert (a - b).abs().max().item() < 1e-6


def test_more_groups_than_one_launch_holds():
    """More size groups than one grouped call takes: the host splits them
    into several calls."""
    from lime_gb300 import _native, engine
    cap = int(_native.require_device().lime_lindblad_stream_max_groups())
    sizes = [65 + 3 * i for i in range(cap + 2)]
    H, C, R, E = _batch(sizes, 9, n_ops=1)
    a = engine.propagate_ragged(H, R, 0.05, 6, C, E, precision='split',
                                schedule={'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True})
    b = engine.propagate_ragged(H, R, 0.05, 6, C, E, precision='split',
                                schedule={'mode': 'streams', 'pack': True})
    _same(a, b)


def test_autotune_writes_the_cache(tmp_path):
    from lime_gb300 import engine, tuning
    H, C, R, E = _batch([8, 64, 130, 130, 16], 4)
    cache = tuning.TuneCache(str(tmp_path / 'tune.json'))
    choice, times = engine.autotune_ragged(H, R, 0.05, C, E, precision='split', steps=4, cache=cache)
    assert choice in [dict(c) for c in engine.UNEVEN_CANDIDATES]
    assert len(times) == len(engine.UNEVEN_CANDIDATES) and all(t is not None for t in times)
    k = tuning.key('lindblad_uneven', engine.uneven_class(H, C, 'split'), 'split', tuning.arch_tag())
    assert tuning.TuneCache(str(tmp_path / 'tune.json')).get(k) == choice
    # propagate_ragged picks the cached choice up through the cache file
    import os
    old = os.environ.get(tuning.CACHE_ENV)
    os.environ[tuning.CACHE_ENV] = str(tmp_path / 'tune.json')
    try:
        o, _, _ = engine.propagate_ragged(H, R, 0.05, 4, C, E, precision='split')
        ref, _, _ = engine.propagate_ragged(H, R, 0.05, 4, C, E, precision='split', schedule=choice)
        for x, y in zip(o, ref):
            assert torch.equal(x, y)
    finally:
        if old is None:
            del os.environ[tuning.CACHE_ENV]
        else:
            os.environ[tuning.CACHE_ENV] = old


@pytest.mark.parametrize('n', [200, 256, 300, 384])
def test_hermitian_half_gemm2_vs_fp64(n):
    """Dense collapse operators at dimensions whose padded size is a multiple
    of 128 with two or three row tiles (200, 256 -> 256; 384 -> 384): GEMM 2
    runs over the upper tiles of the Hermitian Z and the lower ones are
    updated from their transposes; 300 (padded 320) takes the full tile set.
    Against the FP64 path, through both the single-group and the grouped
    launch."""
    from lime_gb300 import engine
    H, C, R, E = _batch([n], 10 + n)
    o64, _, r64 = engine.propagate_ragged(H, R, 0.05, 10, C, E, precision='fp64')
    for sched in ({'mode': 'streams', 'pack': True}, {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True}):
        o, _, r = engine.propagate_ragged(H, R, 0.05, 10, C, E, precision='split', schedule=sched)
        assert (o[0] - o64[0]).abs().max().item() < 1e-6
        assert (r[0] - r64[0]).abs().max().item() < 1e-6
        # the final state stays Hermitian to the split precision
        assert (r[0] - r[0].mH).abs().max().item() < 1e-6
