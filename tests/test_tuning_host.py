"""The autotuner's cache and selection (lime_gb300.tuning), on the CPU with
a fake measurement."""
import json

import numpy as np
import pytest

from lime_gb300 import tuning


def test_cache_path_from_env(tmp_path, monkeypatch):
    p = tmp_path / 'x' / 'tune.json'
    monkeypatch.setenv(tuning.CACHE_ENV, str(p))
    assert tuning.cache_path() == str(p)
    monkeypatch.delenv(tuning.CACHE_ENV)
    assert tuning.cache_path().endswith('tune.json')


def test_uneven_class_is_canonical():
    a = tuning.uneven_class([256, 64, 128], [171, 89, 170], 3)
    b = tuning.uneven_class([128, 256, 64], [170, 171, 89], 3)
    assert a == b == '64x128+128x256+256x256|K3'
    # counts are bucketed to powers of two; the operator count is part of the class
    assert tuning.uneven_class([64], [100], 3) == tuning.uneven_class([64], [128], 3)
    assert tuning.uneven_class([64], [100], 3) != tuning.uneven_class([64], [129], 3)
    assert tuning.uneven_class([64], [100], 3) != tuning.uneven_class([64], [100], 2)


def test_tune_picks_the_fastest_and_caches(tmp_path):
    cache = tuning.TuneCache(str(tmp_path / 'tune.json'))
    cands = [{'mode': 'a'}, {'mode': 'b'}, {'mode': 'c'}]
    cost = {'a': 3.0, 'b': 1.0, 'c': 2.0}
    calls = []

    def measure(c):
        calls.append(c['mode'])
        return cost[c['mode']]

    choice, times = tuning.tune('k', 'cls', 'split', cands, measure, arch='sm_103', cache=cache, repeats=2)
    assert choice == {'mode': 'b'} and times == [3.0, 1.0, 2.0]
    assert calls == ['a', 'a', 'b', 'b', 'c', 'c']
    # persisted: a fresh cache object reads the same choice, no measurement
    again = tuning.TuneCache(str(tmp_path / 'tune.json'))
    calls.clear()
    choice2, times2 = tuning.tune('k', 'cls', 'split', cands, measure, arch='sm_103', cache=again)
    assert choice2 == {'mode': 'b'} and times2 is None and calls == []
    data = json.loads((tmp_path / 'tune.json').read_text())
    assert data['version'] == tuning.VERSION
    entry = data['entries'][tuning.key('k', 'cls', 'split', 'sm_103')]
    assert entry['choice'] == {'mode': 'b'} and entry['times'] == [3.0, 1.0, 2.0]
    # force re-measures; a different arch or precision is a different entry
    cost['c'] = 0.5
    choice3, _ = tuning.tune('k', 'cls', 'split', cands, measure, arch='sm_103', cache=again, force=True)
    assert choice3 == {'mode': 'c'}
    assert tuning.choose('k', 'cls', 'split', {'mode': 'dflt'}, arch='sm_100', cache=again) == {'mode': 'dflt'}
    assert tuning.choose('k', 'cls', 'fp64', {'mode': 'dflt'}, arch='sm_103', cache=again) == {'mode': 'dflt'}
    assert tuning.choose('k', 'cls', 'split', {'mode': 'dflt'}, arch='sm_103', cache=again) == {'mode': 'c'}


def test_failing_candidates_are_skipped(tmp_path):
    cache = tuning.TuneCache(str(tmp_path / 't.json'))

    def measure(c):
        if c['mode'] == 'bad':
            raise RuntimeError('unsupported')
        return 1.0

    choice, times = tuning.tune('k', 'c', 'split', [{'mode': 'bad'}, {'mode': 'ok'}], measure, arch='a',
                                cache=cache)
    assert choice == {'mode': 'ok'} and times == [None, 1.0]
    with pytest.raises(RuntimeError):
        tuning.tune('k', 'c2', 'split', [{'mode': 'bad'}], measure, arch='a', cache=cache)
    with pytest.raises(ValueError):
        tuning.tune('k', 'c3', 'split', [], measure, arch='a', cache=cache)


@pytest.mark.parametrize('content', ['not json', '{"version": 99, "entries": {"x": {}}}', '[]',
                                     '{"version": 1, "entries": {"k|c|split|a": {"choice": 3}}}'])
def test_unreadable_cache_is_empty(tmp_path, content):
    p = tmp_path / 't.json'
    p.write_text(content)
    cache = tuning.TuneCache(str(p))
    assert tuning.choose('k', 'c', 'split', {'d': 1}, arch='a', cache=cache) == {'d': 1}
    cache.put('k|c|split|a', {'d': 2})
    cache.save()
    assert tuning.TuneCache(str(p)).get('k|c|split|a') == {'d': 2}


def test_engine_uneven_class_groups_like_the_launch():
    from lime_gb300 import engine
    sizes = [8] * 10 + [16] * 5 + [64] * 3 + [256] * 2
    H = [np.eye(n) for n in sizes]
    C = [[np.eye(n)] * 3 for n in sizes]
    # packed: 8 chains of 8 per 64-dim instance (10 -> 2), 4 of 16 (5 -> 2)
    got = engine.uneven_class(H, C, 'split', pack=True)
    assert got == tuning.uneven_class([64, 64, 64, 256], [2, 2, 3, 2], 3)
    assert engine.uneven_class(H, C, 'split', pack=False) == tuning.uneven_class([64, 64, 64, 256],
                                                                                 [10, 5, 3, 2], 3)


def test_redfield_product_cost_model():
    """The wave-quantised cost model behind the Redfield split path's choice
    of complex product: the 3M form at the 9216-dim, 512-RHS workload (6
    waves of 144 chunks vs 4 of 288), the block form where the 3M tiles
    would spill into a second wave (dim 4096, 256 RHS: measured 0.87 vs
    0.73 ms per step)."""
    from lime_gb300.redfield import split_class, split_cost
    t4, t3 = split_cost(96, 512, 152)
    assert t4 == 4 * 288 and t3 < 0.97 * t4
    t4, t3 = split_cost(64, 256, 152)
    assert t4 == 128 and t3 > 0.97 * t4
    assert split_class(96, 512) == 'D9216|R512' and split_class(12, 130) == 'D256|R192'


def test_default_cache_is_reread_only_when_it_changes(tmp_path, monkeypatch):
    import os
    p = tmp_path / 'tune.json'
    monkeypatch.setenv(tuning.CACHE_ENV, str(p))
    assert tuning.choose('k', 'c', 'split', {'d': 0}, arch='a') == {'d': 0}
    c = tuning.TuneCache(str(p))
    c.put(tuning.key('k', 'c', 'split', 'a'), {'d': 1})
    c.save()
    os.utime(p, (1, 1))                       # a distinct modification time
    assert tuning.choose('k', 'c', 'split', {'d': 0}, arch='a') == {'d': 1}
    c.put(tuning.key('k', 'c', 'split', 'a'), {'d': 2})
    c.save()
    os.utime(p, (2, 2))
    assert tuning.choose('k', 'c', 'split', {'d': 0}, arch='a') == {'d': 2}
