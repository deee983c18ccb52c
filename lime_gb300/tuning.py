"""Autotuning of the free launch choices of the tensor-core paths.

The tile shapes of the kernels follow from the hardware budgets (TMEM
columns, shared memory, registers) and are compiled in; what is left free
at run time is chosen here by measurement and remembered in a JSON cache:

* ``lindblad_uneven`` (an uneven batch on the streaming tensor-core path):
  one grouped persistent launch per GEMM phase for all sizes or one launch
  sequence per size on concurrent streams, the tile order of the grouped
  launch (largest tiles first or as given), the persistent CTA count, and
  whether chains of dimension <= 32 are packed block-diagonally.
* ``redfield_split`` (the tensor-core Redfield RK4): the complex product in
  its block form or its 3M form (``redfield.autotune_split``).

The cache is keyed by (kind, N-class, precision, arch): the N-class of an
uneven batch is its multiset of padded group dimensions with bucketed
instance counts and the collapse-operator count (``uneven_class``), of a
Redfield shape its padded Liouville dimension and right-hand-side count;
the arch is the device's compute capability.  It lives at ``$LIME_GB300_TUNE_CACHE``
or ``~/.cache/lime_gb300/tune.json``; a missing or unreadable file is an
empty cache, writes are atomic (temporary file + rename).
"""
from __future__ import annotations

import json
import math
import os
import tempfile
import time

CACHE_ENV = 'LIME_GB300_TUNE_CACHE'
VERSION = 1


def cache_path() -> str:
    p = os.environ.get(CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'lime_gb300', 'tune.json')


def arch_tag(device=None) -> str:
    """'sm_103' style tag of the device (``'cpu'`` without CUDA)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return 'cpu'
        major, minor = torch.cuda.get_device_capability(device)
        return 'sm_%d%d' % (major, minor)
    except Exception:
        return 'cpu'


def _bucket(count: int) -> int:
    """Instance counts rounded up to a power of two (timings scale smoothly
    with the count; the cache should not miss on 170 vs 171 chains)."""
    return 1 << max(0, math.ceil(math.log2(max(1, count))))


def uneven_class(group_dims, group_counts, n_ops: int) -> str:
    """N-class of an uneven batch: sorted (padded dimension x bucketed
    count) pairs of its groups and the collapse-operator count, e.g.
    ``'64x128+128x256+256x256|K3'``."""
    pairs = sorted((int(d), _bucket(int(c))) for d, c in zip(group_dims, group_counts))
    return '+'.join('%dx%d' % p for p in pairs) + '|K%d' % int(n_ops)


def key(kind: str, n_class: str, precision: str, arch: str) -> str:
    return '%s|%s|%s|%s' % (kind, n_class, precision, arch)


class TuneCache:
    """The JSON cache: {"version": 1, "entries": {key: {"choice": {...},
    "times": [...], "candidates": [...], "when": epoch seconds}}}."""

    def __init__(self, path: str | None = None):
        self.path = path or cache_path()
        self.entries = {}
        self.load()

    def load(self):
        self.entries = {}
        try:
            with open(self.path) as f:
                data = json.load(f)
            if isinstance(data, dict) and data.get('version') == VERSION and isinstance(data.get('entries'), dict):
                self.entries = data['entries']
        except (OSError, ValueError):
            self.entries = {}

    def get(self, k: str):
        e = self.entries.get(k)
        return dict(e['choice']) if isinstance(e, dict) and isinstance(e.get('choice'), dict) else None

    def put(self, k: str, choice: dict, candidates=None, times=None):
        self.entries[k] = {'choice': dict(choice), 'candidates': list(candidates or []),
                           'times': list(times or []), 'when': time.time()}

    def save(self):
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix='.tune', suffix='.json', dir=d)
        try:
            with os.fdopen(fd, 'w') as f:
                json.dump({'version': VERSION, 'entries': self.entries}, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except BaseException:
            try:
                os.unlink(tmp)
            except OSError:
                pass
            raise


_LOADED = {}   # cache path -> (modification time, TuneCache): one file read per change


def _default_cache() -> TuneCache:
    path = cache_path()
    try:
        mtime = os.path.getmtime(path)
    except OSError:
        mtime = None
    hit = _LOADED.get(path)
    if hit is None or hit[0] != mtime:
        hit = (mtime, TuneCache(path))
        _LOADED[path] = hit
    return hit[1]


def choose(kind: str, n_class: str, precision: str, default: dict, arch: str | None = None,
           cache: TuneCache | None = None) -> dict:
    """The cached choice for the key, or ``default`` (no measurement).  The
    default cache file is read again only when it changes."""
    c = cache if cache is not None else _default_cache()
    got = c.get(key(kind, n_class, precision, arch or arch_tag()))
    return got if got is not None else dict(default)


def tune(kind: str, n_class: str, precision: str, candidates, measure, arch: str | None = None,
         cache: TuneCache | None = None, force: bool = False, repeats: int = 2):
    """Measure every candidate (``measure(candidate) -> seconds``, best of
    ``repeats``), store the fastest under the key and return
    ``(choice, times)``.  A cached entry is returned without measuring
    unless ``force``.  A candidate whose measurement raises is skipped (its
    time is recorded as None); if every one fails the error propagates."""
    c = cache if cache is not None else TuneCache()
    k = key(kind, n_class, precision, arch or arch_tag())
    if not force:
        got = c.get(k)
        if got is not None:
            return got, None
    cands = [dict(x) for x in candidates]
    if not cands:
        raise ValueError('no candidates to tune over')
    times, last_err = [], None
    for cand in cands:
        best = None
        for _ in range(max(1, repeats)):
            try:
                t = float(measure(cand))
            except Exception as e:   # noqa: BLE001 - a failing candidate is not chosen
                last_err = e
                best = None
                break
            best = t if best is None else min(best, t)
        times.append(best)
    ok = [(t, i) for i, t in enumerate(times) if t is not None]
    if not ok:
        raise last_err if last_err is not None else RuntimeError('no candidate could be measured')
    choice = cands[min(ok)[1]]
    c.put(k, choice, cands, times)
    c.save()
    return choice, times
