"""Multi-process timing of the NumPy oracle on the host cores (test/bench only).

One process per core (spawn start method, single-threaded BLAS), each
propagating its own realisation of the disorder ensemble through the oracle
restatement of ``_lindblad`` (lime/oqs.py:1590-1688) with population
observables every step, exactly the per-instance work the reference does.
Returns the aggregate instance-steps/s.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time


def _one_instance(args):
    n, b, n_steps, dt, seed_cfg = args
    import numpy as np
    from lime_gb300 import chains
    from oracle import lindblad as ol
    w = chains.disorder_ensemble(n=n, batch=b + 1, n_steps=n_steps, dt=dt, cfg=seed_cfg)
    H = w['H'][b]
    c_ops = chains.dephasing_ops(n, float(w['gamma'][b]))
    e_ops = chains.population_ops(n)
    t0 = time.perf_counter()
    ol.lindblad(H, w['rho0'], c_ops, e_ops, Nt=n_steps, dt=dt, store_states=False)
    return time.perf_counter() - t0


def _timed_instance(args):
    """Warm-up steps, then timed steps, of one realisation; returns the
    timed seconds."""
    n, b, warm_steps, steps, dt, seed_cfg = args
    from lime_gb300 import chains
    from oracle import lindblad as ol
    w = chains.disorder_ensemble(n=n, batch=b + 1, n_steps=steps, dt=dt, cfg=seed_cfg)
    H = w['H'][b]
    c_ops = chains.dephasing_ops(n, float(w['gamma'][b]))
    e_ops = chains.population_ops(n)
    if warm_steps:
        ol.lindblad(H, w['rho0'], c_ops, e_ops, Nt=warm_steps, dt=dt, store_states=False)
    t0 = time.perf_counter()
    ol.lindblad(H, w['rho0'], c_ops, e_ops, Nt=steps, dt=dt, store_states=False)
    return time.perf_counter() - t0


def _single_threaded_pool(cores, fn, tasks):
    env_keys = ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS')
    old = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = '1'
    try:
        ctx = mp.get_context('spawn')
        with ctx.Pool(cores) as pool:
            pool.map(_one_instance, [(tasks[0][0], 0, 1, tasks[0][-2], tasks[0][-1])] * cores)  # imports
            return pool.map(fn, tasks)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def concurrent_steps(n=64, warm_steps=8, steps=64, cores=None, dt=0.05, cfg=2):
    """One realisation per core, all cores at once: ``warm_steps`` untimed
    RK4 steps, then ``steps`` timed ones.  Returns (seconds of the slowest
    core, cores)."""
    cores = cores or os.cpu_count() or 1
    times = _single_threaded_pool(cores, _timed_instance,
                                  [(n, b % 64, warm_steps, steps, dt, cfg) for b in range(cores)])
    return max(times), cores


def ensemble_rate(n=64, n_steps=20, cores=None, dt=0.05, cfg=2):
    """Instance-steps/s of the oracle on ``cores`` processes (one instance each).

    Returns (rate, cores, wall_seconds).
    """
    cores = cores or os.cpu_count() or 1
    env_keys = ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS')
    old = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = '1'
    try:
        ctx = mp.get_context('spawn')
        with ctx.Pool(cores) as pool:
            # warm the workers (imports) before timing
            pool.map(_one_instance, [(n, 0, 1, dt, cfg)] * cores)
            t0 = time.perf_counter()
            pool.map(_one_instance, [(n, b % 64, n_steps, dt, cfg) for b in range(cores)])
            wall = time.perf_counter() - t0
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return cores * n_steps / wall, cores, wall
