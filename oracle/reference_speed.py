"""Speed of the NumPy port against the reference's own solver (test
infrastructure; runs where the reference tree is available, read-only):

    OMP_NUM_THREADS=1 python oracle/reference_speed.py /root/reference

Times lime.oqs._lindblad (lime/oqs.py:1590-1688), imported through the stub
shim of tests/golden/make_golden.py, and oracle.lindblad.lindblad on the same
realisation of the 64-site dephasing ensemble (64 collapse operators, 64
population observables every step), single-threaded, best of three, and
prints both rates and their ratio as one JSON line.  The bench's reference
arm runs the port (the reference tree does not travel with the repository);
this script is the evidence that the two run at the same speed.
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'tests', 'golden'))


def main(ref_root, n=64, steps=30, reps=3):
    import numpy as np
    from make_golden import import_reference
    from lime_gb300 import chains
    from oracle import lindblad as ol
    oqs, _, _ = import_reference(ref_root)
    w = chains.disorder_ensemble(n=n, batch=1, n_steps=steps, cfg=2)
    H = w['H'][0]
    c_ops = chains.dephasing_ops(n, float(w['gamma'][0]))
    e_ops = chains.population_ops(n)

    def best(fn):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            ts.append(time.perf_counter() - t0)
        return min(ts), out

    t_ref, res = best(lambda: oqs._lindblad(H, w['rho0'], c_ops, e_ops=e_ops, Nt=steps, dt=w['dt']))
    t_port, (obs, _) = best(lambda: ol.lindblad(H, w['rho0'], c_ops, e_ops, Nt=steps, dt=w['dt'],
                                                store_states=False))
    diff = float(np.max(np.abs(np.asarray(res.observables) - obs)))
    print(json.dumps({'workload': '%d-site dephasing chain, %d collapse operators, %d population '
                                  'observables every step, %d RK4 steps, one core' % (n, n, n, steps),
                      'reference_steps_per_s': steps / t_ref, 'port_steps_per_s': steps / t_port,
                      'port_over_reference': t_ref / t_port, 'max_observable_difference': diff,
                      'omp_num_threads': os.environ.get('OMP_NUM_THREADS')}))


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
