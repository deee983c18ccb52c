"""Small propagations over every kernel family, for the bounds-checked
build's GPU test (tests/test_bounds_check_gpu.py): run once with the regular
library and once, in a child process with LIME_GB300_LIBRARY pointing at
liblime_gb300_check.so, with the bounds-checked one.  Shapes are chosen to
exercise padding and tile edges: ragged n (1, 5, 20, 33, 63, 70, 130), dense
and diagonal collapse operators, dense and population observables, stored
states, packed uneven batches (grouped persistent launches and per-size
streams), the Redfield tensor-core path in both complex-product forms with
their split-K observable passes, the driven batched kernel and both
adjoints."""
import sys

import numpy as np
import torch


def run_all() -> dict:
    from lime_gb300 import chains, engine
    from lime_gb300.adjoint import chain_observables
    from lime_gb300.redfield import redfield_tensor, propagate_vec, propagate_vec_split
    out = {}
    rng = np.random.default_rng(77)
    # FP64 path: dense operators, stored states, dense observables
    for n in (1, 5, 20, 33):
        H, c = chains.uneven_chain(n, rng, n_ops=2)
        gen = engine.LindbladGenerator.build(np.stack([H, H.T]), c + chains.dephasing_ops(n, 0.02)[:1])
        e = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        E = [e + e.conj().T, chains.population_ops(n)[0]]
        o, s, r = engine.propagate(gen, chains.ground_dm(n), 0.05, 12, E, states_every=4)
        out['f64_n%d' % n] = (o, s, r)
    # batched split kernel: population and dense observables, padded sizes, a drive
    for n in (5, 20, 63, 64):
        w = chains.disorder_ensemble(n=n, batch=7, n_steps=30)
        gen = engine.LindbladGenerator.build(w['H'], [engine.SiteDephasing(np.repeat(w['gamma'][:, None], n, 1))])
        out['split_pop_n%d' % n] = engine.propagate(gen, w['rho0'], 0.05, 30, engine.Populations(n),
                                                    precision='split', obs_every=3)
        e = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        out['split_dense_n%d' % n] = engine.propagate(gen, w['rho0'], 0.05, 30, [e + e.conj().T],
                                                      precision='split')
    mu = np.zeros((20, 20), dtype=np.complex128)
    mu[0, 1:] = mu[1:, 0] = 1.0
    gen = engine.LindbladGenerator.build(chains.exciton_chain(20, rng.normal(0, 0.05, 20)),
                                         chains.dephasing_ops(20, 0.01))
    coef = 0.01 * np.cos(0.1 * np.arange(1, 21))[:, None]
    drive = (torch.as_tensor(mu[None], device='cuda'), torch.as_tensor(coef, device='cuda'))
    for prec in ('fp64', 'split'):
        out['driven_' + prec] = engine.propagate(gen, chains.ground_dm(20), 0.05, 20, chains.population_ops(20)[:3],
                                                 drive=drive, precision=prec)
    # streaming split path: dense operators, n not a multiple of 64, several generators
    for n in (20, 70, 130):
        H, c = chains.uneven_chain(n, rng, n_ops=2)
        gen = engine.LindbladGenerator.build(H, c)
        out['stream_n%d' % n] = engine.propagate(gen, chains.ground_dm(n), 0.05, 8, chains.population_ops(n)[:2],
                                                 precision='split')
    # uneven batch, packed small chains
    ns = (8, 8, 8, 16, 32, 64)
    Hs, Cs, R0, Es = [], [], [], []
    for n in ns:
        H, c = chains.uneven_chain(n, rng)
        Hs.append(H)
        Cs.append(c)
        R0.append(chains.ground_dm(n))
        Es.append(chains.population_ops(n)[:2])
    for nm, sched in (('ragged', {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True}),
                      ('ragged_streams', {'mode': 'streams', 'pack': True}),
                      ('ragged_groups2', {'mode': 'groups', 'order': 0, 'n_ctas': 2, 'pack': False})):
        o, _, r = engine.propagate_ragged(Hs, R0, 0.05, 6, Cs, Es, precision='split', schedule=sched)
        out[nm] = (torch.stack([x[:, :2] for x in o]), None, torch.cat([x.reshape(-1) for x in r]))
    # Redfield: FP64 and the tensor-core path (split-K observable pass)
    rw = chains.redfield_chain(n=6, n_rhs=3, cfg=5)
    R, evecs = redfield_tensor(rw['H'], rw['a_ops'], rw['spectra'])
    V = torch.as_tensor(evecs, dtype=torch.complex128, device='cuda')
    r0 = V.mH @ torch.as_tensor(rw['rho0'], dtype=torch.complex128, device='cuda') @ V
    E = [V.mH @ torch.as_tensor(e, device='cuda') @ V for e in chains.population_ops(6)]
    out['redfield_f64'] = propagate_vec((R.R, 6), r0, 0.05, 10, E)
    out['redfield_split'] = propagate_vec_split((R.R, 6), r0, 0.05, 10, E, product='4m')
    out['redfield_split3'] = propagate_vec_split((R.R, 6), r0, 0.05, 10, E, product='3m')
    # adjoints (FP64 and tensor-core) of the chain model
    n = 12
    eps = torch.tensor(rng.normal(0, 0.05, (2, n)), device='cuda')
    bond = torch.full((2, n - 1), -0.1, dtype=torch.float64, device='cuda')
    gam = torch.full((2, n), 0.01, dtype=torch.float64, device='cuda')
    rho0 = torch.as_tensor(chains.ground_dm(n), device='cuda')
    for prec in ('fp64', 'split'):
        e_, b_, g_ = [x.clone().requires_grad_(True) for x in (eps, bond, gam)]
        obs = chain_observables(torch.zeros((n, n), dtype=torch.complex128, device='cuda'), e_, b_, g_, rho0,
                                chains.population_ops(n)[:3], 0.05, 16, checkpoint=8, precision=prec)
        obs.real.sum().backward()
        out['adjoint_' + prec] = (obs, None, torch.cat([e_.grad.reshape(-1), b_.grad.reshape(-1),
                                                        g_.grad.reshape(-1)]))
    torch.cuda.synchronize()
    return {k: tuple(None if x is None else x.detach().cpu().numpy() for x in v) for k, v in out.items()}


def save(path):
    res = run_all()
    flat = {}
    for k, v in res.items():
        for i, x in enumerate(v):
            if x is not None:
                flat['%s__%d' % (k, i)] = x
    np.savez(path, **flat)


if __name__ == '__main__':
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    save(sys.argv[1])
