"""Generate golden vectors by running the reference lime solvers.

Run in a container where the reference tree is available (read-only):

    python tests/golden/make_golden.py /root/reference

The reference is pure Python.  Three import-time dependencies that are not
installed and are not on the propagation path are replaced by permissive
stubs: ``numba`` (``jit``/``njit`` become identity decorators), ``proplot``
and ``matplotlib`` (plotting only).  ``lime.mol.Result`` raises TypeError
unless ``nout`` and ``t0`` are given (``lime/mol.py:92``); the generator
patches a subclass with ``nout=1, t0=0`` defaults (and ``Nt = len(times)``,
``dt = 0`` when only ``times`` is given, ``lime/superoperator.py:527``) into
``lime.oqs`` and ``lime.superoperator``.

``_lindblad_driven`` (lime/oqs.py:1691) builds H(t) with ``Ht = H[0];
Ht += ...``, which aliases and mutates ``H[0]`` every step.  The driven case
therefore passes ``H[0]`` as an ndarray subclass whose ``+=`` returns a new
array, so the fixture pins the documented H(t) = H0 - f(t) H1.

Every fixture stores its inputs next to the outputs, so the tests do not
depend on the workload builders staying bit-stable.
"""
from __future__ import annotations

import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from lime_gb300 import chains  # noqa: E402


class _Any(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        return _anything


def _anything(*a, **k):
    if len(a) == 1 and callable(a[0]) and not k:
        return a[0]
    return _anything


def import_reference(ref_root):
    for name in ['numba', 'proplot', 'matplotlib', 'matplotlib.pyplot',
                 'matplotlib.cm', 'matplotlib.colors', 'matplotlib.collections',
                 'matplotlib.ticker']:
        sys.modules[name] = _Any(name)
    sys.path.insert(0, ref_root)
    import lime.mol
    import lime.oqs as oqs
    import lime.superoperator as superop
    import lime.fft as lfft

    class Result(lime.mol.Result):
        def __init__(self, *a, **k):
            k.setdefault('nout', 1)
            k.setdefault('t0', 0)
            if k.get('Nt') is None:
                k['Nt'] = len(k['times']) if k.get('times') is not None else 1
            if k.get('dt') is None:
                k['dt'] = 0.0
            super().__init__(*a, **k)

    oqs.Result = Result
    superop.Result = Result
    return oqs, superop, lfft


class NoInplace(np.ndarray):
    def __iadd__(self, other):
        return np.add(np.asarray(self), other).view(NoInplace)


def main(ref_root):
    oqs, superop, lfft = import_reference(ref_root)
    out = {}

    # 1. single 16-site chain, full 2000 steps
    w = chains.single_chain()
    res = oqs.Lindblad_solver(w['H'], c_ops=w['c_ops']).evolve(
        w['rho0'], dt=w['dt'], Nt=w['Nt'], e_ops=w['e_ops'])
    snap = np.array([0, 99, 499, 999, 1999])
    out['lindblad_chain16'] = dict(
        H=w['H'], c_ops=np.array(w['c_ops']), rho0=w['rho0'],
        e_ops=np.array(w['e_ops']), dt=w['dt'], Nt=w['Nt'],
        observables=res.observables, snap=snap,
        rho_snap=np.array([res.rholist[i] for i in snap]))

    # 1b. the file-writing branch (observables before each step, final rho)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        try:
            rho_f = oqs._lindblad(w['H'], w['rho0'], w['c_ops'], e_ops=w['e_ops'][:4],
                                  Nt=50, dt=w['dt'], return_result=False)
            rows = [line.split() for line in open('obs.dat')]
        finally:
            os.chdir(cwd)
    obs_f = np.array([[complex(x) for x in r[1:]] for r in rows])
    out['lindblad_chain16_noresult'] = dict(
        H=w['H'], c_ops=np.array(w['c_ops']), rho0=w['rho0'],
        e_ops=np.array(w['e_ops'][:4]), dt=w['dt'], Nt=50,
        observables=obs_f, rho_final=rho_f)

    # 2. dense collapse operators (uneven-batch model), N = 8
    rng = chains.rng_for(3, child=10_000)
    H, c_ops = chains.uneven_chain(8, rng)
    e_ops = []
    for _ in range(3):
        X = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
        e_ops.append((X + X.conj().T) / 2)
    rho0 = chains.ground_dm(8)
    res = oqs.Lindblad_solver(H, c_ops=c_ops).evolve(rho0, dt=0.05, Nt=300, e_ops=e_ops)
    snap = np.array([0, 49, 149, 299])
    out['lindblad_dense8'] = dict(
        H=H, c_ops=np.array(c_ops), rho0=rho0, e_ops=np.array(e_ops), dt=0.05,
        Nt=300, observables=res.observables, snap=snap,
        rho_snap=np.array([res.rholist[i] for i in snap]))

    # 3. dipole correlation <mu(t) mu(0)> for an 8-site absorption chain
    m = chains.absorption_chain(8, chains.rng_for(4, child=10_000))
    rho_g = chains.ground_dm(9)
    with tempfile.TemporaryDirectory() as td:
        cor = oqs.Lindblad_solver(m['H'], c_ops=m['c_ops']).correlation_2op_1t(
            rho_g, m['mu'], m['mu'], dt=0.05, Nt=400, output=os.path.join(td, 'cor.dat'))
    out['correlation_2op_chain8'] = dict(
        H=m['H'], c_ops=np.array(m['c_ops']), mu=m['mu'], rho0=rho_g, dt=0.05,
        Nt=400, cor=cor)

    # 4. three- and four-operator correlations, N = 4, two dense collapse ops
    rng = chains.rng_for(4, child=20_000)
    H, c_ops = chains.uneven_chain(4, rng, n_ops=2)
    ops = [rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)) for _ in range(4)]
    rho0 = chains.ground_dm(4)
    sol = oqs.Lindblad_solver(H, c_ops=c_ops)
    c3 = sol.correlation_3op_1t(rho0, ops[:3], dt=0.05, Nt=30)
    c4 = sol.correlation_4op_1t(rho0, ops, dt=0.05, nt=30)
    c32 = sol.correlation_3op_2t(rho0, ops[:3], dt=0.05, Nt=12, Ntau=10)
    c42 = sol.correlation_4op_2t(rho0, ops, dt=0.05, nt=12, ntau=10)
    out['correlations_n4'] = dict(
        H=H, c_ops=np.array(c_ops), ops=np.array(ops), rho0=rho0, dt=0.05,
        c3op_1t=c3, c4op_1t=c4, c3op_2t=c32, c4op_2t=c42)

    # 5. Redfield tensor + RK4 + Green's-function route, N = 8 chain
    wr = chains.redfield_chain(n=8, n_rhs=2, cfg=5)
    rs = oqs.Redfield_solver(wr['H'], c_ops=wr['a_ops'], spectra=wr['spectra'])
    R, evecs = rs.redfield_tensor()
    Rd = R.toarray()
    e_ops = chains.population_ops(8)
    rho0 = wr['rho0'][0]
    res = rs.evolve(rho0, dt=0.05, Nt=200, e_ops=e_ops)
    snap = np.array([0, 99, 199])
    tau = np.arange(6) * 0.5
    U = rs.propagator(tau)
    ex = rs.expect(rho0, e_ops[:3])
    mu = np.zeros((8, 8), dtype=complex)
    mu[0, 1:] = 1.0
    mu[1:, 0] = 1.0
    # Redfield_solver.correlation_2op_1t (lime/oqs.py:254-275) cannot run:
    # dm2vec(identity(dim)) is an (N^2, 1) sparse column and idm.dot fails.
    c43 = rs.correlation_4op_3t(rho0, [mu] * 4, 'llll', tau[:4])
    w_grid = -chains.rng_for(5, child=1).uniform(0, 0.3, size=(8, 8))
    out['redfield_chain8'] = dict(
        H=wr['H'], a_ops=np.array(wr['a_ops']), rho0=rho0, dt=0.05, Nt=200,
        R=Rd, evecs=evecs, e_ops=np.array(e_ops), observables=res.observables,
        snap=snap, rho_snap=np.array([res.rholist[i] for i in snap]),
        tau=tau, U=U[:, :, :3], expect=ex, mu=mu, c4op_3t=c43,
        spectrum_w=w_grid, spectrum_S=wr['spectra'][0](w_grid))

    # 6. Liouville-space superoperators and the eigen-series solver, N = 4
    rng = chains.rng_for(1, child=30_000)
    H, c_ops = chains.uneven_chain(4, rng, n_ops=2)
    Ls = superop.liouvillian(H, c_ops).toarray()
    es = superop.Lindblad_solver(H, c_ops=c_ops)
    es.eigenstates()
    tl = np.arange(10) * 0.3
    e_ops = chains.population_ops(4)
    ev = es.evolve(chains.ground_dm(4), tl, e_ops).observables
    a_op = np.zeros((4, 4), dtype=complex)
    a_op[0, 1:] = 1.0
    a_op[1:, 0] = 1.0
    cc = es.correlation_2op_1t(chains.ground_dm(4), [a_op, a_op], tl)
    out['superop_n4'] = dict(H=H, c_ops=np.array(c_ops), L=Ls, t=tl,
                             e_ops=np.array(e_ops), evolve=ev, a=a_op, cor=cc,
                             op2sop_c=superop.op2sop(H).toarray(),
                             op2sop_l=superop.op2sop(H, 'left').toarray(),
                             op2sop_r=superop.op2sop(H, 'right').toarray(),
                             op2sop_a=superop.op2sop(H, 'anticommutator').toarray())

    # 7. driven Lindblad, H(t) = H0 - f(t) H1, f(t) = 0.1 sin(t)
    rng = chains.rng_for(1, child=40_000)
    H0, c_ops = chains.uneven_chain(4, rng, n_ops=2)
    H1 = np.zeros((4, 4), dtype=complex)
    H1[0, 1:] = 1.0
    H1[1:, 0] = 1.0
    f = lambda t: 0.1 * np.sin(t)
    res = oqs._lindblad_driven([np.array(H0).view(NoInplace), [H1, f]],
                               rho0=chains.ground_dm(4), c_ops=c_ops,
                               e_ops=chains.population_ops(4), Nt=100, dt=0.05)
    out['driven_n4'] = dict(H0=H0, H1=H1, c_ops=np.array(c_ops), dt=0.05, Nt=100,
                            observables=res.observables,
                            rho_final=np.asarray(res.rholist[-1]))

    # 8. FFT sign convention
    x = np.arange(64) * 0.5 + 1.25
    sig = np.exp(-0.05 * x) * np.cos(0.7 * x) + 0.2j * np.sin(0.3 * x)
    g, freq = lfft.fft(sig, x)
    out['fft'] = dict(x=x, f=sig, g=g, freq=freq)

    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **d)
        print('wrote', name, {k: np.shape(v) for k, v in d.items()})


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
