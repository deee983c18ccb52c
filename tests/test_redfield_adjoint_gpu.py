"""Gradients of Bloch-Redfield populations through the library's kernels
(lime_gb300.redfield_grad): the assembly adjoint and the discrete RK4
adjoint against

* torch autograd through a plain-torch FP64 restatement of the same
  computation (the generator's closed form and RK4, lime/oqs.py:528-579 and
  453-472) at 1e-9 relative, and
* central finite differences of the library's FP64 forward at 1e-5
  relative,

for site energies, the coupling J, per-site bath coupling strengths and the
reorganisation energy of the Ohmic spectrum."""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
CDT = torch.complex128


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _model(n, seed):
    rng = np.random.default_rng(seed)
    dev = torch.device('cuda')
    eps = torch.tensor(rng.normal(0, 0.05, n), device=dev)
    J = torch.tensor(-0.1, dtype=torch.float64, device=dev)
    s = torch.tensor(rng.uniform(0.8, 1.2, n), device=dev)
    lam = torch.tensor(0.05, dtype=torch.float64, device=dev)
    psi = rng.normal(size=(2, n)) + 1j * rng.normal(size=(2, n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    rho0 = torch.as_tensor(np.einsum('bi,bj->bij', psi, psi.conj()), device=dev)
    E = torch.as_tensor(np.stack(chains.population_ops(n)), device=dev)
    return dict(eps=eps, J=J, s=s, lam=lam, rho0=rho0, E=E, rng=rng)


def _inputs(m, eps, J, s, lam):
    n = eps.shape[0]
    off = torch.diag(torch.ones(n - 1, dtype=torch.float64, device=eps.device), 1)
    H = torch.diag(eps) + J * (off + off.T)
    proj = torch.stack([torch.diag(torch.nn.functional.one_hot(torch.tensor(k), n).to(torch.float64))
                        for k in range(n)]).to(eps.device)
    a_ops = s[:, None, None] * proj
    return H, a_ops


def _loss_lib(m, eps, J, s, lam, weights, n_steps, obs_every, checkpoint, precision='fp64'):
    from lime_gb300.redfield_grad import redfield_observables, ohmic_spectrum
    H, a_ops = _inputs(m, eps, J, s, lam)
    obs = redfield_observables(H, a_ops, ohmic_spectrum(lam, 0.1, 0.025), m['rho0'], m['E'], 0.05, n_steps,
                               obs_every=obs_every, checkpoint=checkpoint, precision=precision)
    return (obs.real * weights).sum()


def _loss_torch(m, eps, J, s, lam, weights, n_steps, obs_every):
    """The same computation in plain torch FP64 (closed-form generator, RK4)."""
    from lime_gb300.redfield_grad import ohmic_spectrum
    H, a_ops = _inputs(m, eps, J, s, lam)
    n = H.shape[0]
    E, V = torch.linalg.eigh(H)
    Vc = V.to(CDT)
    A = Vc.mH @ a_ops.to(CDT) @ Vc
    W = E[:, None] - E[None, :]
    C = ohmic_spectrum(lam, 0.1, 0.025)(-W).to(CDT)
    Lam = C * A
    P = (A @ Lam).sum(0)
    Q = (Lam.mH @ A).sum(0)
    eye = torch.eye(n, dtype=CDT, device=H.device)
    L = (torch.einsum('kac,kbd->abcd', A, Lam.conj()) + torch.einsum('kac,kdb->abcd', Lam, A)
         - torch.einsum('ac,bd->abcd', P, eye) - torch.einsum('ac,db->abcd', eye, Q)
         - 1j * torch.einsum('ac,bd->abcd', torch.diag(E.to(CDT)), eye)
         + 1j * torch.einsum('ac,bd->abcd', eye, torch.diag(E.to(CDT))))
    L = L.reshape(n * n, n * n)
    x = (Vc.mH @ m['rho0'] @ Vc).reshape(-1, n * n).T
    Ee = Vc.mH @ m['E'] @ Vc
    Et = Ee.transpose(-2, -1).reshape(-1, n * n)
    out = []
    for s_ in range(n_steps):
        k1 = L @ x
        k2 = L @ (x + 0.025 * k1)
        k3 = L @ (x + 0.025 * k2)
        k4 = L @ (x + 0.05 * k3)
        x = x + (k1 + 2 * k2 + 2 * k3 + k4) / 6. * 0.05
        if (s_ + 1) % obs_every == 0:
            out.append((Et @ x).T)
    obs = torch.stack(out, 1)
    return (obs.real * weights).sum()


def _grads(fn, params):
    ps = [p.clone().requires_grad_(True) for p in params]
    loss = fn(*ps)
    loss.backward()
    return loss.item(), [p.grad.clone() for p in ps]


def test_redfield_gradients_vs_torch_autograd_and_finite_differences():
    n, steps, obs_every, ckpt = 5, 40, 2, 16
    m = _model(n, 11)
    weights = torch.tensor(m['rng'].normal(size=(2, steps // obs_every, n)), device='cuda')
    params = [m['eps'], m['J'], m['s'], m['lam']]
    l_lib, g_lib = _grads(lambda *p: _loss_lib(m, *p, weights, steps, obs_every, ckpt), params)
    l_ref, g_ref = _grads(lambda *p: _loss_torch(m, *p, weights, steps, obs_every), params)
    assert abs(l_lib - l_ref) < 1e-12 * max(1.0, abs(l_ref))
    for a, b in zip(g_lib, g_ref):
        assert (a - b).abs().max().item() <= 1e-9 * max(b.abs().max().item(), 1e-300)
    # central finite differences of the library's FP64 forward
    h = 1e-6
    for pi, p in enumerate(params):
        flat = p.reshape(-1)
        for j in range(flat.numel()):
            def shifted(delta):
                q = [x.clone() for x in params]
                q[pi].reshape(-1)[j] += delta
                with torch.no_grad():
                    return _loss_lib(m, *q, weights, steps, obs_every, ckpt).item()
            fd = (shifted(h) - shifted(-h)) / (2 * h)
            g = g_lib[pi].reshape(-1)[j].item()
            assert abs(fd - g) <= 1e-5 * max(abs(g), 1e-3 * max(x.abs().max().item() for x in g_lib)), (pi, j, fd, g)


# The tensor-core backward's own outputs (the generator gradient G, the
# gradient of the initial states and of the eigenbasis observables) agree
# with the FP64 backward to ~1e-7 of their largest element
# (test_redfield_split_adjoint_raw_outputs).  The parameter gradients are
# that G contracted with dL/dtheta through the assembly, the spectral factors
# and the eigenvector derivative of eigh(H) (terms in 1 / (E_a - E_b)),
# sums of both signs that are much smaller than their terms: the ~1e-7
# relative error of G reaches them amplified, measured 1.1e-5 relative on the
# 6-site chain.  Bar for the split path's parameter gradients: 3e-5.
SPLIT_PARAM_TOL = 3e-5


def test_redfield_split_adjoint_raw_outputs():
    """G, dl/drho0 and dl/dE of the tensor-core backward against the FP64
    backward, over 1, 3, 20 and 60 steps (one and two checkpoint segments)."""
    from lime_gb300.redfield import redfield_tensor
    from lime_gb300.redfield_grad import _Propagate
    n = 6
    rw = chains.redfield_chain(n=n, n_rhs=2, cfg=5)
    R, evecs = redfield_tensor(rw['H'], rw['a_ops'], rw['spectra'])
    V = torch.as_tensor(evecs, dtype=CDT, device='cuda')
    r0 = V.mH @ torch.as_tensor(rw['rho0'], dtype=CDT, device='cuda') @ V
    E = torch.stack([V.mH @ torch.as_tensor(e, device='cuda') @ V for e in chains.population_ops(n)])
    for steps, ck in ((1, 1), (3, 3), (20, 10), (60, 30)):
        out = {}
        for prec in ('fp64', 'split'):
            leaves = [x.clone().requires_grad_(True) for x in (R.R, r0, E)]
            obs = _Propagate.apply(*leaves, 0.05, steps, 1, ck, prec, 0)
            g = torch.tensor(np.random.default_rng(1).normal(size=tuple(obs.shape)), device='cuda').to(CDT)
            (obs.conj() * g).real.sum().backward()
            out[prec] = [x.grad for x in leaves]
        for a, b in zip(out['split'], out['fp64']):
            assert ((a - b).abs().max() / b.abs().max()).item() < 1e-6, steps


def test_redfield_gradients_split():
    """The tensor-core forward and backward against the FP64 gradients
    (SPLIT_PARAM_TOL relative)."""
    n, steps, obs_every, ckpt = 6, 60, 3, 30
    m = _model(n, 12)
    weights = torch.tensor(m['rng'].normal(size=(2, steps // obs_every, n)), device='cuda')
    params = [m['eps'], m['J'], m['s'], m['lam']]
    _, g64 = _grads(lambda *p: _loss_lib(m, *p, weights, steps, obs_every, ckpt), params)
    _, gsp = _grads(lambda *p: _loss_lib(m, *p, weights, steps, obs_every, ckpt, 'split'), params)
    for a, b in zip(gsp, g64):
        assert (a - b).abs().max().item() <= SPLIT_PARAM_TOL * max(b.abs().max().item(), 1e-300)


def test_redfield_split_adjoint_larger_block():
    """The tensor-core backward on a 12-site chain (Liouville dimension 144,
    padded to 256) with 70 right-hand sides (two column tiles) and uneven
    segments, against the FP64 backward."""
    n, steps, obs_every, ckpt = 12, 50, 1, 20
    m = _model(n, 13)
    rng = m['rng']
    psi = rng.normal(size=(70, n)) + 1j * rng.normal(size=(70, n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    m['rho0'] = torch.as_tensor(np.einsum('bi,bj->bij', psi, psi.conj()), device='cuda')
    weights = torch.tensor(rng.normal(size=(70, steps // obs_every, n)), device='cuda')
    params = [m['eps'], m['J'], m['s'], m['lam']]
    _, g64 = _grads(lambda *p: _loss_lib(m, *p, weights, steps, obs_every, ckpt), params)
    _, gsp = _grads(lambda *p: _loss_lib(m, *p, weights, steps, obs_every, ckpt, 'split'), params)
    for a, b in zip(gsp, g64):
        assert (a - b).abs().max().item() <= SPLIT_PARAM_TOL * max(b.abs().max().item(), 1e-300)


def test_redfield_split_kept_stage_inputs_give_the_same_gradients():
    """Stage inputs kept from the forward pass (no recomputation) against
    recomputed ones: bitwise the same gradients, with every segment kept and
    with only the last one kept."""
    n, steps, obs_every, ckpt = 7, 45, 1, 20
    m = _model(n, 14)
    weights = torch.tensor(m['rng'].normal(size=(2, steps // obs_every, n)), device='cuda')
    params = [m['eps'], m['J'], m['s'], m['lam']]

    def grads(keep):
        from lime_gb300.redfield_grad import redfield_observables, ohmic_spectrum
        ps = [p.clone().requires_grad_(True) for p in params]
        H, a_ops = _inputs(m, *ps)
        obs = redfield_observables(H, a_ops, ohmic_spectrum(ps[3], 0.1, 0.025), m['rho0'], m['E'], 0.05, steps,
                                   obs_every=obs_every, checkpoint=ckpt, precision='split', keep_stages=keep)
        (obs.real * weights).sum().backward()
        return [p.grad for p in ps]

    from lime_gb300.redfield import stage_buffer_floats
    g0 = grads(0)
    last = stage_buffer_floats(n, 2, steps - 2 * ckpt) * 4
    for keep in ('auto', last):
        for a, b in zip(grads(keep), g0):
            assert torch.equal(a, b)
