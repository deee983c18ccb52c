"""Throughput benchmark of the lime_gb300 density-matrix propagator.

Workload: the static-disorder ensemble — 4096 realisations of a 64-site
Frenkel exciton chain (site energies ~ N(0, 0.05), J = -0.1, open ends),
pure dephasing gamma_b ~ U(0.005, 0.02), rho0 = |0><0|, dt = 0.05, site
populations recorded.  A bench "step" is one RK4 time step of the whole
ensemble; ``--steps K`` RK4 steps are timed (the full workload is 4000).

Metric: instance-steps/s (one RK4 step of one density matrix).

Arms:
  (default)          lime_gb300 CUDA path (``--path split`` once available,
                     else the plain FP64 kernel); also reports the plain FP64
                     GPU rate, the roofline of the dominant kernel, an
                     end-to-end number through the public API with host
                     buffers, and the CPU oracle baseline.
  --impl reference   the reference algorithm on the host cores (the NumPy
                     restatement in oracle/, one process per core).

Multi-GPU: instances are independent, so N ranks run disjoint slices of the
ensemble (weak scaling, no collective); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'batched rho RK4 instance-steps/s'
N_SITES = 64
BATCH = 4096
DT = 0.05
FULL_STEPS = 4000
CPU_SAMPLE_STEPS = 150   # ~10 s of oracle work per host core


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=None)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='lime', choices=['lime', 'reference'])
    p.add_argument('--path', default='auto', choices=['auto', 'fp64', 'split'])
    p.add_argument('--batch', type=int, default=BATCH)
    p.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--no-adjoint', action='store_true')
    p.add_argument('--no-redfield', action='store_true')
    p.add_argument('--no-ragged', action='store_true')
    p.add_argument('--no-rows', action='store_true', help='skip the small other-workload leg')
    p.add_argument('--rows-only', action='store_true',
                   help='run only the single-chain / driven / two-time leg and print its JSON')
    p.add_argument('--redfield-only', action='store_true',
                   help='run only the dense Redfield leg and print its JSON')
    p.add_argument('--ragged-only', action='store_true',
                   help='run only the uneven-batch leg and print its JSON')
    p.add_argument('--adjoint-only', action='store_true',
                   help='run only the adjoint/forward leg and print its JSON')
    p.add_argument('--errors-only', action='store_true',
                   help='run only the full-horizon split-vs-FP64 error leg and print its JSON')
    p.add_argument('--no-errors', action='store_true')
    p.add_argument('--redfield-adjoint-only', action='store_true',
                   help='run only the Redfield adjoint/forward leg and print its JSON')
    p.add_argument('--no-redfield-adjoint', action='store_true')
    p.add_argument('--redfield-adjoint-steps', type=int, default=128)
    p.add_argument('--redfield-adjoint-checkpoint', type=int, default=64)
    p.add_argument('--adjoint-batch', type=int, default=256)
    p.add_argument('--ragged-batch', type=int, default=1024)
    p.add_argument('--ragged-sizes', default='8,16,32,64,128,256',
                   help='comma-separated chain sizes of the uneven batch')
    p.add_argument('--redfield-n', type=int, default=96)
    p.add_argument('--redfield-rhs', type=int, default=512)
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in open(self.path):
            f = [x.strip() for x in line.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), samples=len(sm))
        out['reasons'] = sorted(reasons)
        return out


def flush_l2(torch, dev):
    buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    buf.fill_(1)
    del buf


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f)
    except Exception:
        return {}


# ------------------------------------------------------------------ workload
def make_workload(batch, rank=0, world=1):
    import numpy as np
    from lime_gb300 import chains
    from lime_gb300.replicas import shard_range
    w = chains.disorder_ensemble(n=N_SITES, batch=BATCH if batch is None else batch, n_steps=FULL_STEPS)
    lo, hi = shard_range(len(w['H']), rank, world)
    H = w['H'][lo:hi]
    # collapse operators sqrt(gamma_b)|k><k| for every site k: one rate per
    # realisation, broadcast to the sites (the generator's compact form)
    g = np.repeat(w['gamma'][lo:hi, None], N_SITES, axis=1)
    return dict(H=H, rho0=w['rho0'], gamma=g)


def gpu_arm(args, rank, world, local):
    import numpy as np
    import torch
    from lime_gb300 import _native as nat
    from lime_gb300 import build as lbuild
    from lime_gb300 import chains, engine
    from lime_gb300.engine import Populations, SiteDephasing

    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=dev)
    lbuild.build()
    nat.require_device()

    if args.adjoint_only:
        if rank == 0:
            print(json.dumps(adjoint_leg(torch, dev, batch=args.adjoint_batch)))
        return
    if args.errors_only:
        if rank == 0:
            print(json.dumps(full_horizon_leg(torch, dev)))
        return
    if args.redfield_adjoint_only:
        if rank == 0:
            print(json.dumps(redfield_adjoint_leg(torch, dev, steps=args.redfield_adjoint_steps,
                                                  checkpoint=args.redfield_adjoint_checkpoint)))
        return
    if args.ragged_only:
        if rank == 0:
            print(json.dumps(ragged_leg(torch, dev, batch=args.ragged_batch,
                                        sizes=tuple(int(x) for x in args.ragged_sizes.split(',')))))
        return
    if args.rows_only:
        if rank == 0:
            print(json.dumps(rows_leg(torch, dev)))
        return
    if args.redfield_only:
        if rank == 0:
            print(json.dumps(redfield_leg(torch, dev, measured_peaks(), n=args.redfield_n,
                                          n_rhs=args.redfield_rhs)))
        return

    path = 'split' if args.path in ('auto', 'split') else 'fp64'
    K = args.steps if args.steps is not None else (FULL_STEPS if path == 'split' else 8)
    W = max(3, args.warmup)
    wl = make_workload(args.batch, rank, world)
    B = wl['H'].shape[0]
    pop_ops = Populations(N_SITES)

    gen = engine.LindbladGenerator.build(wl['H'], [SiteDephasing(wl['gamma'])], device=dev)
    rho0 = torch.as_tensor(np.broadcast_to(wl['rho0'], (B, N_SITES, N_SITES)).copy(),
                           dtype=torch.complex128, device=dev)
    obs_every = max(1, K // 100)

    def run(nsteps, events=None):
        return engine.propagate(gen, rho0, DT, nsteps, pop_ops, precision=path,
                                obs_every=max(1, min(obs_every, nsteps)), events=events)

    run(W)
    torch.cuda.synchronize()
    flush_l2(torch, dev)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    n0 = nat.launch_count()
    with ClockSampler(local) as clk:
        ev0.record()
        obs, _, _ = run(K, events=kev)
        ev1.record()
        torch.cuda.synchronize()
    launches = nat.launch_count() - n0
    t = ev0.elapsed_time(ev1) / 1e3
    tk = kev[0].elapsed_time(kev[1]) / 1e3
    if world > 1:
        from lime_gb300.replicas import max_over_ranks
        t = max_over_ranks(t, device=dev)
    total_instances = B * world
    value = total_instances * K / t
    clocks = clk.summary()

    # plain FP64 GPU rate on the same ensemble (the metric's denominator) and
    # the split path's error against it over the full K-step horizon
    fp64 = None
    if path == 'fp64':
        fp64 = {'value': value}
    elif rank == 0:
        fp64 = fp64_leg(gen, rho0, pop_ops, K, obs_every, obs, torch, engine)
    e2e = None
    if not args.no_e2e:
        # every rank runs its shard through the public API; whole-job rate
        # from the slowest rank
        if world > 1:
            torch.distributed.barrier()
        e2e = e2e_leg(wl, K, path, dev)
        if world > 1:
            from lime_gb300.replicas import max_over_ranks
            t_max = max_over_ranks(e2e.pop('wall_s'), device=dev)
            e2e['value'] = B * world * K / t_max
        else:
            e2e.pop('wall_s')
    # single-GPU legs (other workloads of the path), at N = 1 only
    single = world == 1
    adj = None
    if not args.no_adjoint and single:
        adj = adjoint_leg(torch, dev, batch=args.adjoint_batch)
    red = None
    if not args.no_redfield and single:
        red = redfield_leg(torch, dev, measured_peaks(), n=args.redfield_n, n_rhs=args.redfield_rhs)
    rag = None
    if not args.no_ragged and single:
        rag = ragged_leg(torch, dev, batch=args.ragged_batch,
                         sizes=tuple(int(x) for x in args.ragged_sizes.split(',')))
    rows = None
    if not args.no_rows and single:
        rows = rows_leg(torch, dev)
    errors = None
    if not args.no_errors and single:
        errors = full_horizon_leg(torch, dev)
    radj = None
    if not args.no_redfield_adjoint and single:
        radj = redfield_adjoint_leg(torch, dev, steps=args.redfield_adjoint_steps,
                                    checkpoint=args.redfield_adjoint_checkpoint)
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        from oracle import pool
        rate, cores, wall = pool.ensemble_rate(n=N_SITES, n_steps=CPU_SAMPLE_STEPS)
        cpu = {'value': rate, 'unit': 'instance-steps/s', 'cores': cores, 'kind': 'port',
               'sample': '%d realisations x %d RK4 steps, one process per core (%.1f s)'
                         % (cores, CPU_SAMPLE_STEPS, wall)}

    # roofline of the dominant kernel
    peaks = measured_peaks()
    flop_per_inst_step = 64 * N_SITES ** 3   # 2 complex N^3 GEMMs per RHS, 4 RHS
    achieved_tf = B * K * flop_per_inst_step / tk / 1e12
    if path == 'fp64':
        pk64 = fp64_gemm_tflops(torch, dev)
        roof = {'bound': 'fp64', 'achieved': achieved_tf, 'peak': pk64, 'unit': 'TFLOP/s',
                'frac': achieved_tf / pk64, 'traffic': None,
                'peak_source': 'cuBLAS DGEMM 4096^3 measured in this run, of measured'}
    else:
        pk = peaks.get('bf16_tflops_sustained') or 1700.0
        # issued tensor work: per stage 5 fp16 products of the 128x64x128 real block
        issued = 4 * 5 * 2 * 128 * 64 * 128
        # DRAM traffic per launch: 185.5 KB per instance (ncu capture of 304
        # instances x 400 steps: 50.5 MB read + 5.9 MB written: the prepared A
        # pieces and rho in, rho out), scaled by the instances one full-size
        # launch processes; it does not grow with steps
        traffic = 185.5e3 * B
        roof = {'bound': 'tensor', 'achieved': achieved_tf, 'peak': pk, 'unit': 'TFLOP/s',
                'frac': achieved_tf / pk, 'traffic': traffic,
                'traffic_source': 'ncu dram__bytes_read+write of a 304-instance launch, '
                                  'scaled by instances (per-instance, not per-step, traffic)',
                'peak_source': ('measured bf16 dense sustained (fp16 runs at the same rate), '
                                'of measured') if peaks else 'fallback 1.7 PFLOP/s',
                'algorithmic_flop_per_instance_step': flop_per_inst_step,
                'issued_tensor_flop_per_instance_step': issued,
                'issued_tflops': B * K * issued / tk / 1e12}

    line = {
        'metric': METRIC, 'value': value, 'unit': 'instance-steps/s', 'n_gpus': world,
        'steps': K, 'warmup': W, 'ms_per_step': t / K * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64' if path == 'fp64' else 'f32 (split 16-bit tensor operands)',
        'data': 'synthetic (seeded disorder ensemble)',
        'config': {'workload': 'dephasing exciton-chain ensemble N=64, 4096 realisations, '
                               'dt=0.05 (4000-step workload; K steps timed)',
                   'n_sites': N_SITES, 'batch': total_instances, 'path': path,
                   'l2': 'flushed before the timed launch; rho stays on chip across steps',
                   'observables': 'site populations every %d steps' % obs_every},
        'kernel_s': tk,
        'fp64_gpu': fp64,
        'speedup_vs_fp64_gpu': (value / fp64['value']) if fp64 and fp64.get('value') else None,
        'gpu_launches': launches,
        'clocks': clocks,
        'roofline': roof,
        'e2e': e2e,
        'adjoint': adj,
        'redfield': red,
        'uneven_batch': rag,
        'other_workloads': rows,
        'full_horizon_errors': errors,
        'redfield_adjoint': radj,
        'cpu_baseline': cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def fp64_leg(gen, rho0, pop_ops, K, obs_every, obs_split, torch, engine, k64=4, n_err=152):
    """Plain FP64 GPU rate on the full ensemble (k64 steps) and the split
    path's max population error against FP64 on the first n_err realisations
    over the full K-step horizon."""
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    engine.propagate(gen, rho0, DT, 1, pop_ops)
    torch.cuda.synchronize()
    engine.propagate(gen, rho0, DT, k64, pop_ops, events=ev)
    torch.cuda.synchronize()
    t = ev[0].elapsed_time(ev[1]) / 1e3
    rate = rho0.shape[0] * k64 / t
    sub = engine.LindbladGenerator(n=gen.n, P=n_err, heff=gen.heff[:n_err].contiguous(),
                                   m=None if gen.m is None else gen.m[:n_err].contiguous(),
                                   l_dense=None, k_dense=0, shared=False)
    o64, _, _ = engine.propagate(sub, rho0[:n_err], DT, K, pop_ops, obs_every=max(1, min(obs_every, K)))
    err = (obs_split[:n_err] - o64).abs().max().item()
    # the FP64 kernel's roofline: the algorithmic 64 N^3 flop per instance-step
    # against the measured FP64 peak (the kernel performs half of them: one
    # GEMM per stage through the Hermitian shortcut)
    pk64 = fp64_gemm_tflops(torch, rho0.device)
    alg = rate * 64 * gen.n ** 3 / 1e12
    return {'value': rate, 'unit': 'instance-steps/s',
            'sample': 'full ensemble, %d RK4 steps' % k64,
            'roofline': {'bound': 'fp64', 'achieved_algorithmic': alg, 'achieved_performed': alg / 2,
                         'peak': pk64, 'frac_performed': alg / 2 / pk64, 'unit': 'TFLOP/s',
                         'peak_source': 'cuBLAS DGEMM 4096^3 measured in this run, of measured'},
            'split_max_population_error': err,
            'error_sample': 'first %d realisations, all %d steps, every %d-th step recorded'
                            % (n_err, K, max(1, min(obs_every, K)))}


def adjoint_leg(torch, dev, n_sites=128, batch=256, steps=4096, checkpoint=64, sample=64, dt=0.05):
    """Adjoint/forward cost on the differentiated absorption workload:
    129-dim chains (|g> + 128 sites), 256 disorder samples, dipole
    correlation <mu(t) mu(0)>, gradients w.r.t. every site energy, the bond
    couplings and the dephasing rates, checkpoint every 64 steps.  The
    tensor-core path runs the full 4096-step horizon; the FP64 path (about
    85 ms a step at this size) a ``sample``-step window with the same
    checkpoint interval, on which the tensor-core gradients are also compared
    with the FP64 ones."""
    from lime_gb300 import chains
    from lime_gb300.adjoint import chain_observables
    w = chains.absorption_ensemble(n_sites=n_sites, batch=batch, n_steps=steps, dt=dt)
    N = n_sites + 1
    H0 = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    eps = torch.tensor(w['eps'], device=dev)
    bond = torch.full((batch, n_sites - 1), w['J'], dtype=torch.float64, device=dev)
    gamma = torch.full((batch, n_sites), w['gamma'], dtype=torch.float64, device=dev)
    mu = torch.as_tensor(w['mu'], device=dev)
    rho0 = mu @ torch.as_tensor(w['rho_g'], device=dev)
    E = [mu]

    def fwd(req, precision, n):
        e = eps.clone().requires_grad_(req)
        b = bond.clone().requires_grad_(req)
        g = gamma.clone().requires_grad_(req)
        return (e, b, g), chain_observables(H0, e, b, g, rho0, E, dt, n, site0=1,
                                            checkpoint=checkpoint, precision=precision)

    def timed(precision, n):
        fwd(False, precision, min(n, checkpoint))   # warm
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        params, obs = fwd(True, precision, n)
        ev[1].record()
        loss = obs.real.sum()   # a linear functional of C(t), as a spectrum is
        loss.backward()
        ev[2].record()
        torch.cuda.synchronize()
        tf = ev[0].elapsed_time(ev[1]) / 1e3
        tb = ev[1].elapsed_time(ev[2]) / 1e3
        return [p.grad for p in params], {'steps': n, 'checkpoint': checkpoint, 'forward_s': tf,
                                          'adjoint_s': tb, 'adjoint_over_forward': tb / tf}

    out = {'workload': 'absorption chain dim %d, %d samples, dipole correlation over %d steps, grads '
                       'w.r.t. %d site energies + %d bonds + %d dephasing rates, checkpoint every %d steps'
                       % (N, batch, steps, n_sites, n_sites - 1, n_sites, checkpoint)}
    g64, out['fp64'] = timed('fp64', sample)
    gsp_s, out['split_sample'] = timed('split', sample)
    _, out['split'] = timed('split', steps)
    out['split_grad_rel_error'] = max(
        float((a - b).abs().max().item() / max(b.abs().max().item(), 1e-300)) for a, b in zip(gsp_s, g64))
    out['split_grad_error_sample'] = '%d-step window, same checkpoint interval' % sample
    out['split_adjoint_speedup_vs_fp64'] = out['fp64']['adjoint_s'] / out['split_sample']['adjoint_s']
    out['adjoint_over_forward'] = out['split']['adjoint_over_forward']
    out['path'] = 'split, full horizon (FP64 on the sample window)'
    return out


def redfield_adjoint_leg(torch, dev, n=96, n_rhs=512, steps=128, checkpoint=64, dt=0.05):
    """Adjoint/forward cost of the differentiable Redfield workload at the
    dense superoperator's size (N = 96, Liouville dimension 9216, 512
    right-hand sides): gradients of all 96 populations' weighted sum with
    respect to the 96 site energies, the coupling J, 96 bath coupling
    strengths and the Ohmic reorganisation energy, on the tensor cores
    (split forward and backward), checkpoint every 64 steps, over a
    ``steps``-step sample of the 2000-step workload (the cost per step does
    not depend on the horizon)."""
    import numpy as np
    from lime_gb300 import chains
    from lime_gb300.redfield_grad import redfield_observables, ohmic_spectrum
    w = chains.redfield_chain(n=n, n_rhs=n_rhs, cfg=5)
    eps0 = torch.tensor(np.real(np.diag(w['H'])).copy(), device=dev)
    off = torch.diag(torch.ones(n - 1, dtype=torch.float64, device=dev), 1)
    proj = torch.eye(n, dtype=torch.float64, device=dev)
    rho0 = torch.as_tensor(w['rho0'], device=dev)
    E = torch.as_tensor(np.stack(chains.population_ops(n)), device=dev)
    wts = torch.tensor(np.random.default_rng(5).normal(size=(n_rhs, steps, n)), device=dev)

    def run(grad, keep=0):
        eps = eps0.clone().requires_grad_(grad)
        J = torch.tensor(-0.1, dtype=torch.float64, device=dev, requires_grad=grad)
        s = torch.ones(n, dtype=torch.float64, device=dev, requires_grad=grad)
        lam = torch.tensor(0.05, dtype=torch.float64, device=dev, requires_grad=grad)
        H = torch.diag(eps) + J * (off + off.T)
        a_ops = s[:, None, None] * torch.diag_embed(proj)
        obs = redfield_observables(H, a_ops, ohmic_spectrum(lam, 0.1, 0.025), rho0, E, dt, steps,
                                   checkpoint=checkpoint, precision='split', keep_stages=keep)
        return (obs.real * wts).sum(), (eps, J, s, lam)

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b) / 1e3

    with torch.no_grad():
        run(False)                      # warm
        _, tf = timed(lambda: run(False))
    def grad_run(keep):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        ev[0].record()
        loss, params = run(True, keep)
        ev[1].record()
        loss.backward()
        ev[2].record()
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / 1e3, ev[1].elapsed_time(ev[2]) / 1e3, params

    tfg, tb, params = grad_run(0)
    free = torch.cuda.mem_get_info(dev)[0] // 2
    tfk, tbk, pk = grad_run(free)
    same = all(torch.equal(a.grad, b.grad) for a, b in zip(params, pk))
    from lime_gb300.redfield import stage_buffer_floats
    seg_gb = stage_buffer_floats(n, n_rhs, checkpoint) * 4 / 1e9
    return {'workload': 'Redfield N=%d (Liouville dim %d), %d right-hand sides, weighted populations; grads '
                        'w.r.t. %d site energies, J, %d bath coupling strengths and the reorganisation energy; '
                        'checkpoint every %d steps; %d-step sample of the 2000-step workload'
                        % (n, n * n, n_rhs, n, n, checkpoint, steps),
            'path': 'split forward and backward (lime_redfield_rk4_split, lime_redfield_adjoint_split)',
            'forward_s': tf, 'forward_with_checkpoints_s': tfg, 'adjoint_s': tb,
            'adjoint_over_forward': tb / tf,
            'kept': {'keep_bytes': int(free), 'segment_gb': seg_gb,
                     'segments_kept': int(min(-(-steps // checkpoint), free // max(1, int(seg_gb * 1e9)))),
                     'forward_keeping_s': tfk, 'adjoint_s': tbk, 'adjoint_over_forward': tbk / tf,
                     'gradients_bitwise_equal_to_recompute': bool(same)},
            'grad_norms': [float(p.grad.abs().max().item()) for p in params]}


def redfield_leg(torch, dev, peaks, n=96, n_rhs=512, dt=0.05, k_split=(4, 12), k64=3):
    """Dense Redfield workload: Liouville dim 9216, 512 initial density
    matrices as one right-hand-side block (2000-step workload; a sample of
    steps is timed).  Tensor-core split path vs the plain FP64 GPU path:
    per-step time from the difference of two split runs (removes the
    one-off operand conversion), FP64 from k64 steps, and the split error on
    populations and final states over those k64 steps."""
    from lime_gb300 import chains
    from lime_gb300.redfield import redfield_tensor, propagate_vec, propagate_vec_split
    w = chains.redfield_chain(n=n, n_rhs=n_rhs, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'], device=dev)
    V = torch.as_tensor(evecs, dtype=torch.complex128, device=dev)
    r0 = V.mH @ torch.as_tensor(w['rho0'], dtype=torch.complex128, device=dev) @ V
    e_eb = [V.mH @ torch.as_tensor(e, dtype=torch.complex128, device=dev) @ V
            for e in chains.population_ops(n)]
    Rg = (R.R, n)

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b) / 1e3

    from lime_gb300 import redfield as rfm
    per_step = {}
    for prod in ('4m', '3m'):
        propagate_vec_split(Rg, r0, dt, 1, e_eb, product=prod)
        _, t1 = timed(lambda: propagate_vec_split(Rg, r0, dt, k_split[0], e_eb, product=prod))
        _, t2 = timed(lambda: propagate_vec_split(Rg, r0, dt, k_split[1], e_eb, product=prod))
        per_step[prod] = (t2 - t1) / (k_split[1] - k_split[0])
    (o64, _, r64), t64 = timed(lambda: propagate_vec(Rg, r0, dt, k64, e_eb))
    errs = {}
    for prod in ('4m', '3m'):
        (osp, _, rsp), _ = timed(lambda: propagate_vec_split(Rg, r0, dt, k64, e_eb, product=prod))
        errs[prod] = ((osp - o64).abs().max().item(), (rsp - r64).abs().max().item())
    D = n * n
    stage_flop = 8.0 * D * D * n_rhs          # one complex D x D x R GEMM
    # issued tensor flops per stage: five fp16 products per real product;
    # the block form multiplies 4 real D x D x R products, the 3M form 3
    issued = {'4m': 5 * stage_flop, '3m': 5 * 0.75 * stage_flop}
    pk = peaks.get('bf16_tflops_sustained') or 1700.0
    prod = rfm.SPLIT_PRODUCT
    if prod == 'auto':
        prod = rfm.split_product(n, n_rhs, dev)
    split_rate = n_rhs / per_step[prod]
    fp64_rate = n_rhs * k64 / t64

    def entry(p):
        return {'value': n_rhs / per_step[p], 'ms_per_step': per_step[p] * 1e3,
                'sample': 'difference of %d- and %d-step runs' % k_split,
                'max_population_error': errs[p][0], 'max_state_error': errs[p][1],
                'achieved_algorithmic_tflops': 4 * stage_flop / per_step[p] / 1e12,
                'achieved_issued_tflops': 4 * issued[p] / per_step[p] / 1e12}

    return {'workload': 'Redfield dense superoperator, spin-boson-like exciton chain N=%d '
                        '(Liouville dim %d), Ohmic bath, %d initial density matrices as one '
                        'right-hand-side block' % (n, D, n_rhs),
            'unit': 'instance-steps/s',
            'split': dict(entry(prod), product=prod),
            'split_4m': entry('4m'), 'split_3m': entry('3m'),
            'fp64_gpu': {'value': fp64_rate, 'ms_per_step': t64 / k64 * 1e3,
                         'sample': '%d RK4 steps' % k64},
            'speedup_vs_fp64_gpu': split_rate / fp64_rate,
            'split_max_population_error': errs[prod][0],
            'split_max_state_error': errs[prod][1],
            'error_sample': 'all %d right-hand sides, %d steps (full horizon: full_horizon_errors)'
                            % (n_rhs, k64),
            'roofline': {'bound': 'tensor', 'unit': 'TFLOP/s',
                         'achieved_algorithmic': 4 * stage_flop / per_step[prod] / 1e12,
                         'achieved_issued': 4 * issued[prod] / per_step[prod] / 1e12,
                         'peak': pk, 'frac_issued': 4 * issued[prod] / per_step[prod] / 1e12 / pk,
                         'note': 'per-step time includes the stage launches and one observable '
                                 'launch'}}


def ragged_leg(torch, dev, batch=1024, sizes=(8, 16, 32, 64, 128, 256), steps_split=40, steps_fp64=2,
               err_steps=200):
    """Uneven batch: 1024 chains with N uniform over {8..256}, three dense
    complex collapse operators each (2000-step workload; samples of steps
    are timed).  The schedule of the split path (one grouped persistent
    launch per GEMM phase for all sizes, or one launch sequence per size on
    concurrent streams; tile order; block-diagonal packing of N <= 32) is
    picked first by the autotuner (``engine.autotune_ragged``, outside the
    timed region); the groups are prepared once; CUDA events on the main
    stream time the GPU work of a whole call (all sizes), and the split
    per-step time is the difference of a 20- and a 40-step call (the
    per-call operand conversion cancels).  The split error on populations
    is taken over err_steps steps on two chains of every N <= 128 through
    the public call."""
    import numpy as np
    from lime_gb300 import chains, engine, tuning
    w = chains.uneven_batch(batch=batch, sizes=sizes, n_steps=steps_split)
    ns = w['ns']
    E = [[chains.population_ops(int(n))[0]] for n in ns]
    main = torch.cuda.current_stream(dev)
    cache = tuning.TuneCache(os.path.join(tempfile.gettempdir(), 'lime_gb300_tune_bench.json'))
    choice, times = engine.autotune_ragged(w['H'], w['rho0'], w['dt'], w['c_ops'], E, precision='split',
                                           device=dev, cache=cache, force=True)
    prepared = {
        'split': engine.ragged_groups(w['H'], w['rho0'], w['c_ops'], E, 'split', dev, pack=choice['pack']),
        'fp64': engine.ragged_groups(w['H'], w['rho0'], w['c_ops'], E, 'fp64', dev),
    }
    sched = {'split': choice, 'fp64': {'mode': 'streams'}}

    def run(steps, precision):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(main)
        fins = engine.ragged_enqueue(prepared[precision], w['dt'], steps, precision, sched[precision],
                                     device=dev)
        b.record(main)
        torch.cuda.synchronize()
        for fin in fins:
            fin(True)
        return a.elapsed_time(b) / 1e3

    run(1, 'split')   # warm
    run(1, 'fp64')
    t1 = min(run(steps_split // 2, 'split') for _ in range(2))
    t2 = min(run(steps_split, 'split') for _ in range(2))
    tf = run(steps_fp64, 'fp64')
    per_step = (t2 - t1) / (steps_split - steps_split // 2)
    small = [s for s in sorted(set(int(n) for n in ns)) if s <= 128] or [int(min(ns))]
    # a full block-diagonal pack plus one more chain for the packed sizes
    sub = [int(i) for s in small
           for i in np.flatnonzero(ns == s)[:(engine.PACK_DIM // s + 1 if 2 * s <= engine.PACK_DIM else 2)]]
    args = ([w['H'][i] for i in sub], [w['rho0'][i] for i in sub], w['dt'], err_steps,
            [w['c_ops'][i] for i in sub], [E[i] for i in sub])
    o64, _, _ = engine.propagate_ragged(*args, precision='fp64')
    osp, _, _ = engine.propagate_ragged(*args, precision='split', schedule=choice)
    err = max(float((x - y).abs().max().item()) for x, y in zip(osp, o64))
    flop = float(sum(256.0 * int(n) ** 3 for n in ns))   # 64 (1 + K) N^3 per instance-step, K = 3
    split_rate = len(ns) / per_step
    fp64_rate = len(ns) * steps_fp64 / tf
    return {'workload': 'uneven batch: %d chains, N uniform over {%s}, tridiagonal + 0.01 GOE, '
                        '3 dense complex collapse operators' % (len(ns), ','.join(str(x) for x in sizes)),
            'unit': 'instance-steps/s',
            'split': {'value': split_rate, 'ms_per_step': per_step * 1e3,
                      'sample': 'difference of %d- and %d-step calls (GPU time, best of 2)'
                                % (steps_split // 2, steps_split),
                      'gpu_s_%d_steps' % steps_split: t2,
                      'algorithmic_tflops': flop / per_step / 1e12,
                      'path': 'streaming tcgen05 GEMMs (Heff rho, L rho L^dag); schedule %s'
                              % json.dumps(choice, sort_keys=True),
                      'schedule': choice,
                      'tuning': {'key': tuning.key('lindblad_uneven',
                                                   engine.uneven_class(w['H'], w['c_ops'], 'split'),
                                                   'split', tuning.arch_tag(dev)),
                                 'ms_per_step': {json.dumps(c, sort_keys=True): (None if t is None else t * 1e3)
                                                 for c, t in zip(engine.UNEVEN_CANDIDATES, times or [])}}},
            'fp64_gpu': {'value': fp64_rate, 'steps': steps_fp64, 'gpu_s': tf},
            'speedup_vs_fp64_gpu': split_rate / fp64_rate,
            'split_max_population_error': err,
            'error_sample': '%d chains (64 // N + 1 of each N <= 32, two of each N <= 128, else of '
                            'the smallest N), %d steps' % (len(sub), err_steps)}


def rows_leg(torch, dev):
    """The other workloads of the path at small sizes, FP64 and split
    precision side by side (GPU time with CUDA events around each public
    call, set-up included; split error against the FP64 path):
    the single 16-site chain (2000 steps, 16 populations every step), the
    driven Lindblad equation (64-site chain, H(t) = H0 - f(t) mu with a
    periodic f, 256 initial states, 1000 steps) and the two-time
    correlation <A(t) B(t+tau) C(t)> (16-site chain, 200 x 200)."""
    import numpy as np
    from lime_gb300 import chains, engine
    from lime_gb300.oqs import Lindblad_solver

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b) / 1e3

    out = {}
    # single chain (latency of one small instance)
    w = chains.single_chain(n=16, n_steps=2000)
    gen = engine.LindbladGenerator.build(w['H'], w['c_ops'], device=dev)
    res = {}
    for prec in ('fp64', 'split', 'fp64', 'split'):   # second pass timed
        (o, _, _), t = timed(lambda: engine.propagate(gen, w['rho0'], w['dt'], w['Nt'], w['e_ops'],
                                                      precision=prec))
        res[prec] = (o, t)
    out['single_chain_n16'] = {
        'steps': w['Nt'], 'fp64_steps_per_s': w['Nt'] / res['fp64'][1],
        'split_steps_per_s': w['Nt'] / res['split'][1],
        'split_max_population_error': float((res['split'][0] - res['fp64'][0]).abs().max())}

    # driven Lindblad: H(t) = H0 - f(t) mu, shared generator, a batch of starts
    n, B, steps, dt = 64, 256, 1000, 0.05
    rng = np.random.default_rng(20261204)
    H0 = chains.exciton_chain(n, rng.normal(0, 0.05, n), -0.1)
    mu = np.zeros((n, n), dtype=np.complex128)
    mu[0, 1:] = mu[1:, 0] = rng.normal(1.0, 0.1, n - 1)
    coef = 0.01 * np.cos(0.1 * dt * np.arange(1, steps + 1))[:, None]
    gen = engine.LindbladGenerator.build(H0, chains.dephasing_ops(n, 0.01), device=dev)
    drive = (torch.as_tensor(mu[None], device=dev), torch.as_tensor(coef, device=dev))
    rho0 = torch.as_tensor(np.stack([chains.ground_dm(n, k % n) for k in range(B)]), device=dev)
    pops = chains.population_ops(n)[:8]
    res = {}
    for prec in ('fp64', 'split'):
        engine.propagate(gen, rho0, dt, 2, pops, drive=(drive[0], drive[1][:2]), precision=prec)
        (o, _, _), t = timed(lambda: engine.propagate(gen, rho0, dt, steps, pops, drive=drive,
                                                      precision=prec))
        res[prec] = (o, t)
    out['driven_n64_b256'] = {
        'steps': steps, 'unit': 'instance-steps/s',
        'fp64': B * steps / res['fp64'][1], 'split': B * steps / res['split'][1],
        'speedup_vs_fp64_gpu': res['fp64'][1] / res['split'][1],
        'split_max_population_error': float((res['split'][0] - res['fp64'][0]).abs().max())}

    # two-time correlation (the Nt inner propagations as one batch)
    w = chains.single_chain(n=16, n_steps=200)
    a = np.zeros((16, 16), dtype=np.complex128)
    a[0, 1:] = a[1:, 0] = 1.0
    res = {}
    for prec in ('fp64', 'split', 'fp64', 'split'):
        sol = Lindblad_solver(w['H'], c_ops=w['c_ops'], precision=prec)
        c, t = timed(lambda: sol.correlation_3op_2t(w['rho0'], [a, a, a], w['dt'], 200, 200))
        res[prec] = (c, t)
    c64, csp = res['fp64'][0], res['split'][0]
    out['two_time_3op_n16'] = {
        'nt': 200, 'ntau': 200, 'fp64_s': res['fp64'][1], 'split_s': res['split'][1],
        'split_rel_error': float(np.max(np.abs(csp - c64)) / np.max(np.abs(c64)))}
    return out


def full_horizon_leg(torch, dev):
    """Split-precision error against FP64 over every configured workload's
    full horizon, on a sample of its instances (the timed legs run shorter
    samples of steps):
      ensemble     32 of the 4096 realisations x 4000 steps, populations every
                   10 steps, vs the library's FP64 kernel
      uneven       one chain of every N in {8..256} (two N = 8 chains packed
                   into one instance), 3 dense collapse operators, 2000
                   steps, 4 populations each, through the public uneven call
      absorption   the dipole correlation of two 129-dimensional chains over
                   4096 steps (relative to max |C|)
      redfield     N = 96 (Liouville dimension 9216), two right-hand sides,
                   all 96 populations every 10 steps, 2000 steps
    The FP64 side of the last three is the PyTorch FP64 RK4 of
    tests/fp64_torch.py (whole-GPU cuBLAS calls; the library's FP64 kernels
    run one CTA per instance and would take minutes on these few large
    instances), which the tests anchor to the library's FP64 kernels at
    1e-12."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, 'tests'))
    import fp64_torch
    from lime_gb300 import chains, engine
    from lime_gb300.engine import Populations, SiteDephasing
    from lime_gb300.redfield import redfield_tensor, propagate_vec_split
    out = {}

    def clock(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    # ensemble (N = 64 dephasing chains)
    w = chains.disorder_ensemble(n=N_SITES, batch=32, n_steps=FULL_STEPS)
    gen = engine.LindbladGenerator.build(w['H'], [SiteDephasing(np.repeat(w['gamma'][:, None], N_SITES, 1))],
                                         device=dev)
    pops = Populations(N_SITES)
    (osp, _, _), tsp = clock(lambda: engine.propagate(gen, w['rho0'], DT, FULL_STEPS, pops,
                                                      precision='split', obs_every=10))
    (o64, _, _), t64 = clock(lambda: engine.propagate(gen, w['rho0'], DT, FULL_STEPS, pops, obs_every=10))
    out['ensemble_n64'] = {'sample': '32 realisations x %d steps, 64 populations every 10 steps' % FULL_STEPS,
                           'max_population_error': (osp - o64).abs().max().item(),
                           'reference': 'library FP64 kernel', 'split_s': tsp, 'fp64_s': t64}

    # uneven batch
    sizes = (8, 8, 16, 32, 64, 128, 256)
    rng = np.random.default_rng(20261203 + 3)
    H, C, R0, E = [], [], [], []
    for n in sizes:
        h, c = chains.uneven_chain(n, rng)
        H.append(h)
        C.append(c)
        R0.append(chains.ground_dm(n))
        E.append(chains.population_ops(n)[:4])
    res, tsp = clock(lambda: engine.propagate_ragged(H, R0, DT, 2000, C, E, precision='split'))
    errs, t64 = {}, 0.0
    for i, n in enumerate(sizes):
        g = engine.LindbladGenerator.build(H[i], C[i], device=dev)
        (o, _), t = clock(lambda: fp64_torch.lindblad_rk4(g, torch.as_tensor(R0[i], device=dev)[None], DT, 2000,
                                                          torch.as_tensor(np.stack(E[i]), device=dev),
                                                          hermitian=True))
        t64 += t
        errs['N%d' % n] = max(errs.get('N%d' % n, 0.0), (res[0][i] - o[0]).abs().max().item())
    out['uneven_batch'] = {'sample': 'chains N = %s, 3 dense collapse operators, 2000 steps, 4 populations each'
                                     % ','.join(str(x) for x in sizes),
                           'max_population_error': max(errs.values()), 'per_size': errs,
                           'reference': 'PyTorch FP64 RK4', 'split_s': tsp, 'fp64_s': t64}

    # absorption shape: dipole correlation, dimension 129
    w = chains.absorption_ensemble(n_sites=128, batch=2, n_steps=4096)
    gen = engine.LindbladGenerator.build(w['H'], [SiteDephasing(np.r_[0.0, np.full(128, w['gamma'])])],
                                         device=dev)
    mu = torch.as_tensor(w['mu'], device=dev)
    rho = mu @ torch.as_tensor(w['rho_g'], device=dev)
    (osp, _, _), tsp = clock(lambda: engine.propagate(gen, rho, w['dt'], 4096, [mu], precision='split'))
    (o64, _), t64 = clock(lambda: fp64_torch.lindblad_rk4(gen, rho, w['dt'], 4096, mu[:, None]))
    out['absorption_dim129'] = {'sample': 'dipole correlation <mu(t) mu(0)> of 2 chains x 4096 steps',
                                'max_correlation_rel_error': ((osp - o64).abs().max() / o64.abs().max()).item(),
                                'reference': 'PyTorch FP64 RK4', 'split_s': tsp, 'fp64_s': t64}

    # dense Redfield superoperator
    w = chains.redfield_chain(n=96, n_rhs=2, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'], device=dev)
    V = torch.as_tensor(evecs, dtype=torch.complex128, device=dev)
    r0 = V.mH @ torch.as_tensor(w['rho0'], dtype=torch.complex128, device=dev) @ V
    Eeb = torch.stack([V.mH @ torch.as_tensor(e, dtype=torch.complex128, device=dev) @ V
                       for e in chains.population_ops(96)])
    (o64, r64), t64 = clock(lambda: fp64_torch.redfield_rk4(R.R, r0, 0.05, 2000, Eeb, obs_every=10))
    for prod in ('4m', '3m'):
        (osp, _, rsp), tsp = clock(lambda: propagate_vec_split((R.R, 96), r0, 0.05, 2000, list(Eeb), obs_every=10,
                                                               product=prod))
        out['redfield_dim9216' + ('' if prod == '4m' else '_3m')] = {
            'sample': '2 right-hand sides x 2000 steps, 96 populations every 10 steps',
            'product': prod,
            'max_population_error': (osp - o64).abs().max().item(),
            'max_state_error': (rsp - r64).abs().max().item(),
            'reference': 'PyTorch FP64 RK4', 'split_s': tsp, 'fp64_s': t64}
    out['bar'] = 'populations <= 1e-6 absolute, correlations <= 1e-6 relative to max |C|'
    return out


def fp64_gemm_tflops(torch, dev, n=4096):
    """Measured FP64 peak of this GPU: cuBLAS DGEMM n^3, best of three
    (CUDA events); the denominator of the FP64 path's roofline."""
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    a @ a
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ a
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        best = t if best is None else min(best, t)
    return 2.0 * n ** 3 / best / 1e12


def e2e_leg(wl, K, path, dev):
    """Same metric through the public API with host (pinned) buffers."""
    import numpy as np
    import torch
    from lime_gb300.oqs import Lindblad_solver, Populations, SiteDephasing
    B = wl['H'].shape[0]
    H = torch.as_tensor(wl['H']).pin_memory()
    g = torch.as_tensor(wl['gamma']).pin_memory()
    rho0 = torch.as_tensor(wl['rho0']).pin_memory()
    pops = Populations(N_SITES)
    nout = max(1, K // 100)
    sol = Lindblad_solver(H, c_ops=[SiteDephasing(g)], precision=path)
    for _ in range(2):   # warm: the same call, so the timed one reuses cached pinned result blocks
        sol.evolve(rho0, dt=DT, Nt=K, e_ops=pops, nout=nout, store_states=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = sol.evolve(rho0, dt=DT, Nt=K, e_ops=pops, nout=nout, store_states=False)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    h2d = H.numel() * 16 + g.numel() * 8 + rho0.numel() * 16
    d2h = res.observables.nbytes + np.asarray(res.rholist).nbytes
    return {'value': B * K / t, 'unit': 'instance-steps/s', 'wall_s': t,
            'h2d_bytes_per_step': h2d / K, 'd2h_bytes_per_step': d2h / K,
            'api': 'lime_gb300.oqs.Lindblad_solver.evolve (pinned host H and dephasing rates '
                   '(SiteDephasing), site populations (Populations), numpy Result out: '
                   'observables and the final states; uploads, launches and copies back '
                   'pipelined over instance ranges)'}


REF_INNER = 8   # RK4 steps per host core in one reference-arm step


def reference_arm(args, rank, world):
    """The reference algorithm on the host cores: the NumPy port of
    ``_lindblad`` (pinned to the reference's own outputs at 1e-10; the
    reference's solver itself runs at 0.92x the port's speed on one core,
    oracle/reference_speed.py), one single-threaded process per core, each
    propagating one realisation of the ensemble.  One arm step = REF_INNER
    RK4 steps on every core at once; W steps of warm-up, then K timed."""
    if rank != 0:
        return
    from oracle import pool
    K = args.steps if args.steps is not None else 20
    W = max(3, args.warmup)
    t, cores = pool.concurrent_steps(n=N_SITES, warm_steps=W * REF_INNER, steps=K * REF_INNER)
    value = cores * K * REF_INNER / t
    sample = ('%d steps, each %d RK4 steps of one realisation on each of %d host cores '
              '(one single-threaded process per core), after %d warm-up steps; %.1f s timed'
              % (K, REF_INNER, cores, W, t))
    line = {
        'metric': METRIC, 'value': value, 'unit': 'instance-steps/s', 'n_gpus': world,
        'steps': K, 'warmup': W, 'ms_per_step': t / K * 1e3,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic (seeded disorder ensemble)', 'impl': 'reference',
        'config': {'workload': 'dephasing exciton-chain ensemble N=64, 4096 realisations, '
                               'dt=0.05 (4000-step workload; a per-core sample of realisations '
                               'is timed)', 'n_sites': N_SITES, 'batch': BATCH,
                   'arm_step': '%d RK4 steps on each of %d cores' % (REF_INNER, cores)},
        'cpu_baseline': {'value': value, 'unit': 'instance-steps/s', 'cores': cores,
                         'kind': 'port', 'sample': sample,
                         'port_speed_vs_reference': 'the reference solver measured at 0.92x '
                                                    'the port on one core (same outputs)'},
        'e2e': {'value': value, 'unit': 'instance-steps/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == 'reference':
        reference_arm(args, rank, world)
        return
    gpu_arm(args, rank, world, local)


if __name__ == '__main__':
    main()
