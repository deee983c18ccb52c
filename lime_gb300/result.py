"""Result container with the fields of ``lime.mol.Result`` (lime/mol.py:78-104).

The reference computes ``times = t0 + arange(Nt // nout) * dt * nout`` and
raises TypeError when ``nout`` or ``t0`` is left at None (lime/mol.py:92);
here they default to 1 and 0.  ``observables[k]`` is recorded after step k,
i.e. at ``t0 + (k + 1) dt``, while ``times[k] = t0 + k dt`` as in the reference.
"""
from __future__ import annotations

import numpy as np


class Result:
    def __init__(self, description=None, psi0=None, rho0=None, dt=None, Nt=None,
                 times=None, t0=None, nout=None):
        self.description = description
        self.dt = dt
        self.timesteps = Nt
        self.observables = None
        self.rholist = None
        self.psilist = [psi0]
        self.psi = None
        self.rho0 = rho0
        self.psi0 = psi0
        self.nout = 1 if nout is None else nout
        t0 = 0.0 if t0 is None else t0
        if times is not None:
            self.times = np.asarray(times)
        elif Nt is not None and dt is not None:
            self.times = t0 + np.arange(Nt // self.nout) * dt * self.nout
        else:
            self.times = None

    def expect(self):
        return self.observables
