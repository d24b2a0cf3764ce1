"""Analytic known answers on the CPU oracle (no GPU).

* dDNKG with every mass equal to m is DNKG with that m: the same states, and the same energy in
  every eigenspace.  DNKG's Fourier modes k and n - k share omega_k, so the basis-independent
  quantity is the energy of each degenerate pair; dDNKG's eigenvalues, sorted ascending, come as
  mode 0, then pairs (1, 2), (3, 4), ..., then mode n/2 for even n.
* FPUT and Toda conserve the total momentum of each chain (the forces are differences of bond
  terms around the ring), up to rounding.
"""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic


def dnkg_pair_sums(lin):
    n = len(lin)
    out = [lin[0]] + [lin[k] + lin[n - k] for k in range(1, (n + 1) // 2)]
    if n % 2 == 0:
        out.append(lin[n // 2])
    return np.array(out)


def sorted_pair_sums(lin):
    n = len(lin)
    out = [lin[0]] + [lin[2 * j - 1] + lin[2 * j] for j in range(1, (n + 1) // 2)]
    if n % 2 == 0:
        out.append(lin[n - 1])
    return np.array(out)


@pytest.mark.parametrize("n", [8, 15, 16])
def test_ddnkg_constant_masses_is_dnkg(n):
    copies, m, steps, b = 6, 0.7, 20, 10
    state = ic.real_ensemble(n, copies, 0.3, ic.low_modes(n, kmax=3), m=m, seed=n)
    dnkg = O.Model("DNKG", n, copies, 0.05, m=m, beta=1.0)
    ddnkg = O.Model("dDNKG", n, copies, 0.05, masses=np.full(n, m), beta=1.0)
    s1 = O.advance(dnkg, state, steps, b, order=O.ORDER_DEVICE)
    s2 = O.advance(ddnkg, state, steps, b, order=O.ORDER_DEVICE)
    assert np.array_equal(s1, s2)
    e1 = dnkg_pair_sums(O.linenergies(dnkg, s1.reshape(copies, n, 2)))
    e2 = sorted_pair_sums(O.linenergies(ddnkg, s2.reshape(copies, n, 2)))
    assert np.abs(e1 - e2).max() <= 1e-12 * np.abs(e1).max()


@pytest.mark.parametrize("name,params", [("FPUT", dict(alpha=0.3, beta=1.0)), ("Toda", dict(alpha=0.5))])
def test_momentum_conserved(name, params):
    n, copies = 16, 4
    state = 0.3 * np.random.default_rng(3).standard_normal((copies, n, 2))
    state[:, :, 1] += 0.2   # a non-zero total momentum
    mdl = O.Model(name, n, copies, 0.05, **params)
    out = O.advance(mdl, state, 200, 100, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    p0, p1 = state[:, :, 1].sum(axis=1), out[:, :, 1].sum(axis=1)
    assert np.abs(p1 - p0).max() <= 1e-12 * np.abs(state[:, :, 1]).sum(axis=1).max()
