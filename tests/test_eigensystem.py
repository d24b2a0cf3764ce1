"""The library's host eigensolver for the dDNKG operator (nlc_eigensystem, device < 0), on the CPU:
against LAPACK (numpy) and the oracle's own solver.  Eigenvectors are compared through quantities
that do not depend on their signs or on the basis chosen inside a degenerate eigenspace: the
residual |A v - omega^2 v|, orthonormality, and the projector onto each eigenspace."""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic


def operator(masses):
    n = len(masses)
    a = np.diag(np.asarray(masses, dtype=np.float64) + 2)
    for i in range(n):
        j = (i + 1) % n
        a[i, j] = a[j, i] = -1.0   # n = 2: the one off-diagonal entry is -1 (eigensystem.cpp:16-18)
    return a


def check_eigensystem(masses, omegas, vecs, tol=1e-12):
    a = operator(masses)
    n = len(masses)
    w2 = np.linalg.eigvalsh(a)
    scale = np.abs(w2).max()
    assert np.all(np.diff(omegas) >= 0)
    assert np.abs(omegas ** 2 - w2).max() <= tol * scale
    assert np.abs(a @ vecs - vecs * omegas ** 2).max() <= 10 * tol * scale
    assert np.abs(vecs.T @ vecs - np.eye(n)).max() <= 10 * tol * n ** 0.5


@pytest.mark.parametrize("n", [2, 3, 5, 16, 64, 255, 300])
def test_host_solver_random_masses(engine, n):
    masses = ic.masses_uniform(n, seed=n)
    om, vecs = engine.eigensystem(masses)
    check_eigensystem(masses, om, vecs)
    # non-degenerate spectrum: every eigenvector equals LAPACK's up to its sign
    _, ref = np.linalg.eigh(operator(masses))
    assert np.abs(np.abs(np.sum(ref * vecs, axis=0)) - 1).max() < 1e-9


@pytest.mark.parametrize("n", [8, 33, 128])
def test_host_solver_degenerate_spectrum(engine, n):
    """Constant masses: DNKG's spectrum, omega_k = omega_{n-k}; compare eigenspace projectors."""
    masses = np.full(n, 0.7)
    om, vecs = engine.eigensystem(masses)
    check_eigensystem(masses, om, vecs)
    k = np.arange(n)
    assert np.allclose(om, np.sort(np.sqrt(0.7 + 4 * np.sin(np.pi * k / n) ** 2)), rtol=0, atol=1e-13)
    w2, ref = np.linalg.eigh(operator(masses))
    groups = np.split(np.arange(n), np.nonzero(np.diff(w2) > 1e-9)[0] + 1)
    for g in groups:
        assert np.abs(vecs[:, g] @ vecs[:, g].T - ref[:, g] @ ref[:, g].T).max() < 1e-10


def test_host_solver_matches_oracle(engine):
    n = 96
    masses = ic.masses_uniform(n, seed=11)
    om, vecs = engine.eigensystem(masses)
    oom, oev = O.eigensystem(n, masses + 2)
    assert np.abs(om - oom).max() <= 1e-13 * om.max()
    oev = oev.reshape(n, n).T   # column k = eigenvector k
    assert np.abs(np.abs(np.sum(oev * vecs, axis=0)) - 1).max() < 1e-9


def mass_pattern(name, n):
    rng = np.random.default_rng(n)
    if name == "uniform":
        return ic.masses_uniform(n, seed=n)
    if name == "constant":         # DNKG: degenerate pairs, deflation everywhere
        return np.full(n, 1.3)
    if name == "near_constant":    # pairs split by 1e-9: near-degenerate poles
        return 1.3 + 1e-9 * rng.standard_normal(n)
    if name == "dimer":            # two alternating masses: two bands
        return np.where(np.arange(n) % 2 == 0, 1.0, 3.0)
    if name == "contrast":         # masses over four decades
        return 10.0 ** rng.uniform(-2, 2, n)
    if name == "impurity":         # one heavy site in a uniform ring
        m = np.full(n, 0.5)
        m[n // 3] = 20.0
        return m
    raise ValueError(name)


PATTERNS = ["uniform", "constant", "near_constant", "dimer", "contrast", "impurity"]


@pytest.mark.parametrize("pattern", PATTERNS)
@pytest.mark.parametrize("n", [64, 97, 128, 255, 256, 401, 512])
def test_divide_and_conquer(engine, monkeypatch, pattern, n):
    """From 64 sites the host solver is divide and conquer; with its fallback switched off it must
    pass on its own: eigenvalues, residuals, orthogonality, and the projector onto every
    eigenspace (which is basis independent) against LAPACK."""
    monkeypatch.setenv("NLC_HOST_EIGEN_DC_ONLY", "1")
    masses = mass_pattern(pattern, n)
    om, vecs = engine.eigensystem(masses)
    check_eigensystem(masses, om, vecs)
    w2, ref = np.linalg.eigh(operator(masses))
    scale = np.abs(w2).max()
    groups = np.split(np.arange(n), np.nonzero(np.diff(w2) > 1e-6 * scale)[0] + 1)
    for g in groups:
        assert np.abs(vecs[:, g] @ vecs[:, g].T - ref[:, g] @ ref[:, g].T).max() < 1e-8


@pytest.mark.parametrize("pattern", ["uniform", "constant"])
def test_divide_and_conquer_equals_dense_qr(engine, monkeypatch, pattern):
    n = 300
    masses = mass_pattern(pattern, n)
    om_dc, v_dc = engine.eigensystem(masses)
    monkeypatch.setenv("NLC_HOST_EIGEN_QR", "1")
    om_qr, v_qr = engine.eigensystem(masses)
    assert np.abs(om_dc - om_qr).max() <= 1e-13 * om_qr.max()
    if pattern == "uniform":
        assert np.abs(np.abs(np.sum(v_dc * v_qr, axis=0)) - 1).max() < 1e-9


def test_device_request_without_a_usable_gpu_uses_the_host(engine):
    """device >= 0 only allows the GPU solver: with no usable GPU (this CPU run) the host answers."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the device path is covered by the GPU tests")
    except ImportError:
        pass
    masses = ic.masses_uniform(300, seed=4)
    om, vecs = engine.eigensystem(masses, device=0)
    check_eigensystem(masses, om, vecs)


def test_host_solver_rejects_bad_arguments(engine):
    for n in (0, 1):
        with pytest.raises(engine.NlcError) as e:
            engine.eigensystem(np.ones(n))
        assert e.value.code == engine.EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("n", [256, 300])
def test_device_solver_equals_host(gpu, n, monkeypatch):
    """device 0 with the device threshold moved to 256 sites: cuSOLVER's divide and conquer; the same
    eigensystem as the host's."""
    monkeypatch.setenv("NLC_DEVICE_EIGEN_FROM", "256")
    masses = ic.masses_uniform(n, seed=n)
    om_d, vec_d = gpu.eigensystem(masses, device=0)
    om_h, vec_h = gpu.eigensystem(masses, device=-1)
    check_eigensystem(masses, om_d, vec_d)
    assert np.abs(om_d - om_h).max() <= 1e-12 * om_h.max()
    assert np.abs(np.abs(np.sum(vec_d * vec_h, axis=0)) - 1).max() < 1e-9
