"""Seeded initial ensembles on the CPU (no GPU).

* The counter generator is SplitMix64 (Steele, Lea and Flood, OOPSLA 2014): from state 0 the
  published generator's first outputs are the mixes of 1, 2, 3 ... times the golden gamma, pinned
  here as known answers.
* Any slice of copies regenerates on its own (the counters are keyed by copy).
* Each recipe puts its energy (norm) exactly where it says: in the harmonic limit (beta = 0) the
  oracle's per-chain energy is energy_density * n, the ensemble-averaged linear-mode energies are
  energy_density * n / (number of excited modes) on the excited modes and zero elsewhere; DNLS
  chains hold norm_density * n.
"""
import numpy as np
import pytest

import oracle as O
from nlchains_gb300 import ic

GOLDEN_GAMMA = np.uint64(0x9E3779B97F4A7C15)
SPLITMIX64_FROM_ZERO = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F,
                        0xF88BB8A8724C81EC, 0x1B39896A51A8749B]


def test_splitmix64_published_sequence():
    with np.errstate(over="ignore"):
        states = np.arange(5, dtype=np.uint64) * GOLDEN_GAMMA
    assert [int(v) for v in ic.splitmix64(states)] == SPLITMIX64_FROM_ZERO


def test_uniform_range_and_slices():
    u = ic.uniform(17, 6, 40, stream=1)
    assert u.shape == (6, 40) and u.min() >= 0.0 and u.max() < 1.0
    assert np.array_equal(u[2:5], ic.uniform(17, 3, 40, stream=1, first_copy=2))
    assert not np.array_equal(u, ic.uniform(17, 6, 40, stream=2))
    assert not np.array_equal(u, ic.uniform(18, 6, 40, stream=1))
    # 53-bit mantissas: every value is an integer multiple of 2^-53
    assert np.all(np.floor(u * 2.0 ** 53) == u * 2.0 ** 53)


@pytest.mark.parametrize("m", [0.0, 0.7])
@pytest.mark.parametrize("n", [31, 32])
def test_real_ensemble_energies(n, m):
    copies, eps = 5, 0.25
    modes = ic.low_modes(n, kmax=3)
    state = ic.real_ensemble(n, copies, eps, modes, m=m, seed=n)
    model = O.Model("DNKG", n, copies, 0.05, m=m, beta=0.0)
    assert np.allclose(O.energies(model, state), eps * n, rtol=1e-12)
    excited = [k for k in modes if ic.dispersion_real(n, m)[k] > 0]
    lin = O.linenergies(model, state)
    want = np.zeros(n)
    want[excited] = eps * n / len(excited)
    assert np.allclose(lin, want, rtol=1e-12, atol=1e-12 * eps * n)
    assert np.array_equal(state[1:3], ic.real_ensemble(n, 2, eps, modes, m=m, seed=n, first_copy=1))


@pytest.mark.parametrize("n", [31, 32])
def test_dnls_ensemble_norm_and_modes(n):
    copies, norm = 4, 0.5
    modes = ic.low_modes(n, kmax=2)
    psi = ic.dnls_ensemble(n, copies, norm, modes, seed=2)
    assert np.allclose((np.abs(psi) ** 2).sum(axis=1), norm * n, rtol=1e-12)
    spectrum = np.abs(np.fft.fft(psi, axis=1)) ** 2
    off = np.setdiff1d(np.arange(n), modes)
    assert np.all(spectrum[:, off] < 1e-20 * spectrum.max())
    assert np.allclose(spectrum[:, modes], spectrum[0, modes[0]], rtol=1e-12)


def test_ddnkg_ensemble_eigenmode_energies():
    n, copies, eps, nmodes = 32, 4, 0.25, 5
    masses = ic.masses_uniform(n, seed=3)
    assert masses.min() >= 1.0 and masses.max() < 3.0
    state = ic.ddnkg_ensemble(masses, copies, eps, nmodes, seed=1)
    model = O.Model("dDNKG", n, copies, 0.05, masses=masses, beta=0.0)
    assert np.allclose(O.energies(model, state), eps * n, rtol=1e-12)
    lin = O.linenergies(model, state)
    want = np.zeros(n)
    want[:nmodes] = eps * n / nmodes
    assert np.allclose(lin, want, rtol=1e-10, atol=1e-10 * eps * n)


def test_state_file_round_trip(tmp_path):
    n = 16
    real = ic.real_ensemble(n, 3, 0.1, ic.low_modes(n, kmax=2), seed=9)
    psi = ic.dnls_ensemble(n, 3, 0.1, ic.low_modes(n, kmax=2), seed=9)
    ic.write_state(tmp_path / "r.bin", real)
    ic.write_state(tmp_path / "c.bin", psi)
    assert (tmp_path / "r.bin").stat().st_size == 3 * n * 2 * 8
    assert np.array_equal(ic.read_state(tmp_path / "r.bin", n), real)
    assert np.array_equal(ic.read_state(tmp_path / "c.bin", n, complex_model=True), psi)
