"""Seeded initial ensembles in the reference's `-i` file format.

The reference reads its initial state as raw doubles, ``double[copies][chain_length][2]`` (phi, pi)
for the real models and ``complex<double>[copies][chain_length]`` for DNLS (README.md:74-82,
common/main.cpp:112-118).  This module builds such ensembles from a seed so that every engine (the
GPU path, the CPU oracle, a user's reference install) integrates identical bytes.

Random numbers come from SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) keyed by (seed, copy, mode), so any slice of copies can be regenerated on
its own.

Recipes (energies follow the reference's diagnostics):

* real models (DNKG, FPUT, Toda): per chain the normal-mode amplitudes z_k = omega_k Phi_k + i Pi_k
  with |z_k|^2 = 2 n E_k, E_k = energy_density * n / (number of excited modes), uniform random phase,
  for the excited wave numbers +-k; then Phi_k = (z_k + conj z_{n-k}) / (2 omega_k),
  Pi_k = (z_k - conj z_{n-k}) / (2i), and phi, pi = inverse DFT.  A mode with omega_k = 0 (k = 0
  when m = 0) is never excited.
* dDNKG: the same in the eigenbasis of the periodic operator diag(m_x + 2) - shift(+-1):
  e_k . phi = sqrt(2 E_k) cos(theta) / omega_k, e_k . pi = sqrt(2 E_k) sin(theta).
* DNLS: psi_hat_k of equal modulus over the excited wave numbers, uniform phases, scaled so that
  sum |psi|^2 = norm_density * n, psi = inverse DFT.
"""
import numpy as np

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x):
    """SplitMix64 finaliser applied elementwise to uint64 counters."""
    with np.errstate(over="ignore"):
        z = (np.asarray(x, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & _MASK64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK64
        return z ^ (z >> np.uint64(31))


def uniform(seed, copies, count, stream=0, first_copy=0):
    """uniform [0, 1) doubles, shape (copies, count), from counters (seed, stream, copy, index)."""
    c = np.arange(first_copy, first_copy + copies, dtype=np.uint64)[:, None]
    i = np.arange(count, dtype=np.uint64)[None, :]
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.uint64(stream))
        ctr = (key + c * np.uint64(count) + i) & _MASK64
    return (splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def low_modes(n, fraction=None, kmax=None, include_zero=True):
    """Wave numbers 0 (optional), +-1 .. +-kmax as DFT indices.

    With `fraction` instead of kmax, the lowest fraction of all n modes is taken, each frequency
    counting twice (+k and -k): kmax = floor(fraction * n / 2), e.g. 10% of n = 1024 gives |k| <= 51.
    """
    if kmax is None:
        kmax = int(np.floor(fraction * n / 2))
    kmax = max(1, min(kmax, (n - 1) // 2 if n > 2 else 1))
    ks = [0] if include_zero else []
    for k in range(1, kmax + 1):
        ks.append(k)
        if n - k != k:
            ks.append(n - k)
    return np.array(sorted(set(ks)), dtype=np.int64)


def dispersion_real(n, m):
    k = np.arange(n)
    s2 = 2 * np.sin(k * np.pi / n)
    return np.sqrt(m + s2 * s2)


def real_ensemble(n, copies, energy_density, modes, m=0.0, seed=0, first_copy=0):
    """planar double2[copies][n] for DNKG / FPUT / Toda (see module docstring)."""
    omega = dispersion_real(n, m)
    modes = np.array([k for k in modes if omega[k] > 0], dtype=np.int64)
    e_k = energy_density * n / len(modes)
    theta = 2 * np.pi * uniform(seed, copies, n, stream=1, first_copy=first_copy)
    z = np.zeros((copies, n), dtype=np.complex128)
    z[:, modes] = np.sqrt(2 * n * e_k) * np.exp(1j * theta[:, modes])
    zc = np.conj(z[:, (-np.arange(n)) % n])
    with np.errstate(divide="ignore", invalid="ignore"):
        phi_k = np.where(omega > 0, (z + zc) / (2 * np.where(omega > 0, omega, 1)), 0)
    pi_k = (z - zc) / 2j
    out = np.empty((copies, n, 2))
    out[:, :, 0] = np.fft.ifft(phi_k, axis=1).real
    out[:, :, 1] = np.fft.ifft(pi_k, axis=1).real
    return out


def periodic_operator(mp2):
    n = len(mp2)
    h = np.diag(np.asarray(mp2, dtype=np.float64))
    for i in range(n):
        j = (i + 1) % n
        h[i, j] = h[j, i] = -1.0
    return h


def ddnkg_ensemble(masses, copies, energy_density, nmodes, seed=0, first_copy=0):
    """planar double2[copies][n] for dDNKG, energy spread over the nmodes lowest eigenmodes."""
    masses = np.asarray(masses, dtype=np.float64)
    n = len(masses)
    w2, vecs = np.linalg.eigh(periodic_operator(masses + 2))
    omega = np.sqrt(w2)
    e_k = energy_density * n / nmodes
    theta = 2 * np.pi * uniform(seed, copies, n, stream=3, first_copy=first_copy)
    amp = np.zeros((copies, n))
    amp_p = np.zeros((copies, n))
    amp[:, :nmodes] = np.sqrt(2 * e_k) * np.cos(theta[:, :nmodes]) / omega[:nmodes]
    amp_p[:, :nmodes] = np.sqrt(2 * e_k) * np.sin(theta[:, :nmodes])
    out = np.empty((copies, n, 2))
    out[:, :, 0] = amp @ vecs.T
    out[:, :, 1] = amp_p @ vecs.T
    return out


def dnls_ensemble(n, copies, norm_density, modes, seed=0, first_copy=0):
    """complex128[copies][n] for DNLS (see module docstring)."""
    theta = 2 * np.pi * uniform(seed, copies, n, stream=2, first_copy=first_copy)
    psik = np.zeros((copies, n), dtype=np.complex128)
    # sum |psi|^2 = (1/n) sum |psi_hat|^2 = norm_density * n  ->  |psi_hat|^2 = n^2 norm_density / M
    psik[:, modes] = np.sqrt(n * n * norm_density / len(modes)) * np.exp(1j * theta[:, modes])
    return np.ascontiguousarray(np.fft.ifft(psik, axis=1))


def masses_uniform(n, lo=1.0, hi=3.0, seed=0):
    """per-site masses m_x ~ U[lo, hi] (the dDNKG -m file content)."""
    return lo + (hi - lo) * uniform(seed, 1, n, stream=4)[0]


def write_state(path, state):
    """Write an ensemble in the reference `-i` / dump format (raw little-endian doubles)."""
    np.ascontiguousarray(state).astype(state.dtype, copy=False).tofile(path)


def read_state(path, n, complex_model=False):
    raw = np.fromfile(path, dtype=np.float64)
    if complex_model:
        return raw.view(np.complex128).reshape(-1, n)
    return raw.reshape(-1, n, 2)
