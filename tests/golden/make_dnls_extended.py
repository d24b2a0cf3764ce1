"""Writes tests/golden/extended/DNLS_n<n>.npz: the DNLS split step in extended precision.

The reference's DNLS step (DNLS/DNLS.cpp:159-175, the CPU form DNLS/cpu-implementation/DNLS.cpp:
110-124): seven pairs of a nonlinear phase rotation psi <- psi exp(-i beta dt c_k |psi|^2) (the first
one's coefficient doubled between steps of a launch) and a linear propagator applied in Fourier
space (forward transform, multiply by exp(-i dt d_k omega_j) / n, backward transform), then the
closing rotation with c_7.  Here every operation is carried out in numpy's longdouble (the x87
80-bit format on x86-64: 64-bit significand, rounding error 2^-64), the transform as a vectorised
radix-2 decimation in time with long-double twiddles, the rotations with long-double sin and cos.

DNLS at these energies is chaotic: two correct double-precision implementations (different FFTs,
different sincos) drift apart from rounding level to 1e-10 in 10^3 steps.  This run, 2^11 times more
precise per operation, is the yardstick the GPU tests measure both the engine and the reference's
own GPU kernels against (tests/test_gpu_reference.py).

Inputs: the seeded DNLS ensembles of nlchains_gb300/ic.py (norm density 1, lowest 10% of modes) at
n = 64 and at the benchmark configuration's n = 1024.  Run from the repository root on an x86-64
host:  python tests/golden/make_dnls_extended.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from nlchains_gb300 import ic  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "extended")
LD = np.longdouble
CHECKPOINTS = (100, 200, 500, 1000)
# name: (n, copies, dt, beta, batching, seed)
CASES = {"DNLS_n64": (64, 8, 0.01, 1.0, 100, 12345), "DNLS_n1024": (1024, 4, 0.01, 1.0, 100, 12345)}


def fft_ld(re, im, sign):
    """Radix-2 DIT DFT along the last axis, sum_j x_j exp(sign 2 pi i j k / n), in long double."""
    n = re.shape[-1]
    bits = n.bit_length() - 1
    rev = np.array([int(format(i, f"0{bits}b")[::-1], 2) for i in range(n)])
    re, im = re[..., rev].copy(), im[..., rev].copy()
    two_pi = LD(2) * np.arccos(LD(-1))
    length = 2
    while length <= n:
        half = length // 2
        ang = two_pi * np.arange(half, dtype=LD) / LD(length)
        wr, wi = np.cos(ang), LD(sign) * np.sin(ang)
        r = re.reshape(re.shape[:-1] + (n // length, length))
        i = im.reshape(im.shape[:-1] + (n // length, length))
        ar, ai = r[..., :half].copy(), i[..., :half].copy()
        br, bi = r[..., half:], i[..., half:]
        tr, ti = br * wr - bi * wi, br * wi + bi * wr
        r[..., :half], i[..., :half] = ar + tr, ai + ti
        r[..., half:], i[..., half:] = ar - tr, ai - ti
        re, im = r.reshape(re.shape), i.reshape(im.shape)
        length *= 2
    return re, im


def rotate(re, im, bds):
    angle = -bds * (re * re + im * im)
    c, s = np.cos(angle), np.sin(angle)
    return re * c - im * s, s * re + im * c


def run(n, copies, dt, beta, batching, seed):
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, fraction=0.1), seed=seed)
    re, im = psi.real.astype(LD), psi.imag.astype(LD)
    c, d = O.coefficients()
    c, d = c.astype(LD), d.astype(LD)
    dt_ld, beta_ld = LD(dt), LD(beta)
    k = np.arange(n, dtype=LD)
    s2 = LD(2) * np.sin(k * np.arccos(LD(-1)) / LD(n))
    omega = s2 * s2
    tab_r = np.stack([np.cos(-dt_ld * d[j] * omega) / LD(n) for j in range(7)])
    tab_i = np.stack([np.sin(-dt_ld * d[j] * omega) / LD(n) for j in range(7)])
    out = {"state_in": np.ascontiguousarray(psi).view(np.float64).reshape(copies, n, 2)}
    t = 0
    for cp in CHECKPOINTS:
        while t < cp:
            for i in range(batching):
                for j in range(7):
                    coef = beta_ld * dt_ld * (LD(2) if (j == 0 and i > 0) else LD(1)) * c[j]
                    re, im = rotate(re, im, coef)
                    re, im = fft_ld(re, im, -1)
                    re, im = re * tab_r[j] - im * tab_i[j], re * tab_i[j] + im * tab_r[j]
                    re, im = fft_ld(re, im, +1)
            re, im = rotate(re, im, beta_ld * dt_ld * c[7])
            t += batching
        out[f"state_{cp}"] = np.stack([re.astype(np.float64), im.astype(np.float64)], axis=-1)
    out.update(n=n, copies=copies, dt=dt, beta=beta, batching=batching, seed=seed,
               checkpoints=np.array(CHECKPOINTS))
    return out


def main():
    if np.finfo(LD).nmant < 63:
        sys.exit("this host's long double is not an extended format")
    os.makedirs(OUT, exist_ok=True)
    for name, args in CASES.items():
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **run(*args))
        print("wrote", name)


if __name__ == "__main__":
    main()
