"""The DNLS linear propagator in real space (nlc_dnls_stencil_coefficients, host only): the taps are
the Bessel values J_x(2 dt d_k) with the signs of i^x, the phase is -2 dt d_k, the radius is where
the taps fall below 2^-64, and the stencil they define equals IFFT diag(exp(-i dt d_k omega)) FFT
(the reference's linear sub-step) to rounding, for smooth and prime lengths (CPU only)."""
import numpy as np
import pytest

import oracle as O

YOSHIDA_D = O.coefficients()[1]


def stencil_apply(psi, c0m1, taps, phase, radius):
    """psi' = exp(i phase) (psi + c0m1 psi + sum_x taps_x i^(x mod 2) (psi_{s+x} + psi_{s-x})), in
    numpy (the kernel's operator, not its rounding)."""
    acc = psi + c0m1 * psi
    for x in range(1, radius + 1):
        s = np.roll(psi, -x, axis=-1) + np.roll(psi, x, axis=-1)
        acc = acc + taps[x - 1] * (1j if x & 1 else 1.0) * s
    return np.exp(1j * phase) * acc


@pytest.mark.parametrize("dt", [0.001, 0.01, 0.05])
def test_taps_are_bessel_values(engine, dt):
    special = pytest.importorskip("scipy.special")
    radius, c0m1, taps, phase = engine.dnls_stencil_coefficients(dt, 11)
    for k in range(7):
        z = 2 * dt * YOSHIDA_D[k]
        assert phase[k] == pytest.approx(-z, rel=1e-15)
        # J_0 - 1 to full relative precision (the series without its leading 1)
        assert c0m1[k] == pytest.approx(special.jv(0, z) - 1, rel=1e-9)
        for x in range(1, 12):
            sign = -1.0 if x & 2 else 1.0
            assert taps[k, x - 1] == pytest.approx(sign * special.jv(x, z), rel=1e-12, abs=1e-300)
    # the radius: the last x with a tap above 2^-64
    above = [x for x in range(1, 12) if np.abs(taps[:, x - 1]).max() > 2.0 ** -64]
    assert radius == (max(above) if above else 0)
    assert radius == {0.001: 5, 0.01: 7, 0.05: 10}[dt]


def test_radius_beyond_the_limit(engine):
    radius, *_ = engine.dnls_stencil_coefficients(0.2, 11)
    assert radius == 12   # max_radius + 1: the stencil form does not apply


@pytest.mark.parametrize("n", [16, 53, 97, 1024, 2953])
@pytest.mark.parametrize("dt", [0.01, 0.05])
def test_stencil_equals_the_fourier_propagator(engine, n, dt):
    radius, c0m1, taps, phase = engine.dnls_stencil_coefficients(dt, 11)
    if n < 2 * radius + 2:
        pytest.skip("too short for this radius")
    rng = np.random.default_rng(n)
    psi = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    omega = 4 * np.sin(np.pi * np.arange(n) / n) ** 2
    for k in range(7):
        ref = np.fft.ifft(np.fft.fft(psi, axis=1) * np.exp(-1j * dt * YOSHIDA_D[k] * omega), axis=1)
        out = stencil_apply(psi, c0m1[k], taps[k], phase[k], radius)
        assert np.abs(out - ref).max() <= 4e-15 * np.abs(ref).max()


def test_invalid_arguments(engine):
    with pytest.raises(engine.NlcError):
        engine.dnls_stencil_coefficients(0.01, 0)
    with pytest.raises(engine.NlcError):
        engine.dnls_stencil_coefficients(-1.0, 11)


@pytest.mark.parametrize("dt", [0.001, 0.01, 0.05, 0.2])
def test_oracle_builds_the_same_coefficients(engine, dt):
    """The oracle's stencil replay uses its own double-double series: the same bits as the engine's."""
    a = engine.dnls_stencil_coefficients(dt, 11)
    b = O.dnls_stencil_coefficients(dt, 11)
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("n", [16, 53, 256])
def test_oracle_stencil_order_agrees_with_the_transform_form(n):
    """The oracle's replay of the stencil form against its transform form (the reference's split step
    with sincos): the same dynamics to rounding after 20 steps."""
    from nlchains_gb300 import ic
    copies, dt = 3, 0.01
    psi = ic.dnls_ensemble(n, copies, 1.0, ic.low_modes(n, 0.1), seed=n)
    mdl = O.Model("DNLS", n, copies, dt, beta=1.0)
    st = np.ascontiguousarray(psi).view(np.float64)
    a = O.advance(mdl, st, 20, 10, order=O.ORDER_STENCIL)
    b = O.advance(mdl, st, 20, 10, order=O.ORDER_DEVICE)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    with pytest.raises(ValueError):
        O.advance(O.Model("DNLS", 12, 1, dt, beta=1.0), np.zeros(24), 1, 1, order=O.ORDER_STENCIL)
