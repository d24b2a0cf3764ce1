"""CPU oracle for the nlchains hot path -- TEST INFRASTRUCTURE ONLY.

A ctypes binding of oracle/nlc_oracle.c, a CPU restatement of the reference's integrators and
diagnostics (each C function cites the reference file:line it follows).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package; the product
(nlchains_gb300) never does.

Parity status: pinned to the reference itself.  oracle/build.py compiles the reference's CPU
program (its nlchains-cpu target) in place from its sources, with stand-ins for Boost, MPI, FFTW3 and
Armadillo (oracle/ref_shim/); the oracle's reference order reproduces that program bit for bit when
the stand-ins' FFT and eigensolver are the oracle's own, and to rounding with the exact transform
(tests/golden/reference, tests/test_reference_pin.py).  The reference's GPU kernels, compiled
unmodified into oracle/_ref/ref_gpu_n<N>.fatbin, run through RefGPU below on the GPU
(tests/test_gpu_reference.py).  The Yoshida tables are pinned to the reference's header as well, and
analytic known answers stay in tests/test_oracle.py and tests/test_known_answers.py.
"""
import ctypes
import os

import numpy as np

from . import build as _build

DNKG, FPUT, TODA, DDNKG, DNLS = range(5)
ORDER_REFERENCE, ORDER_DEVICE, ORDER_STENCIL = 0, 1, 2
MODEL_NAMES = {"DNKG": DNKG, "FPUT": FPUT, "Toda": TODA, "dDNKG": DDNKG, "DNLS": DNLS}


class _Model(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("order", ctypes.c_int32), ("n", ctypes.c_uint32),
                ("copies", ctypes.c_uint32), ("dt", ctypes.c_double), ("m", ctypes.c_double),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("mp2", ctypes.POINTER(ctypes.c_double)), ("threads", ctypes.c_int32)]


_libs = {}


def _lib(mt=False):
    name = "libnlc_oracle_mt.so" if mt else "libnlc_oracle.so"
    if name not in _libs:
        out = _build.build()
        lib = ctypes.CDLL(os.path.join(out, name))
        dp = ctypes.POINTER(ctypes.c_double)
        lib.nlo_advance.argtypes = [ctypes.POINTER(_Model), dp, ctypes.c_uint64, ctypes.c_uint32]
        lib.nlo_linenergies.argtypes = [ctypes.POINTER(_Model), dp, dp, dp, dp]
        lib.nlo_entropies.argtypes = [dp, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_uint8), dp, dp]
        lib.nlo_energy.argtypes = [ctypes.POINTER(_Model), dp]
        lib.nlo_energy.restype = ctypes.c_double
        lib.nlo_eigensystem.argtypes = [ctypes.c_uint32, dp, dp, dp]
        lib.nlo_fft.argtypes = [ctypes.c_uint32, dp, ctypes.c_int]
        lib.nlo_dispersion.argtypes = [ctypes.c_int32, ctypes.c_uint32, ctypes.c_double, dp]
        lib.nlo_exp_table.argtypes = [ctypes.c_double, dp]
        lib.nlo_exp_scaled.argtypes = [ctypes.c_double, dp]
        lib.nlo_exp_scaled.restype = ctypes.c_double
        lib.nlo_coefficients.argtypes = [dp, dp]
        lib.nlo_dnls_stencil_coefficients.argtypes = [ctypes.c_double, ctypes.c_int, dp, dp, dp]
        _libs[name] = lib
    return _libs[name]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Model:
    """Parameters of one ensemble, as the reference's gconf plus the per-model options."""

    def __init__(self, model, n, copies, dt, m=0.0, alpha=0.0, beta=0.0, masses=None,
                 order=ORDER_DEVICE):
        self.model = MODEL_NAMES[model] if isinstance(model, str) else int(model)
        self.n, self.copies, self.dt = int(n), int(copies), float(dt)
        self.m, self.alpha, self.beta = float(m), float(alpha), float(beta)
        self.order = order
        self.mp2 = None
        if self.model == DDNKG:
            if masses is None:
                raise ValueError("dDNKG needs per-site masses")
            # dDNKG.cpp:47: the m file holds m_x and the solver works with m_x + 2
            self.mp2 = np.ascontiguousarray(np.asarray(masses, dtype=np.float64) + 2)

    def _struct(self, threads=1, order=None):
        s = _Model(self.model, self.order if order is None else order, self.n, self.copies, self.dt,
                   self.m, self.alpha, self.beta, None, threads)
        if self.mp2 is not None:
            s.mp2 = _dp(self.mp2)
        return s


def coefficients():
    c, d = np.zeros(8), np.zeros(8)
    _lib().nlo_coefficients(_dp(c), _dp(d))
    return c, d


def dnls_stencil_coefficients(dt, max_radius=11):
    """(radius, c0m1[7], taps[7, max_radius], phase[7]) of the DNLS stencil form, computed by the
    oracle's own double-double series (nlo_dnls_stencil_coefficients)."""
    c0, taps, ph = np.zeros(7), np.zeros(7 * max_radius), np.zeros(7)
    r = _lib().nlo_dnls_stencil_coefficients(float(dt), int(max_radius), _dp(c0), _dp(taps), _dp(ph))
    return r, c0, taps.reshape(7, max_radius), ph


def reference_coefficients():
    """The reference's own (symplectic_c, symplectic_d) from oracle/_ref, or None where it was not
    built for this machine (no reference sources here)."""
    path = os.path.join(_build.REF_OUT, "libref_symplectic.so")
    if not os.path.exists(path):
        return None
    try:
        lib = ctypes.CDLL(path)
    except OSError:   # built for another machine
        return None
    c, d = np.zeros(8), np.zeros(8)
    lib.ref_symplectic(_dp(c), _dp(d))
    return c, d


def advance(model, state, steps, batching, order=None, threads=1):
    """Return a copy of `state` (planar [copies][n][2] float64) advanced by `steps` steps."""
    out = np.ascontiguousarray(np.array(state, dtype=np.float64, copy=True))
    assert out.size == 2 * model.n * model.copies
    s = model._struct(threads, order)
    lib = _lib(mt=threads > 1)
    if lib.nlo_advance(ctypes.byref(s), _dp(out), steps, batching) != 0:
        raise ValueError("nlo_advance rejected its arguments")
    return out


def eigensystem(n, mp2):
    mp2 = np.ascontiguousarray(mp2, dtype=np.float64)
    om, ev = np.zeros(n), np.zeros(n * n)
    if _lib().nlo_eigensystem(n, _dp(mp2), _dp(om), _dp(ev)) != 0:
        raise ValueError("eigensystem failed")
    return om, ev


def linenergies(model, state, eig=None):
    """Normalised per-mode energies of the ensemble (results::calc_linenergies output).  eig: the
    dDNKG (omegas, eigenvectors) of eigensystem(), computed here when not given."""
    state = np.ascontiguousarray(state, dtype=np.float64)
    out = np.zeros(model.n)
    ev = om = None
    if model.model == DDNKG:
        om, ev = eig if eig is not None else eigensystem(model.n, model.mp2)
    s = model._struct()
    rc = _lib().nlo_linenergies(ctypes.byref(s), _dp(state), _dp(ev) if ev is not None else None,
                                _dp(om) if om is not None else None, _dp(out))
    if rc != 0:
        raise ValueError("nlo_linenergies rejected its arguments")
    return out


def a0is0(model):
    """Whether mode 0 has zero frequency and is left out of the entropy (results.cpp:8)."""
    if model.model == DNLS:
        return True
    if model.model == DDNKG:
        return False
    return model.m == 0.0


def entropies(lin, a0is0_flag, mask=None):
    lin = np.ascontiguousarray(lin, dtype=np.float64)
    wt, inf = ctypes.c_double(), ctypes.c_double()
    mp = None
    if mask is not None:
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        mp = mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    if _lib().nlo_entropies(_dp(lin), lin.size, int(a0is0_flag), mp, ctypes.byref(wt), ctypes.byref(inf)) != 0:
        raise ValueError("nlo_entropies rejected its arguments")
    return wt.value, inf.value


def energy(model, chain):
    chain = np.ascontiguousarray(chain, dtype=np.float64)
    s = model._struct()
    return _lib().nlo_energy(ctypes.byref(s), _dp(chain))


def energies(model, state):
    st = np.ascontiguousarray(state, dtype=np.float64).reshape(model.copies, model.n * 2)
    return np.array([energy(model, st[c]) for c in range(model.copies)])


def fft(z, sign=-1):
    z = np.ascontiguousarray(np.asarray(z, dtype=np.complex128).copy())
    _lib().nlo_fft(z.size, z.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sign)
    return z


def dispersion(model_id, n, m=0.0):
    out = np.zeros(n)
    _lib().nlo_dispersion(model_id, n, m, _dp(out))
    return out


def exp_table(scale):
    t = np.zeros(2048)
    _lib().nlo_exp_table(scale, _dp(t))
    return t


def exp_scaled(x, table):
    return _lib().nlo_exp_scaled(x, _dp(np.ascontiguousarray(table)))


class RefGPU:
    """The reference's own GPU kernels (oracle/_ref/ref_gpu_n<N>.fatbin, compiled unmodified from its
    sources) launched by oracle/ref_shim/ref_gpu_host.cpp on device ensembles.  Test infrastructure:
    the checker and the bench's plain-reference line, never the product.

    ``available(n_opt)`` tells whether the fatbin and the harness exist on this machine.
    """

    @staticmethod
    def fatbin(n_opt):
        return os.path.join(_build.REF_OUT, f"ref_gpu_n{n_opt}.fatbin")

    @staticmethod
    def available(n_opt):
        return (os.path.exists(RefGPU.fatbin(n_opt)) and
                os.path.exists(os.path.join(_build.OUT, "libref_gpu_host.so")))

    _host = None

    @classmethod
    def _lib(cls):
        if cls._host is None:
            _build.build()
            lib = ctypes.CDLL(os.path.join(_build.OUT, "libref_gpu_host.so"))
            vp, dp, u32, u64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_uint32, ctypes.c_uint64
            lib.refgpu_open.argtypes = [ctypes.c_char_p, ctypes.c_int, dp, dp, ctypes.POINTER(vp)]
            lib.refgpu_close.argtypes = [vp]
            lib.refgpu_error.argtypes = [vp]
            lib.refgpu_error.restype = ctypes.c_char_p
            lib.refgpu_kernel_count.argtypes = [vp]
            lib.refgpu_advance.argtypes = [vp, ctypes.c_int, vp, u32, u32, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, dp, u64, u32, ctypes.c_int, vp]
            lib.refgpu_move_warp_async.argtypes = [vp, ctypes.c_int, vp, u32, u32, u32, u32, vp, vp]
            lib.refgpu_linenergies.argtypes = [vp, ctypes.c_int, vp, u32, u32, ctypes.c_double, dp, dp, dp, vp]
            lib.refgpu_dnls_advance.argtypes = [vp, vp, u32, u32, ctypes.c_double, ctypes.c_double, u64, u32, vp,
                                                ctypes.c_int]
            cls._host = lib
        return cls._host

    def __init__(self, n_opt):
        self.n_opt = n_opt
        lib = self._lib()
        c, d = coefficients()
        self.h = ctypes.c_void_p()
        rc = lib.refgpu_open(self.fatbin(n_opt).encode(), n_opt, _dp(c), _dp(d), ctypes.byref(self.h))
        if rc != 0:
            msg = lib.refgpu_error(self.h).decode()
            self.close()
            raise RuntimeError("reference GPU module: " + msg)

    def close(self):
        if getattr(self, "h", None):
            self._lib().refgpu_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference GPU path: " + self._lib().refgpu_error(self.h).decode())

    def kernel_count(self):
        return self._lib().refgpu_kernel_count(self.h)

    def advance(self, model, state_ptr, steps, batching, force_split=False, stream=0):
        """move<model> on a device double2[copies][n] (model: an oracle Model), `steps / batching`
        launches; synchronous."""
        mp2 = _dp(model.mp2) if model.mp2 is not None else None
        self._check(self._lib().refgpu_advance(self.h, model.model, state_ptr, model.n, model.copies, model.dt,
                                               model.m, model.alpha, model.beta, mp2, steps, batching,
                                               int(force_split), stream))

    def move_warp_async(self, model_id, state_ptr, n, copies, batching, launches=1, mp2_ptr=None, stream=0):
        """Queue `launches` launches of the reference's warp kernel (move_chain_in_warp) on `stream`;
        constants as the last advance() call set them."""
        self._check(self._lib().refgpu_move_warp_async(self.h, model_id, state_ptr, n, copies, batching, launches,
                                                       mp2_ptr, stream))

    def linenergies(self, model, state_ptr, stream=0):
        out = np.zeros(model.n)
        ev = om = None
        if model.model == DDNKG:
            om, ev = eigensystem(model.n, model.mp2)
        self._check(self._lib().refgpu_linenergies(self.h, model.model, state_ptr, model.n, model.copies, model.m,
                                                   _dp(ev) if ev is not None else None,
                                                   _dp(om) if om is not None else None, _dp(out), stream))
        return out

    def dnls_advance(self, model, state_ptr, steps, batching, stream=0, sync=True):
        self._check(self._lib().refgpu_dnls_advance(self.h, state_ptr, model.n, model.copies, model.dt, model.beta,
                                                    steps, batching, stream, int(sync)))
