"""nlchains_gb300: GB300-native (sm_103a) engine for the nlchains ensemble integrators.

This package is a thin ctypes binding of the C ABI in include/nlchains.h (libnlchains_gb300.so,
built in-tree by nlchains_gb300/builder.py).  It mirrors the reference's interface:

* ``run_program(["FPUT", "-n", "64", ...])`` is the reference command line
  ``nlchains FPUT -n 64 ...`` (common/main.cpp:142-176, same options, files and exit codes);
* ``Plan`` exposes the per-model GPU operators that replace the reference's internal GPU API
  (``move<model>``, ``make_linenergies``, ``DNLS::evolve_*``) on caller-owned device memory;
* ``Context`` / ``Job`` run an ensemble with engine-owned device state, as the reference's main loop.

There is no CPU fallback: every entry point needs the CUDA library, and importing a missing or
stale build raises immediately.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(_HERE, "libnlchains_gb300.so")
EXECUTABLE_PATH = os.path.join(_HERE, "nlchains")

DNKG, FPUT, TODA, DDNKG, DNLS = range(5)
MODELS = {"DNKG": DNKG, "FPUT": FPUT, "Toda": TODA, "dDNKG": DDNKG, "DNLS": DNLS}
MODEL_NAMES = {v: k for k, v in MODELS.items()}

OK, EINVAL, ECUDA, ENOMEM, EIO, ETIMEDOUT, ENOTFOUND, EBLOWUP, EUNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7, -8
FLAG_SPLIT_KERNEL, FLAG_NO_TUNE, FLAG_CANONICAL_SHAPE, FLAG_COMPACT_DIAG = 1, 2, 4, 8
FLAG_SHARED_GPU, FLAG_TENSOR_PROJECTION, FLAG_FP64_PROJECTION, FLAG_BF16X3_PROJECTION = 16, 32, 64, 128
FLAG_FP32_DIAGNOSTICS, FLAG_DNLS_FOURIER = 256, 512
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3

# the exported symbols, as declared in include/nlchains.h
EXPORTS = (
    "nlc_plan_create", "nlc_plan_destroy", "nlc_move", "nlc_linenergies", "nlc_dnls_evolve_nonlinear",
    "nlc_dnls_evolve_linear", "nlc_plan_shape", "nlc_plan_omegas", "nlc_eigensystem", "nlc_create", "nlc_destroy",
    "nlc_job_create", "nlc_job_destroy", "nlc_job_upload", "nlc_job_advance", "nlc_job_linenergies",
    "nlc_job_download", "nlc_job_wait", "nlc_job_state_ptr", "nlc_program_run", "nlc_last_error",
    "nlc_version", "nlc_kernel_launches", "nlc_fp64_peak", "nlc_linenergies_noalloc",
    "nlc_server_create", "nlc_server_destroy", "nlc_server_submit", "nlc_server_poll", "nlc_server_wait",
    "nlc_server_result", "nlc_entropies", "nlc_job_sample_async", "nlc_job_sample_wait", "nlc_energies",
    "nlc_job_energies", "nlc_job_step_async", "nlc_job_after", "nlc_initial_state", "nlc_server_submit_seeded",
    "nlc_dnls_stencil_coefficients",
)


class NlcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class _CModel(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("chain_length", ctypes.c_uint32), ("copies", ctypes.c_uint32),
                ("dt", ctypes.c_double), ("m", ctypes.c_double), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("masses", ctypes.POINTER(ctypes.c_double)),
                ("entropy_mask", ctypes.POINTER(ctypes.c_uint8)), ("flags", ctypes.c_uint32)]


class _CServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_uint64), ("max_active", ctypes.c_int32),
                ("streams", ctypes.c_int32), ("quantum_ms", ctypes.c_double)]


class _CRequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("error", ctypes.c_int32), ("steps_done", ctypes.c_uint64),
                ("samples", ctypes.c_uint64), ("submit_ms", ctypes.c_double), ("start_ms", ctypes.c_double),
                ("ready_ms", ctypes.c_double), ("finish_ms", ctypes.c_double)]


_lib = None


def build(verbose=False):
    """Compile the CUDA extension in-tree (sm_103a) and return the library path."""
    from . import builder as _b
    return _b.build(verbose=verbose)


def lib():
    """Load libnlchains_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBRARY_PATH):
        raise ImportError(f"{LIBRARY_PATH} is missing: run `python -m nlchains_gb300.builder` (needs nvcc)")
    L = ctypes.CDLL(LIBRARY_PATH)
    vp, u64, i32, u32, dp = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double)
    P = ctypes.POINTER
    sig = {
        "nlc_plan_create": ([P(_CModel), P(vp)], i32),
        "nlc_plan_destroy": ([vp], i32),
        "nlc_move": ([vp, vp, u32, vp], i32),
        "nlc_linenergies": ([vp, vp, vp, vp, vp], i32),
        "nlc_dnls_evolve_nonlinear": ([vp, vp, ctypes.c_double, vp], i32),
        "nlc_dnls_evolve_linear": ([vp, vp, vp, vp], i32),
        "nlc_plan_shape": ([vp, P(i32), P(i32), P(i32), P(i32)], i32),
        "nlc_plan_omegas": ([vp, dp], i32),
        "nlc_eigensystem": ([u32, dp, i32, dp, dp], i32),
        "nlc_create": ([P(vp), ctypes.c_int], i32),
        "nlc_destroy": ([vp], i32),
        "nlc_job_create": ([vp, P(_CModel), u32, P(u64)], i32),
        "nlc_job_destroy": ([vp, u64], i32),
        "nlc_job_upload": ([vp, u64, vp], i32),
        "nlc_job_advance": ([vp, u64, u64], i32),
        "nlc_job_linenergies": ([vp, u64, dp, dp, dp], i32),
        "nlc_job_download": ([vp, u64, vp], i32),
        "nlc_job_wait": ([vp, u64, i32], i32),
        "nlc_job_after": ([vp, u64, u64], i32),
        "nlc_initial_state": ([vp, u64, u64, ctypes.c_double, P(ctypes.c_uint32), ctypes.c_uint32, vp, vp], i32),
        "nlc_job_state_ptr": ([vp, u64, P(vp)], i32),
        "nlc_program_run": ([ctypes.c_int, P(ctypes.c_char_p)], ctypes.c_int),
        "nlc_last_error": ([], ctypes.c_char_p),
        "nlc_version": ([], ctypes.c_char_p),
        "nlc_kernel_launches": ([], u64),
        "nlc_fp64_peak": ([ctypes.c_double, dp], i32),
        "nlc_linenergies_noalloc": ([i32, u32, u32, ctypes.c_double, vp, vp, vp, vp, vp], i32),
        "nlc_server_create": ([P(_CServerConfig), P(vp)], i32),
        "nlc_server_destroy": ([vp], i32),
        "nlc_server_submit": ([vp, P(_CModel), u32, u64, vp, P(u64)], i32),
        "nlc_server_submit_seeded": ([vp, P(_CModel), u32, u64, u64, ctypes.c_double, P(ctypes.c_uint32),
                                      ctypes.c_uint32, P(u64)], i32),
        "nlc_server_poll": ([vp, u64, P(_CRequestStatus)], i32),
        "nlc_server_wait": ([vp, u64, i32], i32),
        "nlc_server_result": ([vp, u64, vp, dp, dp, P(u64)], i32),
        "nlc_entropies": ([dp, u32, i32, vp, dp], i32),
        "nlc_job_sample_async": ([vp, u64, i32, i32], i32),
        "nlc_job_sample_wait": ([vp, u64, i32, dp, dp, dp, vp, i32], i32),
        "nlc_energies": ([vp, vp, vp, vp], i32),
        "nlc_job_energies": ([vp, u64, dp], i32),
        "nlc_job_step_async": ([vp, u64, i32, i32], i32),
        "nlc_dnls_stencil_coefficients": ([ctypes.c_double, i32, P(i32), dp, dp, dp], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise NlcError(rc, lib().nlc_last_error().decode(errors="replace"))
    return rc


def entropies(lin, a0is0, entropy_mask=None):
    """(WT, INF) of host linear energies (nlc_entropies); NlcError(EBLOWUP) when not finite."""
    lin = np.ascontiguousarray(lin, dtype=np.float64)
    out = np.zeros(2)
    mask = None if entropy_mask is None else np.ascontiguousarray(entropy_mask, dtype=np.uint8)
    _check(lib().nlc_entropies(lin.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), lin.size, int(bool(a0is0)),
                               None if mask is None else mask.ctypes.data_as(ctypes.c_void_p),
                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return float(out[0]), float(out[1])


def last_error():
    return lib().nlc_last_error().decode(errors="replace")


def kernel_launches():
    return int(lib().nlc_kernel_launches())


def fp64_peak_tflops(ms=200.0):
    out = ctypes.c_double()
    _check(lib().nlc_fp64_peak(ms, ctypes.byref(out)))
    return out.value


def eigensystem(masses, device=-1):
    """(omegas, eigenvectors) of the dDNKG operator diag(masses + 2) - shift(+-1) (nlc_eigensystem):
    omegas ascending, eigenvectors[:, k] the k-th; device >= 0 allows the GPU solver from 256 sites."""
    m = np.ascontiguousarray(masses, dtype=np.float64)
    n = m.size
    om, ev = np.zeros(n), np.zeros(n * n)
    P = ctypes.POINTER(ctypes.c_double)
    _check(lib().nlc_eigensystem(n, m.ctypes.data_as(P), int(device), om.ctypes.data_as(P), ev.ctypes.data_as(P)))
    return om, ev.reshape(n, n).T


def dnls_stencil_coefficients(dt, max_radius=11):
    """The DNLS linear propagators as real-space stencils (nlc_dnls_stencil_coefficients, host only):
    (radius, c0m1[7], taps[7, max_radius], phase[7]) with c0m1 = J_0(2 dt d_k) - 1, taps[k, x - 1] =
    J_x(2 dt d_k) times the sign of i^x, phase = -2 dt d_k."""
    r = ctypes.c_int32()
    c0, taps, ph = np.zeros(7), np.zeros(7 * max_radius), np.zeros(7)
    P = ctypes.POINTER(ctypes.c_double)
    _check(lib().nlc_dnls_stencil_coefficients(float(dt), int(max_radius), ctypes.byref(r), c0.ctypes.data_as(P),
                                               taps.ctypes.data_as(P), ph.ctypes.data_as(P)))
    return r.value, c0, taps.reshape(7, max_radius), ph


class Model:
    """Per-model options plus the gconf fields the kernels read (include/nlchains.h nlc_model)."""

    def __init__(self, model, chain_length, copies, dt, m=0.0, alpha=0.0, beta=0.0, masses=None,
                 entropy_mask=None, flags=0):
        self.model = MODELS[model] if isinstance(model, str) else int(model)
        self.chain_length, self.copies, self.dt = int(chain_length), int(copies), float(dt)
        self.m, self.alpha, self.beta, self.flags = float(m), float(alpha), float(beta), int(flags)
        self.masses = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64)
        self.entropy_mask = None if entropy_mask is None else np.ascontiguousarray(entropy_mask, dtype=np.uint8)

    @property
    def name(self):
        return MODEL_NAMES[self.model]

    @property
    def a0is0(self):
        """Mode 0 has zero frequency and is left out of the entropies (results.cpp:8)."""
        if self.model == MODELS["DNLS"]:
            return True
        if self.model == MODELS["dDNKG"]:
            return False
        return self.model != MODELS["DNKG"] or self.m == 0.0

    @property
    def state_shape(self):
        return (self.copies, self.chain_length, 2)

    def c_struct(self):
        s = _CModel(self.model, self.chain_length, self.copies, self.dt, self.m, self.alpha, self.beta,
                    None, None, self.flags)
        if self.masses is not None:
            s.masses = self.masses.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if self.entropy_mask is not None:
            s.entropy_mask = self.entropy_mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        return s


class Plan:
    """Level-1 operators on caller-owned device memory (pointers as integers, streams as handles)."""

    def __init__(self, model):
        self.model = model
        self._c = model.c_struct()
        self._h = ctypes.c_void_p()
        _check(lib().nlc_plan_create(ctypes.byref(self._c), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lib().nlc_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_state(self, state_ptr, seed, density, modes, first_copy=0, stream=0):
        """Seeded initial ensemble into device memory (nlc_initial_state; the ic.py recipes)."""
        m = np.ascontiguousarray(np.asarray(modes, dtype=np.uint32))
        _check(lib().nlc_initial_state(self._h, int(seed), int(first_copy), float(density),
                                       m.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(m),
                                       ctypes.c_void_p(state_ptr), ctypes.c_void_p(stream)))

    def move(self, state_ptr, steps, stream=0):
        _check(lib().nlc_move(self._h, ctypes.c_void_p(state_ptr), steps, ctypes.c_void_p(stream)))

    def linenergies(self, state_ptr, lin_ptr, entropies_ptr=0, stream=0):
        _check(lib().nlc_linenergies(self._h, ctypes.c_void_p(state_ptr), ctypes.c_void_p(lin_ptr),
                                     ctypes.c_void_p(entropies_ptr or None), ctypes.c_void_p(stream)))

    def energies(self, state_ptr, energies_ptr, stream=0):
        _check(lib().nlc_energies(self._h, ctypes.c_void_p(state_ptr), ctypes.c_void_p(energies_ptr),
                                  ctypes.c_void_p(stream)))

    def dnls_evolve_nonlinear(self, psi_ptr, coef, stream=0):
        _check(lib().nlc_dnls_evolve_nonlinear(self._h, ctypes.c_void_p(psi_ptr), coef, ctypes.c_void_p(stream)))

    def dnls_evolve_linear(self, psi_ptr, table_ptr=0, stream=0):
        _check(lib().nlc_dnls_evolve_linear(self._h, ctypes.c_void_p(psi_ptr), ctypes.c_void_p(table_ptr or None),
                                            ctypes.c_void_p(stream)))

    def shape(self):
        v = [ctypes.c_int32() for _ in range(4)]
        _check(lib().nlc_plan_shape(self._h, *[ctypes.byref(x) for x in v]))
        return {"lanes_per_chain": v[0].value, "sites_per_lane": v[1].value, "threads": v[2].value,
                "tier": v[3].value}

    def omegas(self):
        out = np.zeros(self.model.chain_length)
        _check(lib().nlc_plan_omegas(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out


class Context:
    """Level-2 engine context on one CUDA device."""

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        _check(lib().nlc_create(ctypes.byref(self._h), device))

    def close(self):
        if self._h:
            lib().nlc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def job(self, model, kernel_batching):
        return Job(self, model, kernel_batching)


class Job:
    """An ensemble with engine-owned device state (the reference's main-loop resources)."""

    def __init__(self, ctx, model, kernel_batching):
        self.ctx, self.model, self.batching = ctx, model, int(kernel_batching)
        self._c = model.c_struct()
        self.id = ctypes.c_uint64()
        _check(lib().nlc_job_create(ctx._h, ctypes.byref(self._c), self.batching, ctypes.byref(self.id)))

    def close(self):
        if self.id.value and self.ctx._h:
            lib().nlc_job_destroy(self.ctx._h, self.id)
            self.id = ctypes.c_uint64()

    def upload(self, state, wait=True):
        """Copy the ensemble to the device.  wait=False returns at once (the copy is asynchronous
        when `state` is pinned host memory, which must then stay alive until the job has used it)."""
        state = np.ascontiguousarray(state)
        assert state.nbytes == self.model.copies * self.model.chain_length * 16
        _check(lib().nlc_job_upload(self.ctx._h, self.id, state.ctypes.data_as(ctypes.c_void_p)))
        if wait:
            _check(lib().nlc_job_wait(self.ctx._h, self.id, -1))

    def advance(self, steps):
        _check(lib().nlc_job_advance(self.ctx._h, self.id, int(steps)))

    def wait(self, timeout_ms=-1):
        _check(lib().nlc_job_wait(self.ctx._h, self.id, int(timeout_ms)))

    def after(self, other):
        """Work enqueued on this job from now on starts after everything queued on `other` so far."""
        _check(lib().nlc_job_after(self.ctx._h, self.id, other.id))

    def linenergies(self):
        """(linenergies[n], WT entropy, information entropy); raises NlcError(EBLOWUP) on blow-up."""
        lin = np.zeros(self.model.chain_length)
        wt, inf = ctypes.c_double(), ctypes.c_double()
        _check(lib().nlc_job_linenergies(self.ctx._h, self.id, lin.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         ctypes.byref(wt), ctypes.byref(inf)))
        return lin, wt.value, inf.value

    def energies(self):
        """Energy of every chain of the current state (nlchains.m:40-48 definitions)."""
        out = np.zeros(self.model.copies)
        _check(lib().nlc_job_energies(self.ctx._h, self.id, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def sample_async(self, slot, copy_state=False):
        """Enqueue the diagnostics (and optionally a state copy) of the current state into slot 0/1."""
        _check(lib().nlc_job_sample_async(self.ctx._h, self.id, int(slot), int(bool(copy_state))))

    def step_async(self, slot, copy_state=False):
        """advance(kernel_batching) + sample_async(slot, copy_state) as one CUDA graph launch."""
        _check(lib().nlc_job_step_async(self.ctx._h, self.id, int(slot), int(bool(copy_state))))

    def sample_wait(self, slot, with_state=False, timeout_ms=-1):
        """(linenergies, WT, INF, state or None) of a slot filled by sample_async; EBLOWUP raises."""
        lin = np.zeros(self.model.chain_length)
        wt, inf = ctypes.c_double(), ctypes.c_double()
        state = np.empty((self.model.copies, self.model.chain_length, 2)) if with_state else None
        _check(lib().nlc_job_sample_wait(self.ctx._h, self.id, int(slot),
                                         lin.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(wt),
                                         ctypes.byref(inf), None if state is None else state.ctypes.data_as(ctypes.c_void_p),
                                         int(timeout_ms)))
        return lin, wt.value, inf.value, state

    def download(self, out=None):
        dtype_shape = (self.model.copies, self.model.chain_length, 2)
        out = np.empty(dtype_shape) if out is None else out
        _check(lib().nlc_job_download(self.ctx._h, self.id, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def state_ptr(self):
        p = ctypes.c_void_p()
        _check(lib().nlc_job_state_ptr(self.ctx._h, self.id, ctypes.byref(p)))
        return p.value


def linenergies_noalloc(model, chain_length, copies, m, state_ptr, lin_ptr, entropies_ptr=0, mask_ptr=0, stream=0):
    """nlc_linenergies_noalloc on caller device pointers (no device allocation inside)."""
    mid = MODELS[model] if isinstance(model, str) else int(model)
    _check(lib().nlc_linenergies_noalloc(mid, chain_length, copies, m, ctypes.c_void_p(state_ptr),
                                         ctypes.c_void_p(mask_ptr or None), ctypes.c_void_p(lin_ptr),
                                         ctypes.c_void_p(entropies_ptr or None), ctypes.c_void_p(stream)))


class Server:
    """Continuous-batching request server on one GPU (nlc_server_* in include/nlchains.h)."""

    def __init__(self, device=0, hbm_budget_bytes=0, max_active=0, streams=0, quantum_ms=0.0):
        cfg = _CServerConfig(device, hbm_budget_bytes, max_active, streams, quantum_ms)
        self._h = ctypes.c_void_p()
        _check(lib().nlc_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._models = {}

    def close(self):
        if self._h:
            lib().nlc_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model, kernel_batching, steps, state):
        state = np.ascontiguousarray(state, dtype=np.float64)
        assert state.size == 2 * model.chain_length * model.copies
        c = model.c_struct()
        rid = ctypes.c_uint64()
        _check(lib().nlc_server_submit(self._h, ctypes.byref(c), int(kernel_batching), int(steps),
                                       state.ctypes.data_as(ctypes.c_void_p), ctypes.byref(rid)))
        self._models[rid.value] = (model, int(steps), int(kernel_batching))
        return rid.value

    def submit_seeded(self, model, kernel_batching, steps, seed, density, modes):
        """A request whose initial state the server generates on the device (nlc_initial_state)."""
        m = np.ascontiguousarray(np.asarray(modes, dtype=np.uint32))
        c = model.c_struct()
        rid = ctypes.c_uint64()
        _check(lib().nlc_server_submit_seeded(self._h, ctypes.byref(c), int(kernel_batching), int(steps), int(seed),
                                              float(density), m.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                              len(m), ctypes.byref(rid)))
        self._models[rid.value] = (model, int(steps), int(kernel_batching))
        return rid.value

    def poll(self, rid):
        st = _CRequestStatus()
        _check(lib().nlc_server_poll(self._h, rid, ctypes.byref(st)))
        return {"state": st.state, "error": st.error, "steps_done": st.steps_done, "samples": st.samples,
                "submit_ms": st.submit_ms, "start_ms": st.start_ms, "ready_ms": st.ready_ms,
                "finish_ms": st.finish_ms}

    def wait(self, rid, timeout_ms=-1):
        _check(lib().nlc_server_wait(self._h, rid, int(timeout_ms)))

    def result(self, rid):
        """(final state, final linenergies, entropies[samples, 2], error code); forgets the request."""
        model, steps, b = self._models.pop(rid)
        state = np.empty((model.copies, model.chain_length, 2))
        lin = np.zeros(model.chain_length)
        ent = np.zeros(2 * (steps // b + 1))
        ns = ctypes.c_uint64()
        rc = lib().nlc_server_result(self._h, rid, state.ctypes.data_as(ctypes.c_void_p),
                                     lin.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     ent.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(ns))
        if rc not in (OK, EBLOWUP):
            _check(rc)
        return state, lin, ent[:2 * ns.value].reshape(-1, 2), rc


def run_program(argv):
    """The reference command line: run_program(["FPUT", "-i", "init", ...]) -> exit code."""
    args = [a.encode() if isinstance(a, str) else a for a in argv]
    arr = (ctypes.c_char_p * (len(args) + 1))(*args, None)
    return lib().nlc_program_run(len(args), arr)
