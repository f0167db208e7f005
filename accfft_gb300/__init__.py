"""GB300-native AccFFT single-GPU 3-D FFT path: Python binding of the C ABI.

The native library (accfft_gb300/lib/libaccfft_gb300.so, built by
``accfft_gb300.build``) implements AccFFT's single-rank GPU transforms and
spectral operators with hand-written sm_103a kernels.  This module binds its
C ABI (include/accfft_gb300.h) with ctypes and accepts either raw device
pointers (int) or CUDA torch tensors.  There is no fallback: if the library
is missing, ``lib()`` raises.

Mirrors AccFFT's API (include/accfft_gpu.h, include/accfft_gpuf.h,
include/accfft_operators_gpu.h in the reference):

    plan = PlanR2C((N0, N1, N2), "float32")         # accfft_plan_dft_3d_r2c_gpuf
    plan.r2c(u, u_hat)                              # accfft_execute_r2c_gpuf
    plan.c2r(u_hat, u2)                             # accfft_execute_c2r_gpuf
    plan.laplace(lap_u, u)                          # accfft_laplace_gpuf
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libaccfft_gb300.so")
API_LIB_PATH = os.path.join(HERE, "lib", "libaccfft_gpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "accfft_gb300.h")

ACCFFT_FORWARD = -1
ACCFFT_BACKWARD = +1
ACCFFT_ESTIMATE = 1
ACCFFT_MEASURE = 2
# float r2c plans with radix-16 stages on the tensor cores (include/accfft_gb300.h)
TC_TF32 = 0x100
TC_BF16 = 0x200
F64_DF = 0x400       # double plan computing in double-float on the FP32 pipes

OK, EINVAL, EUNSUPPORTED, ECUDA, ENOTBAKED, EOVERFLOW = range(6)

_lib = None


class AccfftError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"accfft_gb300 error {code}: {msg}")
        self.code = code


def header_symbols() -> list[str]:
    """Names of every function declared in include/accfft_gb300.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(accfft_c_\w+)\s*\(", txt)))


def lib() -> ctypes.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m accfft_gb300.build` first")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    ll, i, u = ctypes.c_longlong, ctypes.c_int, ctypes.c_uint
    sig = {
        "accfft_c_last_error": ([], ctypes.c_char_p),
        "accfft_c_last_error_code": ([], i),
        "accfft_c_version": ([], i),
        "accfft_c_length_supported": ([i], i),
        "accfft_c_length_generic": ([i], i),
        "accfft_c_line_plan": ([i, i, ip, ip, ip], i),
        "accfft_c_kernel_launches": ([], ctypes.c_ulonglong),
        "accfft_c_set_pdl": ([ctypes.c_int], ctypes.c_int),
        "accfft_c_set_wait_limit": ([ll], ll),
        "accfft_c_check": ([vp], i),
        "accfft_c_dfft_get_local_size": ([i, i, i, ip, ip, i], ll),
        "accfft_c_local_size_dft_r2c": ([ip, ip, ip, ip, ip, i], ll),
        "accfft_c_local_size_dft_c2c": ([ip, ip, ip, ip, ip, i], ll),
        "accfft_c_plan_dft_3d_r2c_gpu": ([ip, vp, vp, u], vp),
        "accfft_c_plan_dft_3d_r2c_gpuf": ([ip, vp, vp, u], vp),
        "accfft_c_plan_dft_3d_c2c_gpu": ([ip, vp, vp, u], vp),
        "accfft_c_plan_dft_3d_c2c_gpuf": ([ip, vp, vp, u], vp),
        "accfft_c_destroy_plan": ([vp], None),
        "accfft_c_plan_info": ([vp, ip, ip, ip, ip, ctypes.POINTER(ll)], i),
        "accfft_c_set_stream": ([vp, vp, i], i),
        "accfft_c_set_zy_schedule": ([vp, i], i),
        "accfft_c_set_pass_order": ([vp, i], i),
        "accfft_c_plan_tuning": ([vp, ip, ip, ip], i),
        "accfft_c_set_variants": ([vp, ip], i),
        "accfft_c_set_profiling": ([vp, i], i),
        "accfft_c_profile_read": ([vp, i, ctypes.c_char_p, ctypes.POINTER(ll), dp], i),
        "accfft_c_execute_r2c_gpu": ([vp, vp, vp, dp, u], i),
        "accfft_c_execute_c2r_gpu": ([vp, vp, vp, dp, u], i),
        "accfft_c_execute_gpu": ([vp, i, vp, vp, dp, u], i),
        "accfft_c_execute_c2c_gpu": ([vp, i, vp, vp, dp, u], i),
        "accfft_c_execute_r2c_gpuf": ([vp, vp, vp, dp, u], i),
        "accfft_c_execute_c2r_gpuf": ([vp, vp, vp, dp, u], i),
        "accfft_c_execute_gpuf": ([vp, i, vp, vp, dp, u], i),
        "accfft_c_execute_c2c_gpuf": ([vp, i, vp, vp, dp, u], i),
        "accfft_c_execute_r2c_axis": ([vp, i, vp, vp, dp], i),
        "accfft_c_execute_c2r_axis": ([vp, i, vp, vp, dp], i),
        "accfft_c_grad": ([vp, vp, vp, vp, vp, u, dp], i),
        "accfft_c_grad_slow": ([vp, vp, vp, vp, vp, u, dp], i),
        "accfft_c_laplace": ([vp, vp, vp, dp], i),
        "accfft_c_divergence": ([vp, vp, vp, vp, vp, dp], i),
        "accfft_c_divergence_slow": ([vp, vp, vp, vp, vp, dp], i),
        "accfft_c_biharmonic": ([vp, vp, vp, dp], i),
        "accfft_c_inv_laplace": ([vp, vp, vp, dp], i),
        "accfft_c_inv_biharmonic": ([vp, vp, vp, dp], i),
        "accfft_c_laplace_gpuf_noalloc": ([ip, vp, vp, vp], i),
        "accfft_c_heat": ([vp, vp, vp, ctypes.c_double, dp], i),
        "accfft_c_helmholtz": ([vp, vp, vp, ctypes.c_double, dp], i),
        "accfft_c_poisson": ([vp, vp, vp, i, dp], i),
        "accfft_c_r2c_adjoint": ([vp, vp, vp, dp], i),
        "accfft_c_c2r_adjoint": ([vp, vp, vp, dp], i),
        "accfft_c_grad_adjoint": ([vp, vp, vp, vp, vp, dp], i),
        "accfft_c_divergence_adjoint": ([vp, vp, vp, vp, vp, dp], i),
        "accfft_c_batch_create": ([], vp),
        "accfft_c_batch_destroy": ([vp], None),
        "accfft_c_batch_record": ([vp, vp, i], i),
        "accfft_c_batch_finalize": ([vp], i),
        "accfft_c_batch_run": ([vp, vp], i),
        "accfft_c_batch_info": ([vp, ip, ip, ip, ip], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def last_error() -> str:
    return lib().accfft_c_last_error().decode()


def kernel_launches() -> int:
    return int(lib().accfft_c_kernel_launches())


def line_plan(length: int, precision: str = "float32") -> dict:
    """The compiled radix plan of a line length (no plan, no GPU): first
    radix E, threads per line P and the stage radices.  ``precision`` is
    "float32", "float64" or "double-float"."""
    prec = {"float32": 0, "float64": 1, "double-float": 2}[precision]
    E, P = ctypes.c_int(0), ctypes.c_int(0)
    rad = (ctypes.c_int * 16)()
    ns = lib().accfft_c_line_plan(int(length), prec, ctypes.byref(E), ctypes.byref(P), rad)
    if ns < 0:
        raise AccfftError(EUNSUPPORTED, f"no radix plan for length {length}")
    return {"E": E.value, "P": P.value, "radices": [rad[s] for s in range(ns)]}


def set_pdl(mode: int | None = None) -> int:
    """Programmatic dependent launch of the pass kernels (each pass waits in
    hardware for the one before it): 0 off, 1 the next pass is released as
    this one's CTAs finish (the default), 2 as they start.  ``None`` only
    queries.  Returns the previous mode."""
    return int(lib().accfft_c_set_pdl(-1 if mode is None else int(mode)))


def set_wait_limit(polls: int | None = None) -> int:
    """Polls a bounded device-side wait makes before it gives up (tensor-core
    completion waits, the persistent z+y schedule's waits between items);
    ``None`` restores the default.  A wait that gives up makes the call raise
    AccfftError(ECUDA).  Returns the previous value."""
    return int(lib().accfft_c_set_wait_limit(-1 if polls is None else int(polls)))


def _check(rc: int):
    if rc != OK:
        raise AccfftError(rc, last_error())


def _ints(vals):
    return (ctypes.c_int * len(vals))(*vals)


def _ptr(x) -> int | None:
    """Address of a CUDA tensor or a pinned host tensor, an int pointer, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda and not x.is_pinned():
            raise ValueError("expected a CUDA tensor or a pinned host tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x.data_ptr()
    raise TypeError(f"cannot take a device pointer of {type(x).__name__}")


def local_size_r2c(n, real_bytes=8):
    """accfft_local_size_dft_r2c_gpu[f] (src/accfft_common.cpp:98-192) at P = 1."""
    isz, ist, osz, ost = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    amax = lib().accfft_c_local_size_dft_r2c(_ints(n), isz, ist, osz, ost, real_bytes)
    return int(amax), tuple(isz), tuple(ist), tuple(osz), tuple(ost)


def local_size_c2c(n, real_bytes=8):
    """accfft_local_size_dft_c2c_gpu[f] (src/accfft_common.cpp:203-256) at P = 1."""
    isz, ist, osz, ost = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    amax = lib().accfft_c_local_size_dft_c2c(_ints(n), isz, ist, osz, ost, real_bytes)
    return int(amax), tuple(isz), tuple(ist), tuple(osz), tuple(ost)


class _Plan:
    kind = 0

    # Python plans default to ACCFFT_ESTIMATE (the default kernels, no timing
    # at plan creation); pass flags=ACCFFT_MEASURE, the reference's default
    # and the C++ API's, to have a float r2c plan tune its passes
    def __init__(self, n, dtype="float32", data=None, data_out=None, flags=ACCFFT_ESTIMATE):
        self.n = tuple(int(v) for v in n)
        self.dtype = str(dtype).replace("torch.", "")
        if self.dtype not in ("float32", "float64"):
            raise ValueError("dtype must be float32 or float64")
        self.dbl = self.dtype == "float64"
        L = lib()
        fn = {(1, False): L.accfft_c_plan_dft_3d_r2c_gpuf, (1, True): L.accfft_c_plan_dft_3d_r2c_gpu,
              (2, False): L.accfft_c_plan_dft_3d_c2c_gpuf, (2, True): L.accfft_c_plan_dft_3d_c2c_gpu}[
            (self.kind, self.dbl)]
        d, o = _ptr(data), _ptr(data_out)
        self._h = fn(_ints(self.n), d, o, flags)
        if not self._h:
            raise AccfftError(L.accfft_c_last_error_code() or EINVAL, last_error())
        kind, dbl, inplace = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        amax = ctypes.c_longlong()
        _check(L.accfft_c_plan_info(self._h, None, ctypes.byref(kind), ctypes.byref(dbl), ctypes.byref(inplace),
                                    ctypes.byref(amax)))
        self.inplace = bool(inplace.value)
        self.alloc_max = int(amax.value)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream, blocking=False):
        """Enqueue on a CUDA stream (cudaStream_t as int, or a torch.cuda.Stream)."""
        s = getattr(stream, "cuda_stream", stream)
        _check(lib().accfft_c_set_stream(self._h, s, 1 if blocking else 0))

    def set_profiling(self, on=True):
        """bracket every kernel of this plan with CUDA events (read with profile())"""
        _check(lib().accfft_c_set_profiling(self._h, 1 if on else 0))

    def profile(self):
        """{pass label: (launches, total ms)} since the previous call"""
        n = 64
        labels = ctypes.create_string_buffer(32 * n)
        counts = (ctypes.c_longlong * n)()
        ms = (ctypes.c_double * n)()
        k = lib().accfft_c_profile_read(self._h, n, labels, counts, ms)
        raw = labels.raw
        return {raw[32 * i:32 * i + 32].split(b"\0")[0].decode(): (int(counts[i]), float(ms[i])) for i in range(k)}

    def set_zy_schedule(self, mode):
        """0: separate z and y passes (default); 1: cluster slab kernel;
        2: persistent z+y kernel (r2c plans, where the grid has the kernel)"""
        _check(lib().accfft_c_set_zy_schedule(self._h, int(mode)))

    def set_pass_order(self, order):
        """0: the reference's pass order (z, y, x); 1: packed (y and x over the
        real field viewed as complex, then mirror-paired z lines)"""
        _check(lib().accfft_c_set_pass_order(self._h, int(order)))

    def tuning(self) -> dict:
        """Radix / tile variants of the y, x, z r2c and z c2r passes (chosen by
        timing at plan creation with flags=ACCFFT_MEASURE; defaults otherwise):
        {"tuned": bool, pass: {"variant", "radix", "tile"}}"""
        v, r, t = (ctypes.c_int * 4)(), (ctypes.c_int * 4)(), (ctypes.c_int * 4)()
        tuned = lib().accfft_c_plan_tuning(self._h, v, r, t)
        out = {"tuned": bool(tuned)}
        for k, name in enumerate(("y", "x", "z_r2c", "z_c2r")):
            out[name] = {"variant": v[k], "radix": r[k], "tile": t[k]}
        return out

    def set_variants(self, y=0, x=0, z_r2c=0, z_c2r=0):
        """Force the radix / tile variants of the four passes (0 = default)."""
        _check(lib().accfft_c_set_variants(self._h, _ints([y, x, z_r2c, z_c2r])))

    def check(self):
        """Wait for the plan's stream; raise AccfftError(ECUDA) when a bounded
        device-side wait of an earlier non-blocking call gave up."""
        _check(lib().accfft_c_check(self._h))

    def destroy(self):
        if getattr(self, "_h", None):
            lib().accfft_c_destroy_plan(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    @staticmethod
    def _timer(timer):
        if timer is None:
            return None, None
        buf = (ctypes.c_double * 5)(*timer[:5])
        return buf, ctypes.cast(buf, ctypes.POINTER(ctypes.c_double))

    @staticmethod
    def _timer_back(buf, timer):
        if buf is not None:
            for k in range(5):
                timer[k] = buf[k]


class PlanR2C(_Plan):
    """accfft_plan_dft_3d_r2c_gpu / _gpuf: real [N0][N1][N2] <-> complex [N0][N1][N2/2+1]."""
    kind = 1

    def r2c(self, data, data_out, xyz=7, timer=None):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_execute_r2c_gpu if self.dbl else lib().accfft_c_execute_r2c_gpuf
        _check(f(self._h, _ptr(data), _ptr(data_out), tp, xyz))
        self._timer_back(buf, timer)

    def c2r(self, data, data_out, xyz=7, timer=None):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_execute_c2r_gpu if self.dbl else lib().accfft_c_execute_c2r_gpuf
        _check(f(self._h, _ptr(data), _ptr(data_out), tp, xyz))
        self._timer_back(buf, timer)

    def execute(self, direction, data, data_out, xyz=7, timer=None):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_execute_gpu if self.dbl else lib().accfft_c_execute_gpuf
        _check(f(self._h, direction, _ptr(data), _ptr(data_out), tp, xyz))
        self._timer_back(buf, timer)

    def r2c_axis(self, axis, data, data_out, timer=None):
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_execute_r2c_axis(self._h, axis, _ptr(data), _ptr(data_out), tp))
        self._timer_back(buf, timer)

    def c2r_axis(self, axis, data, data_out, timer=None):
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_execute_c2r_axis(self._h, axis, _ptr(data), _ptr(data_out), tp))
        self._timer_back(buf, timer)

    # ---- operators (accfft_operators_gpu.h)
    def grad(self, ax, ay, az, a, xyz=7, timer=None, slow=False):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_grad_slow if slow else lib().accfft_c_grad
        _check(f(self._h, _ptr(ax), _ptr(ay), _ptr(az), _ptr(a), xyz, tp))
        self._timer_back(buf, timer)

    def divergence(self, div, ax, ay, az, timer=None, slow=False):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_divergence_slow if slow else lib().accfft_c_divergence
        _check(f(self._h, _ptr(div), _ptr(ax), _ptr(ay), _ptr(az), tp))
        self._timer_back(buf, timer)

    # ---- spectral solvers
    def heat(self, out, a, t, timer=None):
        """exact heat propagator exp(t * laplace) applied to a"""
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_heat(self._h, _ptr(out), _ptr(a), float(t), tp))
        self._timer_back(buf, timer)

    def helmholtz(self, out, a, alpha, timer=None):
        """solve (alpha - laplace) out = a (zero mean part dropped where alpha + |k|^2 = 0)"""
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_helmholtz(self._h, _ptr(out), _ptr(a), float(alpha), tp))
        self._timer_back(buf, timer)

    def poisson(self, phi, rho, method=0, timer=None):
        """steps/step4's Poisson solve on the unit cube: method 0 uses the
        finite-difference Laplacian's eigenvalues, method 1 -4 pi^2 |k|^2"""
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_poisson(self._h, _ptr(phi), _ptr(rho), int(method), tp))
        self._timer_back(buf, timer)

    # ---- adjoints (backward passes of accfft_gb300.autograd)
    def r2c_adjoint(self, dX, du, timer=None):
        self._op("r2c_adjoint", dX, du, timer)

    def c2r_adjoint(self, dx, dY, timer=None):
        self._op("c2r_adjoint", dx, dY, timer)

    def grad_adjoint(self, out, gx, gy, gz, timer=None):
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_grad_adjoint(self._h, _ptr(out), _ptr(gx), _ptr(gy), _ptr(gz), tp))
        self._timer_back(buf, timer)

    def divergence_adjoint(self, ax, ay, az, d, timer=None):
        buf, tp = self._timer(timer)
        _check(lib().accfft_c_divergence_adjoint(self._h, _ptr(ax), _ptr(ay), _ptr(az), _ptr(d), tp))
        self._timer_back(buf, timer)

    def _op(self, name, first, second, timer):
        buf, tp = self._timer(timer)
        _check(getattr(lib(), "accfft_c_" + name)(self._h, _ptr(first), _ptr(second), tp))
        self._timer_back(buf, timer)

    def laplace(self, out, a, timer=None):
        self._op("laplace", out, a, timer)

    def biharmonic(self, out, a, timer=None):
        self._op("biharmonic", out, a, timer)

    def inv_laplace(self, out, a, timer=None):
        self._op("inv_laplace", out, a, timer)

    def inv_biharmonic(self, out, a, timer=None):
        self._op("inv_biharmonic", out, a, timer)


class PlanC2C(_Plan):
    """accfft_plan_dft_3d_c2c_gpu / _gpuf: complex [N0][N1][N2] (interleaved)."""
    kind = 2

    def c2c(self, direction, data, data_out, xyz=7, timer=None):
        buf, tp = self._timer(timer)
        f = lib().accfft_c_execute_c2c_gpu if self.dbl else lib().accfft_c_execute_c2c_gpuf
        _check(f(self._h, direction, _ptr(data), _ptr(data_out), tp, xyz))
        self._timer_back(buf, timer)


class Batch:
    """Independent transforms recorded pass by pass and run level by level,
    one grouped kernel per (pass kind, line length) and level
    (accfft_c_batch_* in include/accfft_gb300.h).

        b = Batch()
        with b.recording(plan):      # the plan's calls are recorded, not run
            plan.r2c(u, spec)
            plan.c2r(spec, back)
        b.finalize()
        b.run(stream)                # capturable into a CUDA graph
    """

    def __init__(self):
        self._b = lib().accfft_c_batch_create()

    def record(self, plan, on=True):
        _check(lib().accfft_c_batch_record(self._b, plan.handle, 1 if on else 0))

    def recording(self, plan):
        batch = self

        class _Rec:
            def __enter__(self):
                batch.record(plan, True)
                return plan

            def __exit__(self, *exc):
                batch.record(plan, False)
                return False

        return _Rec()

    def finalize(self):
        _check(lib().accfft_c_batch_finalize(self._b))

    def run(self, stream=None):
        s = 0 if stream is None else getattr(stream, "cuda_stream", stream)
        _check(lib().accfft_c_batch_run(self._b, s))

    def info(self) -> dict:
        vals = [ctypes.c_int() for _ in range(4)]
        _check(lib().accfft_c_batch_info(self._b, *[ctypes.byref(v) for v in vals]))
        return dict(zip(("instances", "levels", "launches", "tasks"), (v.value for v in vals)))

    def destroy(self):
        if getattr(self, "_b", None):
            lib().accfft_c_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
