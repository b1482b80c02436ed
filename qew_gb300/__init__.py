"""qew_gb300 -- GB300-native hot path of the quenched Edwards-Wilkinson line.

Python mirror of the reference's operator API (IMTEK-Simulation/qEW,
src/qew_model.h, src/filtered_noise.h, src/lbfgs.h, src/dynamics.h,
src/rosso_krauth.h) over the C ABI of ``include/qew_gpu.h``. Lines are CUDA
float64 torch tensors (torch supplies device memory and streams only); all
arithmetic runs in this package's own sm_103a kernels. Names, argument
meaning, defaults and error behaviour follow the reference:

=========================================  ====================================
reference                                  here
=========================================  ====================================
``Params``, ``Model``                      :class:`Params`, :class:`Model`
``FilteredNoise(field, nx, ny, Lx, Ly)``   :class:`FilteredNoise`
test stubs (ZeroNoise, HarmonicWell, ...)  :func:`ZeroNoise` etc.
``objective(h, p, noise)``                 :func:`objective`
``objective(x0, d, alpha, p, noise)``      :func:`objective_trial`
``gradient(h, p, noise, grad)``            :func:`gradient`
``lbfgs_minimize(h, p, noise, lp)``        :func:`lbfgs_minimize`
``LangevinDynamics(n, seed).step(...)``    :class:`LangevinDynamics`
``rk_site_velocity`` / ``rk_block``        :func:`rk_site_velocity`, :func:`rk_block`
``fire_minimize(h, p, noise, fp)``         :func:`fire_minimize`
``static_sweep`` / ``dynamic_anneal`` /    :func:`static_sweep`, :func:`dynamic_anneal`,
``depinning_ramp`` (qew_runs.h)            :func:`depinning_ramp`
=========================================  ====================================

``rk_block`` raises ``ValueError`` on an odd line length where the reference
throws ``std::invalid_argument``.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, fields

import numpy as np

from . import _capi
from ._capi import (QEW_FIELD_BSPLINE, QEW_FIELD_CONST, QEW_FIELD_HARMONIC,  # noqa: F401
                    QEW_FIELD_SINCOS, QEW_FIELD_WASHBOARD, QEW_FIELD_ZERO,
                    QEW_LBFGS_PLAIN, QEW_LBFGS_RESIDENT, QEW_PREC_FP32_SPLIT,
                    QEW_PREC_FP64, QEW_PREC_FP64_REFERENCE, QEW_RK_PLAIN, QEW_RK_RESIDENT,
                    QEW_STORE_FP32, QEW_STORE_FP32_EDGE, QEW_STORE_FP64, QEW_STORE_FP64_POLY,
                    QEW_TUNE_GRADIENT_POLY, QEW_TUNE_GRADIENT_SPLIT, QEW_TUNE_RK_SEARCH,
                    QEW_TUNE_LANGEVIN_RUN,
                    QewError)

__all__ = [
    "Model", "Params", "FilteredNoise", "ZeroNoise", "ConstNoise", "HarmonicWell",
    "SinusoidNoise", "AnalyticNoise", "objective", "objective_trial", "gradient",
    "gradient_batch", "gradient_host", "gradient_host_batch", "split_heights", "join_heights", "gradient_split", "gradient_split_batch",
    "LbfgsParams", "LbfgsResult", "lbfgs_minimize", "ensemble_minimize",
    "precond_apply",
    "LangevinDynamics", "RkParams", "RkResult", "rk_site_velocity", "rk_block",
    "depinning_bisect", "depinning_bisect_report", "BisectResult", "Context", "default_context", "QewError", "Server",
    "StaticConfig", "StaticProfile", "static_sweep", "DynamicConfig", "DynamicSnapshot",
    "DynamicResult", "dynamic_anneal", "DepinningConfig", "DepinningStep", "DepinningResult",
    "depinning_ramp", "FireParams", "FireResult", "fire_minimize", "line_statistics",
    "tune_report",
]


def _torch():
    import torch
    return torch


class Model(enum.IntEnum):  # qew_model.h:20
    Linear = 0
    Arclength = 1


@dataclass
class Params:  # qew_model.h:22-27
    physical_size: float = 1.0
    line_tension: float = 1.0
    driving_force: float = 0.0
    model: Model = Model.Linear

    def c(self) -> _capi.qew_params:
        return _capi.qew_params(float(self.physical_size), float(self.line_tension),
                                float(self.driving_force), int(self.model))


@dataclass
class LbfgsParams:  # lbfgs.h:32-52
    m: int = 8
    ftol: float = 1e-6
    max_iter: int = 10000
    c1: float = 1e-4
    ls_shrink: float = 0.5
    max_ls: int = 30
    curvature_eps: float = 1e-12
    precondition: bool = False
    precond_shift: float = 0.0
    ls_fallback: bool = False  # extension: approximate-Wolfe fallback (see qew_gpu.h)

    def c(self) -> _capi.qew_lbfgs_params:
        return _capi.qew_lbfgs_params(int(self.m), float(self.ftol), int(self.max_iter),
                                      float(self.c1), float(self.ls_shrink), int(self.max_ls),
                                      float(self.curvature_eps), int(bool(self.precondition)),
                                      float(self.precond_shift), int(bool(self.ls_fallback)))


@dataclass
class LbfgsResult:  # lbfgs.h:54-61
    iterations: int = 0
    max_force: float = 0.0
    converged: bool = False
    n_func_evals: int = 0
    n_curvature_skips: int = 0
    n_ls_restarts: int = 0


@dataclass
class RkParams:  # rosso_krauth.h:34-41
    dstep: float = 0.0
    max_advance: float = 0.0
    root_tol: float = 1e-10
    sweep_tol: float = 1e-9
    runaway: float = 0.0
    max_sweeps: int = 200000

    def c(self) -> _capi.qew_rk_params:
        return _capi.qew_rk_params(float(self.dstep), float(self.max_advance),
                                   float(self.root_tol), float(self.sweep_tol),
                                   float(self.runaway), int(self.max_sweeps))


@dataclass
class RkResult:  # rosso_krauth.h:43-49
    blocked: bool = False
    runaway: bool = False
    sweeps: int = 0
    total_advance: float = 0.0
    mean_h: float = 0.0


# ---------------------------------------------------------------- context
class Context:
    """One qew_ctx (device, stream, reduction and workspace arenas)."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        self.device = device
        h = C.c_void_p()
        _capi.check(self.lib.qew_ctx_create(device, C.byref(h)), None, "qew_ctx_create")
        self.h = h

    def sync_stream(self):
        """Run subsequent work on torch's current stream of this device."""
        torch = _torch()
        s = torch.cuda.current_stream(self.device).cuda_stream
        self.lib.qew_ctx_set_stream(self.h, C.c_void_p(s))

    def launches(self) -> int:
        return int(self.lib.qew_ctx_launch_count(self.h))

    def synchronize(self):
        _capi.check(self.lib.qew_ctx_synchronize(self.h), self.h, "synchronize")

    def set_barrier_limits(self, max_polls: int = 0, skip_block: int = -1):
        """Grid-barrier poll limit (0: default) and a CTA that skips its
        arrival (-1: none) for this context's later persistent launches."""
        _capi.check(self.lib.qew_ctx_set_barrier_limits(self.h, int(max_polls), int(skip_block)),
                    self.h, "set_barrier_limits")

    def set_autotune(self, on: bool = True):
        """Launch shapes by measurement (True) or the hand-chosen defaults."""
        _capi.check(self.lib.qew_ctx_set_autotune(self.h, int(bool(on))), self.h, "autotune")

    def force_tune_candidate(self, kernel: int, candidate: int = -1):
        """Fix one tuned kernel's launch shape for this context (-1: release)."""
        _capi.check(self.lib.qew_ctx_force_tune_candidate(self.h, int(kernel), int(candidate)),
                    self.h, "force_tune_candidate")

    def measure_fp64_fma_rate(self, iters: int = 4096):
        """(FP64 FMA instructions per second, timed ms) of this GPU."""
        self.sync_stream()
        rate, ms = C.c_double(), C.c_double()
        _capi.check(self.lib.qew_measure_fp64_fma_rate(self.h, int(iters), C.byref(rate),
                                                       C.byref(ms)),
                    self.h, "measure_fp64_fma_rate")
        return rate.value, ms.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.lib.qew_ctx_destroy(self.h)
                self.h = None
        except Exception:
            pass


def tune_report() -> str:
    """The autotuner's choices in this process (qew_tune_report)."""
    lib = _capi.load()
    n = lib.qew_tune_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    lib.qew_tune_report(buf, n + 1)
    return buf.value.decode()


def bounds_check_report() -> dict | None:
    """Out-of-range device indices since the last call (qew_bounds_check_report):
    {"count", "index", "bound", "line"}; None in the normal (unchecked) build."""
    out = (C.c_longlong * 4)()
    st = _capi.load().qew_bounds_check_report(out)
    if st == _capi.QEW_ERR_UNSUPPORTED:
        return None
    _capi.check(st, None, "bounds_check_report")
    return dict(zip(("count", "index", "bound", "line"), (int(v) for v in out)))


_contexts: dict[int, Context] = {}


def default_context(device: int | None = None) -> Context:
    torch = _torch()
    if device is None:
        device = torch.cuda.current_device()
    ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        _contexts[device] = ctx
    ctx.sync_stream()
    return ctx


def _ptr(t) -> C.c_void_p:
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if t.dtype != torch.float64 or not t.is_contiguous():
        raise ValueError("expected a contiguous float64 CUDA tensor")
    return C.c_void_p(t.data_ptr())


# ------------------------------------------------------------------ noise
class _Noise:
    kind: int = -1

    def __init__(self):
        self.h = None
        self.ctx = None

    def __del__(self):
        try:
            if self.h:
                self.ctx.lib.qew_field_destroy(self.h)
                self.h = None
        except Exception:
            pass


class FilteredNoise(_Noise):
    """FilteredNoise(field, nx, ny, Lx, Ly) (filtered_noise.h:183-189).

    ``field`` is the real-space field in the reference's host layout
    ``field[i, j]`` (i along x, j along y), as a numpy array or a CUDA tensor.
    The periodic cubic B-spline prefilter runs on the GPU. ``store`` selects
    FP64 and/or FP32 coefficient storage; QEW_STORE_FP32_EDGE (with FP32) adds
    the x-filtered copy that the split-form gradient reads on a line with one
    point per field column (4 taps per edge instead of 16); QEW_STORE_FP64_POLY
    (with FP64) adds the FP64 cell polynomials of the x-filtered field, which
    the FP64 gradient on such a line reads (one 32-byte cell and two FMAs per
    edge instead of the 16-tap sum).
    """

    kind = QEW_FIELD_BSPLINE

    def __init__(self, field, Lx: float, Ly: float, store: int = QEW_STORE_FP64,
                 ctx: Context | None = None):
        super().__init__()
        self.ctx = ctx or default_context()
        torch = _torch()
        h = C.c_void_p()
        if isinstance(field, torch.Tensor):
            f = field.contiguous()
            nx, ny = f.shape
            _capi.check(self.ctx.lib.qew_field_create_from_device(
                self.ctx.h, _ptr(f), nx, ny, float(Lx), float(Ly), store, C.byref(h)),
                self.ctx.h, "FilteredNoise")
        else:
            f = np.ascontiguousarray(field, dtype=np.float64)
            nx, ny = f.shape
            _capi.check(self.ctx.lib.qew_field_create_from_host(
                self.ctx.h, f.ctypes.data_as(_capi.PD), nx, ny, float(Lx), float(Ly), store,
                C.byref(h)), self.ctx.h, "FilteredNoise")
        self.h = h
        self.nx, self.ny, self.Lx, self.Ly = nx, ny, float(Lx), float(Ly)
        self.dx, self.dy = self.Lx / nx, self.Ly / ny
        self.store = store

    @classmethod
    def generated(cls, nx: int, ny: int, Lx: float, Ly: float, amplitude: float,
                  xi_x_cells: float, xi_y_cells: float, seed: int,
                  store: int = QEW_STORE_FP64, ctx: Context | None = None) -> "FilteredNoise":
        """A synthetic Gaussian-filtered field generated on the device."""
        self = cls.__new__(cls)
        _Noise.__init__(self)
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _capi.check(self.ctx.lib.qew_field_create_generated(
            self.ctx.h, int(nx), int(ny), float(Lx), float(Ly), float(amplitude),
            float(xi_x_cells), float(xi_y_cells), int(seed), int(store), C.byref(h)),
            self.ctx.h, "FilteredNoise.generated")
        self.h = h
        self.nx, self.ny, self.Lx, self.Ly = int(nx), int(ny), float(Lx), float(Ly)
        self.dx, self.dy = self.Lx / nx, self.Ly / ny
        self.store = store
        return self

    @classmethod
    def seeded(cls, nx: int, ny: int, Lx: float, Ly: float, amplitude: float, xi_x: float,
               xi_y: float, seed: int, store: int = QEW_STORE_FP64,
               ctx: Context | None = None) -> "FilteredNoise":
        """FilteredNoise(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed): the
        reference's seeded constructor (filtered_noise.cpp:25-82)."""
        self = cls.__new__(cls)
        _Noise.__init__(self)
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _capi.check(self.ctx.lib.qew_field_create_seeded(
            self.ctx.h, int(nx), int(ny), float(Lx), float(Ly), float(amplitude),
            float(xi_x), float(xi_y), int(seed), int(store), C.byref(h)),
            self.ctx.h, "FilteredNoise.seeded")
        self.h = h
        self.nx, self.ny, self.Lx, self.Ly = int(nx), int(ny), float(Lx), float(Ly)
        self.dx, self.dy = self.Lx / nx, self.Ly / ny
        self.store = store
        return self

    def coefficients(self) -> np.ndarray:
        """The FP64 B-spline coefficients in the host layout [nx][ny]."""
        out = np.empty((self.nx, self.ny))
        _capi.check(self.ctx.lib.qew_field_get_coefficients(
            self.ctx.h, self.h, out.ctypes.data_as(_capi.PD)), self.ctx.h, "coefficients")
        return out

    def sample(self, x, y):
        return sample(self, x, y)


class _Analytic(_Noise):
    def __init__(self, kind, p0=0.0, p1=0.0, p2=0.0, ctx: Context | None = None):
        super().__init__()
        self.ctx = ctx or default_context()
        self.kind = kind
        self.params = (p0, p1, p2)
        h = C.c_void_p()
        _capi.check(self.ctx.lib.qew_field_create_analytic(self.ctx.h, kind, p0, p1, p2,
                                                           C.byref(h)), self.ctx.h, "noise")
        self.h = h

    def sample(self, x, y):
        return sample(self, x, y)


def ZeroNoise(ctx=None):  # test_lbfgs.cpp:24-27
    return _Analytic(QEW_FIELD_ZERO, ctx=ctx)


def ConstNoise(v0: float = 0.0, ctx=None):  # test_qew_model.cpp:38-42
    return _Analytic(QEW_FIELD_CONST, v0, ctx=ctx)


def HarmonicWell(k: float = 2.0, y0: float = 0.5, ctx=None):  # test_lbfgs.cpp:30-38
    return _Analytic(QEW_FIELD_HARMONIC, k, y0, ctx=ctx)


def SinusoidNoise(A: float = 0.1, k: float = 2.0 * 3.14159265358979323846, ctx=None):
    return _Analytic(QEW_FIELD_WASHBOARD, A, k, ctx=ctx)  # test_rosso_krauth.cpp:24-31


def AnalyticNoise(amp: float = 0.3, kx: float = 0.7, ky: float = 1.3, ctx=None):
    return _Analytic(QEW_FIELD_SINCOS, amp, kx, ky, ctx=ctx)  # test_qew_model.cpp:22-34


def sample(noise: _Noise, x, y):
    """DeviceNoise::sample at points (x, y): returns (v, dv_dx, dv_dy) tensors."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    x = torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()
    y = torch.as_tensor(y, dtype=torch.float64, device="cuda").contiguous()
    v, dx, dy = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    _capi.check(ctx.lib.qew_field_sample(ctx.h, noise.h, _ptr(x), _ptr(y), x.numel(), _ptr(v),
                                         _ptr(dx), _ptr(dy)), ctx.h, "sample")
    return v, dx, dy


# ------------------------------------------------------------------ model
def objective(h, p: Params, noise: _Noise) -> float:
    ctx = noise.ctx
    ctx.sync_stream()
    out = C.c_double()
    pc = p.c()
    _capi.check(ctx.lib.qew_objective(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                      C.byref(out)), ctx.h, "objective")
    return out.value


def objective_trial(x0, d, alpha: float, p: Params, noise: _Noise) -> float:
    ctx = noise.ctx
    ctx.sync_stream()
    out = C.c_double()
    pc = p.c()
    _capi.check(ctx.lib.qew_objective_trial(ctx.h, noise.h, _ptr(x0), _ptr(d), float(alpha),
                                            x0.numel(), C.byref(pc), C.byref(out)),
                ctx.h, "objective_trial")
    return out.value


def gradient(h, p: Params, noise: _Noise, grad=None, precision: int = QEW_PREC_FP64):
    """gradient(h, p, noise, grad) -- writes and returns grad (allocated if None)."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    if grad is None:
        grad = torch.empty_like(h)
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_prec(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                          precision, _ptr(grad)), ctx.h, "gradient")
    return grad


def gradient_batch(h, p: Params, noise: _Noise, grad=None, precision: int = QEW_PREC_FP64):
    """gradient() of every row of a contiguous [count, n] FP64 CUDA tensor,
    one launch when the field's FP64 cell-polynomial store serves the lines."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    if h.dim() != 2 or not h.is_contiguous() or h.dtype != torch.float64:
        raise ValueError("expected a contiguous float64 [count, n] tensor")
    if grad is None:
        grad = torch.empty_like(h)
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_batch(ctx.h, noise.h, h.shape[0], _ptr(h), h.shape[1],
                                           C.byref(pc), precision, _ptr(grad)),
                ctx.h, "gradient_batch")
    return grad


def gradient_host(h: np.ndarray, p: Params, noise: _Noise, out: np.ndarray | None = None,
                  precision: int = QEW_PREC_FP64) -> np.ndarray:
    """Gradient of a host (numpy, ideally pinned) line into a host array."""
    ctx = noise.ctx
    ctx.sync_stream()
    if out is None:
        out = np.empty_like(h)
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_host(ctx.h, noise.h, C.c_void_p(h.ctypes.data), h.size,
                                          C.byref(pc), precision, C.c_void_p(out.ctypes.data)),
                ctx.h, "gradient_host")
    return out


def gradient_host_batch(h: np.ndarray, p: Params, noise: _Noise, out: np.ndarray | None = None,
                        precision: int = QEW_PREC_FP64) -> np.ndarray:
    """Gradients of the rows of a host array h[count, n] (ideally pinned), the
    copies of consecutive rows overlapped with the gradients on the device."""
    ctx = noise.ctx
    ctx.sync_stream()
    h = np.ascontiguousarray(h, dtype=np.float64)
    if h.ndim != 2:
        raise ValueError("h must be [count, n]")
    if out is None:
        out = np.empty_like(h)
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_host_batch(ctx.h, noise.h, h.shape[0],
                                                C.c_void_p(h.ctypes.data), h.shape[1],
                                                C.byref(pc), precision,
                                                C.c_void_p(out.ctypes.data)),
                ctx.h, "gradient_host_batch")
    return out


def split_heights(h, noise: "FilteredNoise"):
    """FP64 heights -> (int32 cell, float32 fraction) in field y-cells."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    cell = torch.empty(h.numel(), dtype=torch.int32, device="cuda")
    frac = torch.empty(h.numel(), dtype=torch.float32, device="cuda")
    _capi.check(ctx.lib.qew_split_heights(ctx.h, noise.h, _ptr(h), h.numel(),
                                          C.c_void_p(cell.data_ptr()),
                                          C.c_void_p(frac.data_ptr())), ctx.h, "split_heights")
    return cell, frac


def join_heights(cell, frac, noise: "FilteredNoise"):
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    h = torch.empty(cell.numel(), dtype=torch.float64, device="cuda")
    _capi.check(ctx.lib.qew_join_heights(ctx.h, noise.h, C.c_void_p(cell.data_ptr()),
                                         C.c_void_p(frac.data_ptr()), cell.numel(), _ptr(h)),
                ctx.h, "join_heights")
    return h


def gradient_split(cell, frac, p: Params, noise: "FilteredNoise", grad=None):
    """gradient() on split heights with FP32 output (the bandwidth form)."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    if cell.dtype != torch.int32 or frac.dtype != torch.float32:
        raise ValueError("expected int32 cells and float32 fractions")
    if grad is None:
        grad = torch.empty(cell.numel(), dtype=torch.float32, device="cuda")
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_split(ctx.h, noise.h, C.c_void_p(cell.data_ptr()),
                                           C.c_void_p(frac.data_ptr()), cell.numel(),
                                           C.byref(pc), C.c_void_p(grad.data_ptr())),
                ctx.h, "gradient_split")
    return grad


def gradient_split_batch(cells, fracs, p: Params, noise: "FilteredNoise", grads=None):
    """gradient_split for a [count, n] batch of lines on one field, one launch."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    if cells.dim() != 2 or cells.shape != fracs.shape or not cells.is_contiguous() \
            or not fracs.is_contiguous():
        raise ValueError("expected contiguous [count, n] cells and fractions")
    if cells.dtype != torch.int32 or fracs.dtype != torch.float32:
        raise ValueError("expected int32 cells and float32 fractions")
    count, n = cells.shape
    if grads is None:
        grads = torch.empty((count, n), dtype=torch.float32, device="cuda")
    pc = p.c()
    _capi.check(ctx.lib.qew_gradient_split_batch(ctx.h, noise.h, count,
                                                 C.c_void_p(cells.data_ptr()),
                                                 C.c_void_p(fracs.data_ptr()), n, C.byref(pc),
                                                 C.c_void_p(grads.data_ptr())),
                ctx.h, "gradient_split_batch")
    return grads


# ----------------------------------------------------------------- L-BFGS
def lbfgs_minimize(h, p: Params, noise: _Noise, lp: LbfgsParams | None = None,
                   form: int = QEW_LBFGS_RESIDENT) -> LbfgsResult:
    """lbfgs_minimize(h, p, noise, lp): relaxes h in place (lbfgs.h:94-96)."""
    ctx = noise.ctx
    ctx.sync_stream()
    lp = lp or LbfgsParams()
    lpc, pc, res = lp.c(), p.c(), _capi.qew_lbfgs_result()
    _capi.check(ctx.lib.qew_lbfgs_minimize_form(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                                C.byref(lpc), form, C.byref(res)),
                ctx.h, "lbfgs_minimize")
    return LbfgsResult(res.iterations, res.max_force, bool(res.converged), res.n_func_evals,
                       res.n_curvature_skips, res.n_ls_restarts)


def ensemble_minimize(lines, lp: LbfgsParams, ftol_fp32: float = 0.0, max_iter_fp32: int = 0,
                      ctx: Context | None = None) -> list[LbfgsResult]:
    """Relax many independent lines in one persistent launch.

    ``lines`` is a list of (h, params, noise, precond_shift) with h a CUDA
    float64 tensor relaxed in place. With ftol_fp32 > 0 each line is first
    relaxed on the FP32 split gather, then refined in FP64 to lp.ftol.
    """
    ctx = ctx or default_context()
    ctx.sync_stream()
    n = len(lines)
    arr = (_capi.qew_ensemble_line * max(n, 1))()
    for k, (h, p, noise, shift) in enumerate(lines):
        arr[k].field = noise.h
        arr[k].d_h = _ptr(h)
        arr[k].n = h.numel()
        arr[k].p = p.c()
        arr[k].precond_shift = float(shift)
    ep = _capi.qew_ensemble_params(lp.c(), float(ftol_fp32), int(max_iter_fp32))
    res = (_capi.qew_lbfgs_result * max(n, 1))()
    _capi.check(ctx.lib.qew_ensemble_minimize(ctx.h, n, arr, C.byref(ep), res), ctx.h,
                "ensemble_minimize")
    return [LbfgsResult(r.iterations, r.max_force, bool(r.converged), r.n_func_evals,
                        r.n_curvature_skips, r.n_ls_restarts) for r in res[:n]]


def precond_apply(q, line_tension: float, physical_size: float, shift: float,
                  form: int = QEW_LBFGS_RESIDENT, ctx: Context | None = None):
    """The L-BFGS preconditioner d = M^{-1} q alone (lbfgs.h:116-146, 173-180)."""
    torch = _torch()
    ctx = ctx or default_context()
    ctx.sync_stream()
    out = torch.empty_like(q)
    _capi.check(ctx.lib.qew_precond_apply(ctx.h, _ptr(q), q.numel(), float(line_tension),
                                          float(physical_size), float(shift), form, _ptr(out)),
                ctx.h, "precond_apply")
    return out


# --------------------------------------------------------------- Langevin
class LangevinDynamics:
    """LangevinDynamics(n, seed) (dynamics.h:27-70)."""

    def __init__(self, n: int, seed: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _capi.check(self.ctx.lib.qew_langevin_create(self.ctx.h, int(n), int(seed), C.byref(h)),
                    self.ctx.h, "LangevinDynamics")
        self.h = h
        self.n = int(n)

    def step(self, h, p: Params, noise: _Noise, drift_coeff: float, diff_coeff: float):
        self.ctx.sync_stream()
        if h.numel() != self.n:
            raise ValueError("line length %d != %d" % (h.numel(), self.n))
        pc = p.c()
        _capi.check(self.ctx.lib.qew_langevin_step(self.h, noise.h, _ptr(h), C.byref(pc),
                                                   float(drift_coeff), float(diff_coeff)),
                    self.ctx.h, "langevin step")

    def step_with_increments(self, h, p: Params, noise: _Noise, drift_coeff: float,
                             diff_coeff: float, xi):
        self.ctx.sync_stream()
        if h.numel() != self.n or xi.numel() != self.n:
            raise ValueError("line/increment length mismatch")
        pc = p.c()
        _capi.check(self.ctx.lib.qew_langevin_step_increments(
            self.h, noise.h, _ptr(h), C.byref(pc), float(drift_coeff), float(diff_coeff),
            _ptr(xi)), self.ctx.h, "langevin step")

    def run(self, h, p: Params, noise: _Noise, drift, diff, precision: int = QEW_PREC_FP64):
        """len(drift) steps with per-step coefficients, in one device-resident launch."""
        self.ctx.sync_stream()
        drift = np.ascontiguousarray(drift, dtype=np.float64)
        diff = np.ascontiguousarray(diff, dtype=np.float64)
        if drift.shape != diff.shape or drift.ndim != 1 or h.numel() != self.n:
            raise ValueError("schedule / line length mismatch")
        pc = p.c()
        _capi.check(self.ctx.lib.qew_langevin_run(
            self.h, noise.h, _ptr(h), C.byref(pc), drift.size, drift.ctypes.data_as(_capi.PD),
            diff.ctypes.data_as(_capi.PD), int(precision)), self.ctx.h, "langevin run")

    def peek_increments(self):
        torch = _torch()
        self.ctx.sync_stream()
        out = torch.empty(self.n, dtype=torch.float64, device="cuda")
        _capi.check(self.ctx.lib.qew_langevin_peek_increments(self.h, _ptr(out)), self.ctx.h,
                    "peek_increments")
        return out

    @property
    def steps(self) -> int:
        return int(self.ctx.lib.qew_langevin_steps(self.h))

    def __del__(self):
        try:
            if self.h:
                self.ctx.lib.qew_langevin_destroy(self.h)
                self.h = None
        except Exception:
            pass


# ----------------------------------------------------------- Rosso-Krauth
def rk_site_velocity(h, p: Params, noise: _Noise):
    """rk_site_velocity (rosso_krauth.h:51-82) of every site of h."""
    torch = _torch()
    ctx = noise.ctx
    ctx.sync_stream()
    out = torch.empty_like(h)
    pc = p.c()
    _capi.check(ctx.lib.qew_rk_site_velocity(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                             _ptr(out)), ctx.h, "rk_site_velocity")
    return out


def rk_block(h, p: Params, noise: _Noise, rp: RkParams, form: int | None = None,
             precision: int = QEW_PREC_FP64) -> RkResult:
    """rk_block(h, p, noise, rp) (rosso_krauth.h:128-194); ValueError on odd n.

    form: None (the library default, the resident kernel), QEW_RK_PLAIN or
    QEW_RK_RESIDENT; precision QEW_PREC_FP32_SPLIT needs FP32 storage."""
    ctx = noise.ctx
    ctx.sync_stream()
    pc, rpc, res = p.c(), rp.c(), _capi.qew_rk_result()
    if form is None and precision == QEW_PREC_FP64:
        st = ctx.lib.qew_rk_block(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc), C.byref(rpc),
                                  C.byref(res))
    else:
        st = ctx.lib.qew_rk_block_form(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                       C.byref(rpc), _capi.QEW_RK_RESIDENT if form is None else
                                       int(form), int(precision), C.byref(res))
    _capi.check(st, ctx.h, "rk_block")
    return RkResult(bool(res.blocked), bool(res.runaway), res.sweeps, res.total_advance,
                    res.mean_h)


def depinning_bisect(h, p: Params, noise: _Noise, rp: RkParams, f_lo: float, f_hi: float,
                     rtol: float = 1e-10, max_steps: int = 200,
                     precision: int = QEW_PREC_FP64):
    """Bisect the depinning force from a blocked h at f_lo; see qew_gpu.h."""
    ctx = noise.ctx
    ctx.sync_stream()
    pc, rpc = p.c(), rp.c()
    fc, flo, fhi, nb = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    _capi.check(ctx.lib.qew_depinning_bisect_prec(
        ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc), C.byref(rpc), float(f_lo), float(f_hi),
        float(rtol), int(max_steps), int(precision), C.byref(fc), C.byref(flo), C.byref(fhi),
        C.byref(nb)), ctx.h, "depinning_bisect")
    return fc.value, flo.value, fhi.value, nb.value


@dataclass
class BisectResult:
    """qew_bisect_result plus the verdict of every block (0 blocked, 1
    runaway, 2 max_sweeps reached)."""
    f_c: float
    f_lo: float
    f_hi: float
    blocks: int
    n_blocked: int
    n_runaway: int
    n_timeout: int
    f_hi_verdict: int
    sweeps: int
    verdicts: list


def depinning_bisect_report(h, p: Params, noise: _Noise, rp: RkParams, f_lo: float,
                            f_hi: float, rtol: float = 1e-10, max_steps: int = 200,
                            precision: int = QEW_PREC_FP64) -> BisectResult:
    """depinning_bisect with each block's verdict (qew_depinning_bisect_ex)."""
    ctx = noise.ctx
    ctx.sync_stream()
    pc, rpc = p.c(), rp.c()
    r = _capi.qew_bisect_result()
    verdicts = (C.c_int * max(int(max_steps), 1))()
    _capi.check(ctx.lib.qew_depinning_bisect_ex(
        ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc), C.byref(rpc), float(f_lo), float(f_hi),
        float(rtol), int(max_steps), int(precision), C.byref(r), verdicts),
        ctx.h, "depinning_bisect")
    return BisectResult(r.f_c, r.f_lo, r.f_hi, r.blocks, r.n_blocked, r.n_runaway, r.n_timeout,
                        r.f_hi_verdict, r.sweeps, list(verdicts[:r.blocks]))


# ------------------------------------------------------------------- FIRE
@dataclass
class FireParams:  # fire.h:21-31
    dt_max: float = 0.0  # required, > 0
    dt_init: float = 0.0
    ftol: float = 1e-6
    max_iter: int = 100000
    n_min: int = 5
    f_inc: float = 1.1
    f_dec: float = 0.5
    alpha_start: float = 0.1
    f_alpha: float = 0.99

    def c(self) -> _capi.qew_fire_params:
        return _capi.qew_fire_params(float(self.dt_max), float(self.dt_init), float(self.ftol),
                                     int(self.max_iter), int(self.n_min), float(self.f_inc),
                                     float(self.f_dec), float(self.alpha_start),
                                     float(self.f_alpha))


@dataclass
class FireResult:  # fire.h:33-37
    iterations: int = 0
    max_force: float = 0.0
    converged: bool = False


def fire_minimize(h, p: Params, noise: _Noise, fp: FireParams) -> FireResult:
    """fire_minimize(h, p, noise, fp), fire.h:41-131: relaxes h in place."""
    ctx = noise.ctx
    ctx.sync_stream()
    pc, fc, res = p.c(), fp.c(), _capi.qew_fire_result()
    _capi.check(ctx.lib.qew_fire_minimize(ctx.h, noise.h, _ptr(h), h.numel(), C.byref(pc),
                                          C.byref(fc), C.byref(res)), ctx.h, "fire_minimize")
    return FireResult(res.iterations, res.max_force, bool(res.converged))


# ------------------------------------------------------------- statistics
def line_statistics(h, physical_size: float, ctx: Context | None = None):
    """(ell, acf, q, psd) of periodic lines h[n] or h[count, n] (CUDA float64),
    with the definitions of qew_line_statistics in include/qew_gpu.h."""
    torch = _torch()
    ctx = ctx or default_context()
    ctx.sync_stream()
    h2 = h.reshape(1, -1) if h.dim() == 1 else h
    h2 = h2.contiguous()
    count, n = h2.shape
    nh = n // 2 + 1
    kw = dict(dtype=torch.float64, device=h2.device)
    ell, q = torch.empty(nh, **kw), torch.empty(nh, **kw)
    acf, psd = torch.empty((count, nh), **kw), torch.empty((count, nh), **kw)
    _capi.check(ctx.lib.qew_line_statistics(ctx.h, count, _ptr(h2), n, float(physical_size),
                                            _ptr(ell), _ptr(acf), _ptr(q), _ptr(psd)),
                ctx.h, "line_statistics")
    if h.dim() == 1:
        acf, psd = acf[0], psd[0]
    return ell, acf, q, psd


# ---------------------------------------------------------------- drivers
# static_sweep / dynamic_anneal / depinning_ramp, qew_runs.h:45-243 (same
# configuration fields and defaults; the additive knobs are marked).
def _lbfgs_result(r) -> LbfgsResult:
    return LbfgsResult(r.iterations, r.max_force, bool(r.converged), r.n_func_evals,
                       r.n_curvature_skips, r.n_ls_restarts)


def _rk_result(r) -> RkResult:
    return RkResult(bool(r.blocked), bool(r.runaway), r.sweeps, r.total_advance, r.mean_h)


@dataclass
class StaticConfig:  # qew_runs.h:48-61
    model: Model = Model.Arclength
    amplitude: float = 1.0
    xi: float = 0.1
    Lx: float = 32.0
    Ly: float = 1.0
    nx: int = 4096
    ny: int = 512
    driving_force: float = 0.0
    pinning_lengths_over_xi: tuple = (0.01, 0.1, 1.0, 10.0, 100.0)
    ftol: float = 1e-6
    max_iter: int = 5000
    lbfgs_m: int = 8  # additive


@dataclass
class StaticProfile:  # qew_runs.h:63-68
    pinning_length_over_xi: float
    line_tension: float
    h: np.ndarray
    result: LbfgsResult


def static_sweep(c: StaticConfig, noise: _Noise) -> list[StaticProfile]:
    """static_sweep(c, noise), qew_runs.h:70-102 (one persistent launch for all
    ratios on a B-spline field)."""
    ctx = noise.ctx
    ctx.sync_stream()
    ratios = np.ascontiguousarray(c.pinning_lengths_over_xi, dtype=np.float64)
    K = len(ratios)
    cc = _capi.qew_static_config(int(c.model), float(c.amplitude), float(c.xi), float(c.Lx),
                                 float(c.Ly), int(c.nx), int(c.ny), float(c.driving_force),
                                 ratios.ctypes.data_as(_capi.PD), K, float(c.ftol),
                                 int(c.max_iter), int(c.lbfgs_m))
    prof = (_capi.qew_static_profile * max(K, 1))()
    h = np.empty((K, int(c.nx)))
    _capi.check(ctx.lib.qew_static_sweep(ctx.h, noise.h, C.byref(cc), prof,
                                         h.ctypes.data_as(_capi.PD)), ctx.h, "static_sweep")
    return [StaticProfile(prof[k].pinning_length_over_xi, prof[k].line_tension, h[k].copy(),
                          _lbfgs_result(prof[k].result)) for k in range(K)]


@dataclass
class DynamicConfig:  # qew_runs.h:107-122
    model: Model = Model.Arclength
    amplitude: float = 1.0
    xi: float = 0.1
    pinning_length_over_xi: float = 0.1
    driving_force: float = 0.0
    Lx: float = 2.0
    Ly: float = 1.0
    nx: int = 2048
    ny: int = 1024
    seed: int = 1
    tau: float = 1.0
    tl_start: float = 0.01
    tl_end: float = 0.0001
    total_time: float = 1000.0
    dt: float = 0.0  # additive: > 0 replaces the timestep heuristic
    precision: int = QEW_PREC_FP64  # additive


@dataclass
class DynamicSnapshot:  # qew_runs.h:124-127
    t: float
    h: np.ndarray


@dataclass
class DynamicResult:  # qew_runs.h:129-134
    dt: float
    total_time: float
    line_tension: float
    snapshots: list
    steps: int = 0


def dynamic_anneal(c: DynamicConfig, noise: _Noise) -> DynamicResult:
    """dynamic_anneal(c, noise), qew_runs.h:136-177."""
    ctx = noise.ctx
    ctx.sync_stream()
    cc = _capi.qew_dynamic_config(int(c.model), float(c.amplitude), float(c.xi),
                                  float(c.pinning_length_over_xi), float(c.driving_force),
                                  float(c.Lx), float(c.Ly), int(c.nx), int(c.ny), int(c.seed),
                                  float(c.tau), float(c.tl_start), float(c.tl_end),
                                  float(c.total_time), float(c.dt), int(c.precision))
    snaps = []

    def on(user, t, h, n):
        snaps.append(DynamicSnapshot(t, np.ctypeslib.as_array(h, shape=(n,)).copy()))

    cb = _capi.SNAPSHOT_FN(on)
    r = _capi.qew_dynamic_result()
    _capi.check(ctx.lib.qew_dynamic_anneal(ctx.h, noise.h, C.byref(cc), cb, None, C.byref(r)),
                ctx.h, "dynamic_anneal")
    return DynamicResult(r.dt, r.total_time, r.line_tension, snaps, r.steps)


@dataclass
class DepinningConfig:  # qew_runs.h:182-194
    model: Model = Model.Arclength
    amplitude: float = 1.0
    xi: float = 0.1
    pinning_length_over_xi: float = 5.0
    Lx: float = 8.0
    Ly: float = 1.0
    nx: int = 1024
    ny: int = 256
    f_step: float = 1.0
    f_max: float = 40.0
    rp: RkParams = None  # the caller fills it, as the reference's
    bisect_rtol: float = 0.0  # additive: > 0 bisects f_c after the ramp
    precision: int = QEW_PREC_FP64  # additive


@dataclass
class DepinningStep:  # qew_runs.h:196-200
    f: float
    result: RkResult
    h: np.ndarray | None  # blocked steps only


@dataclass
class DepinningResult:  # qew_runs.h:202-206
    line_tension: float
    f_c_upper_bound: float
    steps: list
    f_c: float = -1.0  # additive (bisection)
    f_c_bracket: tuple = (-1.0, -1.0)
    bisect_blocks: int = 0


def depinning_ramp(c: DepinningConfig, noise: _Noise) -> DepinningResult:
    """depinning_ramp(c, noise), qew_runs.h:208-243; raises ValueError on odd nx."""
    ctx = noise.ctx
    ctx.sync_stream()
    rp = c.rp if c.rp is not None else RkParams()
    cc = _capi.qew_depinning_config(int(c.model), float(c.amplitude), float(c.xi),
                                    float(c.pinning_length_over_xi), float(c.Lx), float(c.Ly),
                                    int(c.nx), int(c.ny), float(c.f_step), float(c.f_max),
                                    rp.c(), float(c.bisect_rtol), int(c.precision))
    steps = []

    def on(user, st, h, n):
        s = st.contents
        steps.append(DepinningStep(s.f, _rk_result(s.result),
                                   np.ctypeslib.as_array(h, shape=(n,)).copy() if h else None))

    cb = _capi.DEPINNING_FN(on)
    r = _capi.qew_depinning_result()
    _capi.check(ctx.lib.qew_depinning_ramp(ctx.h, noise.h, C.byref(cc), cb, None, C.byref(r)),
                ctx.h, "depinning_ramp")
    return DepinningResult(r.line_tension, r.f_c_upper_bound, steps, r.f_c,
                           (r.f_c_lo, r.f_c_hi), r.bisect_blocks)


# ---------------------------------------------------------------- serving
class Server:
    """Continuous-batching server over the C ABI (see qew_server_* in qew_gpu.h)."""

    def __init__(self, hbm_budget_bytes: float = 150e9, max_inflight: int = 32,
                 device: int | None = None):
        torch = _torch()
        self.lib = _capi.load()
        self.device = torch.cuda.current_device() if device is None else device
        h = C.c_void_p()
        _capi.check(self.lib.qew_server_create(self.device, float(hbm_budget_bytes),
                                               int(max_inflight), C.byref(h)), None,
                    "qew_server_create")
        self.h = h

    def submit(self, kind: int, n: int, rows: int, xi: float, seed: int, *, model: int = 0,
               line_tension: float = 1.0, driving_force: float = 0.0, ftol: float = 1e-8,
               steps: int = 10000, temperature: float = 0.0, dt: float = 0.01,
               f_step: float = 0.1, f_max: float = 10.0, bisect_rtol: float = 1e-10,
               max_sweeps: int = 200000, max_advance: float = 0.0, runaway: float = 0.0,
               h_out: np.ndarray | None = None) -> int:
        r = _capi.qew_request(int(kind), int(n), int(rows), float(xi), int(seed), int(model),
                              float(line_tension), float(driving_force), float(ftol), int(steps),
                              float(temperature), float(dt), float(f_step), float(f_max),
                              float(bisect_rtol), int(max_sweeps), float(max_advance),
                              float(runaway),
                              None if h_out is None else C.c_void_p(h_out.ctypes.data))
        rid = C.c_uint64()
        _capi.check(self.lib.qew_server_submit(self.h, C.byref(r), C.byref(rid)), None,
                    "qew_server_submit")
        return rid.value

    def poll(self, max_items: int = 1024) -> list:
        buf = (_capi.qew_response * max_items)()
        k = self.lib.qew_server_poll(self.h, buf, max_items)
        return [dict(id=b.id, kind=b.kind, status=b.status, t_submit=b.t_submit,
                     t_start=b.t_start, t_end=b.t_end, iterations=b.iterations, value=b.value,
                     max_force=b.max_force, converged=bool(b.converged)) for b in buf[:k]]

    def lane_stats(self) -> dict:
        """Requests served by the device-resident static loop, and its launches."""
        served, launches = C.c_uint64(), C.c_uint64()
        st = self.lib.qew_server_lane_stats(self.h, C.byref(served), C.byref(launches))
        return {"available": st == _capi.QEW_OK, "served": served.value,
                "launches": launches.value}

    def set_lane_limit(self, max_n: int) -> None:
        """Static requests on lines of at most max_n points go to the
        device-resident loop (qew_server_set_lane_limit; 0: none)."""
        _capi.check(self.lib.qew_server_set_lane_limit(self.h, int(max_n)), None,
                    "set_lane_limit")

    def drain(self, timeout_s: float = 600.0) -> None:
        _capi.check(self.lib.qew_server_drain(self.h, float(timeout_s)), None, "drain")

    def clock(self) -> float:
        return float(self.lib.qew_server_clock(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.qew_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
