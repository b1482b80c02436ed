"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker. The product
(``qew_gb300``) never imports it and has no CPU fallback.

Arrays are numpy float64. Fields use the reference's host layout
``field[i, j]`` with i the x (column) index and j the y (row) index.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field as dc_field

import numpy as np

from . import build as _build

_lib = None

D = C.c_double
I = C.c_int
PD = C.POINTER(C.c_double)


class QoNoise(C.Structure):
    _fields_ = [("kind", I), ("coef", PD), ("nx", I), ("ny", I), ("dx", D),
                ("dy", D), ("p0", D), ("p1", D), ("p2", D)]


class QoParams(C.Structure):
    _fields_ = [("physical_size", D), ("line_tension", D),
                ("driving_force", D), ("model", I)]


class QoLbfgsParams(C.Structure):
    _fields_ = [("m", I), ("ftol", D), ("max_iter", I), ("c1", D),
                ("ls_shrink", D), ("max_ls", I), ("curvature_eps", D),
                ("precondition", I), ("precond_shift", D), ("ls_fallback", I)]


class QoLbfgsResult(C.Structure):
    _fields_ = [("iterations", I), ("max_force", D), ("converged", I),
                ("n_func_evals", C.c_long), ("n_curvature_skips", C.c_long),
                ("n_ls_restarts", C.c_long)]


class QoFireParams(C.Structure):
    _fields_ = [("dt_max", D), ("dt_init", D), ("ftol", D), ("max_iter", I), ("n_min", I),
                ("f_inc", D), ("f_dec", D), ("alpha_start", D), ("f_alpha", D)]


class QoFireResult(C.Structure):
    _fields_ = [("iterations", I), ("max_force", D), ("converged", I)]


class QoRkParams(C.Structure):
    _fields_ = [("dstep", D), ("max_advance", D), ("root_tol", D),
                ("sweep_tol", D), ("runaway", D), ("max_sweeps", I)]


class QoRkResult(C.Structure):
    _fields_ = [("blocked", I), ("runaway", I), ("sweeps", I),
                ("total_advance", D), ("mean_h", D)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        L = _lib
        L.qo_sample_many.argtypes = [C.POINTER(QoNoise), PD, PD, I, PD, PD, PD]
        L.qo_prefilter.argtypes = [PD, I, I, PD]
        L.qo_prefilter.restype = I
        L.qo_fft.argtypes = [PD, PD, I, I]
        L.qo_rfft.argtypes = [PD, I, PD, PD]
        L.qo_irfft.argtypes = [PD, PD, I, PD]
        for fn in ("qo_objective", "qo_objective_omp"):
            getattr(L, fn).argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise)]
            getattr(L, fn).restype = D
        L.qo_objective_trial.argtypes = [PD, PD, D, I, C.POINTER(QoParams), C.POINTER(QoNoise)]
        L.qo_objective_trial.restype = D
        for fn in ("qo_gradient", "qo_gradient_omp"):
            getattr(L, fn).argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise), PD]
        L.qo_omp_max_threads.restype = I
        L.qo_lbfgs_default_params.argtypes = [C.POINTER(QoLbfgsParams)]
        L.qo_lbfgs_minimize.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                        C.POINTER(QoLbfgsParams), C.POINTER(QoLbfgsResult)]
        L.qo_precond_apply.argtypes = [PD, I, D, D, D, PD]
        L.qo_langevin_step.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                       D, D, PD, PD]
        L.qo_rk_site_velocity.argtypes = [I, I, D, D, D, I, D, D, D, C.POINTER(QoNoise)]
        L.qo_rk_site_velocity.restype = D
        L.qo_rk_block.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                  C.POINTER(QoRkParams), C.POINTER(QoRkResult)]
        L.qo_rk_block.restype = I
        L.qo_depinning_bisect.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                          C.POINTER(QoRkParams), D, D, D, I,
                                          PD, PD, PD, C.POINTER(I)]
        L.qo_depinning_bisect.restype = I
        L.qo_depinning_bisect_ex.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                             C.POINTER(QoRkParams), D, D, D, I,
                                             PD, PD, PD, C.POINTER(I), C.POINTER(I),
                                             C.POINTER(C.c_long)]
        L.qo_depinning_bisect_ex.restype = I
        L.qo_philox_normals.argtypes = [C.c_uint64, C.c_uint64, I, PD]
        L.qo_langevin_step_philox.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise), D,
                                              D, C.c_uint64, C.c_uint64, PD, PD, I]
        L.qo_omp_set_threads.argtypes = [I]
        L.qo_fire_minimize.argtypes = [PD, I, C.POINTER(QoParams), C.POINTER(QoNoise),
                                       C.POINTER(QoFireParams), C.POINTER(QoFireResult)]
        L.qo_mt64_seed.argtypes = [C.c_void_p, C.c_uint64]
        L.qo_mt64_next.argtypes = [C.c_void_p]
        L.qo_mt64_next.restype = C.c_uint64
        L.qo_seeded_field.argtypes = [I, I, D, D, D, D, D, C.c_uint64, PD]
        L.qo_seeded_field.restype = I
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(PD)


# --------------------------------------------------------------------------
# Noise descriptors (the production field and the reference tests' stubs)
# --------------------------------------------------------------------------
class Noise:
    """Base: holds a QoNoise struct (and keeps the coefficient array alive)."""

    def __init__(self, kind: int, p0=0.0, p1=0.0, p2=0.0):
        self.s = QoNoise(kind, None, 0, 0, 1.0, 1.0, p0, p1, p2)
        self._keep = None


class BSplineField(Noise):
    """FilteredNoise(field, nx, ny, Lx, Ly), filtered_noise.cpp:84-90."""

    def __init__(self, field_xy: np.ndarray | None, Lx: float, Ly: float,
                 coef: np.ndarray | None = None):
        """field_xy may be None when the prefiltered coefficients are given."""
        if field_xy is None:
            field_xy = np.empty((0, 0))
            nx, ny = np.shape(coef)
        else:
            field_xy = np.ascontiguousarray(field_xy, dtype=np.float64)
            nx, ny = field_xy.shape
        super().__init__(0)
        if coef is None:
            coef = prefilter(field_xy)
        self.field = field_xy
        self.coef = np.ascontiguousarray(coef, dtype=np.float64)
        self.nx, self.ny, self.Lx, self.Ly = nx, ny, Lx, Ly
        self.s.coef = _p(self.coef)
        self.s.nx, self.s.ny = nx, ny
        self.s.dx, self.s.dy = Lx / nx, Ly / ny
        self._keep = self.coef


def ZeroNoise():
    return Noise(1)


def ConstNoise(v0):
    return Noise(2, v0)


def HarmonicWell(k=2.0, y0=0.5):
    return Noise(3, k, y0)


def SinusoidNoise(A=0.1, k=2.0 * 3.14159265358979323846):
    return Noise(4, A, k)


def AnalyticNoise(amp=0.3, kx=0.7, ky=1.3):
    return Noise(5, amp, kx, ky)


def prefilter(field_xy: np.ndarray) -> np.ndarray:
    field_xy = np.ascontiguousarray(field_xy, dtype=np.float64)
    nx, ny = field_xy.shape
    coef = np.empty_like(field_xy)
    rc = lib().qo_prefilter(_p(field_xy), nx, ny, _p(coef))
    assert rc == 0
    return coef


def sample(noise: Noise, x: np.ndarray, y: np.ndarray):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    m = x.size
    v, dx, dy = np.empty(m), np.empty(m), np.empty(m)
    lib().qo_sample_many(C.byref(noise.s), _p(x), _p(y), m, _p(v), _p(dx), _p(dy))
    return v, dx, dy


# --------------------------------------------------------------------------
# Model / solvers
# --------------------------------------------------------------------------
def params(physical_size=1.0, line_tension=1.0, driving_force=0.0, model=0):
    return QoParams(physical_size, line_tension, driving_force, int(model))


def objective(h, p: QoParams, noise: Noise, omp=False) -> float:
    h = np.ascontiguousarray(h, dtype=np.float64)
    fn = lib().qo_objective_omp if omp else lib().qo_objective
    return fn(_p(h), h.size, C.byref(p), C.byref(noise.s))


def objective_trial(x0, d, alpha, p: QoParams, noise: Noise) -> float:
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    return lib().qo_objective_trial(_p(x0), _p(d), alpha, x0.size, C.byref(p), C.byref(noise.s))


def gradient(h, p: QoParams, noise: Noise, omp=False, out=None) -> np.ndarray:
    h = np.ascontiguousarray(h, dtype=np.float64)
    g = np.empty_like(h) if out is None else out
    fn = lib().qo_gradient_omp if omp else lib().qo_gradient
    fn(_p(h), h.size, C.byref(p), C.byref(noise.s), _p(g))
    return g


def omp_max_threads() -> int:
    return lib().qo_omp_max_threads()


def lbfgs_default_params(**kw) -> QoLbfgsParams:
    lp = QoLbfgsParams()
    lib().qo_lbfgs_default_params(C.byref(lp))
    for k, v in kw.items():
        setattr(lp, k, v)
    return lp


def lbfgs_minimize(h: np.ndarray, p: QoParams, noise: Noise, lp: QoLbfgsParams):
    """Relaxes h in place (numpy float64); returns a QoLbfgsResult."""
    assert h.dtype == np.float64 and h.flags["C_CONTIGUOUS"]
    res = QoLbfgsResult()
    lib().qo_lbfgs_minimize(_p(h), h.size, C.byref(p), C.byref(noise.s), C.byref(lp), C.byref(res))
    return res


def precond_apply(q, kappa, physical_size, shift) -> np.ndarray:
    q = np.ascontiguousarray(q, dtype=np.float64)
    d = np.empty_like(q)
    lib().qo_precond_apply(_p(q), q.size, kappa, physical_size, shift, _p(d))
    return d


def langevin_step(h: np.ndarray, p: QoParams, noise: Noise, drift, diff, xi):
    xi = np.ascontiguousarray(xi, dtype=np.float64)
    g = np.empty_like(h)
    lib().qo_langevin_step(_p(h), h.size, C.byref(p), C.byref(noise.s), drift, diff, _p(xi), _p(g))


def langevin_step_philox(h: np.ndarray, p: QoParams, noise: Noise, drift, diff, seed, step,
                         omp=False, work=None):
    """LangevinDynamics::step with the Philox normals of (seed, step) drawn in
    the step (the increments the GPU's step uses); omp=True on all threads."""
    g, xi = work if work is not None else (np.empty_like(h), np.empty_like(h))
    lib().qo_langevin_step_philox(_p(h), h.size, C.byref(p), C.byref(noise.s), drift, diff,
                                  seed, step, _p(g), _p(xi), 1 if omp else 0)


def set_threads(k: int) -> None:
    """OpenMP threads of the oracle's parallel forms."""
    lib().qo_omp_set_threads(int(k))


def rk_params(dstep=0.0, max_advance=0.0, root_tol=1e-10, sweep_tol=1e-9,
              runaway=0.0, max_sweeps=200000) -> QoRkParams:
    return QoRkParams(dstep, max_advance, root_tol, sweep_tol, runaway, max_sweeps)


def rk_site_velocity(i, n, dx, lt, f, model, hi, hl, hr, noise: Noise) -> float:
    return lib().qo_rk_site_velocity(i, n, dx, lt, f, model, hi, hl, hr, C.byref(noise.s))


def rk_block(h: np.ndarray, p: QoParams, noise: Noise, rp: QoRkParams):
    assert h.dtype == np.float64 and h.flags["C_CONTIGUOUS"]
    res = QoRkResult()
    rc = lib().qo_rk_block(_p(h), h.size, C.byref(p), C.byref(noise.s), C.byref(rp), C.byref(res))
    if rc != 0:
        raise ValueError("rk_block: line length must be even for the red-black sweep")
    return res


def depinning_bisect(h: np.ndarray, p: QoParams, noise: Noise, rp: QoRkParams,
                     f_lo, f_hi, rtol=1e-10, max_steps=200):
    fc, flo, fhi = D(), D(), D()
    nb = I()
    rc = lib().qo_depinning_bisect(_p(h), h.size, C.byref(p), C.byref(noise.s), C.byref(rp),
                                   f_lo, f_hi, rtol, max_steps, C.byref(fc), C.byref(flo),
                                   C.byref(fhi), C.byref(nb))
    if rc != 0:
        raise ValueError("depinning_bisect: line length must be even")
    return fc.value, flo.value, fhi.value, nb.value


def depinning_bisect_verdicts(h: np.ndarray, p: QoParams, noise: Noise, rp: QoRkParams,
                              f_lo, f_hi, rtol=1e-10, max_steps=200):
    """depinning_bisect plus each block's verdict (0 blocked, 1 runaway, 2
    max_sweeps reached) and the sweeps of all blocks together."""
    fc, flo, fhi = D(), D(), D()
    nb = I()
    verdicts = (I * max(max_steps, 1))()
    sweeps = C.c_long()
    rc = lib().qo_depinning_bisect_ex(_p(h), h.size, C.byref(p), C.byref(noise.s), C.byref(rp),
                                      f_lo, f_hi, rtol, max_steps, C.byref(fc), C.byref(flo),
                                      C.byref(fhi), C.byref(nb), verdicts, C.byref(sweeps))
    if rc != 0:
        raise ValueError("depinning_bisect: line length must be even")
    return fc.value, flo.value, fhi.value, list(verdicts[:nb.value]), sweeps.value


def philox_normals(seed: int, step: int, n: int) -> np.ndarray:
    out = np.empty(n)
    lib().qo_philox_normals(seed, step, n, _p(out))
    return out


def fft(re, im, inverse=False):
    re = np.array(re, dtype=np.float64)
    im = np.array(im, dtype=np.float64)
    lib().qo_fft(_p(re), _p(im), re.size, 1 if inverse else 0)
    return re, im


def mt64_outputs(seed: int, count: int) -> np.ndarray:
    """The first `count` outputs of std::mt19937_64(seed), restated."""
    st = C.create_string_buffer(312 * 8 + 16)
    lib().qo_mt64_seed(st, seed)
    return np.array([lib().qo_mt64_next(st) for _ in range(count)], dtype=np.uint64)


def seeded_field(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed) -> np.ndarray:
    """FilteredNoise's seeded field (filtered_noise.cpp:25-82), [nx][ny]."""
    out = np.empty((nx, ny))
    if lib().qo_seeded_field(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed, _p(out)) != 0:
        raise MemoryError("qo_seeded_field")
    return out


def fire_params(dt_max, **kw) -> QoFireParams:
    """FireParams with the defaults of fire.h:21-31."""
    fp = QoFireParams(float(dt_max), 0.0, 1e-6, 100000, 5, 1.1, 0.5, 0.1, 0.99)
    for k, v in kw.items():
        setattr(fp, k, v)
    return fp


def fire_minimize(h: np.ndarray, p: QoParams, noise: Noise, fp: QoFireParams) -> QoFireResult:
    """Relaxes h in place (numpy float64)."""
    assert h.dtype == np.float64 and h.flags["C_CONTIGUOUS"]
    res = QoFireResult()
    lib().qo_fire_minimize(_p(h), h.size, C.byref(p), C.byref(noise.s), C.byref(fp), C.byref(res))
    return res
