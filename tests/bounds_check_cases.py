"""Small cases run on the bounds-checked build of the library (imported with
QEW_GB300_VARIANT=bounds_check by tests/test_gpu_bounds_check.py): every
gather form, the objective and the persistent solvers, on fields and heights
that exercise the wrapped and folded paths. Prints one JSON line: the
results' largest errors against the oracle and the device's bounds report."""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from conftest import band_limited_field, gaussian_field  # noqa: E402


def main():
    import torch

    import qew_gb300 as Q
    from oracle import oracle as O

    def t64(a):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")

    def rel(a, b, scale=None):
        if scale is None:
            scale = np.max(np.abs(b))
        return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(scale, 1e-300))

    def term_scale(h, po, of):
        """Largest magnitude among the gradient's terms (the FP32 bar's scale)."""
        g_el = O.gradient(h, po, O.ZeroNoise())
        return max(np.max(np.abs(g_el)), np.max(np.abs(O.gradient(h, po, of) - g_el)))

    errs = {}
    # 16-tap FP64 and reference-exact, a line that is not on the field's grid
    nx, ny, Lx, Ly = 96, 40, 4.8, 1.3
    fld = band_limited_field(nx, ny, Lx, Ly, 1.0, 0.3, 5)
    f = Q.FilteredNoise(fld, Lx, Ly, store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(1)
    h = rng.uniform(-2 * Ly, 3 * Ly, 257)
    for model in (0, 1):
        p, po = Q.Params(Lx, 1.3, 0.2, Q.Model(model)), O.params(Lx, 1.3, 0.2, model)
        go = O.gradient(h, po, of)
        errs["fp64_16tap_%d" % model] = rel(Q.gradient(t64(h), p, f).cpu().numpy(), go)
        errs["fp64_reference_%d" % model] = rel(
            Q.gradient(t64(h), p, f, precision=Q.QEW_PREC_FP64_REFERENCE).cpu().numpy(), go)
        errs["fp32split_16tap_%d" % model] = rel(
            Q.gradient(t64(h), p, f, precision=Q.QEW_PREC_FP32_SPLIT).cpu().numpy(), go,
            term_scale(h, po, of))
        eo = O.objective(h, po, of)
        errs["objective_16tap_%d" % model] = abs(Q.objective(t64(h), p, f) - eo) / max(abs(eo), 1)
    # a line on the field's grid: the cell-polynomial store, the x-filtered
    # FP32 store in a batched persistent launch
    nx, ny = 2048, 32
    fld = gaussian_field(nx, ny, 3.0, 7)
    f = Q.FilteredNoise(fld, float(nx), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY | Q.QEW_STORE_FP32 |
                        Q.QEW_STORE_FP32_EDGE)
    of = O.BSplineField(fld, float(nx), float(ny), coef=f.coefficients())
    hb = np.stack([rng.uniform(-ny, 2 * ny, nx), ny / 2 + rng.standard_normal(nx),
                   rng.uniform(0, ny, nx)])
    for model in (0, 1):
        p, po = Q.Params(float(nx), 1.0, 0.1, Q.Model(model)), O.params(float(nx), 1.0, 0.1, model)
        gb = Q.gradient_batch(t64(hb), p, f).cpu().numpy()
        errs["fp64_poly_%d" % model] = max(rel(gb[k], O.gradient(hb[k], po, of)) for k in range(3))
        cells = torch.stack([Q.split_heights(t64(hb[k]), f)[0] for k in range(3)])
        fracs = torch.stack([Q.split_heights(t64(hb[k]), f)[1] for k in range(3)])
        g32 = Q.gradient_split_batch(cells, fracs, p, f).cpu().numpy().astype(np.float64)
        errs["fp32split_store_%d" % model] = max(
            rel(g32[k], O.gradient(hb[k], po, of), term_scale(hb[k], po, of)) for k in range(3))
        eo = O.objective(hb[1], po, of)
        errs["objective_poly_%d" % model] = abs(Q.objective(t64(hb[1]), p, f) - eo) / max(abs(eo), 1)
    # persistent solvers
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=200)
    p = Q.Params(float(nx), 1.0, 0.05, Q.Model.Linear)
    for prec in (Q.QEW_PREC_FP64, Q.QEW_PREC_FP32_SPLIT, Q.QEW_PREC_FP64_REFERENCE):
        Q.rk_block(t64(np.full(nx, ny / 2)), p, f, rp, precision=prec)
    dyn = Q.LangevinDynamics(nx, 3)
    for prec in (Q.QEW_PREC_FP64, Q.QEW_PREC_FP32_SPLIT):
        dyn.run(t64(np.full(nx, ny / 2)), p, f, np.full(20, 0.01), np.full(20, 0.05),
                precision=prec)
    lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=500, precondition=True, precond_shift=0.05,
                       ls_fallback=True)
    r = Q.lbfgs_minimize(t64(np.full(nx, ny / 2)), Q.Params(float(nx), 1.0, 0.0), f, lp)
    lines = [(t64(np.full(n, ny / 2)), Q.Params(float(nx), 1.0, 0.0), f, 0.05) for n in (nx,)]
    re = Q.ensemble_minimize(lines, lp, ftol_fp32=2e-5)
    torch.cuda.synchronize()
    print(json.dumps({"report": Q.bounds_check_report(), "errors": errs,
                      "lbfgs_converged": bool(r.converged),
                      "ensemble_converged": bool(re[0].converged)}))


if __name__ == "__main__":
    main()
