"""Benchmark: line-point gradient evaluations per second on one GB300.

Workload (the gather-roofline configuration): a periodic line of L = 2^20
points on a 2^20 x 1024 pinning field (Gaussian-filtered white noise,
correlation length xi = 4 cells, unit variance, seed 5, grid spacing 1). A
step evaluates the gradient of 8 independent line instances (h = band centre
+ a smooth random walk of std 8 cells; the 8 lines sit in 8 disjoint row
bands), so every step touches ~8x the per-instance footprint, more than twice
the 129 MB L2: inputs larger than L2, no flush needed.

Reports (one JSON line on rank 0): value = points/s with inputs resident in
HBM; e2e = the same through the host-buffer C-ABI call (qew_gradient_host,
pinned host buffers, copies inside the timed region); roofline of the
dominant gradient kernel against the measured HBM copy bandwidth;
cpu_baseline = the CPU oracle's OpenMP gradient on the machine's host cores.

``--impl reference`` times the CPU implementation of the path (the oracle's
restatement of the reference, OpenMP on all host cores) on the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "line-point gradient evals/s"
UNIT = "points/s"
L_FULL, NY_FULL, XI, SEED, N_INST = 1 << 20, 1024, 4.0, 5, 8
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_reference", "fp32split"],
                    help="headline form of the gather: fp64 (FP64 drop-in on the cell-"
                         "polynomial store), fp64_reference (FP64 with the reference's "
                         "arithmetic bit for bit) or fp32split (FP32 split-index gather)")
    ap.add_argument("--small", action="store_true",
                    help="small case for profiling: the same batched launch (8 lines of "
                         "L=2^20) on a 64-row field (about 3 GB of field stores)")
    ap.add_argument("--no-poly-store", action="store_true",
                    help="field without the FP64 cell-polynomial store: the fp64 form sums the "
                         "16 taps in the reference's order")
    ap.add_argument("--no-edge-store", action="store_true",
                    help="field without the x-filtered FP32 copy: the split gather reads the 16 "
                         "B-spline taps per edge (the form used on lines that do not have one "
                         "point per field column)")
    ap.add_argument("--no-headline", action="store_true",
                    help="run only the --sections configurations (profiling), no headline")
    ap.add_argument("--profile-run", action="store_true",
                    help="GPU timed loop only (no e2e, CPU baseline or clock sampling)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ensemble-lines", type=int, default=4096,
                    help="lines of the batched-statics section (0 skips it)")
    ap.add_argument("--ensemble-store", default="poly", choices=["fp64", "poly"],
                    help="the ensemble fields' FP64 store: coefficients only (16 taps per "
                         "edge), or with the cell polynomials the FP64 refinement then reads")
    ap.add_argument("--ensemble-ref", type=int, default=16,
                    help="lines timed with the plain one-line-per-launch form")
    ap.add_argument("--sections", default="refshape,static,ensemble,dynamics,depinning,serving",
                    help="extra configurations reported beside the headline")
    ap.add_argument("--refshape-cpu-reps", type=int, default=20,
                    help="oracle calls per kernel on one core in the reference-shape section "
                         "(four times as many on all cores)")
    ap.add_argument("--dyn-steps", type=int, default=100000)
    ap.add_argument("--dyn-plain-steps", type=int, default=2000)
    ap.add_argument("--dyn-cpu-steps", type=int, default=400,
                    help="oracle Langevin steps timed for the dynamics section's CPU baseline")
    ap.add_argument("--dep-size", type=int, default=2048,
                    help="line length and field size of the depinning section (16384: C2)")
    ap.add_argument("--dep-max-sweeps", type=int, default=20000,
                    help="RkParams::max_sweeps of the depinning section (200000: C2)")
    ap.add_argument("--dep-fstep", type=float, default=0.05)
    ap.add_argument("--dep-fmax", type=float, default=20.0)
    ap.add_argument("--dep-rate-sweeps", type=int, default=2000)
    ap.add_argument("--dep-forms", default="fp64,fp64_poly,fp32split",
                    help="velocity forms of the depinning section")
    ap.add_argument("--serve-rates", default="100,10000")
    ap.add_argument("--serve-requests", type=int, default=500)
    ap.add_argument("--serve-inflight", type=int, default=32)
    ap.add_argument("--serve-lane-max", type=int, default=2048,
                    help="static requests on lines of at most this many points go to the "
                         "device-resident loop (0: none, at most 16384)")
    ap.add_argument("--serve-lsteps", type=int, default=10000)
    return ap.parse_args()


# ----------------------------------------------------------------- helpers
_T0 = time.time()


def log(msg: str) -> None:
    """Progress to stderr (the JSON result line goes to stdout)."""
    print("[bench %7.1fs] %s" % (time.time() - _T0, msg), file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(torch, t_ms: float, device) -> float:
    """The slowest replica's time: the whole job ends when it does."""
    t = torch.tensor([t_ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ws: int, steps: int, lines: int, L: int, t_ms: float) -> float:
    """Points per second of all replicas together (each does the same work)."""
    return ws * steps * lines * L / (t_ms * 1e-3)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def smooth_walk(rng, n, std, corr):
    """A smooth periodic random line: Gaussian-filtered white noise, given std."""
    w = rng.standard_normal(n)
    k = np.fft.rfftfreq(n)
    f = np.fft.irfft(np.fft.rfft(w) * np.exp(-0.5 * (2 * np.pi * corr * k) ** 2), n)
    return f * (std / f.std())


def gaussian_field_gpu(torch, nx, ny, xi, seed):
    """Seeded white noise, Gaussian filter exp(-(2 pi xi f)^2/2) (f in cycles
    per cell) applied axis by axis in Fourier space, unit population std.
    Layout (nx, ny), y fastest (the reference's host layout)."""
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    w = torch.randn((nx, ny), dtype=torch.float64, device="cuda", generator=g)
    ky = torch.fft.rfftfreq(ny, device="cuda", dtype=torch.float64)
    w = torch.fft.irfft(torch.fft.rfft(w, dim=1) * torch.exp(-0.5 * (2 * math.pi * xi * ky) ** 2),
                        n=ny, dim=1)
    kx = torch.fft.rfftfreq(nx, device="cuda", dtype=torch.float64)[:, None]
    w = torch.fft.irfft(torch.fft.rfft(w, dim=0) * torch.exp(-0.5 * (2 * math.pi * xi * kx) ** 2),
                        n=nx, dim=0)
    w -= w.mean()
    w /= w.std(unbiased=False)
    return w.contiguous()


# ---------------------------------------------------------- reference arm
def cpu_gradient_rate(seconds: float, L: int = L_FULL, ny: int = 64):
    """The CPU oracle's OpenMP gradient on a bounded sample: a 2^20-point line
    on a 2^20 x 64 field. The raw synthetic field serves as the coefficient
    array (the gather's cost does not depend on the values)."""
    from oracle import oracle as O
    rng = np.random.default_rng(SEED)
    coef = rng.standard_normal((L, ny))
    f = O.BSplineField(coef, float(L), float(ny), coef=coef)
    h = ny / 2 + smooth_walk(rng, L, 8.0, 64.0)
    p = O.params(float(L), 1.0, 0.0, 0)
    out = np.empty(L)
    O.gradient(h, p, f, omp=True, out=out)  # warm
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.gradient(h, p, f, omp=True, out=out)
        reps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": reps * L / dt, "unit": UNIT, "cores": O.omp_max_threads(), "kind": "port",
            "sample": "%d gradient evals of a 2^20-point line on a 2^20x%d FP64 field "
                      "(OpenMP, %.1f s)" % (reps, ny, dt)}


def headline_config(L, ny, n_inst, precision, ws):
    """The headline workload's description (both arms print the same)."""
    return {"workload": "gradient of %d line instances of L=2^20 points on a 2^20x%d field "
                        "(xi=4 cells), %s gather" % (n_inst, ny, precision),
            "L": L, "rows": ny, "instances_per_step": n_inst, "model": "linear",
            "l2": "inputs larger than L2 (8 disjoint row bands per step)",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    rng = np.random.default_rng(SEED)
    L, ny = L_FULL, 64
    coef = rng.standard_normal((L, ny))
    f = O.BSplineField(coef, float(L), float(ny), coef=coef)
    h = ny / 2 + smooth_walk(rng, L, 8.0, 64.0)
    p = O.params(float(L), 1.0, 0.0, 0)
    out = np.empty(L)
    for _ in range(max(args.warmup, 0)):
        O.gradient(h, p, f, omp=True, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.gradient(h, p, f, omp=True, out=out)
    dt = time.perf_counter() - t0
    val = args.steps * L / dt
    line = {"metric": METRIC, "value": val, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(L, NY_FULL, N_INST, args.precision, ws),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": O.omp_max_threads(),
                             "kind": "port",
                             "sample": "per step one of the workload's 2^20-point lines (FP64, the "
                                       "reference algorithm restated in the CPU oracle, OpenMP) "
                                       "on a 2^20x64 field: the gather's cost does not depend "
                                       "on the field height"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------- static (C0)
def host_gaussian_field(nx, ny, xi, seed):
    """Seeded N(0,1) white noise, Gaussian filter exp(-(2 pi xi f)^2 / 2) in
    Fourier space (f in cycles per cell), unit population std; [nx][ny]."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nx, ny))
    fx = np.fft.fftfreq(nx)[:, None]
    fy = np.fft.rfftfreq(ny)[None, :]
    filt = np.exp(-0.5 * (2 * np.pi * xi) ** 2 * (fx ** 2 + fy ** 2))
    f = np.fft.irfft2(np.fft.rfft2(w) * filt, s=(nx, ny))
    return f / f.std()


def run_static(args, Q, torch):
    """C0: L = 1024, linear elasticity of stiffness 1, 1024 x 1024 field
    (seed 0, xi in {2, 4, 8} cells, unit variance), h0 = 0, L-BFGS m = 10
    with the preconditioner (shift 0.5 dx A / xi^2), to max|g| < 1e-8 — on
    the GPU (resident form) and with the CPU oracle (serial), the same field
    coefficients on both sides. With the reference's Armijo search alone the
    solve can stall just above 1e-8 (energy differences below the energy's
    rounding); the approximate-Wolfe fallback is on for both sides, and the
    Armijo-only GPU run is reported beside it."""
    from oracle import oracle as O
    n = 1024
    out = {"metric": "static solves/s at max|g| < 1e-8", "unit": "solves/s",
           "workload": "L=1024, 1024x1024 field seed 0, xi in {2,4,8}, linear, h0=0, m=10, "
                       "preconditioned", "xi": {}}
    gpu_total = cpu_total = 0.0
    for xi in (2.0, 4.0, 8.0):
        field = host_gaussian_field(n, n, xi, 0)
        f = Q.FilteredNoise(field, float(n), float(n))
        p = Q.Params(float(n), 1.0, 0.0, Q.Model.Linear)
        shift = 0.5 * 1.0 * 1.0 / xi ** 2
        lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True,
                           precond_shift=shift, ls_fallback=True)
        h = torch.zeros(n, dtype=torch.float64, device="cuda")
        Q.lbfgs_minimize(h.clone(), p, f, lp)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = Q.lbfgs_minimize(h, p, f, lp)
        torch.cuda.synchronize()
        tg = time.perf_counter() - t0
        e_gpu = Q.objective(h, p, f)
        h_ref = torch.zeros(n, dtype=torch.float64, device="cuda")
        lp_ref = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True,
                               precond_shift=shift)
        rr = Q.lbfgs_minimize(h_ref, p, f, lp_ref)
        of = O.BSplineField(field, float(n), float(n), coef=f.coefficients())
        hc = np.zeros(n)
        op = O.params(float(n), 1.0, 0.0, 0)
        olp = O.lbfgs_default_params(m=10, ftol=1e-8, max_iter=20000, precondition=1,
                                     precond_shift=shift, ls_fallback=1)
        t0 = time.perf_counter()
        rc = O.lbfgs_minimize(hc, op, of, olp)
        tc = time.perf_counter() - t0
        e_cpu = O.objective(hc, op, of)
        gpu_total += tg
        cpu_total += tc
        out["xi"][str(int(xi))] = {
            "gpu_s": tg, "gpu_iterations": r.iterations, "gpu_max_grad": r.max_force,
            "gpu_converged": bool(r.converged), "cpu_s": tc, "cpu_iterations": rc.iterations,
            "cpu_max_grad": rc.max_force, "cpu_converged": bool(rc.converged),
            "energy_rel_diff": abs(e_gpu - e_cpu) / abs(e_cpu),
            "armijo_only_gpu": {"iterations": rr.iterations, "max_grad": rr.max_force,
                                "converged": bool(rr.converged)}}
    out["value"] = 3.0 / gpu_total
    out["cpu_solves_per_s"] = 3.0 / cpu_total
    out["cpu"] = {"cores": 1, "kind": "port", "sample": "the three solves, serial oracle"}
    # The reference's published end-to-end L-BFGS case (3.55 s, 2470 iterations,
    # Kokkos Serial): qew_static's defaults (seeded FilteredNoise 4096 x 512,
    # Lx = 32, xi = 0.1, arclength) at lambda_p/xi = 1 (Gamma = 1), m = 8,
    # preconditioned, ftol 1e-6, through static_sweep.
    fld = Q.FilteredNoise.seeded(4096, 512, 32.0, 1.0, 1.0, 0.1, 0.1, 1)
    cfg = Q.StaticConfig(model=Q.Model.Arclength, nx=4096, ny=512, Lx=32.0, Ly=1.0, xi=0.1,
                         pinning_lengths_over_xi=(1.0,), ftol=1e-6, max_iter=20000)
    Q.static_sweep(cfg, fld)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prof = Q.static_sweep(cfg, fld)[0]
    tg = time.perf_counter() - t0
    of = O.BSplineField(np.zeros((4096, 512)), 32.0, 1.0, coef=fld.coefficients())
    hc = np.full(4096, 0.5)
    olp = O.lbfgs_default_params(m=8, ftol=1e-6, max_iter=20000, precondition=1,
                                 precond_shift=0.5 * (32.0 / 4096) * 1.0 / 0.01)
    t0 = time.perf_counter()
    rc = O.lbfgs_minimize(hc, O.params(32.0, 1.0, 0.0, 1), of, olp)
    tc = time.perf_counter() - t0
    out["reference_case"] = {
        "workload": "qew_static defaults at lambda_p/xi=1: n=4096, 4096x512 seeded field, "
                    "Lx=32, xi=0.1, arclength, m=8, preconditioned, ftol 1e-6",
        "gpu_s": tg, "gpu_iterations": prof.result.iterations,
        "gpu_converged": bool(prof.result.converged), "cpu_oracle_s": tc,
        "cpu_oracle_iterations": rc.iterations, "cpu_oracle_converged": bool(rc.converged),
        "max_abs_h_diff": float(np.max(np.abs(prof.h - hc))),
        "published_reference_s": 3.55, "published_reference_iterations": 2470,
        "published_reference_hardware": "Kokkos Serial, one CPU core (docs/fix_plan.md)"}
    return out


# ----------------------------------------------------------- ensemble (C3)
def run_ensemble(args, Q, torch):
    """Batched statics: `lines` realisations, L log-uniform in [256, 16384]
    (even), each on its own 256-row field (Gaussian filter, xi ~ U[2, 8]
    cells, unit variance, generated on the device), linear or arclength with
    probability 1/2, Gamma = 1, f = 0, h0 = 0; L-BFGS m = 10, preconditioned
    (shift 0.5/xi^2), FP32 split-gather phase to 2e-5 then FP64 refinement to
    max|g| < 1e-8. Compared with the plain one-line-per-launch FP64 form
    (same parameters) on a uniform random sample of the lines."""
    rng = np.random.default_rng(3)
    n_lines = args.ensemble_lines
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32
    if args.ensemble_store == "poly":
        store |= Q.QEW_STORE_FP64_POLY
    specs, lines = [], []
    for k in range(n_lines):
        L = int(round(np.exp(rng.uniform(np.log(256), np.log(16384))) / 2)) * 2
        xi = float(rng.uniform(2, 8))
        model = Q.Model(int(rng.integers(0, 2)))
        f = Q.FilteredNoise.generated(L, 256, float(L), 256.0, 1.0, xi, xi, 30000 + k, store=store)
        p = Q.Params(float(L), 1.0, 0.0, model)
        specs.append((L, xi, p, f))
        lines.append((torch.zeros(L, dtype=torch.float64, device="cuda"), p, f, 0.5 / xi ** 2))
    lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True, ls_fallback=True)
    torch.cuda.synchronize()
    ctx = Q.default_context()
    l0 = ctx.launches()
    t0 = time.perf_counter()
    res = Q.ensemble_minimize(lines, lp, ftol_fp32=2e-5)
    torch.cuda.synchronize()
    t_ens = time.perf_counter() - t0
    launches = ctx.launches() - l0
    conv = sum(r.converged for r in res)
    gmax = max(float(Q.gradient(h, p, f).abs().max()) for h, p, f, _ in lines)
    iters = [r.iterations for r in res]
    # plain comparator on a sample
    sample = rng.choice(n_lines, size=min(args.ensemble_ref, n_lines), replace=False)
    t_plain, conv_plain, gmax_plain = [], 0, 0.0
    for k in sample:
        L, xi, p, f = specs[k]
        h = torch.zeros(L, dtype=torch.float64, device="cuda")
        lpk = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True,
                            precond_shift=0.5 / xi ** 2, ls_fallback=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = Q.lbfgs_minimize(h, p, f, lpk, form=Q.QEW_LBFGS_PLAIN)
        torch.cuda.synchronize()
        t_plain.append(time.perf_counter() - t1)
        conv_plain += int(r.converged)
        gmax_plain = max(gmax_plain, float(Q.gradient(h, p, f).abs().max()))
    plain_rate = 1.0 / float(np.mean(t_plain))
    rate = n_lines / t_ens
    for h, p, f, _ in lines:
        del h
    return {"metric": "ensemble solves/s at max|grad| < 1e-8 (FP64-refined)", "value": rate,
            "unit": "solves/s", "lines": n_lines, "wall_s": t_ens, "converged": conv,
            "verified_max_grad": gmax, "iterations_median": float(np.median(iters)),
            "gpu_launches": launches,
            "workload": "L log-uniform [256,16384], 256-row fields, xi~U[2,8], h0=0, m=10, "
                        "preconditioned, FP32 phase to 2e-5 then FP64 to 1e-8",
            "field_store": ("FP64 coefficients + FP32 (16 FP64 taps per edge in the refinement)"
                            if args.ensemble_store == "fp64" else
                            "FP64 coefficients + cell polynomials + FP32 (the refinement reads "
                            "one 32-byte cell per edge)"),
            "plain_fp64_one_line_per_launch": {
                "value": plain_rate, "unit": "solves/s", "sample_lines": int(len(sample)),
                "converged": conv_plain, "verified_max_grad": gmax_plain,
                "mean_s_per_solve": float(np.mean(t_plain))},
            "speedup_vs_plain": rate / plain_rate}


# ------------------------------------------- the reference's benchmark shape
def run_reference_shape(args, Q, torch):
    """The reference's own timing harness (executables/benchmark/main.cpp:19-72):
    the seeded FilteredNoise(262144, 64, Lx = 256, Ly = 1, A = 1, xi = 0.1,
    seed 1), Params{Lx, Gamma = 1, f = 0.1, arclength}, h = Ly/2, one warm-up
    gradient, then 200 gradient() calls, 200 objective() calls and 200
    LangevinDynamics::step(0.01, 0.01) calls, ms per call. The reference
    publishes 26.5 ms (gradient) and 34.4 ms (step) on one core
    (docs/fix_plan.md:12-13). GPU: FP64 on the cell-polynomial store (the
    line has one point per field column) and in the reference's exact
    arithmetic; CPU: the oracle on one core and on all cores (the step draws
    its normals from the same Philox stream as the GPU's step)."""
    from oracle import oracle as O
    nx, ny, Lx, Ly, reps = 262144, 64, 256.0, 1.0, 200
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY
    f = Q.FilteredNoise.seeded(nx, ny, Lx, Ly, 1.0, 0.1, 0.1, 1, store=store)
    p = Q.Params(Lx, 1.0, 0.1, Q.Model.Arclength)
    h = torch.full((nx,), 0.5 * Ly, dtype=torch.float64, device="cuda")
    g = torch.empty_like(h)
    stream = torch.cuda.current_stream()

    def gpu_ms(fn, n):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    out = {"workload": "FilteredNoise(262144, 64, 256, 1, 1, 0.1, 0.1, seed 1), arclength, "
                       "Gamma=1, f=0.1, h=Ly/2; 200 calls each (benchmark/main.cpp)",
           "unit": "ms per call",
           "published_reference_1core": {"gradient": 26.5, "step": 34.4,
                                         "source": "docs/fix_plan.md:12-13 (Kokkos Serial)"}}
    gpu = {}
    gpu["gradient_fp64"] = gpu_ms(lambda: Q.gradient(h, p, f, g), reps)
    gpu["gradient_fp64_reference_exact"] = gpu_ms(
        lambda: Q.gradient(h, p, f, g, precision=Q.QEW_PREC_FP64_REFERENCE), reps)
    t0 = time.perf_counter()
    for _ in range(reps):
        Q.objective(h, p, f)  # returns the energy to the host, as the reference does
    gpu["objective_fp64"] = 1e3 * (time.perf_counter() - t0) / reps
    dyn = Q.LangevinDynamics(nx, 7)
    hs = h.clone()
    gpu["step_fp64"] = gpu_ms(lambda: dyn.step(hs, p, f, 0.01, 0.01), reps)
    out["gpu"] = gpu
    # the oracle on the same coefficients
    of = O.BSplineField(None, Lx, Ly, coef=f.coefficients())
    op = O.params(Lx, 1.0, 0.1, 1)
    hh = np.full(nx, 0.5 * Ly)
    go = np.empty(nx)
    work = (np.empty(nx), np.empty(nx))
    cpu = {}
    nthreads = O.omp_max_threads()
    for label, threads, nrep in (("1core", 1, max(3, args.refshape_cpu_reps)),
                                 ("all_cores", nthreads, 4 * max(3, args.refshape_cpu_reps))):
        O.set_threads(threads)
        par = threads > 1
        O.gradient(hh, op, of, omp=par, out=go)
        t0 = time.perf_counter()
        for _ in range(nrep):
            O.gradient(hh, op, of, omp=par, out=go)
        tg = 1e3 * (time.perf_counter() - t0) / nrep
        t0 = time.perf_counter()
        for _ in range(nrep):
            O.objective(hh, op, of, omp=par)
        to = 1e3 * (time.perf_counter() - t0) / nrep
        hs_c = hh.copy()
        t0 = time.perf_counter()
        for k in range(nrep):
            O.langevin_step_philox(hs_c, op, of, 0.01, 0.01, 7, k, omp=par, work=work)
        ts = 1e3 * (time.perf_counter() - t0) / nrep
        cpu[label] = {"threads": threads, "calls": nrep, "gradient": tg, "objective": to,
                      "step": ts}
    O.set_threads(nthreads)
    out["cpu_oracle"] = cpu
    # the GPU's gradient against the oracle's on this field
    gq = Q.gradient(h, p, f).cpu().numpy()
    O.gradient(hh, op, of, omp=True, out=go)
    out["gradient_max_rel_diff_vs_oracle"] = float(np.max(np.abs(gq - go)) / np.max(np.abs(go)))
    out["speedup_gradient_vs_1core"] = cpu["1core"]["gradient"] / gpu["gradient_fp64"]
    out["speedup_step_vs_1core"] = cpu["1core"]["step"] / gpu["step_fp64"]
    out["value"] = gpu["gradient_fp64"]
    return out


# ------------------------------------------------------------ dynamics (C1)
def run_dynamics(args, Q, torch):
    """Annealed overdamped Langevin: L = 65536, 65536 x 4096 field (xi = 4
    cells, seed 1), arclength, f = 0.5, Gamma = 1, T from 0.5 to 0 linearly
    over the steps, dt = 0.01 (drift = dt, diff = sqrt(2 T dt)), Philox
    increments of seed 1. Device-resident runs (one launch each): FP64 in the
    reference's 16-tap order, FP64 on the cell-polynomial store (the line has
    one point per field column), FP32 split gather; the plain per-step form
    (gradient + update launches) on the first steps; and the CPU oracle's
    step (the same Philox increments, all host cores) on a bounded sample."""
    from oracle import oracle as O
    n, ny, K = 65536, 4096, args.dyn_steps
    f = Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 1,
                                  store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 |
                                  Q.QEW_STORE_FP64_POLY)
    f16 = Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 1,
                                    store=Q.QEW_STORE_FP64)
    p = Q.Params(float(n), 1.0, 0.5, Q.Model.Arclength)
    dt = 0.01
    T = 0.5 * (1.0 - np.arange(K) / K)
    drift = np.full(K, dt)
    diff = np.sqrt(2.0 * T * dt)
    out = {"metric": "Langevin steps/s (L=65536)", "unit": "steps/s", "steps": K,
           "workload": "L=65536, 65536x4096 field xi=4, arclength, f=0.5, T 0.5->0, dt=0.01"}
    finals = {}
    for name, fld, prec in (("fp64", f16, Q.QEW_PREC_FP64), ("fp64_poly", f, Q.QEW_PREC_FP64),
                            ("fp32split", f, Q.QEW_PREC_FP32_SPLIT)):
        h = torch.full((n,), 0.5 * ny, dtype=torch.float64, device="cuda")
        dyn = Q.LangevinDynamics(n, 1)
        dyn.run(h.clone(), p, fld, drift[:10], diff[:10], precision=prec)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dyn.run(h, p, fld, drift, diff, precision=prec)
        torch.cuda.synchronize()
        dt_s = time.perf_counter() - t0
        finals[name] = h
        out[name] = {"value": K / dt_s, "points_per_s": K * n / dt_s, "wall_s": dt_s,
                     "final_mean_h": float(h.mean()), "final_std_h": float(h.std())}
    out["fp64_poly"]["vs_fp64_16tap"] = {
        "max_abs_h_diff": float((finals["fp64_poly"] - finals["fp64"]).abs().max()),
        "roughness_rel_diff": abs(out["fp64_poly"]["final_std_h"] - out["fp64"]["final_std_h"])
        / out["fp64"]["final_std_h"]}
    Kp = min(K, args.dyn_plain_steps)
    h = torch.full((n,), 0.5 * ny, dtype=torch.float64, device="cuda")
    dyn = Q.LangevinDynamics(n, 1)
    dyn.step(h, p, f16, drift[0], diff[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(Kp):
        dyn.step(h, p, f16, drift[k], diff[k])
    torch.cuda.synchronize()
    out["plain_fp64_per_step_launches"] = {"value": Kp / (time.perf_counter() - t0),
                                           "steps": Kp}
    # CPU oracle: LangevinDynamics::step on all host cores, the same Philox
    # increments drawn inside the step, on the same coefficients
    of = O.BSplineField(None, float(n), float(ny), coef=f16.coefficients())
    op = O.params(float(n), 1.0, 0.5, 1)
    hc = np.full(n, 0.5 * ny)
    work = (np.empty(n), np.empty(n))
    kc = max(10, args.dyn_cpu_steps)
    O.langevin_step_philox(hc, op, of, drift[0], diff[0], 1, 0, omp=True, work=work)
    t0 = time.perf_counter()
    for k in range(1, kc + 1):
        O.langevin_step_philox(hc, op, of, drift[k], diff[k], 1, k, omp=True, work=work)
    tc = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": kc / tc, "unit": "steps/s", "cores": O.omp_max_threads(),
                           "kind": "port",
                           "sample": "%d steps of the oracle's LangevinDynamics::step (gradient, "
                                     "Philox increments, update; OpenMP) at L=65536 from the "
                                     "flat line" % kc}
    del of
    out["value"] = out["fp64"]["value"]
    return out


# ----------------------------------------------------------- depinning (C2)
def run_depinning(args, Q, torch):
    """Rosso-Krauth depinning: L = 16384, 16384^2 field (xi = 4 cells, seed 2,
    unit variance), linear, Gamma = 1, flat start at Ly/2; dstep = 0.5 cell,
    max_advance = Ly, runaway = 2 Ly, root_tol 1e-10, sweep_tol 1e-8. Ramp f
    by f_step until a block fails, then bisect f to 1e-10 relative from the
    last blocked line. Velocities in FP64 in the reference's 16-tap order
    (the form whose f_c the tests pin to the oracle's), in FP64 on the
    cell-polynomial store, and from the FP32 coefficients; the plain
    host-driven form is timed on one block for its sweep rate."""
    n = ny = args.dep_size
    dep_forms = [x.strip() for x in args.dep_forms.split(",") if x.strip()]
    fld = Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 2,
                                    store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    fld_poly = (Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 2,
                                          store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY)
                if "fp64_poly" in dep_forms else None)
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=args.dep_max_sweeps)
    out = {"metric": "time to f_c (ramp + bisection to 1e-10)", "unit": "s",
           "workload": "L=%d, %dx%d field xi=4, linear, Gamma=1, f_step=%g" % (n, n, ny, args.dep_fstep)}
    crit = {}
    for name, prec in (("fp64", Q.QEW_PREC_FP64), ("fp64_poly", Q.QEW_PREC_FP64),
                       ("fp32split", Q.QEW_PREC_FP32_SPLIT)):
        if name not in dep_forms:
            continue
        fld_k = fld_poly if name == "fp64_poly" else fld
        h = torch.full((n,), 0.5 * ny, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sweeps, blocks, f_lo, f_hi, h_lo = 0, 0, None, None, None
        k = 0
        while k * args.dep_fstep <= args.dep_fmax:
            fk = k * args.dep_fstep
            r = Q.rk_block(h, Q.Params(float(n), 1.0, fk, Q.Model.Linear), fld_k, rp, precision=prec)
            sweeps += r.sweeps
            blocks += 1
            log("  depinning %s f=%.3f blocked=%d sweeps=%d" % (name, fk, r.blocked, r.sweeps))
            if not r.blocked:
                f_hi = fk
                break
            f_lo, h_lo = fk, h.clone()
            k += 1
        res = {"ramp_blocks": blocks, "ramp_sweeps": sweeps, "f_lo": f_lo, "f_hi": f_hi,
               "ramp_end_verdict": None if f_hi is None else
               ("runaway" if r.runaway else "max_sweeps")}
        if f_lo is not None and f_hi is not None:
            br = Q.depinning_bisect_report(h_lo, Q.Params(float(n), 1.0, 0.0, Q.Model.Linear),
                                           fld_k, rp, f_lo, f_hi, rtol=1e-10, max_steps=64,
                                           precision=prec)
            torch.cuda.synchronize()
            res.update({"f_c": br.f_c, "bracket": [br.f_lo, br.f_hi], "bisect_blocks": br.blocks,
                        "bisect_sweeps": br.sweeps,
                        "verdicts": {"blocked": br.n_blocked, "runaway": br.n_runaway,
                                     "max_sweeps": br.n_timeout},
                        "f_hi_set_by": {0: "ramp", 1: "runaway", 2: "max_sweeps"}[br.f_hi_verdict],
                        "f_c_limited_by_max_sweeps": br.f_hi_verdict == 2 or
                        (br.f_hi_verdict == 0 and not r.runaway),
                        "mean_h_critical": float(h_lo.mean())})
            crit[name] = h_lo
        res["wall_s"] = time.perf_counter() - t0
        out[name] = res
    if "fp64" in crit and "fp64_poly" in crit:
        out["fp64_poly_vs_fp64"] = {
            "f_c_rel_diff": abs(out["fp64_poly"]["f_c"] - out["fp64"]["f_c"]) / out["fp64"]["f_c"],
            "max_abs_h_diff_critical": float((crit["fp64"] - crit["fp64_poly"]).abs().max())}
    if "fp64" in crit and "fp32split" in crit:
        out["fp32_vs_fp64"] = {
            "f_c_rel_diff": abs(out["fp32split"]["f_c"] - out["fp64"]["f_c"]) / out["fp64"]["f_c"],
            "max_abs_h_diff_critical": float((crit["fp64"] - crit["fp32split"]).abs().max())}

    if "fp64" in crit:
        # sweep rate: resident vs plain host-driven, one block at the last blocked force
        p_lo = Q.Params(float(n), 1.0, out["fp64"]["f_lo"], Q.Model.Linear)
        rates = {}
        for label, form, fk, prec in (
                ("resident", Q.QEW_RK_RESIDENT, fld, Q.QEW_PREC_FP64),
                ("resident_poly", Q.QEW_RK_RESIDENT, fld_poly, Q.QEW_PREC_FP64),
                ("resident_reference_exact", Q.QEW_RK_RESIDENT, fld, Q.QEW_PREC_FP64_REFERENCE),
                ("plain", Q.QEW_RK_PLAIN, fld, Q.QEW_PREC_FP64)):
            if fk is None:
                continue
            rpp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                             runaway=2.0 * ny, max_sweeps=args.dep_rate_sweeps)
            # one untimed block first: a class's first call runs the autotuner's probe
            Q.rk_block(crit["fp64"].clone(),
                       Q.Params(float(n), 1.0, out["fp64"]["f_c"], Q.Model.Linear), fk,
                       Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10,
                                  sweep_tol=1e-8, runaway=2.0 * ny, max_sweeps=32),
                       form=form, precision=prec)
            h = crit["fp64"].clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = Q.rk_block(h, Q.Params(float(n), 1.0, out["fp64"]["f_c"], Q.Model.Linear), fk,
                           rpp, form=form, precision=prec)
            torch.cuda.synchronize()
            rates[label] = r.sweeps / (time.perf_counter() - t0)
        out["sweeps_per_s"] = rates
    first = next((k for k in ("fp64", "fp64_poly", "fp32split") if k in out), None)
    out["value"] = out[first]["wall_s"] if first else None
    return out


# ------------------------------------------------------------- serving (C4)
def run_serving(args, Q, torch):
    """Poisson request streams (seed 4) at each rate: 50% static minimise
    (FP64-refined to max|g| < 1e-8), 30% Langevin (serve_lsteps steps, T ~
    U[0, 0.5], dt 0.01), 20% depinning f_c (line relaxed at f = 0, ramp 0.05,
    bisection to 1e-2, 500 sweeps per block, FP32 velocities); L
    log-uniform in [512, 65536] (even), 256 or 1024
    rows, xi ~ U[2, 8]; each field generated on the device per request;
    admission by a 150 GB HBM budget; static lines shorter than 2048 points
    through the device-resident loop, the rest over serve_inflight workers.
    Every rate serves the same request list (only the arrival times differ),
    so the rates are compared on the same work."""
    rng = np.random.default_rng(4)
    rates = [float(x) for x in args.serve_rates.split(",") if x]
    N = args.serve_requests
    reqs = []
    for k in range(N):
        kind = int(rng.choice(3, p=[0.5, 0.3, 0.2]))
        n = int(round(np.exp(rng.uniform(np.log(512), np.log(65536))) / 2)) * 2
        r = dict(kind=kind, n=n, rows=int(rng.choice([256, 1024])),
                 xi=float(rng.uniform(2, 8)), seed=100000 + k, model=int(rng.integers(0, 2)))
        if kind == 1:
            r.update(steps=args.serve_lsteps, temperature=float(rng.uniform(0, 0.5)), dt=0.01)
        elif kind == 2:
            r.update(model=0, f_step=0.05, f_max=5.0, bisect_rtol=1e-2, max_sweeps=500,
                     max_advance=32.0, runaway=float(r["rows"]) / 4)
        reqs.append(r)
    gaps_unit = rng.exponential(1.0, N)
    out = {"metric": "serving latency p50/p99 and solves/s", "unit": "s",
           "budget_GB": 150, "inflight": args.serve_inflight, "requests_per_rate": N,
           "rates": [],
           "mix": "50%% static (1e-8), 30%% Langevin (%d steps), 20%% depinning f_c "
                  "(relaxed start, ramp 0.05, bisection to 1e-2, 500 sweeps per block)"
                  % args.serve_lsteps,
           "request_counts": {name: int(sum(r["kind"] == kind for r in reqs))
                              for kind, name in ((0, "static"), (1, "langevin"),
                                                 (2, "depinning"))},
           "device_loop_limit": args.serve_lane_max,
           "static_on_device_loop": int(sum(r["kind"] == 0 and r["n"] <= args.serve_lane_max
                                            for r in reqs))}
    for rate in rates:
        srv = Q.Server(hbm_budget_bytes=150e9, max_inflight=args.serve_inflight)
        srv.set_lane_limit(args.serve_lane_max)
        try:
            gaps = gaps_unit / rate
            t_next = srv.clock()
            for k in range(N):
                t_next += gaps[k]
                while srv.clock() < t_next:
                    time.sleep(min(1e-3, max(0.0, t_next - srv.clock())))
                srv.submit(**reqs[k])
            t_last_submit = srv.clock()
            srv.drain(3600)
            resps = srv.poll(N + 16)
            lane = srv.lane_stats()
        finally:
            srv.close()
        log("  serving rate %g: %d responses" % (rate, len(resps)))
        lat = np.array([r["t_end"] - r["t_submit"] for r in resps])
        t0 = min(r["t_submit"] for r in resps)
        span = max(r["t_end"] for r in resps) - t0
        per_kind = {}
        for kind, name in ((0, "static"), (1, "langevin"), (2, "depinning")):
            lk = [r["t_end"] - r["t_submit"] for r in resps if r["kind"] == kind]
            svc = [r["t_end"] - r["t_start"] for r in resps if r["kind"] == kind]
            if lk:
                per_kind[name] = {"count": len(lk), "p50_s": float(np.percentile(lk, 50)),
                                  "p99_s": float(np.percentile(lk, 99)),
                                  "service_p50_s": float(np.percentile(svc, 50))}
        out["rates"].append({
            "rate_per_s": rate, "requests": N, "arrival_span_s": t_last_submit - t0,
            "ok": int(sum(r["status"] == 0 for r in resps)),
            "static_converged_1e8": int(sum(r["kind"] == 0 and r["converged"] and
                                            r["max_force"] < 1e-8 for r in resps)),
            "depinning_with_f_c": int(sum(r["kind"] == 2 and r["converged"] for r in resps)),
            "service_s_total": float(sum(r["t_end"] - r["t_start"] for r in resps)),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "solves_per_s": N / span, "makespan_s": span, "per_kind": per_kind,
            "device_loop": lane})
    return out


# ---------------------------------------------------------------- our arm
def timed(torch, fn, steps, ctx):
    """Run fn() `steps` times between CUDA events on the current stream;
    returns (elapsed ms, number of this library's kernel launches)."""
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = ctx.launches()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), ctx.launches() - l0


def fp64_peak(Q, ctx):
    """FP64 FMA instructions/s of this GPU from the library's microbenchmark
    (best of three timed launches)."""
    best, ms = 0.0, None
    for _ in range(3):
        r, m = ctx.measure_fp64_fma_rate(4096)
        if r > best:
            best, ms = r, m
    return best, ms


# FP64 instructions (DFMA + DADD + DMUL, thread level) per line point of each
# FP64 kernel on the headline workload, from ncu's
# smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum of one
# launch divided by its points. For k_gradient these counters leave out its
# FP64 floor, conversions and compares, so its fraction reads low.
# k_gradient_poly: 7 on the headline's lines (f = 0, dx = 1: the zero-force
# form, 4 DFMA + 3 DADD); 8 at f != 0.
FP64_INST_PER_POINT = {"k_gradient_poly": 7.0, "k_gradient": 49.15}


def run_sections_only(args, Q, torch, rank):
    """The --sections configurations without the headline measurement: one
    JSON line of their results (for profiling a section's kernels)."""
    runners = {"refshape": run_reference_shape, "static": run_static,
               "ensemble": run_ensemble, "dynamics": run_dynamics,
               "depinning": run_depinning, "serving": run_serving}
    out = {}
    for name in [x.strip() for x in args.sections.split(",") if x.strip()]:
        log("%s section" % name)
        out[name] = runners[name](args, Q, torch)
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps({"sections": out,
                          "autotune": [ln for ln in Q.tune_report().splitlines() if ln]}),
              flush=True)
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from qew_gb300 import build as qbuild
    qbuild.build()
    import qew_gb300 as Q

    if args.no_headline:  # one configuration section alone (profiling runs)
        return run_sections_only(args, Q, torch, rank)
    if args.small:
        L, ny, n_inst = L_FULL, 64, N_INST
    else:
        L, ny, n_inst = L_FULL, NY_FULL, N_INST
    field = gaussian_field_gpu(torch, L, ny, XI, SEED + rank)
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32
    if not args.no_edge_store:
        store |= Q.QEW_STORE_FP32_EDGE
    if not args.no_poly_store:
        store |= Q.QEW_STORE_FP64_POLY
    torch.cuda.synchronize()
    t_setup = time.perf_counter()
    noise = Q.FilteredNoise(field, float(L), float(ny), store=store)
    torch.cuda.synchronize()
    field_setup = {"ms": 1e3 * (time.perf_counter() - t_setup),
                   "what": "prefilter of the resident field and every store the run reads "
                           "(FP64, FP32, x-filtered FP32, FP64 cell polynomials as selected)"}
    del field
    torch.cuda.empty_cache()
    rng = np.random.default_rng(SEED + 1000 * rank)
    band = ny / n_inst
    hs_host = [np.ascontiguousarray(band * (k + 0.5) + smooth_walk(rng, L, min(8.0, band / 8), 64.0))
               for k in range(n_inst)]
    H = torch.as_tensor(np.stack(hs_host), device="cuda")  # [n_inst, L], line k at k * L
    G = torch.empty_like(H)
    cells = torch.empty((n_inst, L), dtype=torch.int32, device="cuda")
    fracs = torch.empty((n_inst, L), dtype=torch.float32, device="cuda")
    for k in range(n_inst):
        c, fr = Q.split_heights(H[k], noise)
        cells[k].copy_(c)
        fracs[k].copy_(fr)
    g32 = torch.empty((n_inst, L), dtype=torch.float32, device="cuda")
    p = Q.Params(float(L), 1.0, 0.0, Q.Model.Linear)
    ctx = noise.ctx

    # The three forms of the gather on the same lines, each one step = the
    # gradients of all n_inst lines:
    #   fp64            FP64 drop-in: the cell-polynomial store, one batched
    #                   persistent launch (k_gradient_poly)
    #   fp64_reference  FP64 with the reference's arithmetic bit for bit (its
    #                   16-tap order, true divisions, no fused multiply-adds),
    #                   one launch per line (k_gradient)
    #   fp32split       FP32 split-index gather on the x-filtered FP32 store,
    #                   one batched persistent launch (k_gradient_split_persist)
    def step_fp64():
        Q.gradient_batch(H, p, noise, G)

    def step_fp64_ref():
        Q.gradient_batch(H, p, noise, G, precision=Q.QEW_PREC_FP64_REFERENCE)

    def step_split():
        Q.gradient_split_batch(cells, fracs, p, noise, g32)

    poly_kernel = "k_gradient" if args.no_poly_store else "k_gradient_poly"
    forms = {
        "fp64": (step_fp64, 48.0, poly_kernel, "f64"),
        "fp64_reference": (step_fp64_ref, 48.0, "k_gradient (reference-exact arithmetic)",
                           "f64"),
        "fp32split": (step_split, 28.0,
                      "k_gradient_split" if args.no_edge_store else "k_gradient_split_persist",
                      "f32"),
    }
    # The energy of the same lines, objective() once per line (each call
    # reads its scalar back to the host, as the reference's reduction does):
    # 40 B per point algorithmic (the 4 field rows' 32 B and the height).
    energies = np.empty(n_inst)

    def step_objective():
        for k in range(n_inst):
            energies[k] = Q.objective(H[k], p, noise)

    forms_extra = {"objective_fp64": (step_objective, 40.0, "k_objective", "f64")}
    head = args.precision
    warm = max(args.warmup, 3)
    for _ in range(warm):
        for fn, _, _, _ in forms.values():
            fn()
    torch.cuda.synchronize()
    step_main = forms[head][0]
    clocks = ClockSampler(local)
    if not args.profile_run:
        clocks.start()  # untimed warm-up steps keep the GPU loaded while the sampler starts
        t_end = time.perf_counter() + 0.8
        while time.perf_counter() < t_end:
            for _ in range(warm):
                step_main()
            torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t_ms, launches = timed(torch, step_main, args.steps, ctx)
    if ws > 1:
        t_ms = max_over_ranks(torch, t_ms, "cuda")
        torch.distributed.barrier()
    clk = clocks.stop() if not args.profile_run else None
    value = whole_job_rate(ws, args.steps, n_inst, L, t_ms)

    peak, peak_kind = measured_peak()
    fma_rate, fma_ms = fp64_peak(Q, ctx)

    def roofline(ms, nl, bpp, name):
        launch_ms = ms / max(nl, 1)
        points_per_launch = args.steps * n_inst * L / max(nl, 1)
        ach = bpp * points_per_launch / (launch_ms * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "traffic": None, "kernel": name, "bytes_per_point": bpp,
                "launch_us": launch_ms * 1e3, "launches": nl, "peak_source": peak_kind}

    def fp64_roofline(rate, name):
        ipp = FP64_INST_PER_POINT.get(name)
        if ipp is None:
            return None
        ach = ipp * rate
        return {"bound": "fp64", "achieved": ach / 1e9, "peak": fma_rate / 1e9,
                "unit": "G FP64 inst/s", "frac": ach / fma_rate, "kernel": name,
                "fp64_inst_per_point": ipp,
                "peak_source": "measured in this run: qew_measure_fp64_fma_rate, %d CTAs x 256 "
                               "threads x 8 independent FMA chains, CUDA events (%.2f ms)"
                               % (8 * torch.cuda.get_device_properties(local).multi_processor_count,
                                  fma_ms)}

    # DRAM bytes (read + write) per line point of each kernel from one ncu
    # capture of the bench's batched launch (8 lines of 2^20 points) on the
    # small field (each point touches the same number of rows whatever the
    # field height), scaled to the points of one launch. k_gradient_poly: a
    # warm launch inside the timed loop (--cache-control none); the others
    # cold (ncu's cache flush, which leaves out the previous launch's
    # write-back).
    dram_per_point = {
        "k_gradient_poly": (342.719232e6 + 69.857280e6) / (8 * L_FULL),
        "k_gradient_split_persist": (237.686784e6 + 22.566656e6) / (8 * L_FULL),
        "k_gradient_split": (241.858816e6 + 20.879104e6) / (8 * L_FULL),
        "k_gradient": (43.320832e6 + 0.039936e6) / L_FULL,
    }
    results = {}
    for name, (fn, bpp, kern, dt) in list(forms.items()) + list(forms_extra.items()):
        if name == head:
            ms, nl, val = t_ms, launches, value
        else:
            ms, nl = timed(torch, fn, args.steps, ctx)
            val = whole_job_rate(ws, args.steps, n_inst, L, ms)
        roof = roofline(ms, nl, bpp, kern)
        pts = args.steps * n_inst * L / max(nl, 1)
        if kern in dram_per_point:
            roof["traffic"] = dram_per_point[kern] * pts
        results[name] = {"value": val, "unit": UNIT, "ms_per_step": ms / args.steps,
                         "dtype": dt, "roofline": roof,
                         "fp64_roofline": fp64_roofline(val / max(ws, 1), kern)}
    # The split form's API takes heights already split into (int32 cell,
    # FP32 fraction) and returns FP32 gradients; the split of the FP64 heights
    # is timed on its own here (one qew_split_heights call per line).
    ms_split, _ = timed(torch, lambda: [Q.split_heights(H[k], noise) for k in range(n_inst)],
                        args.steps, ctx)
    results["fp32split"]["timed_region"] = (
        "qew_gradient_split_batch on (cell, fraction) heights; the FP64 -> (cell, fraction) "
        "split of the step's lines (qew_split_heights) is outside it: %.1f us per step, "
        "timed alone" % (1e3 * ms_split / args.steps))
    results["fp32split"]["roofline"]["field_store"] = (
        "FP32 coefficients: 16 taps per edge" if args.no_edge_store else
        "FP32 coefficients plus the x-filtered copy: 4 taps per edge (the same rows, so the "
        "same DRAM bytes, as 16 taps)")
    results["fp64"]["roofline"]["field_store"] = (
        "FP64 coefficients: 16 taps per edge in the reference's order" if args.no_poly_store else
        "FP64 cell polynomials of the x-filtered field: one 32-byte cell per edge (the "
        "algorithmic 4 rows x 8 B of the reference's gather)")
    e2e = None
    cpu = None
    if not args.profile_run:
        # two sets of pinned host buffers, used in turn (256 MB per step pair:
        # nothing of one step's host data can still sit in L2 at the next)
        hh = [torch.as_tensor(np.stack(hs_host)).pin_memory().numpy() for _ in range(2)]
        gh = [torch.empty((n_inst, L), dtype=torch.float64).pin_memory().numpy()
              for _ in range(2)]

        def e2e_rate(name, prec):
            for k in range(2):
                Q.gradient_host_batch(hh[k], p, noise, gh[k], precision=prec)
            torch.cuda.synchronize()
            e2e_steps = max(4, args.steps)
            if ws > 1:
                torch.distributed.barrier()
            t0 = time.perf_counter()
            for k in range(e2e_steps):
                Q.gradient_host_batch(hh[k & 1], p, noise, gh[k & 1], precision=prec)
            dt = time.perf_counter() - t0
            if ws > 1:  # the slowest replica's time, as for the device-timed value
                dt = max_over_ranks(torch, dt * 1e3, "cuda") * 1e-3
            return {"value": ws * e2e_steps * n_inst * L / dt, "unit": UNIT,
                    "h2d_bytes_per_step": n_inst * L * 8, "d2h_bytes_per_step": n_inst * L * 8,
                    "call": "qew_gradient_host_batch (precision %s): the step's 8 lines as "
                            "FP64 pinned host heights in, FP64 pinned host gradients out; the "
                            "kernels read and write the mapped host buffers over the host link "
                            "(no staging copies)" % name}

        e2e_prec = {"fp64": Q.QEW_PREC_FP64, "fp64_reference": Q.QEW_PREC_FP64_REFERENCE,
                    "fp32split": Q.QEW_PREC_FP32_SPLIT}
        for name in (head,) + tuple(k for k in ("fp64", "fp32split") if k != head):
            results[name]["e2e"] = e2e_rate(name, e2e_prec[name])
        e2e = results[head]["e2e"]
    refshape = static = ensemble = dynamics = depinning = serving = None
    sections = set(s.strip() for s in args.sections.split(",") if s.strip())
    if not args.profile_run and sections:
        del noise, cells, fracs, g32, G, H
        torch.cuda.empty_cache()
        if "refshape" in sections:
            log("reference benchmark shape section")
            refshape = run_reference_shape(args, Q, torch)
            torch.cuda.empty_cache()
        if "static" in sections:
            log("static section")
            static = run_static(args, Q, torch)
            torch.cuda.empty_cache()
        if "ensemble" in sections and args.ensemble_lines > 0:
            log("ensemble section")
            ensemble = run_ensemble(args, Q, torch)
            torch.cuda.empty_cache()
        if "dynamics" in sections:
            log("dynamics section")
            dynamics = run_dynamics(args, Q, torch)
            torch.cuda.empty_cache()
        if "depinning" in sections:
            log("depinning section")
            depinning = run_depinning(args, Q, torch)
            torch.cuda.empty_cache()
        if "serving" in sections:
            log("serving section")
            serving = run_serving(args, Q, torch)
            log("serving done")
    if not args.profile_run:
        if rank == 0 and args.cpu_seconds > 0:
            cpu = cpu_gradient_rate(args.cpu_seconds)

    if rank == 0:
        if cpu is not None:
            for name in results:
                results[name]["cpu_baseline"] = cpu
        head_r = results[head]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": warm, "ms_per_step": t_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": head_r["dtype"], "data": "synthetic",
                "config": headline_config(L, ny, n_inst, head, ws),
                "roofline": head_r["roofline"], "fp64_roofline": head_r["fp64_roofline"],
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "field_setup": field_setup, "forms": {k: v for k, v in results.items() if k != head},
                "autotune": [ln for ln in Q.tune_report().splitlines() if ln],
                "reference_shape": refshape, "static": static, "ensemble": ensemble,
                "dynamics": dynamics,
                "depinning": depinning, "serving": serving}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
