"""SGDLM filtering throughput on GB300: time-steps/s at m = 400 with 10k IS draws.

One time step = computePosterior + computeVBPosterior(10k) + ESS-gated
setPosteriorParameters + computePrior + computeForecast(10k, 1 step), the loop
of the reference's README (README.md:103-154), at m = 400 series with
p_j <= 20 (3 external predictors + Uniform{0..17} simultaneous parents).
Data: synthetic, simulated from a true SGDLM (Gamma off-diagonals ~ N(0, 0.1^2)
rescaled to spectral radius 0.5, external coefficients ~ N(0, 0.3^2), precisions
lambda_j ~ Gamma(5, rate 5/400)); priors a = 0, R = 0.1 I, r = 2, c = 0.0025;
beta = 0.97, Delta = 0.98.  Seeds are recorded in the output line.

  value : fused device-resident step (sgdlm_filter_step_device), inputs staged in
          HBM before the timed region;
  e2e   : the same steps through the C ABI with host buffers (pinned), H2D of
          y_t, F_t, F_t+1 and D2H of the VB results and the forecast draws inside
          the timed region.
  fp64_gpu : the plain FP64 form (every kernel in FP64) on the same workload.
  precision_config_50k_draws : 50 000 IS draws and forecasts 1..5 steps ahead
          (10 000 draws each) per step, mixed and plain FP64 forms, C ABI calls
          with page-locked host outputs.
--impl reference runs the FP64 CPU implementation of the same step (the oracle
port: the reference has no CPU path and its CUDA build cannot be built on the
Arm GPU host) on all host cores: whole time steps at the full draw counts after
a reduced-draw burn-in; the line reports the steps that ran.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "time-steps/s at m=400, 10k IS draws"
LU_FLOPS_PER_DRAW = lambda m: 2.0 / 3.0 * m ** 3  # noqa: E731  dense LU of (I - Gamma)


# ----------------------------------------------------------------- workload
def make_workload(m=400, n_ext=3, kmax=17, T=16, seed=20261203):
    """True-SGDLM synthetic series (the C1 recipe at m series)."""
    rng = np.random.default_rng(seed)
    ks = rng.integers(0, kmax + 1, size=m)
    p = (n_ext + ks).astype(np.uint32)
    P = int(n_ext + kmax)
    NA = 2147483648
    sp = np.full((P, m), NA, dtype=np.uint32, order="F")
    Gam = np.zeros((m, m))
    for j in range(m):
        others = np.delete(np.arange(m), j)
        pars = rng.choice(others, size=ks[j], replace=False)
        for t, par in enumerate(pars):
            sp[n_ext + t, j] = j + m * par
            Gam[j, par] = rng.normal(0, 0.1)
    rho = np.max(np.abs(np.linalg.eigvals(Gam)))
    if rho > 0.5:
        Gam *= 0.5 / rho
    phi = rng.normal(0, 0.3, size=(m, n_ext))
    lam = rng.gamma(5.0, 1.0 / (5.0 / 400.0), size=m)  # E lambda = 400 (sd 0.05)
    ImG = np.eye(m) - Gam
    y = np.zeros((T + 2, m))
    X = np.zeros((T + 2, m, n_ext))
    for t in range(1, T + 2):
        X[t, :, 0] = 1.0
        X[t, :, 1] = y[t - 1]
        X[t, :, 2] = rng.normal(0, 1, m)
        nu = (X[t] * phi).sum(1) + rng.normal(0, 1, m) / np.sqrt(lam)
        y[t] = np.linalg.solve(ImG, nu)

    def F_of(t, with_parents=True):
        F = np.zeros((P, m), order="F")
        F[:n_ext, :] = X[t].T
        if with_parents:
            for j in range(m):
                for k in range(n_ext, p[j]):
                    F[k, j] = y[t, sp[k, j] // m]
        return F

    return dict(m=m, P=P, p=p, sp=sp, y=y, F_of=F_of, seed=seed, n_ext=n_ext)


def prior_arrays(m, P):
    a = np.zeros((P, m), order="F")
    R = np.asfortranarray(np.repeat((0.1 * np.eye(P))[:, :, None], m, axis=2))
    return a, R, np.full(m, 2.0), np.full(m, 0.0025)


# --------------------------------------------------------------- clock sampler
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx, self.rows, self.proc = device_index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def ready(self, timeout=3.0):
        """Waits for nvidia-smi's first sample (its start-up takes longer than a
        short timed region), then forgets the samples taken so far, so that the
        ones kept are those of the region that follows."""
        t_end = time.time() + timeout
        while self.proc and not self.rows and time.time() < t_end:
            time.sleep(0.01)
        self.rows = []

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d, "of measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "of fallback"


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, rank, world):
    import torch

    from gpusgdlm_gb300 import SGDLM
    from gpusgdlm_gb300 import _lib as L

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    T_total = args.burn_in + args.warmup + args.steps + args.e2e_steps + args.fp64_steps + 12
    wl = make_workload(m=args.m, T=T_total, seed=args.seed + rank)
    m, P, n = wl["m"], wl["P"], args.nsim
    s = SGDLM(1, strict=True, precision=args.precision)
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    a, R, r, c = prior_arrays(m, P)
    s.setPriorParameters(a, R, r, c)
    s.setRngState(1234 + 100 * rank, 0)
    s._ensure_sim(n, n)
    lib, h = s._lib, s._h
    stream = torch.cuda.ExternalStream(s.stream(), device=dev)
    ess_thr = n / 2.0

    # stage every step's inputs in HBM (burn-in, warm-up and timed steps)
    nsteps = args.burn_in + args.warmup + args.steps
    ys = torch.tensor(np.stack([wl["y"][t] for t in range(1, nsteps + 1)]), dtype=torch.float64, device=dev)
    Fs = torch.tensor(np.stack([wl["F_of"](t).ravel(order="F") for t in range(1, nsteps + 1)]),
                      dtype=torch.float64, device=dev)
    Xs = torch.tensor(np.stack([wl["F_of"](t + 1, False).ravel(order="F") for t in range(1, nsteps + 1)]),
                      dtype=torch.float64, device=dev)
    yout = torch.zeros(n * m, dtype=torch.float64, device=dev)
    wout = torch.zeros(n, dtype=torch.float64, device=dev)
    stout = torch.zeros(8, dtype=torch.float64, device=dev)

    def step(t):
        ok = s.filterStepDevice(ys[t].data_ptr(), Fs[t].data_ptr(), Xs[t].data_ptr(), ess_thr,
                                yout.data_ptr(), wout.data_ptr(), stout.data_ptr())
        assert ok

    torch.cuda.synchronize()
    # burn-in: filter past the diffuse-prior transient (setup, untimed), then warm-up
    for t in range(args.burn_in + args.warmup):
        step(t)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    clocks.ready()
    launches0 = s.launchCount()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for t in range(args.burn_in + args.warmup, nsteps):
        step(t)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = s.launchCount() - launches0
    barrier(world)
    clk = clocks.stop()
    accepted = float(stout[2].item())
    ess_last = float(stout[0].item())

    # e2e through the C ABI with pinned host buffers, continuing the same filter
    e2e = run_e2e(args, s, wl, rank, world, t0=nsteps + 1)

    # per-kernel timing of the dominant kernel (batched LU) with CUDA events on
    # the engine's stream (the API path records them around its phases)
    lu_ms, vb_ms, sample_ms, fc_ms, pivoted, ess_rate = [], [], [], [], [], []
    for k in range(3):
        t = nsteps + 1 + args.e2e_steps + 2 + k
        s.computePosterior(wl["y"][t], wl["F_of"](t))
        s.computeVBPosterior(n, n)
        st = s.getStats()
        lu_ms.append(st["ms_lu"]); vb_ms.append(st["ms_vb"]); sample_ms.append(st["ms_sample"])
        pivoted.append(st["draws_pivoted"])
        ess_rate.append(st["ess"] / (st["ms_total"] / 1000.0))  # ESS per second of VB device time
        s.computePrior()
        s.computeForecast(n, n, wl["F_of"](t + 1, False))
        fc_ms.append(s.getStats()["ms_lu_forecast"])
    info = s.getEliminationInfo()
    dpad = (info["core_n"] + 31) // 32 * 32
    exec_flops = n * (2.0 / 3.0 * dpad ** 3)
    fp64 = None
    if args.precision == "mixed" and args.fp64_steps > 0:
        t_next = nsteps + 1 + args.e2e_steps + 2 + 3
        fp64 = run_fp64_form(args, s, wl, t_next, dev, rank)
    return dict(ms=ms, launches=launches, clocks=clk, accepted=accepted, ess=ess_last, fp64=fp64,
                exec_flops=exec_flops, core_n=info["core_n"], levels=info["levels"],
                lu_ms=statistics.median(lu_ms), vb_ms=statistics.median(vb_ms),
                sample_ms=statistics.median(sample_ms), fc_ms=statistics.median(fc_ms),
                pivoted=int(max(pivoted)), e2e=e2e, m=m, P=P,
                ess_per_s=statistics.median(ess_rate))


def run_fp64_form(args, s_mixed, wl, t0, dev, rank):
    """The plain FP64 form (every kernel in FP64, the reference's arithmetic) on
    the same workload, continuing from the mixed engine's current prior state:
    fused device steps with inputs staged in HBM, CUDA events on the engine's
    stream."""
    import torch

    from gpusgdlm_gb300 import SGDLM

    m, P, n = wl["m"], wl["P"], args.nsim
    st = s_mixed.getParameters()
    s = SGDLM(1, strict=True, precision="fp64")
    s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
    s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
    s.setPriorParameters(st["m"], st["C"], st["n"], st["s"])
    s.setRngState(5678 + 100 * rank, 0)
    s._ensure_sim(n, n)
    stream = torch.cuda.ExternalStream(s.stream(), device=dev)
    k_warm, k = 1, args.fp64_steps
    ts = range(t0, t0 + k_warm + k)
    ys = torch.tensor(np.stack([wl["y"][t] for t in ts]), dtype=torch.float64, device=dev)
    Fs = torch.tensor(np.stack([wl["F_of"](t).ravel(order="F") for t in ts]), dtype=torch.float64,
                      device=dev)
    Xs = torch.tensor(np.stack([wl["F_of"](t + 1, False).ravel(order="F") for t in ts]),
                      dtype=torch.float64, device=dev)
    yout = torch.zeros(n * m, dtype=torch.float64, device=dev)
    wout = torch.zeros(n, dtype=torch.float64, device=dev)

    def step(i):
        assert s.filterStepDevice(ys[i].data_ptr(), Fs[i].data_ptr(), Xs[i].data_ptr(), n / 2.0,
                                  yout.data_ptr(), wout.data_ptr(), None)

    for i in range(k_warm):
        step(i)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(k_warm, k_warm + k):
        step(i)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    s.close()
    return dict(ms=ms, steps=k)


def run_c2(args):
    """The precision configuration at its stated per-step sizes: m = 400, p_j <= 20,
    50 000 IS draws per VB call and forecasts 1..5 steps ahead with 10 000 samples
    each, through the C ABI with page-locked host outputs (the VB results and the
    forecast draws of all five horizons, 160 MB, written to host memory every
    step), the mixed form and the plain FP64 form from the same prior state after
    a 30-step burn-in (2 000 draws); wall clock per time step, every call
    synchronous."""
    import torch

    from gpusgdlm_gb300 import SGDLM
    from gpusgdlm_gb300 import _lib as L

    m, n_vb, n_fc, K = 400, 50000, 10000, 5
    wl = make_workload(m=m, T=60, seed=args.seed)
    P = wl["P"]

    def engine(precision):
        # corrected samplers: the reference's beta sampler of the evolution
        # (make_beta, kernel_functions.cuh:725-798; Marsaglia-Tsang without the
        # boost below shape one) gives NaN for shapes below 1/3, which (1 - beta) r / 2
        # reaches here, and would make every 2..5-step forecast draw NaN
        s = SGDLM(1, strict=True, precision=precision, compat=L.COMPAT_NONE)
        s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
        s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
        return s

    pin = lambda shape: torch.zeros(int(np.prod(shape)), dtype=torch.float64).pin_memory().numpy()  # noqa: E731
    dp = C.POINTER(C.c_double)
    ptr = lambda a: a.ctypes.data_as(dp)  # noqa: E731
    om, oC, on, os_, ow = pin((P, m)), pin((P, P, m)), pin((m,)), pin((m,)), pin((n_vb,))
    ofc = [pin((m, n_fc)) for _ in range(K)]
    sw = C.c_double()
    staged = {}
    for t in range(1, 50):
        yb, Fb = pin((m,)), pin((P, m))
        yb[:] = wl["y"][t]
        Fb[:] = wl["F_of"](t).ravel(order="F")
        Xs = []
        for k in range(1, K + 1):
            Xb = pin((P, m))
            Xb[:] = wl["F_of"](t + k, False).ravel(order="F")
            Xs.append(Xb)
        staged[t] = (yb, Fb, Xs)

    def step(s, t):
        lib, h = s._lib, s._h
        yb, Fb, Xs = staged[t]
        assert lib.sgdlm_compute_posterior(h, ptr(yb), ptr(Fb)) == 0
        s._ensure_sim(n_vb, n_vb)
        assert lib.sgdlm_compute_vb_posterior(h, ptr(om), ptr(oC), ptr(on), ptr(os_), ptr(ow),
                                              C.byref(sw)) == 0
        if 1.0 / float(np.dot(ow, ow)) > n_vb / 2:
            assert lib.sgdlm_set_parameters(h, ptr(om), ptr(oC), ptr(on), ptr(os_)) == 0
            lib.sgdlm_set_is_prior(h, 0)
        assert lib.sgdlm_compute_prior(h, 0) == 0
        s._ensure_sim(n_fc, n_fc)
        assert lib.sgdlm_init_forecast_priors(h) == 0
        for k in range(K):  # RcppWrapper.cpp:455-472
            if k > 0:
                assert lib.sgdlm_evolve_forecast_samples(h) == 0
            assert lib.sgdlm_compute_forecast(h, ptr(ofc[k]), ptr(Xs[k]), None, None,
                                              1 if k > 0 else 0) == 0

    s = engine("mixed")
    a, R, r, c = prior_arrays(m, P)
    s.setPriorParameters(a, R, r, c)
    s.setRngState(1234, 0)
    t = 1
    for _ in range(30):
        s.computePosterior(wl["y"][t], wl["F_of"](t))
        vb = s.computeVBPosterior(2000, 2000)
        if 1.0 / np.sum(vb["IS_weights"] ** 2) > 1000:
            s.setPosteriorParameters(vb["m"], vb["C"], vb["n"], vb["s"])
        s.computePrior()
        t += 1
    st = s.getParameters()
    seed, epoch = s.getRngState()
    f = engine("fp64")
    f.setPriorParameters(st["m"], st["C"], st["n"], st["s"])
    f.setRngState(seed, epoch)
    out = {}
    for name, e, k in (("mixed", s, args.c2_steps), ("fp64", f, max(1, args.c2_steps // 2))):
        step(e, t)  # warm-up: allocations of both draw counts
        t0 = time.perf_counter()
        for q in range(k):
            step(e, t + 1 + q)
        dt = time.perf_counter() - t0
        out[name] = {"time_steps_per_s": k / dt, "ms_per_step": 1000.0 * dt / k, "timed_steps": k}
        e.close()
    return {"workload": f"m={m}, p_j<=20, {n_vb} IS draws + forecasts k=1..{K} x {n_fc} draws per "
                        "step, C ABI with page-locked host outputs, corrected samplers (compat off)",
            "mixed": out["mixed"], "fp64": out["fp64"],
            "speedup_mixed_vs_fp64": out["mixed"]["time_steps_per_s"] / out["fp64"]["time_steps_per_s"],
            "burn_in_steps": 30}


def run_c3(args):
    """The batched form: 64 independent instances with m_i ~ Uniform{20..400}
    (p_j <= 20, the true-SGDLM data with per-instance seeds), 10k IS draws and a
    10k-draw one-step forecast per instance per step, mixed precision.  After a
    few burn-in steps, timed time steps of (a) every instance one at a time
    (its fused device step, synchronised before the next instance), (b) the
    batch: one CUDA-graph launch per time step whose branches run concurrently,
    (c) the batch after the autotuner (LU plan per m bucket, LU grid
    concurrency).  Inputs of each step are staged in HBM beforehand and copied
    into the recorded buffers with one device copy per step."""
    import torch

    from gpusgdlm_gb300 import Batch, SGDLM

    K, n = args.c3_instances, args.nsim
    rng = np.random.default_rng(args.seed + 3)
    ms = rng.integers(20, 401, size=K)
    T = args.c3_burn_in + args.c3_steps + 2
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    engines, wls = [], []
    for k, m in enumerate(ms):
        m = int(m)
        wl = make_workload(m=m, kmax=17, T=T + 1, seed=args.seed + 1000 + k)
        P = wl["P"]
        s = SGDLM(1, strict=True, precision="mixed")
        s.setSimultaneousParents(wl["p"], np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float))
        s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
        a, R, r, c = prior_arrays(m, P)
        s.setPriorParameters(a, R, r, c)
        s.setRngState(5000 + k, 0)
        s._ensure_sim(n, n)
        engines.append(s)
        wls.append(wl)
    # packed per-step inputs: for instance k, y (m), F (P m), x (P m)
    sizes = [wl["m"] * (1 + 2 * wl["P"]) for wl in wls]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    staged = np.zeros((T, offs[-1]))
    for t in range(1, T):
        for k, wl in enumerate(wls):
            m, P = wl["m"], wl["P"]
            o = offs[k]
            staged[t, o:o + m] = wl["y"][t]
            staged[t, o + m:o + m + P * m] = wl["F_of"](t).ravel(order="F")
            staged[t, o + m + P * m:o + m + 2 * P * m] = wl["F_of"](t + 1, False).ravel(order="F")
    staged = torch.tensor(staged, dtype=torch.float64, device=dev)
    cur = torch.zeros(offs[-1], dtype=torch.float64, device=dev)
    fcs = [torch.zeros(n * wl["m"], dtype=torch.float64, device=dev) for wl in wls]
    base = cur.data_ptr()
    yp = [base + 8 * int(offs[k]) for k in range(K)]
    Fp = [base + 8 * int(offs[k] + wls[k]["m"]) for k in range(K)]
    xp = [base + 8 * int(offs[k] + wls[k]["m"] * (1 + wls[k]["P"])) for k in range(K)]
    b = Batch(engines)
    b.record(yp, Fp, xp, n / 2.0, [f.data_ptr() for f in fcs], None, None)

    def load(t):
        cur.copy_(staged[t])
        torch.cuda.synchronize()

    def batched(t0, t1):
        for t in range(t0, t1):
            load(t)
            b.step()
        for s in engines:
            s.synchronize()

    def one_at_a_time(t0, t1):
        for t in range(t0, t1):
            load(t)
            for k, s in enumerate(engines):
                assert s.filterStepDevice(yp[k], Fp[k], xp[k], n / 2.0, fcs[k].data_ptr(), None, None)
                s.synchronize()

    t = 1
    batched(t, t + args.c3_burn_in)
    t += args.c3_burn_in
    # every form runs the same time steps from the same state (parameters and
    # Philox position of every instance restored before each)
    snap = [(s.getParameters(), s.getRngState()) for s in engines]

    def restore():
        for s, (p, rs) in zip(engines, snap):
            s.setPriorParameters(p["m"], p["C"], p["n"], p["s"])
            s.setRngState(*rs)
        torch.cuda.synchronize()

    res = {}
    tune = None
    for name, fn in (("one_at_a_time", one_at_a_time), ("batched", batched),
                     ("batched_autotuned", batched)):
        if name == "batched_autotuned":
            tune = b.autotune(replays=3)
        restore()
        fn(t, t + 1)  # warm-up
        t0 = time.perf_counter()
        fn(t + 1, t + args.c3_steps)
        res[name] = (args.c3_steps - 1) / (time.perf_counter() - t0)
    b.close()
    for s in engines:
        s.close()
    return {"workload": f"{K} instances, m in [{int(ms.min())}, {int(ms.max())}] (Uniform{{20..400}}), "
                        f"p_j<=20, {n} IS + {n} forecast draws per instance per step, mixed",
            "time_steps_per_s": res,
            "instance_steps_per_s": {k: v * K for k, v in res.items()},
            "speedup_batched_autotuned_vs_one_at_a_time": res["batched_autotuned"] / res["one_at_a_time"],
            "autotune": tune, "timed_steps": args.c3_steps - 1, "burn_in_steps": args.c3_burn_in,
            "note": "wall clock per time step (a host synchronisation per step for the input copy); "
                    "the three forms run the same time steps from the same restored state"}


def run_c4(args):
    """The learned-proposal configuration: m = 200, p_j <= 15 (3 external +
    Uniform{0..12} simultaneous parents), the true-SGDLM data, T = 2000 steps of
    computePosterior + computeVBPosterior(10k) + ESS-gated update + computePrior,
    once with the plain proposal and once with the learned one (trained on the
    first 500 calls' pairs with Adam, lr 1e-3, batch 4096, then deployed with the
    plain fallback below ESS = 50 %).  ESS/s = ESS / VB device time, over the
    deployed calls 501..2000.  Moment accuracy: at a few deployed steps both
    proposals' VB posteriors (10k draws, mixed) from the learned run's naive
    posterior against plain IS with 200,000 FP64 draws (rms error of the means in
    units of the judge's posterior sd)."""
    from gpusgdlm_gb300 import SGDLM

    m, T, n, train = 200, args.c4_steps, args.nsim, min(500, args.c4_steps // 4)
    wl = make_workload(m=m, kmax=12, T=T + 2, seed=args.seed + 4)
    P = wl["P"]
    sp = np.where(wl["sp"] >= m * m, np.nan, wl["sp"]).astype(float)

    def engine(precision="mixed", seed=4321):
        s = SGDLM(1, strict=True, precision=precision)
        s.setSimultaneousParents(wl["p"], sp)
        s.setDiscountFactors(np.full(m, 0.97), np.full((P, P, m), 0.98))
        a, R, r, c = prior_arrays(m, P)
        s.setPriorParameters(a, R, r, c)
        s.setRngState(seed, 0)
        return s

    evals = sorted({train + (T - train) // 4, train + (T - train) // 2, T - 1})
    judge = engine("fp64", seed=777)
    plain_at = engine("mixed", seed=999)
    mask = np.zeros((P, m), dtype=bool)
    for j in range(m):
        mask[: wl["p"][j], j] = True
    out = {}
    for mode in ("plain", "learned"):
        s = engine()
        if mode == "learned":
            s.setProposal("learned", train_steps=train, iters_per_step=4, batch=4096, lr=1e-3,
                          ess_fraction=0.5, seed=args.seed)
        ess_rate, ess_frac, errs = [], [], {"learned": [], "plain": []}
        t0 = time.perf_counter()
        for t in range(1, T):
            s.computePosterior(wl["y"][t], wl["F_of"](t))
            post = s.getParameters() if (mode == "learned" and t in evals) else None
            vb = s.computeVBPosterior(n, n)
            st = s.getStats()
            if t > train:
                ess_rate.append(st["ess"] / (st["ms_total"] / 1000.0))
                ess_frac.append(st["ess"] / n)
            if post is not None:
                judge.setPosteriorParameters(post["m"], post["C"], post["n"], post["s"])
                ref = judge.computeVBPosterior(200000, 200000)
                plain_at.setPosteriorParameters(post["m"], post["C"], post["n"], post["s"])
                pv = plain_at.computeVBPosterior(n, n)
                sd = np.sqrt(np.stack([np.diag(ref["C"][:, :, j]) for j in range(m)], 1))
                for key, v in (("learned", vb), ("plain", pv)):
                    z = (v["m"] - ref["m"])[mask] / sd[mask]  # active coefficients only
                    errs[key].append(float(np.sqrt(np.mean(z ** 2))))
            if 1.0 / np.sum(vb["IS_weights"] ** 2) > n / 2:
                s.setPosteriorParameters(vb["m"], vb["C"], vb["n"], vb["s"])
            s.computePrior()
        wall = time.perf_counter() - t0
        info = s.getProposalInfo()
        out[mode] = dict(ess_per_s=statistics.median(ess_rate), ess_fraction=statistics.median(ess_frac),
                         wall_s=wall, info=info, moment_rms_sd={k: v for k, v in errs.items() if v})
        s.close()
    judge.close()
    plain_at.close()
    return {"workload": f"m={m}, p_j<=15, T={T}, {n} VB draws, learned proposal trained on calls "
                        f"1..{train}, ESS/s over calls {train + 1}..{T - 1} (VB device time)",
            "plain": out["plain"]["ess_per_s"], "learned": out["learned"]["ess_per_s"],
            "ratio": out["learned"]["ess_per_s"] / out["plain"]["ess_per_s"],
            "ess_fraction": {k: out[k]["ess_fraction"] for k in out},
            "learned_calls": int(out["learned"]["info"]["learned_calls"]),
            "fallbacks": int(out["learned"]["info"]["fallbacks"]),
            "final_training_loss": out["learned"]["info"]["last_loss"],
            "moment_rms_error_vs_200k_fp64_judge": out["learned"]["moment_rms_sd"],
            "eval_steps": evals,
            "wall_s": {k: out[k]["wall_s"] for k in out}}


def run_e2e(args, s, wl, rank, world, t0):
    import torch

    lib, h = s._lib, s._h
    m, P, n = wl["m"], wl["P"], args.nsim
    pin = lambda shape: torch.zeros(int(np.prod(shape)), dtype=torch.float64).pin_memory().numpy()  # noqa: E731
    om, oC, on, os_, ow, of = pin((P, m)), pin((P, P, m)), pin((m,)), pin((m,)), pin((n,)), pin((m, n))
    sw = C.c_double()
    dp = C.POINTER(C.c_double)
    ptr = lambda a: a.ctypes.data_as(dp)  # noqa: E731
    h2d = d2h = 0
    steps = args.e2e_steps

    # every step's inputs sit in pinned host buffers before the timed region (the
    # synthetic data is generated outside it); the calls copy them to the device
    staged = {}
    for t in range(t0, t0 + steps + 1):
        yb, Fb, Xb = pin((m,)), pin((P, m)), pin((P, m))
        yb[:] = wl["y"][t]
        Fb[:] = wl["F_of"](t).ravel(order="F")
        Xb[:] = wl["F_of"](t + 1, False).ravel(order="F")
        staged[t] = (yb, Fb, Xb)

    def one(t):
        nonlocal h2d, d2h
        y_h, F_h, X_h = staged[t]
        assert lib.sgdlm_compute_posterior(h, ptr(y_h), ptr(F_h)) == 0
        assert lib.sgdlm_compute_vb_posterior(h, ptr(om), ptr(oC), ptr(on), ptr(os_), ptr(ow), C.byref(sw)) == 0
        ess = 1.0 / float(np.dot(ow, ow))
        b_in = (m + 2 * P * m) * 8
        b_out = (P * m + P * P * m + 2 * m + n + 1 + n * m) * 8
        if ess > n / 2:
            assert lib.sgdlm_set_parameters(h, ptr(om), ptr(oC), ptr(on), ptr(os_)) == 0
            lib.sgdlm_set_is_prior(h, 0)
            b_in += (P * m + P * P * m + 2 * m) * 8
        assert lib.sgdlm_compute_prior(h, 0) == 0
        assert lib.sgdlm_init_forecast_priors(h) == 0
        assert lib.sgdlm_compute_forecast(h, ptr(of), ptr(X_h), None, None, 0) == 0
        return b_in, b_out

    one(t0)  # untimed: first call of this path
    barrier(world)
    start = time.perf_counter()
    for k in range(steps):
        bi, bo = one(t0 + 1 + k)
        h2d += bi; d2h += bo
    dt = time.perf_counter() - start
    return dict(seconds=dt, steps=steps, h2d=h2d / steps, d2h=d2h / steps)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    """The largest value of x over the ranks (the replicas' timing is the slowest one)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(ms_max, steps, world):
    """Whole-job time-steps/s: every replica advances its own filter `steps` times;
    the job's time is the slowest rank's."""
    return world * steps / (ms_max / 1000.0)


# --------------------------------------------------------------- CPU arms
def cpu_filter(m, nsim, threads, seed, burn_in, burn_in_draws, warmup, steps, single=None):
    """The FP64 oracle (tests/oracle_model.py over oracle/) running the same README
    time step on the host cores: burn_in untimed steps with burn_in_draws draws
    (the filter past the diffuse-prior transient, as the GPU arm), then warmup
    untimed and `steps` timed steps at the full nsim VB + nsim forecast draws.
    Returns the seconds of each timed step."""
    import oracle  # noqa: F401  (builds the oracle library if needed)

    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_model import OracleSGDLM

    wl = make_workload(m=m, T=burn_in + warmup + steps + 4, seed=seed)
    P = wl["P"]
    o = OracleSGDLM(wl["p"], wl["sp"], np.full(m, 0.97), np.full((P, P, m), 0.98), seed=77, epoch=0,
                    nthreads=threads)
    a, R, r, c = prior_arrays(m, P)
    o.set_parameters(a, R, r, c)

    def step(t, n):
        o.posterior(wl["y"][t], wl["F_of"](t))
        vb = o.vb(n)
        if 1.0 / np.sum(vb["IS_weights"] ** 2) > n / 2:
            o.set_parameters(vb["m"], vb["C"], vb["n"], vb["s"])
        o.prior()
        o.forecast(n, wl["F_of"](t + 1, False))

    t = 1
    for _ in range(burn_in):
        step(t, burn_in_draws)
        t += 1
    for _ in range(warmup):
        step(t, nsim)
        t += 1
    secs = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step(t, single or nsim)
        secs.append(time.perf_counter() - t0)
        t += 1
    return secs


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(args):
    """One measured full-size step of the FP64 oracle on all host threads after a
    reduced-draw burn-in (about 15 s of host work at m = 400), plus a one-thread
    sample scaled to the workload."""
    threads = host_threads()
    t0 = time.perf_counter()
    secs = cpu_filter(args.m, args.nsim, threads, args.seed, args.burn_in, args.cpu_burn_in_draws,
                      0, 1)
    total = time.perf_counter() - t0
    sample1 = max(50, args.cpu_sample // 10)
    secs1 = cpu_filter(args.m, args.nsim, 1, args.seed, 0, 0, 0, 1, single=sample1)
    return {"value": 1.0 / secs[0], "unit": "time-steps/s", "cores": threads, "kind": "port",
            "precision": "fp64",
            "sample": f"one full step ({args.nsim} VB + {args.nsim} forecast draws, m={args.m}) of "
                      f"the FP64 oracle on {threads} threads (OpenMP), measured: {secs[0]:.2f} s, "
                      f"after {args.burn_in} burn-in steps with {args.cpu_burn_in_draws} draws "
                      f"({total:.1f} s in all)",
            "single_thread": {"value": 1.0 / (secs1[0] * (args.nsim / sample1)), "unit": "time-steps/s",
                              "sample": f"{sample1} VB + {sample1} forecast draws from the prior in "
                                        f"{secs1[0]:.2f} s on 1 thread, scaled linearly to "
                                        f"{args.nsim} draws"}}


def run_reference_arm(args, config):
    """The reference arm: the FP64 CPU implementation of the step (the oracle port,
    the reference having no CPU path of its own), on all host threads, at the full
    workload: every timed step is one whole time step with nsim VB + nsim forecast
    draws.  A reduced-draw burn-in first takes the filter to the GPU arm's regime;
    warm-up and timed steps are capped (1 and 8) so that the run stays within a few
    minutes, and the line reports the counts that ran."""
    threads = host_threads()
    warm = min(args.warmup, 1)
    k = max(1, min(args.steps, args.ref_max_steps))
    t0 = time.perf_counter()
    secs = cpu_filter(args.m, args.nsim, threads, args.seed, args.burn_in, args.cpu_burn_in_draws,
                      warm, k)
    wall = time.perf_counter() - t0
    ms = 1000.0 * sum(secs)
    value = k / (ms / 1000.0)
    cfg = dict(config, precision="fp64")
    cb = {"value": value, "unit": "time-steps/s", "cores": threads, "kind": "port",
          "sample": f"{k} full time steps ({args.nsim} VB + {args.nsim} forecast draws, m={args.m}) "
                    f"of the FP64 oracle on {threads} threads, after {args.burn_in} untimed burn-in "
                    f"steps with {args.cpu_burn_in_draws} draws and {warm} untimed full step; "
                    f"{wall:.1f} s wall in all"}
    return {"metric": METRIC, "value": value, "unit": "time-steps/s", "n_gpus": args.gpus,
            "steps": k, "warmup": warm, "ms_per_step": ms / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (true-SGDLM simulation)", "config": cfg, "impl": "reference",
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "time-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "requested": {"steps": args.steps, "warmup": args.warmup}}


# --------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--m", type=int, default=400)
    ap.add_argument("--nsim", type=int, default=10000)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--burn-in", type=int, default=30,
                    help="untimed filter steps run first to reach the steady state")
    ap.add_argument("--cpu-sample", type=int, default=1000,
                    help="draws of the one-thread CPU sample (a tenth of this)")
    ap.add_argument("--cpu-burn-in-draws", type=int, default=1000,
                    help="draws per burn-in step of the CPU arms")
    ap.add_argument("--ref-max-steps", type=int, default=8,
                    help="cap on the reference arm's timed full-size steps")
    ap.add_argument("--fp64-steps", type=int, default=3,
                    help="timed steps of the plain FP64 form (0: skip)")
    ap.add_argument("--c2-steps", type=int, default=4,
                    help="timed steps of the 50k-draw, five-horizon configuration (0: skip)")
    ap.add_argument("--c3-instances", type=int, default=64,
                    help="instances of the batched-form comparison (0: skip)")
    ap.add_argument("--c3-steps", type=int, default=12)
    ap.add_argument("--c3-burn-in", type=int, default=10)
    ap.add_argument("--c4-steps", type=int, default=2000,
                    help="time steps of the learned-proposal comparison (0: skip)")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", 1))
    rank = int(os.environ.get("RANK", 0))
    config = {"workload": f"SGDLM filter step, m={args.m}, p_j<=20 (3 external + Uniform{{0..17}} "
                          f"simultaneous parents), {args.nsim} IS draws + {args.nsim} 1-step forecast draws",
              "m": args.m, "max_p": 20, "nsim": args.nsim, "precision": args.precision,
              "parallelism": f"replicas x{world}", "l2": "working set > L2 (theta draws "
              f"{args.m * args.nsim * 20 * 4 / 1e6:.0f} MB rewritten per pass)",
              "burn_in_steps": args.burn_in, "seeds": {"data": args.seed, "philox": 1234}}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference_arm(args, config)))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    r = run_gpu(args, rank, world)
    ms = max_over_ranks(r["ms"], world)
    e2e_s = max_over_ranks(r["e2e"]["seconds"], world)
    if rank != 0:
        return
    value = job_value(ms, args.steps, world)
    pk, which = peaks()
    lu_flops = args.nsim * LU_FLOPS_PER_DRAW(args.m)
    achieved = lu_flops / (r["lu_ms"] / 1000.0) / 1e12
    peak = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    traffic_file = ROOT / "profiles" / "lu_traffic.json"
    traffic = None
    if traffic_file.exists():
        tj = json.loads(traffic_file.read_text())
        if tj.get("m") == args.m:
            traffic = tj["bytes_per_draw"] * args.nsim
    line = {
        "metric": METRIC, "value": value, "unit": "time-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 draws/LU + f64 state/LSE/Newton" if args.precision == "mixed" else "f64",
        "data": "synthetic (true-SGDLM simulation)", "config": config,
        "clocks": r["clocks"], "gpu_launches": r["launches"],
        "e2e": {"value": world * r["e2e"]["steps"] / e2e_s, "unit": "time-steps/s",
                "h2d_bytes_per_step": int(r["e2e"]["h2d"]), "d2h_bytes_per_step": int(r["e2e"]["d2h"])},
        "roofline": {"kernel": "k_lu (batched LU, log|det| of 10k draws)", "bound": "tensor",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_note": f"bf16 dense sustained {which}",
                     "traffic": traffic, "algorithmic_flops": lu_flops,
                     "note": "achieved = dense-equivalent n*(2/3)m^3 flop / LU time; the kernel "
                             "executes the sparse pre-elimination plus a dense LU of the core",
                     "executed_flops": r["exec_flops"],
                     "executed_tflops": r["exec_flops"] / (r["lu_ms"] / 1000.0) / 1e12},
        "phases_ms": {"sample": r["sample_ms"], "lu": r["lu_ms"], "vb": r["vb_ms"],
                      "forecast_lu_solve": r["fc_ms"]},
        "draws_pivoted_max": r["pivoted"],
        "elimination": {"levels": r["levels"], "dense_core": r["core_n"]},
        "is_draws_per_s": value * args.nsim,
        "fp64_gpu": None if r["fp64"] is None else {
            "value": r["fp64"]["steps"] / (r["fp64"]["ms"] / 1000.0), "unit": "time-steps/s",
            "steps": r["fp64"]["steps"], "ms_per_step": r["fp64"]["ms"] / r["fp64"]["steps"],
            "speedup_of_value": value / (r["fp64"]["steps"] / (r["fp64"]["ms"] / 1000.0)),
            "note": "plain FP64 form: every kernel in FP64 (draws, LU, solves, moments), "
                    "same workload and fused device step, continuing from the mixed run's state"},
        "ess_last": r["ess"], "accepted_last": r["accepted"],
        "ess_per_s_m400": {"plain": r["ess_per_s"],
                           "note": "ESS of the decoupled (plain) proposal per second of "
                                   "computeVBPosterior device time at this workload"},
    }
    if args.c2_steps > 0:
        line["precision_config_50k_draws"] = run_c2(args)
    if args.c4_steps > 0:
        line["ess_per_s"] = run_c4(args)
    if args.c3_instances > 0:
        line["batched_instances"] = run_c3(args)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
