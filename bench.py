#!/usr/bin/env python
"""Benchmark of the 4D time-resolved TV reconstruction (rectv::run hot path).

Workload (one GPU): N=1024, Nz=64, Nzp=16, Ntheta=2880 over Nrot=8 half-turns,
M=16 time samples, titer=4, lambda0=1e-3, lambda1=4, centre N/2; synthetic
data = our forward operator applied to a seeded phantom of 10 moving
ellipsoids plus 1% Gaussian noise.  One step = one outer ADMM iteration over
the whole volume (titer forward/adjoint pairs, gradient-divergence steps,
shrink, dual update, rho rule).

  value  iterations/s with data resident in HBM (device-side session API),
         timed with CUDA events on the library's stream.
  e2e    iterations/s through the reference-facing C-ABI call rectv_run with
         pinned host buffers: upload, set-up, K iterations, download.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
For N > 1 launch with torch.distributed.run; every rank reconstructs its own
volume (independent replicas, weak scaling).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# hardware work queues for the concurrent streams of the multi-problem engine
# (read at CUDA initialisation; a per-process setting)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

WORKLOAD = dict(n=1024, nz=64, nzp=16, ntheta=2880, nrot=8, m=16, titer=4, lambda0=1e-3, lambda1=4.0)
SMALL = dict(n=256, nz=16, nzp=8, ntheta=720, nrot=8, m=16, titer=4, lambda0=1e-3, lambda1=4.0)
METRIC = "ADMM iters/s (outer iterations, titer=4) of the 4D TV reconstruction"
# launch groups timed by rectv_launch_kernel: 0 = forward gather, 1 = adjoint
# scatter, 2 = fused inner TV step, 3 = shrink / dual update, 4 / 5 = forward /
# inverse padded-grid 2D FFT (when 2n is a power of two).  The USFFT kernels
# depend on the geometry: scans that revisit their directions interpolate once
# per position (k_gather_dir; k_adj_mix + k_scatter_dir), others per ray on
# the tensor cores (k_gather_tc, plus k_gather_fwd for the few items near the
# centre of the spectrum; k_scatter_tc).
KERNEL_NAMES = {0: "k_gather_tc", 1: "k_scatter_tc", 2: "k_graddiv", 3: "k_shrink",
                4: "k_fft_rows_fwd+k_fft_cols_fwd", 5: "k_fft_cols_inv+k_fft_rows_inv", 6: "k_graddiv (first step)"}
KERNEL_NAMES_DIR = {**KERNEL_NAMES, 0: "k_gather_dir", 1: "k_adj_mix+k_scatter_dir"}


def workload_of(args):
    """The timed workload; --nz/--nzp override the slice counts (small cases for ncu captures)."""
    w = dict(SMALL if args.small else WORKLOAD)
    if getattr(args, "nz", None):
        w["nz"] = args.nz
    if getattr(args, "nzp", None):
        w["nzp"] = args.nzp
    return w


def workload_name(w):
    return ("N=%(n)d Nz=%(nz)d Nzp=%(nzp)d Ntheta=%(ntheta)d Nrot=%(nrot)d M=%(m)d titer=%(titer)d" % w)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, wl):
    """DRAM bytes per launch of `kernel` recorded from an ncu capture (profiles/)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        e = d.get(kernel, {}).get(wl)
        return None if e is None else float(e)
    except Exception:
        return None


# ---------------------------------------------------------------------------
# multi-rank aggregation (independent replicas, one per GPU)
# ---------------------------------------------------------------------------
def max_over_ranks(x, dist, device):
    """Largest value of x over all ranks (x unchanged without a process group)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(steps, world, ms):
    """Units all ranks processed (each rank: `steps` iterations) per second."""
    return world * steps / (ms * 1e-3)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1].split()[0]))
                    mx.append(float(p[2].split()[0]))
                except ValueError:
                    continue
                try:
                    pw.append(float(p[3].split()[0]))
                except ValueError:
                    pass
                for nm, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(mx),
                "power_w": statistics.median(pw) if pw else None, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# synthetic input on the device
# ---------------------------------------------------------------------------
def phantom_device(torch, w, seed, device):
    """phantom4d (rectv_gpu_gb300.phantom) evaluated on the GPU: same seeded
    parameter draws, ellipsoids rasterised with torch."""
    n, nz, m, ntheta = w["n"], w["nz"], w["m"], w["ntheta"]
    rng = np.random.default_rng(seed)
    x = torch.arange(n, dtype=torch.float32, device=device) - n / 2 + 0.5
    z = torch.arange(nz, dtype=torch.float32, device=device) - nz / 2 + 0.5
    u = torch.zeros((nz, m, n, n), dtype=torch.float32, device=device)
    tj = (np.arange(m) * ntheta) // m
    Y = x.view(1, n, 1)
    X = x.view(1, 1, n)
    Z = z.view(nz, 1, 1)
    for _ in range(10):
        c0 = np.array([rng.uniform(-0.3, 0.3) * nz, rng.uniform(-0.3, 0.3) * n, rng.uniform(-0.3, 0.3) * n])
        ax = np.array([rng.uniform(0.05, 0.3) * nz, rng.uniform(0.05, 0.3) * n, rng.uniform(0.05, 0.3) * n])
        ax = np.maximum(ax, 0.75)
        dens = rng.uniform(0.1, 1.0)
        ang = rng.uniform(0, np.pi)
        direc = rng.normal(size=2)
        direc /= np.linalg.norm(direc) + 1e-12
        disp = direc * rng.uniform(0, 0.1 * n)
        ca, sa = float(np.cos(ang)), float(np.sin(ang))
        for j in range(m):
            tau = tj[j] / ntheta
            cy = float(c0[1] + tau * disp[0])
            cx = float(c0[2] + tau * disp[1])
            dy, dx = Y - cy, X - cx
            ry = ca * dy - sa * dx
            rx = sa * dy + ca * dx
            inside = ((Z - float(c0[0])) / float(ax[0])) ** 2 + (ry / float(ax[1])) ** 2 + \
                (rx / float(ax[2])) ** 2 <= 1.0
            u[:, j] += dens * inside.to(torch.float32)
    return u


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 oracle on a bounded sample, extrapolated
# ---------------------------------------------------------------------------
def cpu_sample(w, angle_stride=30):
    """Time one basis function of the oracle's fwdR and adjR for one slice on
    every `angle_stride`-th angle, plus one slice of gradient/divergence, and
    extrapolate to one outer ADMM iteration of the whole workload."""
    import scipy.fft as sfft
    from oracle import rectv_oracle as orc
    n, ntheta, m, nz, titer = w["n"], w["ntheta"], w["m"], w["nz"], w["titer"]
    theta = np.linspace(0, w["nrot"] * np.pi, ntheta, endpoint=False).astype(np.float32)
    sub = theta[::angle_stride]
    frac = ntheta / sub.size
    U = orc.USFFT(n, sub, n / 2)
    rng = np.random.default_rng(0)
    f = rng.standard_normal((1, n, n)) + 0j
    g = rng.standard_normal((1, sub.size, n)) + 0j
    workers = os.cpu_count() or 1
    with sfft.set_workers(workers):
        orig_fft2, orig_ifft2 = np.fft.fft2, np.fft.ifft2
        np.fft.fft2 = lambda a: sfft.fft2(a, workers=workers)
        np.fft.ifft2 = lambda a: sfft.ifft2(a, workers=workers)
        try:
            t0 = time.perf_counter()
            U.fwd(f)
            t1 = time.perf_counter()
            U.adj(g)
            t2 = time.perf_counter()
        finally:
            np.fft.fft2, np.fft.ifft2 = orig_fft2, orig_ifft2
    # split the measured times into the angle-proportional and fixed parts
    P = 2 * n
    a = rng.standard_normal((P, P)) + 0j
    t3 = time.perf_counter()
    sfft.fft2(a, workers=workers)
    t4 = time.perf_counter()
    tfft2 = t4 - t3
    fwd = max(tfft2, t1 - t0)
    adj = max(tfft2, t2 - t1)
    per_slice_basis = 2 * tfft2 + (fwd - tfft2) * frac + (adj - tfft2) * frac
    # gradient + divergence of one slice chunk (the TV part)
    fm = rng.standard_normal((3, m, n, n))
    t5 = time.perf_counter()
    h = orc.gradient(fm, w["lambda1"], 0, 0)
    orc.divergent(h, w["lambda1"], -0.5)
    t6 = time.perf_counter()
    tv_slice = t6 - t5
    t_iter = titer * nz * (m * per_slice_basis + tv_slice) + nz * tv_slice
    sample = ("FP64 oracle: fwdR+adjR of 1 slice x 1 basis on %d of %d angles (+ one 2048^2 FFT pair), "
              "gradient/divergence of 1 slice; extrapolated x%d bases x%d slices x%d inner steps"
              % (sub.size, ntheta, m, nz, titer))
    return 1.0 / t_iter, t6 - t0 + (t4 - t3), sample, workers


def fp64_accuracy(torch, w, g_h, theta, phi, iters, nsub=2):
    """Relative L2 error of the GPU reconstruction against the FP64 oracle
    after every outer iteration, on a subset of the workload: `nsub` middle
    slices of the same data, solved as one chunk of the same geometry (N,
    Ntheta, M, titer, lambdas).  The FP64 side is the PyTorch transcription of
    the oracle in float64 on the GPU, run in lockstep; it follows its own rho
    rule, and whether both sides took the same rho decisions is reported."""
    from oracle import rectv_oracle_torch as ort
    from rectv_gpu_gb300 import rectv
    n, ntheta, m, nz, titer = w["n"], w["ntheta"], w["m"], w["nz"], w["titer"]
    lam0, lam1 = w["lambda0"] * w["lambda1"], w["lambda1"]
    z0 = nz // 2 - nsub // 2
    g = np.ascontiguousarray(g_h[z0:z0 + nsub].numpy())
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.perf_counter()
    obj = rectv(n, ntheta, m, nsub, nsub, 1)
    obj.set_verbose(False)
    dg = torch.from_numpy(g).to(dev)
    dth = torch.from_numpy(theta).to(dev)
    dph = torch.from_numpy(phi).to(dev)
    out = torch.empty((nsub, m, n, n), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    obj.setup_device(dg.data_ptr(), dth.data_ptr(), dph.data_ptr(), n / 2, lam0, lam1, titer)
    errs = []

    def step(it, f):
        obj.iterate(1)
        obj.result_device(out.data_ptr())
        obj.synchronize()
        errs.append(float(torch.linalg.vector_norm(out.to(torch.float64) - f) / torch.linalg.vector_norm(f)))

    try:
        _, h64 = ort.run(g, theta, phi, n / 2, lam0, lam1, iters, titer, nsub, device=dev, return_history=True,
                         callback=step)
        hist = obj.history()
    finally:
        obj.free()
    return {"max": max(errs), "final": errs[-1], "iterations": iters, "per_iteration": errs,
            "subset": "slices %d-%d of the workload's data as one chunk (Nz=Nzp=%d), same N, Ntheta, M, titer, "
                      "lambdas; FP64 oracle (PyTorch transcription, float64 on the GPU) in lockstep"
                      % (z0, z0 + nsub - 1, nsub),
            "same_rho_decisions": list(hist["rho"]) == [x["rho"] for x in h64],
            "seconds": time.perf_counter() - t0}


# ---------------------------------------------------------------------------
# batched form and serving loop (many problems of uneven size on one GPU)
# ---------------------------------------------------------------------------
MIX = dict(n=(256, 512, 1024), nz=(4, 64), ntheta=(720, 1440, 2880), m=(8, 16), nrot=8, titer=4, lambda0=1e-3,
           lambda1=4.0)


def draw_jobs(seed, count, iters):
    """Problems of the batched / serving mix: N from {256, 512, 1024}, Nz
    uniform in [4, 64] (one chunk: Nzp = Nz), Ntheta from {720, 1440, 2880},
    M from {8, 16}; `iters` = (lo, hi) outer iterations, uniform."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        n = int(rng.choice(MIX["n"]))
        nz = int(rng.integers(MIX["nz"][0], MIX["nz"][1] + 1))
        ntheta = int(rng.choice(MIX["ntheta"]))
        m = int(rng.choice(MIX["m"]))
        niter = int(rng.integers(iters[0], iters[1] + 1))
        jobs.append(dict(n=n, nz=nz, nzp=nz, ntheta=ntheta, m=m, nrot=MIX["nrot"], niter=niter,
                         titer=MIX["titer"], seed=seed * 1000 + i))
    return jobs


def make_job_data(torch, jobs, device):
    """Per job: its own seeded phantom, forward-projected with this library's
    operator plus 1% Gaussian noise, in page-locked host memory; and a
    page-locked output array."""
    from rectv_gpu_gb300 import rectv, takephi
    from rectv_gpu_gb300.phantom import scan_angles
    groups = {}
    for j in jobs:
        groups.setdefault((j["n"], j["ntheta"], j["m"]), []).append(j)
    for (n, ntheta, m), js in groups.items():
        nzmax = max(j["nz"] for j in js)
        theta = scan_angles(ntheta, MIX["nrot"])
        phi = takephi(ntheta, m)
        obj = rectv(n, ntheta, m, nzmax, nzmax, 1)
        d_th = torch.from_numpy(theta).to(device)
        d_ph = torch.from_numpy(phi).to(device)
        torch.cuda.synchronize()
        obj.op_set_geometry(d_th.data_ptr(), d_ph.data_ptr(), n / 2)
        for j in js:
            w = dict(n=n, nz=j["nz"], m=m, ntheta=ntheta)
            u = phantom_device(torch, w, seed=j["seed"], device=device)
            dg = torch.empty((j["nz"], ntheta, n), dtype=torch.float32, device=device)
            torch.cuda.synchronize()
            obj.op_radonapr(dg.data_ptr(), u.data_ptr(), j["nz"], 1.0)
            gen = torch.Generator(device=device).manual_seed(j["seed"])
            dg += 0.01 * float(dg.abs().max()) * torch.randn(dg.shape, generator=gen, device=device)
            gh = torch.empty(dg.shape, dtype=torch.float32, pin_memory=True)
            gh.copy_(dg)
            j["g"] = gh
            j["out"] = torch.empty((j["nz"], m, n, n), dtype=torch.float32, pin_memory=True)
            j["theta"], j["phi"] = theta, phi
            del u, dg
        obj.free()
        del obj
        torch.cuda.synchronize()
    torch.cuda.empty_cache()  # the engine's budget is the free device memory
    return jobs


def run_engine(jobs, arrivals, max_resident=0, autotune=False, largest_first=False, age_priority=True, keep=None,
               shortest_first=False):
    """Runs the jobs through the engine; returns per-job info and stats."""
    from rectv_gpu_gb300.engine import Engine
    with Engine(max_resident=max_resident, autotune=autotune, largest_first=largest_first,
                age_priority=age_priority, shortest_first=shortest_first) as eng:
        ids = []
        for j, a in zip(jobs, arrivals):
            ids.append(eng.submit(j["g"].numpy(), j["theta"], j["phi"], nzp=j["nzp"], niter=j["niter"],
                                  titer=j["titer"], lambda0=MIX["lambda0"], lambda1=MIX["lambda1"], arrival=a,
                                  out=j["out"].numpy(), copy_input=False))
        eng.run()
        infos = [eng.info(i) for i in ids]
        st = eng.stats()
        if keep is not None:
            keep.extend(j["out"].numpy().copy() for j in jobs)
    bad = [x for x in infos if x["status"] != "done"]
    if bad:
        raise RuntimeError("engine jobs failed: %s" % bad[0]["error"])
    return infos, st


def job_work(j):
    return float(j["n"]) ** 2 * j["m"] * j["nz"] * j["niter"]


def pretune(torch, jobs, device):
    """Autotunes the launch shapes of every distinct problem shape once, in
    isolation (the engine then applies the cached shapes at admission)."""
    from rectv_gpu_gb300 import rectv
    seen = {}
    t0 = time.perf_counter()
    for j in jobs:
        key = (j["n"], j["ntheta"], j["m"], j["nz"], j["nzp"])
        if key in seen:
            continue
        obj = rectv(j["n"], j["ntheta"], j["m"], j["nz"], j["nzp"], 1)
        obj.set_verbose(False)
        dg = j["g"].to(device)
        d_th = torch.from_numpy(j["theta"]).to(device)
        d_ph = torch.from_numpy(j["phi"]).to(device)
        torch.cuda.synchronize()
        obj.setup_device(dg.data_ptr(), d_th.data_ptr(), d_ph.data_ptr(), j["n"] / 2,
                         MIX["lambda0"] * MIX["lambda1"], MIX["lambda1"], j["titer"])
        seen[key] = obj.autotune()
        obj.free()
        del obj, dg
    torch.cuda.synchronize()
    return {"%dx%dx%dx%d" % k[:4]: v for k, v in seen.items()}, time.perf_counter() - t0


SCHEDULES = [("all_concurrent", 0), ("two_concurrent", 2)]  # candidates of the chunk schedule (max running jobs)


def batched_form(torch, device, count=32, iters=8, seed=4):
    """Config 4: `count` slice chunks of the mix, all arriving at once, run
    by the engine (autotuned launch shapes, most work first, age priority)
    under each candidate chunk schedule -- every chunk concurrently, or at
    most two at a time -- and one at a time.  The faster schedule is the one
    reported (and the one the serving run uses)."""
    jobs = make_job_data(torch, draw_jobs(seed, count, (iters, iters)), device)
    tuned, tune_s = pretune(torch, jobs, device)
    work = sum(job_work(j) for j in jobs)
    run_engine(jobs[:2], [0.0, 0.0], autotune=True)  # warm-up of the engine path
    outs, runs = {}, {}
    for name, mr in SCHEDULES + [("one_at_a_time", 1)]:
        keep = []
        infos, st = run_engine(jobs, [0.0] * len(jobs), max_resident=mr, autotune=True, largest_first=True,
                               keep=keep)
        outs[name] = keep
        runs[name] = {"max_running": mr or "all", "makespan_s": st["makespan"],
                      "voxel_updates_per_s": work / st["makespan"], "peak_running": st["peak_running"],
                      "peak_bytes": st["peak_bytes"]}
    best = min((n for n, _ in SCHEDULES), key=lambda n: runs[n]["makespan_s"])
    same = all(all(np.array_equal(a, b) for a, b in zip(outs[n], outs["one_at_a_time"])) for n in outs)
    return {
        "workload": "%d slice chunks: N from {256,512,1024}, Nz uniform in [4,64] (Nzp=Nz), Ntheta from "
                    "{720,1440,2880}, M from {8,16}, Nrot=8, titer=4, %d outer iterations each, seeded phantoms "
                    "(seed %d)" % (count, iters, seed),
        "voxel_updates": work,
        "schedule": best,
        "voxel_updates_per_s": runs[best]["voxel_updates_per_s"], "makespan_s": runs[best]["makespan_s"],
        "one_at_a_time_voxel_updates_per_s": runs["one_at_a_time"]["voxel_updates_per_s"],
        "speedup_vs_one_at_a_time": runs["one_at_a_time"]["makespan_s"] / runs[best]["makespan_s"],
        "runs": runs,
        "results_equal_one_at_a_time": same,
        "autotune": {"shapes": tuned, "seconds": tune_s,
                     "note": "(gather slices per block, scatter persistent blocks; 0 = the default: two per SM "
                             "on the direction path, one per SM on the per-ray path) per NxNthetaxMxNz, timed in "
                             "isolation before the runs"},
        "shapes": [[j["n"], j["nz"], j["ntheta"], j["m"]] for j in jobs],
    }, jobs


def serving_form(torch, device, throughput, count, iters, max_running, seed=5, load=0.8):
    """Config 5: a Poisson stream of `count` requests of the mix with `iters`
    outer iterations each, at `load` times the rate the batched throughput
    sustains; continuous batching (admission by the HBM budget as memory and
    slots free up, resident state, up to `max_running` jobs overlapping on
    the device, age priority) against one request at a time (same arrivals),
    each with requests admitted in arrival order and with the arrived request
    of least work first."""
    jobs = make_job_data(torch, draw_jobs(seed, count, iters), device)
    mean_work = sum(job_work(j) for j in jobs) / count
    rate = load * throughput / mean_work
    rng = np.random.default_rng(seed + 77)
    arrivals = list(np.cumsum(rng.exponential(1.0 / rate, size=count)))
    work = sum(job_work(j) for j in jobs)
    out = {"workload": "%d requests of the batched mix with %d-%d outer iterations each (titer=4), Poisson "
                       "arrivals at %.3f requests/s (%.0f%% of the batched throughput)"
                       % (count, iters[0], iters[1], rate, 100 * load),
           "rate_per_s": rate}
    for name, mr, sjf in (("continuous_batching", max_running, False), ("one_at_a_time", 1, False),
                          ("continuous_batching_shortest_first", max_running, True),
                          ("one_at_a_time_shortest_first", 1, True)):
        infos, st = run_engine(jobs, arrivals, max_resident=mr, autotune=True, shortest_first=sjf)
        lat = np.array([x["latency"] for x in infos])
        out[name] = {"max_running": mr or "all", "admission": "least work first" if sjf else "arrival order",
                     "p50_latency_s": float(np.percentile(lat, 50)),
                     "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
                     "makespan_s": st["makespan"], "requests_per_s": count / st["makespan"],
                     "voxel_updates_per_s": work / st["makespan"], "peak_running": st["peak_running"]}
    return out


CONFIG2 = dict(n=512, nz=32, nzp=8, ntheta=1440, nrot=8, m=16, titer=4, lambda0=1e-3, lambda1=4.0)


def _ref_seconds_per_iter(g, theta, phi, w, iters):
    """Seconds per outer iteration of the reference's CUDA build on g:
    (time of run(1 + iters) - time of run(1)) / iters, in a child process."""
    from oracle import ref_run
    n = g.shape[2]
    _, info = ref_run.run(g, theta, phi, n / 2, w["lambda0"] * w["lambda1"], w["lambda1"], 1, w["titer"], w["nzp"],
                          time_niters=[1, 1 + iters], timeout=3000)
    return (info["times"][1] - info["times"][0]) / iters


def plain_fp32(torch, device, w, value, iters=2, steps=10):
    """The reference's own CUDA build -- the plain FP32 form, src/cuda/*.cu
    unchanged, compiled for sm_103a by oracle/ref_build.py -- timed through
    rectv::run in a child process, beside this library:

    * config 2 (N=512, Nz=32, Nzp=8, Ntheta=1440, M=16): both on the same
      data, both measured;
    * the benchmark workload: the reference cannot allocate it -- the size of
      psi and mu, (n+1)^2 (m+1)(nzp+1) nz/nzp float4 (rectv.cu:15-16), is
      computed in 32-bit int and overflows for n=1024, m=16, nz=64 (19.4e9),
      so the allocation fails and run() faults on the host.  Its time per
      outer iteration is extrapolated from single-chunk runs of the same
      geometry (Nz = Nzp = 2, 4, 7, a least-squares line a + b Nz per chunk)
      to 4 chunks of 16 slices."""
    from oracle import ref_build
    from rectv_gpu_gb300 import rectv, takephi
    from rectv_gpu_gb300.phantom import scan_angles
    if ref_build.build() is None:
        return {"unavailable": "the reference's CUDA sources are not on this machine"}
    out = {"what": "reference CUDA build (src/cuda/*.cu unchanged, nvcc sm_103a) through rectv::run: includes its "
                   "host-side norm loop and managed-memory prefetches"}
    t0 = time.perf_counter()
    # ---- config 2, measured on both sides ----
    c2 = CONFIG2
    theta2 = scan_angles(c2["ntheta"], c2["nrot"])
    phi2 = takephi(c2["ntheta"], c2["m"])
    obj = rectv(c2["n"], c2["ntheta"], c2["m"], c2["nz"], c2["nzp"], 1)
    obj.set_verbose(False)
    d_th = torch.from_numpy(theta2).to(device)
    d_ph = torch.from_numpy(phi2).to(device)
    u = phantom_device(torch, c2, seed=0, device=device)
    dg = torch.empty((c2["nz"], c2["ntheta"], c2["n"]), dtype=torch.float32, device=device)
    torch.cuda.synchronize()
    obj.op_set_geometry(d_th.data_ptr(), d_ph.data_ptr(), c2["n"] / 2)
    obj.op_radonapr(dg.data_ptr(), u.data_ptr(), c2["nz"], 1.0)
    gen = torch.Generator(device=device).manual_seed(7)
    dg += 0.01 * float(dg.abs().max()) * torch.randn(dg.shape, generator=gen, device=device)
    del u
    obj.setup_device(dg.data_ptr(), d_th.data_ptr(), d_ph.data_ptr(), c2["n"] / 2, c2["lambda0"] * c2["lambda1"],
                     c2["lambda1"], c2["titer"])
    obj.autotune()
    obj.iterate(3)
    stream = torch.cuda.ExternalStream(obj.stream, device=device)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    obj.iterate(steps)
    b.record(stream)
    torch.cuda.synchronize()
    ours2 = steps / (a.elapsed_time(b) * 1e-3)
    g2 = dg.cpu().numpy()
    obj.free()
    del obj, dg
    torch.cuda.empty_cache()
    ref2 = 1.0 / _ref_seconds_per_iter(g2, theta2, phi2, c2, iters)
    out["config2"] = {"workload": workload_name(c2), "reference_iter_per_s": ref2, "ours_iter_per_s": ours2,
                      "speedup": ours2 / ref2}
    # ---- the benchmark workload: single-chunk runs, extrapolated ----
    theta = scan_angles(w["ntheta"], w["nrot"])
    phi = takephi(w["ntheta"], w["m"])
    rng = np.random.default_rng(11)
    pts = []
    for nzs in (2, 4, 7):
        g = (0.01 * rng.standard_normal((nzs, w["ntheta"], w["n"]))).astype(np.float32)
        ws = dict(w, nz=nzs, nzp=nzs)
        pts.append((nzs, _ref_seconds_per_iter(g, theta, phi, ws, iters)))
    x = np.array([p[0] for p in pts], dtype=np.float64)
    y = np.array([p[1] for p in pts])
    bcoef, acoef = np.polyfit(x, y, 1)
    chunks = w["nz"] // w["nzp"]
    per = chunks * (acoef + bcoef * w["nzp"])
    out["workload"] = {"workload": workload_name(w), "reference_iter_per_s": 1.0 / per,
                       "reference_seconds_per_iteration": per, "kind": "extrapolated",
                       "single_chunk_runs": [{"nz": int(p[0]), "seconds_per_iteration": p[1]} for p in pts],
                       "model": "per chunk a + b*Nzp, a=%.3f s, b=%.3f s/slice, x%d chunks of %d slices"
                                % (acoef, bcoef, chunks, w["nzp"]),
                       "speedup": value * per}
    out["value"] = 1.0 / per
    out["unit"] = "iter/s"
    out["seconds"] = time.perf_counter() - t0
    return out


def run_reference_arm(args, rank):
    """--impl reference: the reference's algorithm (FP64 oracle restatement; the
    reference has no CPU path and its CUDA build cannot travel) on host cores."""
    if rank != 0:
        return 0
    w = workload_of(args)
    for _ in range(args.warmup):
        cpu_sample(w)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        v, s, sample, workers = cpu_sample(w)
        vals.append(v)
        secs += s
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(w), "kind": "cpu oracle sample, extrapolated"},
        "cpu_baseline": {"value": value, "unit": "iter/s", "cores": workers, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch

    import __graft_entry__
    __graft_entry__.build()
    from rectv_gpu_gb300 import rectv, takephi
    from rectv_gpu_gb300 import _lib
    from rectv_gpu_gb300.phantom import scan_angles

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    w = workload_of(args)
    n, nz, nzp, ntheta, m, titer = w["n"], w["nz"], w["nzp"], w["ntheta"], w["m"], w["titer"]
    lam0, lam1 = w["lambda0"] * w["lambda1"], w["lambda1"]
    center = n / 2
    theta = scan_angles(ntheta, w["nrot"])
    phi = takephi(ntheta, m)

    obj = rectv(n, ntheta, m, nz, nzp, 1)
    obj.set_verbose(False)
    lib = _lib.load()
    stream = torch.cuda.ExternalStream(obj.stream, device=dev)

    # synthetic data: phantom -> our forward operator -> +1% noise
    d_theta = torch.from_numpy(theta).to(dev)
    d_phi = torch.from_numpy(phi).to(dev)
    u = phantom_device(torch, w, seed=rank, device=dev)
    d_g = torch.empty((nz, ntheta, n), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    obj.op_set_geometry(d_theta.data_ptr(), d_phi.data_ptr(), center)
    obj.op_radonapr(d_g.data_ptr(), u.data_ptr(), nz, 1.0)
    gen = torch.Generator(device=dev).manual_seed(1000 + rank)
    sigma = 0.01 * float(d_g.abs().max())
    d_g += sigma * torch.randn(d_g.shape, generator=gen, device=dev)
    del u
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    obj.setup_device(d_g.data_ptr(), d_theta.data_ptr(), d_phi.data_ptr(), center, lam0, lam1, titer)
    ndir = obj.directions()
    names = KERNEL_NAMES_DIR if ndir > 0 else KERNEL_NAMES
    t_tune = time.perf_counter()
    tuned = obj.autotune()
    t_tune = time.perf_counter() - t_tune
    obj.iterate(args.warmup)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    obj.iterate(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    if dist:
        dist.barrier()
    hist = obj.history()

    kern = ctypes_int()
    ffts = ctypes_int()
    zbs = ctypes_int()
    _lib.check(lib.rectv_get_launch_counts(obj._h, kern[1], ffts[1], zbs[1]))
    launches_per_iter = kern[0].value

    # ---- per-kernel timing (roofline of the dominant kernel) ----
    import ctypes
    reps = 3
    ktimes = {}
    kids = (0, 1, 2, 3, 6) + ((4, 5) if lib.rectv_launch_kernel(obj._h, 4, 0) == 0 else ())
    for kid in kids:
        lib.rectv_launch_kernel(obj._h, kid, 1)  # warm
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        _lib.check(lib.rectv_launch_kernel(obj._h, kid, reps))
        b.record(stream)
        torch.cuda.synchronize()
        ktimes[kid] = a.elapsed_time(b) / reps
    # launches per outer iteration of each kernel: titer*nbatch (0,1,2), nbatch (3)
    nbatch = nz // zbs[0].value if zbs[0].value else 1
    share = {k: (nbatch if k == 3 else titer * nbatch) * ktimes[k] for k in ktimes if k != 6}
    if titer > 0:  # one first inner step (6) and titer - 1 later ones (2)
        share[2] = nbatch * (ktimes[6] + (titer - 1) * ktimes[2])
    dom = max(share, key=share.get)
    bytes_ = ctypes.c_double()
    flops = ctypes.c_double()
    _lib.check(lib.rectv_kernel_cost(obj._h, dom, ctypes.byref(bytes_), ctypes.byref(flops)))
    peak, peak_kind = measured_peaks()
    achieved = bytes_.value / (ktimes[dom] * 1e-3) / 1e9
    limiter = {
        "k_adj_mix+k_scatter_dir": "k_scatter_dir (~90% of the pair): per-cell FP32 sums of w E + w_perp E_perp "
                                   "over the entries touching each 4x4-cell block (two lanes per cell) -- latency of "
                                   "the shared-memory loads of E and of the packed-FMA chains with 16 warps per SM "
                                   "(two 8-warp blocks at 128 registers; issue ~54% active, L1/shared ~73% busy, FMA "
                                   "pipe ~38%); float2 atomics into the Hermitian half planes; DRAM ~20% of peak, so "
                                   "not DRAM-bound",
        "k_gather_dir": "latency of the footprint loads and block barriers (two 8-warp blocks per SM at 121 "
                        "registers, ~30 positions per tile and slice) and shared-memory bandwidth of the 81-tap "
                        "reads (L1/shared pipe ~70% busy); DRAM ~14% of peak",
        "k_scatter_tc": "block barriers and the per-cell ray sums on the CUDA cores (shared-memory loads), "
                        "the tcgen05 time-sample GEMM (3xTF32) at ~14% of the tensor pipe; DRAM traffic 4.0x "
                        "the algorithmic bytes (float2 atomics read and write every Hermitian half-plane cell "
                        "twice), about 1.7 TB/s (25% of the DRAM peak) at full size, so not DRAM-bound",
        "k_gather_tc": "shared-memory bandwidth of the per-sample 81-tap sums and of the TMEM -> shared "
                       "read-out of G, block barriers; TMA-staged footprints, DRAM traffic 3.0x the spectra "
                       "(overlapping footprints) at 8% of the DRAM peak",
        "k_graddiv": "HBM bandwidth", "k_shrink": "HBM bandwidth",
        KERNEL_NAMES[4]: "HBM bandwidth", KERNEL_NAMES[5]: "HBM bandwidth"}[names[dom]]
    fma = ctypes.c_double()
    fma2 = ctypes.c_double()
    _lib.check(lib.rectv_measure_fp32_peak(ctypes.byref(fma), ctypes.byref(fma2)))
    fp32_rate = flops.value / (ktimes[dom] * 1e-3) / 1e12
    roofline = {"bound": "hbm", "limiter": limiter, "kernel": names[dom], "achieved": achieved,
                "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(names[dom], workload_name(w)),
                "algorithmic_bytes": bytes_.value, "fp32_tflops": fp32_rate,
                "compute": {"fp32_equivalent_tflops": fp32_rate, "fp32_peak_tflops": fma2.value,
                            "fp32_peak_scalar_tflops": fma.value, "frac": fp32_rate / fma2.value,
                            "note": "flops of the direct formulation (81 taps x M time samples per polar sample, "
                                    "complex); the kernels do fewer (per-ray path: time samples mixed on the "
                                    "tensor cores; direction path: taps once per position for all rays of a "
                                    "direction). Peaks measured in this run (rectv_measure_fp32_peak): packed "
                                    "fma.rn.f32x2 and scalar fma.rn chains on every SM"},
                "ms_per_launch": ktimes[dom],
                "per_iteration_ms": {names[k]: share[k] for k in share}}

    # ---- the same workload on the per-ray tensor-core kernels (3xTF32 time-sample
    # mixing), for comparison: the geometry is rebuilt without direction sharing ----
    per_ray = None
    if ndir > 0 and rank == 0 and world == 1 and args.per_ray_steps > 0:
        os.environ["RECTV_DIRS"] = "0"
        try:
            obj.setup_device(d_g.data_ptr(), d_theta.data_ptr(), d_phi.data_ptr(), center, lam0, lam1, titer)
            obj.autotune()
            obj.iterate(2)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            obj.iterate(args.per_ray_steps)
            b.record(stream)
            torch.cuda.synchronize()
            pr_ms = a.elapsed_time(b) / args.per_ray_steps
            per_ray = {"value": 1e3 / pr_ms, "unit": "iter/s", "ms_per_step": pr_ms, "steps": args.per_ray_steps,
                       "what": "the same workload with RECTV_DIRS=0: every ray interpolated on its own, time "
                               "samples mixed on the tensor cores (k_gather_tc, k_scatter_tc)"}
        finally:
            os.environ.pop("RECTV_DIRS", None)
        obj.setup_device(d_g.data_ptr(), d_theta.data_ptr(), d_phi.data_ptr(), center, lam0, lam1, titer)
        obj.autotune()

    # ---- end-to-end through rectv_run with pinned host buffers ----
    g_h = torch.empty((nz, ntheta, n), dtype=torch.float32, pin_memory=True)
    g_h.copy_(d_g.cpu())
    th_h = torch.from_numpy(theta).pin_memory()
    ph_h = torch.from_numpy(phi).pin_memory()
    f_h = torch.empty((nz, m, n, n), dtype=torch.float32, pin_memory=True)
    del d_g
    # untimed warm-up call with the same arguments: the timed call then finds
    # the geometry, plans and captured graphs in place (as every call after a
    # user's first does; the first call is timed separately below)
    obj.run(f_h.data_ptr(), g_h.data_ptr(), th_h.data_ptr(), ph_h.data_ptr(), center, lam0, lam1,
            max(1, min(args.warmup, 3)), titer)
    if dist:
        dist.barrier()
    e2e_sampler = ClockSampler(local_rank)
    e2e_sampler.start()
    ea = torch.cuda.Event(enable_timing=True)
    eb = torch.cuda.Event(enable_timing=True)
    ea.record(stream)
    t0 = time.perf_counter()
    obj.run(f_h.data_ptr(), g_h.data_ptr(), th_h.data_ptr(), ph_h.data_ptr(), center, lam0, lam1, args.steps,
            titer)
    t1 = time.perf_counter()
    eb.record(stream)
    torch.cuda.synchronize()
    e2e_clocks = e2e_sampler.stop()
    e2e_gpu_s = ea.elapsed_time(eb) * 1e-3  # the call's span on the library's stream (copies and kernels)
    e2e_s = max_over_ranks(t1 - t0, dist, dev)
    h2d = g_h.numel() * 4 + th_h.numel() * 4 + ph_h.numel() * 4
    d2h = f_h.numel() * 4
    finite = bool(np.isfinite(f_h[:, :, ::64, ::64].numpy()).all())

    acc = None
    if rank == 0 and world == 1 and args.acc_iters > 0:
        acc = fp64_accuracy(torch, w, g_h, theta, phi, args.acc_iters)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu_sample(w)  # warm: FFT plans, thread pool
        v, s, sample, workers = cpu_sample(w)
        cpu = {"value": v, "unit": "iter/s", "cores": workers, "kind": "port", "sample": sample}

    value = whole_job_rate(args.steps, world, ms)
    voxels = float(n) * n * m * nz
    line = {
        "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: 10 moving ellipsoids, forward-projected with this library + 1% Gaussian noise",
        "config": {"workload": workload_name(w), "lambda0": w["lambda0"], "lambda1": lam1, "center": center,
                   "chunks": nz // nzp, "batch_slices": zbs[0].value,
                   "usfft_path": ("directions: %d directions x %d rays share their sample positions" %
                                  (ndir, ntheta // ndir)) if ndir > 0 else "per ray (tensor cores)",
                   "l2": "inputs larger than L2 (iterate 4.3 GB, dual variables 3x19 GB)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "voxel_updates_per_s": value * voxels,
        "e2e": {"value": whole_job_rate(args.steps, world, e2e_s * 1e3), "unit": "iter/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps, "seconds": e2e_s, "stream_seconds": e2e_gpu_s,
                "api": "rectv_run (C ABI)", "clocks": e2e_clocks},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches_per_iter * args.steps,
        "cufft_execs": ffts[0].value * args.steps,
        "rho_final": float(hist["rho"][-1]) if len(hist["rho"]) else None,
        "rel_err_vs_fp64": acc,
        "per_ray_path": per_ray,
        "autotune": {"gather_slices_per_block": tuned[0],
                     "scatter_blocks": tuned[1] or ("two per SM" if ndir > 0 else "one per SM"),
                     "seconds": t_tune},
        "result_finite": finite,
    }
    obj.free()
    del obj
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    if rank == 0 and world == 1:
        # first call: a fresh object (allocation, angle plan, adjoint records,
        # graph capture) and rectv_run, as a user's first reconstruction runs
        t0 = time.perf_counter()
        fresh = rectv(n, ntheta, m, nz, nzp, 1)
        fresh.set_verbose(False)
        fresh.run(f_h.data_ptr(), g_h.data_ptr(), th_h.data_ptr(), ph_h.data_ptr(), center, lam0, lam1,
                  args.steps, titer)
        t1 = time.perf_counter()
        fresh.free()
        del fresh
        line["e2e"]["first_call"] = {"value": args.steps / (t1 - t0), "unit": "iter/s", "seconds": t1 - t0,
                                     "what": "rectv(...) creation + rectv_run of the same steps"}
    del g_h, f_h
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and args.plain_iters > 0:
        line["plain_fp32"] = plain_fp32(torch, dev, w, value, args.plain_iters)
        if "value" in line["plain_fp32"]:
            line["plain_fp32"]["speedup_e2e"] = line["e2e"]["value"] / line["plain_fp32"]["value"]
    if rank == 0 and world == 1 and args.batched > 0:
        line["batched"], _ = batched_form(torch, dev, count=args.batched, iters=args.batched_iters)
        if args.serve > 0:
            mr = dict(SCHEDULES)[line["batched"]["schedule"]]
            line["serving"] = serving_form(torch, dev, line["batched"]["voxel_updates_per_s"], args.serve,
                                           tuple(args.serve_iters), mr)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def ctypes_int():
    import ctypes
    v = ctypes.c_int(0)
    return v, ctypes.byref(v)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--small", action="store_true", help="N=256 workload (quick check)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--plain-iters", type=int, default=2,
                    help="outer iterations of the reference CUDA build timed on the same data (0: skip)")
    ap.add_argument("--batched", type=int, default=32, help="slice chunks of the batched form (0: skip)")
    ap.add_argument("--batched-iters", type=int, default=8, help="outer iterations per batched chunk")
    ap.add_argument("--serve", type=int, default=32, help="requests of the serving run (0: skip)")
    ap.add_argument("--serve-iters", type=int, nargs=2, default=[8, 16],
                    help="range of outer iterations per request (the full serving config: 200 requests, 32 128)")
    ap.add_argument("--per-ray-steps", type=int, default=3,
                    help="outer iterations timed on the per-ray tensor-core kernels for comparison (0: skip)")
    ap.add_argument("--acc-iters", type=int, default=64,
                    help="outer iterations of the FP64 accuracy check on a 2-slice subset (0: skip)")
    ap.add_argument("--nz", type=int, default=None, help="slices (default: the workload's); for small ncu cases")
    ap.add_argument("--nzp", type=int, default=None, help="slices per chunk (default: the workload's)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference_arm(args, rank)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
