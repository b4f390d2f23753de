#!/usr/bin/env python
"""Benchmark of the 2-point hot path: GG on a 10M-point curved-sky catalog.

Workload (the curved-sky precision configuration): N = 10,000,000 points uniform on a
1000 deg^2 spherical cap; shear = an E-mode Gaussian random field with
xi+(theta) = 1e-4 (theta/1')^-0.8 drawn on a 4096^2 grid, plus N(0, 0.25) shape noise;
w ~ U[0.5, 1.5]; GG auto-correlation, Arc metric, 30 Log bins from 1 to 300 arcmin,
bin_slop 0.1, angle_slop 0.1 (the reference's defaults), split 'mean', min_top 3,
max_top 10.  The catalog is synthetic (seeded); no public dataset is involved.

One step = one pass of the hot path over the catalog: field construction from the
catalog columns (normalisation, float payloads), ball-tree build, dual-tree traversal,
accumulation and the final reduction into the caller's 8 output arrays.

metric: pair evaluations per second -- accepted cell pairs (directProcess11 calls in the
reference, src/Corr2.cpp:476-525) per second of the whole step.  The GPU path takes the
reference's accept/split decisions, so its count equals the reference's.

value: inputs resident in HBM (device columns), timed with CUDA events on the library's
stream.  e2e: the same step through the C ABI with host columns (pinned: the preparation
kernel reads them over the host link), the host->device transfer and the device->host read
of the results inside the timed region.  point_pairs_per_s counts the same step in point
pairs in range (sum of npairs), which does not depend on how pairs are grouped into cells.

Before the timed steps each entry runs the library's autotuner (tile leaf size and
expansion chunk, on 2% of the top-level pairs; reported in `tuning`).  The library's
default fixed-order expansion is on (bit-identical repeats; --fixed-order 0 turns it off).

The metric's accuracy clause (xi err <= 1e-4 vs FP64): bin_slop 0.1 redistributes the
shape noise of the pairs it accepts whole, and its xi differs from the all-pairs result by
a few percent of max|xi+|.  The line therefore carries
  * xi_err: the headline's max over bins of |d xi+-| / max|xi+| against the exact result
    (bin_slop 0, angle_slop 0) on the same catalog;
  * accurate: that exact configuration timed the same way (every pair in range counted at
    its own separation, the leaf-pair tiles), with its own e2e, its k_tiles roofline (FP32
    issue), its error against the FP64 oracle on a 200,000-point random subsample
    (xi_err_fp64) and the oracle's CPU rate there (cpu_baseline, vs_cpu).

The inputs (10M x 6 float64 columns = 480 MB, plus a tree of ~1.3 GB) are larger than L2,
so no L2 flush is needed between steps.

--impl reference times the reference algorithm's CPU implementation (the oracle port of
TreeCorr's C++, OpenMP on all host cores) on a bounded sample of the same workload: each
step processes a fixed set of top-level rows of the auto-correlation loop; value = pair
evaluations in the sample / time of the sample (the tree build is excluded, which favours
the CPU).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ARCMIN = np.pi / 180.0 / 60.0
METRIC = ("GG wall-s & pair-evals/s at N=10M, xi err<=1e-4 vs FP64; learned vs plain split "
          "(curved sky, Arc, 30 Log bins 1-300'; headline bin_slop 0.1, accurate entry "
          "bin_slop 0 / angle_slop 0)")
UNIT = "pair-evals/s"


# ----------------------------------------------------------------------------------------
# Synthetic catalog

def grf_shear(ngrid, pix_arcmin, rng, amp=1e-4, alpha=0.8):
    """E-mode shear field on a periodic ngrid^2 grid whose xi+ is amp*(theta/1')^-alpha.

    The 2D Fourier transform of theta^-alpha is 2^(2-alpha) pi Gamma(1-alpha/2) /
    Gamma(alpha/2) k^(alpha-2), which is the convergence power spectrum P(k) (k in 1/arcmin);
    gamma(k) = exp(2 i phi_k) kappa(k)."""
    from math import gamma, pi
    try:
        import scipy.fft as sfft
        fft2 = lambda a: sfft.fft2(a, workers=-1)       # noqa: E731
        ifft2 = lambda a: sfft.ifft2(a, workers=-1)     # noqa: E731
    except Exception:                                    # pragma: no cover
        fft2, ifft2 = np.fft.fft2, np.fft.ifft2
    k1 = 2 * np.pi * np.fft.fftfreq(ngrid, d=pix_arcmin)
    kx, ky = np.meshgrid(k1, k1, indexing="xy")
    ksq = kx * kx + ky * ky
    ksq[0, 0] = 1.0
    pk = amp * 2 ** (2 - alpha) * pi * gamma(1 - alpha / 2) / gamma(alpha / 2) * ksq ** ((alpha - 2) / 2)
    pk[0, 0] = 0.0
    noise = rng.standard_normal((ngrid, ngrid))
    w = fft2(noise)
    w *= np.sqrt(pk) * ((kx * kx - ky * ky) + 2j * kx * ky) / ksq
    g = ifft2(w) / pix_arcmin
    return g.real.astype(np.float64), g.imag.astype(np.float64)


def curved_sky_catalog(n, seed=20261203, area_deg2=1000.0, ngrid=4096):
    rng = np.random.default_rng(seed)
    r = np.arccos(1 - area_deg2 * (np.pi / 180) ** 2 / (2 * np.pi))   # cap radius (rad)
    u = rng.uniform(np.cos(r), 1.0, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    th = np.arccos(u)
    # Cap around the pole, rotated to (ra, dec) = (180, -30) deg.
    s = np.sin(th)
    v = np.stack([s * np.cos(phi), s * np.sin(phi), u])
    dec0, ra0 = np.radians(-30.0), np.radians(180.0)
    a = np.pi / 2 - dec0
    Ry = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    Rz = np.array([[np.cos(ra0), -np.sin(ra0), 0], [np.sin(ra0), np.cos(ra0), 0], [0, 0, 1]])
    v = Rz @ Ry @ v
    # Shear: GRF on the azimuthal-equidistant plane of the cap, plus shape noise.
    half = r / ARCMIN
    pix = 2 * half / ngrid
    g1f, g2f = grf_shear(ngrid, pix, rng)
    px = np.clip(((th / ARCMIN) * np.cos(phi) + half) / pix, 0, ngrid - 1).astype(np.int64)
    py = np.clip(((th / ARCMIN) * np.sin(phi) + half) / pix, 0, ngrid - 1).astype(np.int64)
    g1 = g1f[py, px] + rng.normal(0, 0.25, n)
    g2 = g2f[py, px] + rng.normal(0, 0.25, n)
    w = rng.uniform(0.5, 1.5, n)
    return dict(x=np.ascontiguousarray(v[0]), y=np.ascontiguousarray(v[1]),
                z=np.ascontiguousarray(v[2]), g1=g1, g2=g2, w=w)


def binning(bin_slop):
    min_sep, max_sep, nbins = 1.0 * ARCMIN, 300.0 * ARCMIN, 30
    bin_size = np.log(max_sep / min_sep) / nbins
    return dict(min_sep=min_sep, max_sep=max_sep, nbins=nbins, bin_size=bin_size,
                b=bin_slop * bin_size, a=0.1)


# ----------------------------------------------------------------------------------------
# Clock sampling during the timed region

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                p = [t.strip() for t in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ----------------------------------------------------------------------------------------
# GPU arm

def run_gpu(args, rank, world):
    import torch
    from treecorr_gb300 import _treecorr as T
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    T.SetDeterministic(bool(args.fixed_order))
    cat = curved_sky_catalog(args.n, seed=args.seed + rank)
    bins = binning(args.bin_slop)
    nb = bins["nbins"]
    cols = ["x", "y", "z", "g1", "g2", "w"]
    dcols = {k: torch.from_numpy(cat[k]).to(dev) for k in cols}
    hcols = {k: torch.from_numpy(cat[k]).pin_memory() for k in cols}
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(T.stream_handle(), device=dev)

    def outputs():
        return {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                          "weight", "npairs")}

    def corr_for(out):
        return T.GGCorr(T.Log, bins["min_sep"], bins["max_sep"], nb, bins["bin_size"],
                        bins["b"], bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0.,
                        0., out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"],
                        out["meanlogr"], out["weight"], out["npairs"])

    def device_field():
        return T.DeviceField(2, T.Sphere, args.n, dcols["x"].data_ptr(), dcols["y"].data_ptr(),
                             dcols["z"].data_ptr(), dcols["g1"].data_ptr(),
                             dcols["g2"].data_ptr(), dcols["w"].data_ptr(), 0, 0.0, 0.0, T.Mean,
                             0, False, 3, 10)

    # The autotuner picks the tile leaf size and expansion chunk on a sample of the top-level
    # pairs, once, outside the timed region; every step then uses its choice.
    t0 = time.perf_counter()
    f, c = device_field(), corr_for(outputs())
    tune = c.autotune(f, metric=T.Arc, frac=args.tune_frac) if args.tune_frac > 0 else \
        {"tile_leaf": 0, "chunk": 0, "ms": 0.}
    tune["tune_s"] = round(time.perf_counter() - t0, 2)
    tune["frac"] = args.tune_frac
    del f, c

    def step_device():
        out = outputs()
        f = device_field()
        c = corr_for(out)
        c.setTuning(tune["tile_leaf"], tune["chunk"])
        c.processAuto(f, False, False, T.Arc)
        st = c.stats()
        del f, c
        return out, st

    def step_host():
        out = outputs()
        e = np.array([])
        f = T.GFieldSphere(hcols["x"].numpy(), hcols["y"].numpy(), hcols["z"].numpy(),
                           hcols["g1"].numpy(), hcols["g2"].numpy(), hcols["w"].numpy(), e,
                           0.0, 0.0, T.Mean, 0, False, 3, 10)
        c = corr_for(out)
        c.setTuning(tune["tile_leaf"], tune["chunk"])
        c.processAuto(f, False, False, T.Arc)
        st = c.stats()
        del f, c
        return out, st

    def timed(fn, k):
        """k steps bracketed by barrier + synchronize; CUDA events on the library stream."""
        res = []
        launches0 = T.launch_count()
        barrier(world)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            res.append(fn())
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        ms = e0.elapsed_time(e1)
        return ms, res, T.launch_count() - launches0

    for _ in range(args.warmup):
        step_device()
    with ClockSampler(dev.index) as clk:
        ms, res, launches = timed(step_device, args.steps)
        # The accuracy clause: the same catalog with bin_slop 0 and angle_slop 0, where every
        # pair is added at its own separation (the leaf-pair tiles); timed inside the same
        # clock sampling.
        exact = None if args.no_exact else exact_entry(args, T, dcols, hcols, timed, world)
    clocks = clk.summary()
    if exact is not None:
        rf = exact["roofline"]
        rf["peak"] = round(rf["sms"] * 128 * 2 * (clocks.get("sm_mhz") or 2070.0) * 1e6 / 1e12, 1)
        rf["frac"] = round(rf["achieved"] / rf["peak"], 4)
    ms = allreduce_max(ms, world)
    acc_per_step = res[-1][1]["accepted"]
    value = world * acc_per_step * args.steps / (ms / 1e3)
    # e2e: host columns through the C ABI.
    for _ in range(max(1, args.warmup // 2)):
        step_host()
    ms_e2e, res_e2e, _ = timed(step_host, args.steps)
    ms_e2e = allreduce_max(ms_e2e, world)
    e2e = world * res_e2e[-1][1]["accepted"] * args.steps / (ms_e2e / 1e3)
    out, st = res[-1]
    # Roofline of the dominant kernel (k_expand, the breadth-first traversal): algorithmic
    # bytes = cell pairs evaluated x two 48-byte node reads (centre, size, weight, payload and
    # children of both cells), over k_expand's own device time, measured by the library with
    # CUDA events around every expansion launch on its stream (per launch: both divided by
    # the number of expansion launches).
    tr_ms = st["traverse_ms"]
    bytes_per_launch = st["cell_pairs"] * (2 * 48) / max(st["launches"], 1)
    per_launch_ms = st["expand_ms"] / max(st["launches"], 1)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    traffic = args.traffic
    if traffic is None and args.n == 10_000_000 and abs(args.bin_slop - 0.1) < 1e-12:
        # DRAM bytes per launch: 25.3 bytes per evaluated cell pair measured with ncu over a
        # whole 1M-point traversal, times the cell pairs per launch of this workload.
        traffic = round(25.3 * st["cell_pairs"] / max(st["launches"], 1))
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": traffic,
                "traffic_source": "ncu DRAM bytes per cell pair at 1M points, scaled"
                                  if args.traffic is None and traffic is not None else
                                  ("--traffic" if traffic is not None else None),
                "kernel": "k_expand",
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    h2d = sum(cat[k].nbytes for k in cols)
    d2h = 8 * nb * 8
    if exact is not None:
        # xi error of this line against the exact result on the same catalog (whose own
        # error against FP64 is measured on a subsample below): max over bins of |d xi+-|,
        # relative to max |xi+|.
        ex = exact.pop("_out")
        exact_xip, exact_xim = ex["xi0"] / ex["weight"], ex["xi2"] / ex["weight"]
        mx = float(np.abs(exact_xip).max())
        xip, xim = out["xi0"] / out["weight"], out["xi2"] / out["weight"]
        xi_err = {"vs": "bin_slop 0 / angle_slop 0 on the same catalog (the accurate entry)",
                  "xip": float(np.abs(xip - exact_xip).max() / mx),
                  "xim": float(np.abs(xim - exact_xim).max() / mx)}
        xi_err["max"] = max(xi_err["xip"], xi_err["xim"])
        xi_err["meets_1e-4"] = xi_err["max"] <= 1e-4
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded curved-sky GRF catalog)",
        "config": {"workload": "GG auto, 10M-point 1000 deg^2 cap, Arc, 30 Log bins 1-300', "
                               f"bin_slop {args.bin_slop}, angle_slop 0.1",
                   "n": args.n, "nbins": nb, "bin_slop": args.bin_slop,
                   "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (480 MB columns + 1.3 GB tree); no flush"},
        "fixed_order": bool(args.fixed_order),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e / args.steps},
        "gpu_launches": launches,
        # The same step counted in point pairs in range (sum of npairs): independent of how
        # an implementation groups them into cell pairs.
        "point_pairs_per_s": world * float(out["npairs"].sum()) * args.steps / (ms / 1e3),
        "tuning": tune,
        "roofline": roofline,
        "clocks": clocks,
        "detail": {"accepted_per_step": acc_per_step, "cell_pairs_per_step": st["cell_pairs"],
                   "escalated_per_step": st["escalated"],
                   "traverse_launches_per_step": st["launches"], "build_ms": st["build_ms"],
                   "traverse_ms": tr_ms, "npairs_total": float(out["npairs"].sum()),
                   "xip_bin10": float(out["xi0"][10] / out["weight"][10])},
    }
    if exact is not None:
        line["xi_err"] = xi_err
        if rank == 0 and not args.no_cpu_baseline:
            exact.update(exact_fp64_check(args, T, cat))
        line["accurate"] = exact
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(cat, bins, args, budget_s=args.cpu_budget)
        line["vs_cpu"] = value / line["cpu_baseline"]["value"]
        if exact is not None and exact.get("cpu_baseline"):
            exact["vs_cpu"] = exact["value"] / exact["cpu_baseline"]["value"]
    return line


def exact_entry(args, T, dcols, hcols, timed, world):
    """The same 10M catalog with bin_slop 0 and angle_slop 0: every pair in range is counted at
    its own separation, which is what the metric's xi err <= 1e-4 asks for.  Timed like the
    headline (device columns, field construction + tree build + tiles + reduction per step,
    CUDA events on the library's stream) over args.exact_steps steps after one warm-up, plus
    one end-to-end step through the host-array API."""
    import torch
    bins = binning(0.0)
    bins["a"] = 0.0
    nb = bins["nbins"]

    def corr_for(out):
        return T.GGCorr(T.Log, bins["min_sep"], bins["max_sep"], nb, bins["bin_size"],
                        bins["b"], bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0.,
                        0., out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"],
                        out["meanlogr"], out["weight"], out["npairs"])

    def outputs():
        return {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                          "weight", "npairs")}

    def device_field():
        return T.DeviceField(2, T.Sphere, args.n, dcols["x"].data_ptr(), dcols["y"].data_ptr(),
                             dcols["z"].data_ptr(), dcols["g1"].data_ptr(),
                             dcols["g2"].data_ptr(), dcols["w"].data_ptr(), 0, 0.0, 0.0, T.Mean,
                             0, False, 3, 10)

    # The autotuner picks the tile leaf size and expansion chunk on a sample of the top-level
    # pairs, once, outside the timed region; every step then uses its choice.
    t0 = time.perf_counter()
    f, c = device_field(), corr_for(outputs())
    tune = c.autotune(f, metric=T.Arc, frac=args.tune_frac) if args.tune_frac > 0 else \
        {"tile_leaf": 0, "chunk": 0, "ms": 0.}
    tune["tune_s"] = round(time.perf_counter() - t0, 2)
    tune["frac"] = args.tune_frac
    del f, c

    def step_device():
        out = outputs()
        f = device_field()
        c = corr_for(out)
        c.setTuning(tune["tile_leaf"], tune["chunk"])
        c.processAuto(f, False, False, T.Arc)
        st = c.stats()
        del f, c
        return out, st

    def step_host():
        out = outputs()
        e = np.array([])
        f = T.GFieldSphere(hcols["x"].numpy(), hcols["y"].numpy(), hcols["z"].numpy(),
                           hcols["g1"].numpy(), hcols["g2"].numpy(), hcols["w"].numpy(), e,
                           0.0, 0.0, T.Mean, 0, False, 3, 10)
        c = corr_for(out)
        c.setTuning(tune["tile_leaf"], tune["chunk"])
        c.processAuto(f, False, False, T.Arc)
        st = c.stats()
        del f, c
        return out, st

    step_device()
    ms, res, launches = timed(step_device, args.exact_steps)
    ms = allreduce_max(ms, world)
    out, st = res[-1]
    value = world * st["accepted"] * args.exact_steps / (ms / 1e3)
    ms_e2e, res_e2e, _ = timed(step_host, 1)
    ms_e2e = allreduce_max(ms_e2e, world)
    e2e = world * res_e2e[-1][1]["accepted"] / (ms_e2e / 1e3)
    # Roofline of k_tiles: FP32 issue (the pair math; no HBM traffic to speak of).
    # Algorithmic work = leaf pairs evaluated x 80 FLOP (a curved-sky GG pair: separation,
    # chord-to-arc, log, two spin-2 directions and rotations, both products, 8 sums), over
    # k_tiles' own device time (events around every tile launch), per launch.
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    tl = max(st["launches"], 1)
    achieved = st["tile_pairs"] * 80.0 / tl / (st["tiles_ms"] / tl / 1e3) / 1e12
    return {
        "config": "bin_slop 0, angle_slop 0 (every pair at its own separation), same catalog, "
                  "binning and step as the headline",
        "value": value, "unit": UNIT, "ms_per_step": ms / args.exact_steps,
        "steps": args.exact_steps, "warmup": 1, "gpu_launches": launches,
        "e2e": {"value": e2e, "unit": UNIT, "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": sum(v.numel() * 8 for v in hcols.values()),
                "d2h_bytes_per_step": 8 * nb * 8, "steps": 1},
        "roofline": {"bound": "fp32", "kernel": "k_tiles", "achieved": round(achieved, 2),
                     "peak": None, "unit": "TFLOP/s", "frac": None,
                     "sms": props.multi_processor_count, "flop_per_pair": 80, "traffic": None,
                     "peak_source": "SMs x 128 FP32 lanes x 2 flop x the median SM clock "
                                    "sampled under load (MEASURED_PEAKS.json has no FP32 "
                                    "figure)"},
        "tuning": tune,
        "detail": {"accepted_per_step": st["accepted"], "tile_pairs": st["tile_pairs"],
                   "tiles": st["tiles"], "tile_escalated": st["tile_escalated"],
                   "cell_pairs": st["cell_pairs"], "build_ms": st["build_ms"],
                   "traverse_ms": st["traverse_ms"], "tiles_ms": st["tiles_ms"],
                   "expand_ms": st["expand_ms"], "launches": st["launches"],
                   "npairs_total": float(out["npairs"].sum())},
        "_out": out,
    }


def exact_fp64_check(args, T, cat, n_sub=200_000):
    """The exact mode against FP64 on a random subsample of the catalog: the GPU result and
    the oracle's (the reference algorithm in FP64 on the host, pinned to the reference's own
    outputs by the tests) on the same 200,000 points.  Also times the oracle there: the CPU
    rate of this configuration."""
    from oracle import oracle as O
    rng = np.random.default_rng(args.seed + 77)
    idx = np.sort(rng.choice(args.n, n_sub, replace=False))
    sub = {k: np.ascontiguousarray(cat[k][idx]) for k in ("x", "y", "z", "g1", "g2", "w")}
    bins = binning(0.0)
    bins["a"] = 0.0
    nb = bins["nbins"]
    e = np.array([])
    out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr", "weight",
                                     "npairs")}
    f = T.GFieldSphere(sub["x"], sub["y"], sub["z"], sub["g1"], sub["g2"], sub["w"], e, 0.0,
                       0.0, T.Mean, 0, False, 3, 10)
    c = T.GGCorr(T.Log, bins["min_sep"], bins["max_sep"], nb, bins["bin_size"], bins["b"], 0.0,
                 -sys.float_info.max, sys.float_info.max, 0., 0., 0., out["xi0"], out["xi1"],
                 out["xi2"], out["xi3"], out["meanr"], out["meanlogr"], out["weight"],
                 out["npairs"])
    c.processAuto(f, False, False, T.Arc)
    nthreads = os.cpu_count() or 1
    of = O.OracleField("G", "spherical", sub["x"], sub["y"], sub["z"], sub["g1"], sub["g2"],
                       sub["w"], None, 0.0, 0.0, "mean", False, 3, 10)
    of.ntop()
    t0 = time.perf_counter()
    ref = O.process("G", "Arc", bins, of, nthreads=nthreads)
    cpu_s = time.perf_counter() - t0
    mx = float(np.abs(ref["xi0"] / ref["weight"]).max())

    def d(k):
        return float(np.abs(out[k] / out["weight"] - ref[k] / ref["weight"]).max() / mx)

    err = {"vs": f"FP64 oracle (the reference algorithm in double precision) on a "
                 f"{n_sub}-point random subsample of the catalog",
           "xip": d("xi0"), "xim": d("xi2"),
           "npairs_identical": bool(np.array_equal(out["npairs"], ref["npairs"])),
           "weight_rel": float(np.abs(out["weight"] - ref["weight"]).max() /
                               np.abs(ref["weight"]).max())}
    err["max"] = max(err["xip"], err["xim"])
    err["meets_1e-4"] = err["max"] <= 1e-4
    return {"xi_err_fp64": err,
            "cpu_baseline": {"value": ref["_accepted"] / cpu_s, "unit": UNIT, "cores": nthreads,
                             "kind": "port",
                             "sample": f"the {n_sub}-point subsample, whole correlation "
                                       f"({ref['_accepted']} pair evaluations, {cpu_s:.1f} s; "
                                       "tree build excluded)"}}


def ggg_catalog(n, seed, side=600.0):
    """The multipole configuration's catalog: x, y ~ U[0, side] arcmin, g1, g2 ~ N(0, 0.25),
    w ~ U[0.5, 1.5] (flat sky)."""
    rng = np.random.default_rng(seed)
    return {"x": rng.uniform(0, side, n), "y": rng.uniform(0, side, n),
            "g1": rng.normal(0, 0.25, n), "g2": rng.normal(0, 0.25, n),
            "w": rng.uniform(0.5, 1.5, n)}


def ggg_bins():
    lo, hi, nb, max_n = 1.0, 50.0, 20, 30
    bs = np.log(hi / lo) / nb
    b = min(bs, 0.1)                      # bin_slop default 0.1/bin_size (bin_size > 0.1)
    a = np.pi / (2 * max_n + 1)           # angle_slop default
    b1 = min(a, b)
    return dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bs, b=b, a=a, max_n=max_n,
                min_size=2 * lo * b1 / (2 + 3 * b1), max_size=hi * b1)


def run_gpu_ggg(args, rank, world):
    """GGG LogMultipole (2M flat-sky points, 20 Log bins 1-50', max_n 30): triangles
    accumulated per second (sum of ntri over all outputs per step time)."""
    import torch
    from treecorr_gb300 import _treecorr as T
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    n = args.n if args.n != 10_000_000 else 2_000_000
    cat = ggg_catalog(n, args.seed + rank, side=600.0 * np.sqrt(n / 2e6))
    B = ggg_bins()
    nb, mn = B["nbins"], B["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    keys = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i", "meand1",
            "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu", "meanv",
            "weight", "weight_im", "ntri")
    hcols = {k: torch.from_numpy(cat[k]).pin_memory() for k in ("x", "y", "g1", "g2", "w")}
    stream = torch.cuda.ExternalStream(T.stream_handle(), device=dev)
    e = np.array([])

    def step():
        out = {k: np.zeros(shape) for k in keys}
        c = T.GGGCorr(T.LogMultipole, B["min_sep"], B["max_sep"], nb, B["bin_size"], B["b"],
                      B["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0., -sys.float_info.max,
                      sys.float_info.max, 0., 0., 0., *[out[k] for k in keys])
        f = T.GFieldFlat(hcols["x"].numpy(), hcols["y"].numpy(), e, hcols["g1"].numpy(),
                         hcols["g2"].numpy(), hcols["w"].numpy(), e, B["min_size"],
                         B["max_size"], T.Mean, 0, False, 3, 10)
        c.processAuto(f, False, False, T.Euclidean)
        del c, f
        return out

    for _ in range(args.warmup):
        step()
    launches0 = T.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        e0.record(stream)
        outs = [step() for _ in range(args.steps)]
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = allreduce_max(e0.elapsed_time(e1), world)
    ntri = float(outs[-1]["ntri"].sum())
    value = world * ntri * args.steps / (ms / 1e3)
    unit = "triangles/s"
    line = {
        "metric": "GGG multipole triangles/s at N=2M (flat, 20 Log bins 1-50', max_n 30)",
        "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded uniform flat catalog)",
        "config": {"workload": f"GGG LogMultipole auto, {n} points U[0,{600*np.sqrt(n/2e6):.0f}']^2, "
                               "20 Log bins 1-50', max_n 30, bin_slop 0.1/bin_size",
                   "n": n, "parallelism": f"replicas{world}",
                   "l2": "tree, c2 lists and vertex records larger than L2; no flush"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 5 * 8 * n,
                "d2h_bytes_per_step": 15 * 8 * nb * nb * (2 * mn + 1)},
        "gpu_launches": T.launch_count() - launches0,
        "clocks": clk.summary(),
        "detail": {"ntri_per_step": ntri, "gam0r_sum": float(outs[-1]["gam0r"].sum())},
    }
    if rank == 0 and not args.no_cpu_baseline:
        # The oracle port on a smaller catalog of the same density (the triangle rate per
        # second is what is compared).
        from oracle import oracle as O
        nthreads = os.cpu_count() or 1
        ns = 100_000
        cs = ggg_catalog(ns, args.seed, side=600.0 * np.sqrt(ns / 2e6))
        f = O.OracleField("G", "flat", cs["x"], cs["y"], None, cs["g1"], cs["g2"], cs["w"],
                          None, B["min_size"], B["max_size"], "mean", False, 3, 10)
        f.ntop()
        t0 = time.perf_counter()
        o = O.multipole("Euclidean", B, mn, f, nthreads=nthreads)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": float(o["ntri"].sum()) / dt, "unit": unit,
                                "cores": nthreads, "kind": "port",
                                "sample": f"{ns}-point catalog of the same density "
                                          f"({dt:.1f} s, tree build excluded)"}
    return line


def run_exact(args, rank, world):
    """One exact-mode GG correlation (bin_slop 0, angle_slop 0; the leaf-pair tiles) of a
    curved-sky catalog of --n points on --area deg^2, 30 Log bins 1-300' -- at --n 1000000
    --area 100 the same density (so the same tiles) as the 10M-point headline catalog, the
    small case the k_tiles profiles are taken on.  Times args.steps correlations after
    args.warmup with CUDA events on the library's stream."""
    import torch
    from treecorr_gb300 import _treecorr as T
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    cat = curved_sky_catalog(args.n, seed=args.seed + rank, area_deg2=args.area,
                             ngrid=1024 if args.area < 500 else 4096)
    e = np.array([])
    f = T.GFieldSphere(cat["x"], cat["y"], cat["z"], cat["g1"], cat["g2"], cat["w"], e, 0.0,
                       0.0, T.Mean, 0, False, 3, 10)
    f.getNTopLevel()
    B = binning(0.0)
    nb = B["nbins"]
    out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr", "weight",
                                     "npairs")}
    c = T.GGCorr(T.Log, B["min_sep"], B["max_sep"], nb, B["bin_size"], 0.0, 0.0,
                 -sys.float_info.max, sys.float_info.max, 0., 0., 0., out["xi0"], out["xi1"],
                 out["xi2"], out["xi3"], out["meanr"], out["meanlogr"], out["weight"],
                 out["npairs"])
    stream = torch.cuda.ExternalStream(T.stream_handle(), device=dev)
    for _ in range(args.warmup):
        c.processAuto(f, False, False, T.Arc)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        c.processAuto(f, False, False, T.Arc)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    st = c.stats()
    return {"metric": "GG exact-mode pair-evals/s (bin_slop 0, angle_slop 0)",
            "value": st["accepted"] / (ms / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded curved-sky GRF catalog)",
            "config": {"workload": f"GG auto, {args.n} points on a {args.area:g} deg^2 cap, Arc, "
                                   "30 Log bins 1-300', bin_slop 0, angle_slop 0 (tree built "
                                   "once, correlation per step)"},
            "detail": {k: st[k] for k in ("accepted", "tile_pairs", "tiles", "tile_escalated",
                                          "cell_pairs", "launches", "tiles_ms", "expand_ms",
                                          "traverse_ms")}}


def clumped_catalog(n, seed, side=3000.0, nclump=100_000, sigma=2.0, frac=0.4):
    """The learned-criterion configuration's catalog: flat U[0, side]^2 positions with
    nclump Gaussian clumps (sigma arcmin) holding frac of the points; g ~ N(0, 0.25); w = 1."""
    rng = np.random.default_rng(seed)
    nc = int(n * frac)
    cen = rng.uniform(0, side, size=(nclump, 2))
    k = rng.integers(0, nclump, size=nc)
    xy_c = cen[k] + rng.normal(0, sigma, size=(nc, 2))
    xy_u = rng.uniform(0, side, size=(n - nc, 2))
    xy = np.concatenate([xy_c, xy_u])
    return dict(x=np.ascontiguousarray(xy[:, 0]), y=np.ascontiguousarray(xy[:, 1]), z=None,
                g1=rng.normal(0, 0.25, n), g2=rng.normal(0, 0.25, n), w=np.ones(n))


def run_learned(args, rank, world):
    """Learned vs plain split.  The network (5-64-64-1, trained by this library's kernels on
    split candidates of plain traversals of a 1M-point catalog of the same distribution)
    accepts candidate pairs -- pairs the bin_slop rule splits with s <= cand_factor b r --
    whose predicted leak into other bins is below 10^threshold.

    Equal accuracy at the metric's target (|d xi+-| <= 1e-4 max|xi+|): on these shape-noise-
    dominated catalogs only bin_slop 0 / angle_slop 0 meets it (any accepted cell pair moves
    its pairs' noise between bins or directions), and at bin_slop 0 the network has no
    candidates, so learned and plain are the same computation; `value` is their time ratio
    there.  `looser` compares the plain rule at bin_slop 0.1, 0.05 and 0.2 with the network on
    a 0.1 base, each with its error against the exact result: the gain at equal accuracy is
    the time of the fastest plain setting at least as accurate as the learned run, over the
    learned run's time.  Curved sky (the 10M-point cap, 30 bins 1-300') by default;
    --config5: 50M flat clumped points, 40 bins 0.5-500' (times on the full catalog, errors on
    a 600' x 600' corner of it, where the exact result fits in seconds)."""
    import torch
    from treecorr_gb300 import _treecorr as T, learned
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    e = np.array([])
    c5 = args.config5
    if c5:
        nb, lo, hi = 40, 0.5, 500.0
        metric = T.Euclidean
    else:
        nb, lo, hi = 30, ARCMIN, 300 * ARCMIN
        metric = T.Arc
    bsz = np.log(hi / lo) / nb

    def field(cat):
        if c5:
            f = T.GFieldFlat(cat["x"], cat["y"], e, cat["g1"], cat["g2"], cat["w"], e, 0.0, 0.0,
                             T.Mean, 0, False, 3, 10)
        else:
            f = T.GFieldSphere(cat["x"], cat["y"], cat["z"], cat["g1"], cat["g2"], cat["w"], e,
                               0.0, 0.0, T.Mean, 0, False, 3, 10)
        f.getNTopLevel()
        return f

    def corr(slop, a=0.1):
        out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                          "weight", "npairs")}
        c = T.GGCorr(T.Log, lo, hi, nb, bsz, slop * bsz, a, -sys.float_info.max,
                     sys.float_info.max, 0., 0., 0., out["xi0"], out["xi1"], out["xi2"],
                     out["xi3"], out["meanr"], out["meanlogr"], out["weight"], out["npairs"])
        return c, out

    def run(f, c, out, reps):
        c.processAuto(f, False, False, metric)
        ts = []
        for _ in range(reps):
            for k in out:
                out[k][:] = 0.
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            c.processAuto(f, False, False, metric)
            ts.append(time.perf_counter() - t1)
        st = c.stats()
        return {"wall_s": float(np.median(ts)), "cell_pairs": st["cell_pairs"],
                "accepted": st["accepted"], "learned": st["learned"],
                "xip": out["xi0"] / out["weight"], "xim": out["xi2"] / out["weight"]}

    def make(n, seed):
        return clumped_catalog(n, seed) if c5 else curved_sky_catalog(n, seed=seed)

    t0 = time.perf_counter()
    ftrain = field(clumped_catalog(1_000_000, args.seed + 1000, side=3000.0 / np.sqrt(50))
                   if c5 else curved_sky_catalog(1_000_000, seed=args.seed + 1000))
    ct, _ = corr(0.1)
    x, y = learned.collect(ct, ftrain, metric, sample_mod=4, max_samples=4 << 20)
    params, loss = learned.train(x, y, steps=4000, batch=8192, lr=2e-3, seed=0)
    t_train = time.perf_counter() - t0
    del ftrain
    n = 50_000_000 if c5 else args.n
    cat = make(n, args.seed + rank)
    if c5:
        sel = (cat["x"] < 600.0) & (cat["y"] < 600.0)
        sub = {k: (np.ascontiguousarray(v[sel]) if v is not None else None) for k, v in cat.items()}
    f = field(cat)
    setups = [("plain_bs0.1", 0.1, None), ("plain_bs0.05", 0.05, None),
              ("plain_bs0.2", 0.2, None), ("learned_bs0.1", 0.1, params)]
    res = {}
    for name, slop, prm in setups:
        c, o = corr(slop)
        if prm is not None:
            c.setLearned(prm, threshold=args.learned_threshold, cand_factor=4.0)
        res[name] = run(f, c, o, args.steps)
    if c5:
        # Errors (and the exact-mode comparison) on the corner sub-catalog; the times of the
        # setups above stay the full catalog's.
        del f
        f = field(sub)
        for name, slop, prm in setups:
            c, o = corr(slop)
            if prm is not None:
                c.setLearned(prm, threshold=args.learned_threshold, cand_factor=4.0)
            r = run(f, c, o, 1)
            res[name]["xip"], res[name]["xim"] = r["xip"], r["xim"]
    ce, oe = corr(0.0, a=0.0)
    ex = run(f, ce, oe, 1)
    cl, ol = corr(0.0, a=0.0)
    cl.setLearned(params, threshold=args.learned_threshold, cand_factor=4.0)
    ex_l = run(f, cl, ol, 1)
    mx = float(np.abs(ex["xip"]).max())
    for r in res.values():
        r["xi_err"] = float(max(np.abs(r["xip"] - ex["xip"]).max(),
                                np.abs(r["xim"] - ex["xim"]).max()) / mx)
        del r["xip"], r["xim"]
    lr = res["learned_bs0.1"]
    ok = [r for k, r in res.items() if k.startswith("plain") and r["xi_err"] <= lr["xi_err"]]
    eq_gain = (min(r["wall_s"] for r in ok) / lr["wall_s"]) if ok else None
    value = ex["wall_s"] / ex_l["wall_s"]
    wl = ("GG auto, 50M flat clumped points (1e5 clumps of 2', 40%), 40 Log bins 0.5-500'"
          if c5 else f"GG auto, {n}-point curved sky, Arc, 30 Log bins 1-300'")
    return {"metric": "GG wall-s, learned vs plain split at equal accuracy "
                      "(|d xi+-| <= 1e-4 max|xi+|; ratio plain/learned)",
            "value": value, "unit": "x", "n_gpus": world, "steps": args.steps,
            "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f16 network", "data": "synthetic (seeded)",
            "config": {"workload": wl + "; network trained on a 1M-point catalog of the same "
                                        "distribution",
                       "threshold": args.learned_threshold, "cand_factor": 4.0},
            "at_1e-4": {"plain_exact_s": ex["wall_s"], "learned_exact_s": ex_l["wall_s"],
                        "learned_accepted": ex_l["learned"],
                        "note": "bin_slop 0 / angle_slop 0: the network has no candidates"
                                + (" (on the 600' x 600' corner)" if c5 else "")},
            "looser": res, "gain_at_equal_accuracy_looser": eq_gain,
            "reference_result": "bin_slop 0, angle_slop 0 on the same catalog"
                                + (" (errors on the 600' x 600' corner)" if c5 else ""),
            "train": {"samples": int(len(y)), "seconds": t_train,
                      "loss_first": float(loss[0]), "loss_last": float(loss[-20:].mean())}}


def run_patches(args, rank, world):
    """Batched patches: the curved-sky GG catalog split into 150 patches (Voronoi cells of
    150 random centres on the cap, so the counts are uneven), every patch-pair correlation
    within max_sep in one GPU expansion, then the jackknife covariance of (xip, xim) on the
    device.  Compared with one GPU call per patch pair (the reference's loop structure,
    corr2base.py:929-950) and with the CPU restatement of the jackknife."""
    import torch
    from treecorr_gb300 import _treecorr as T
    from oracle import jackknife_oracle as J
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    cat = curved_sky_catalog(args.n, seed=args.seed + rank)
    npatch = 150
    rng = np.random.default_rng(args.seed + 7)
    cen_idx = rng.choice(args.n, npatch, replace=False)
    cen = np.stack([cat["x"][cen_idx], cat["y"][cen_idx], cat["z"][cen_idx]], axis=1)
    pid = np.empty(args.n, dtype=np.int32)
    for s0 in range(0, args.n, 1 << 20):
        p = np.stack([cat["x"][s0:s0 + (1 << 20)], cat["y"][s0:s0 + (1 << 20)],
                      cat["z"][s0:s0 + (1 << 20)]], axis=1)
        pid[s0:s0 + len(p)] = (p @ cen.T).argmax(axis=1)
    counts = np.bincount(pid, minlength=npatch)
    e = np.array([])
    B = binning(args.bin_slop)
    nb = B["nbins"]

    def corr():
        out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                          "weight", "npairs")}
        return T.GGCorr(T.Log, B["min_sep"], B["max_sep"], nb, B["bin_size"], B["b"], B["a"],
                        -sys.float_info.max, sys.float_info.max, 0., 0., 0., out["xi0"],
                        out["xi1"], out["xi2"], out["xi3"], out["meanr"], out["meanlogr"],
                        out["weight"], out["npairs"]), out

    order = np.argsort(pid, kind="stable")
    starts = np.concatenate([[0], np.cumsum(counts)])
    fields = []
    for p in range(npatch):
        sel = order[starts[p]:starts[p + 1]]
        fields.append(T.GFieldSphere(cat["x"][sel], cat["y"][sel], cat["z"][sel],
                                     cat["g1"][sel], cat["g2"][sel], cat["w"][sel], e, 0.0, 0.0,
                                     T.Mean, 0, False, 3, 10))
    for f in fields:
        f.getNTopLevel()
    c, _ = corr()
    pairs, res = c.processPatches(fields, T.Arc)          # warm-up
    torch.cuda.synchronize()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        pairs, res = c.processPatches(fields, T.Arc)
        v, cov = T.jackknife_cov(res, pairs, npatch, 2, "simple")
        ts.append(time.perf_counter() - t0)
    st = c.stats()
    t_batched = float(np.median(ts))
    t0 = time.perf_counter()
    v, cov = T.jackknife_cov(res, pairs, npatch, 2, "simple")
    t_jk_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    v0 = J.design_matrix(res, pairs, npatch, gg=True, cpw="simple")
    c0 = J.cov_jackknife(v0)
    t_jk_cpu = time.perf_counter() - t0
    # One GPU call per pair, as the reference's Python loop does (not timed for all pairs
    # when that takes long: the first 200 pairs, scaled).
    npp = min(len(pairs), 200)
    t0 = time.perf_counter()
    for (i, j) in pairs[:npp]:
        cc, _ = corr()
        if i == j:
            cc.processAuto(fields[i], False, False, T.Arc)
        else:
            cc.processCross(fields[i], fields[j], False, False, T.Arc)
    t_loop = (time.perf_counter() - t0) * len(pairs) / npp
    return {"metric": "GG patch-pair correlations + jackknife covariance, wall-s per step",
            "value": t_batched, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": 1,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic (seeded curved-sky GRF catalog)",
            "config": {"workload": f"GG auto, {args.n}-point curved sky in {npatch} Voronoi "
                                   "patches, Arc, 30 Log bins 1-300', bin_slop 0.1",
                       "patch_counts_min_median_max": [int(counts.min()), int(np.median(counts)),
                                                       int(counts.max())]},
            "detail": {"patch_pairs": len(pairs), "cell_pairs": st["cell_pairs"],
                       "accepted": st["accepted"], "traverse_ms": st["traverse_ms"],
                       "per_pair_calls_s": t_loop, "jackknife_gpu_s": t_jk_gpu,
                       "jackknife_cpu_restatement_s": t_jk_cpu,
                       "jackknife_max_rel_diff": float(np.abs(cov - c0).max() / np.abs(c0).max())}}


def run_kmeans(args, rank, world):
    """k-means patches of the curved-sky catalog (150 patches, the jackknife configuration):
    the N field k-means builds (min_size 0, max_size inf, min_top 4, max_top 7 =
    bit_length(150) - 1), KMeansInitTree, KMeansRun for a fixed number of iterations
    (tol 0, so both sides iterate alike) and KMeansAssign.  Metric: point-iterations of
    KMeansRun per second."""
    import torch
    from treecorr_gb300 import _treecorr as T
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    cat = curved_sky_catalog(args.n, seed=args.seed + rank)
    npatch, iters = 150, 20
    e = np.array([])
    f = T.NFieldSphere(cat["x"], cat["y"], cat["z"], cat["w"], e, 0.0, np.inf, T.Mean, 0, False,
                       4, 7)
    t0 = time.perf_counter()
    f.getNTopLevel()
    build_s = time.perf_counter() - t0
    c0 = np.zeros((npatch, 3))
    t0 = time.perf_counter()
    f.KMeansInitTree(c0, npatch, 1234)
    init_s = time.perf_counter() - t0
    c = c0.copy()
    f.KMeansRun(c, npatch, 2, 0.0, False)          # warm-up
    launches0 = T.launch_count()
    ts = []
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            c = c0.copy()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            f.KMeansRun(c, npatch, iters, 0.0, False)
            ts.append(time.perf_counter() - t0)
    launches = T.launch_count() - launches0
    pat = np.zeros(args.n, dtype=np.int64)
    t0 = time.perf_counter()
    f.KMeansAssign(c, npatch, pat)
    assign_s = time.perf_counter() - t0
    q = np.zeros(args.n, dtype=np.int64)
    t0 = time.perf_counter()
    T.QuickAssign(c, npatch, cat["x"], cat["y"], cat["z"], q)
    quick_s = time.perf_counter() - t0
    t_run = float(np.median(ts))
    value = world * args.n * iters / t_run
    unit = "point-iterations/s"
    line = {"metric": "k-means KMeansRun point-iterations/s at N=10M, 150 patches (curved sky)",
            "value": value, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": 1,
            "ms_per_step": 1e3 * t_run, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded curved-sky catalog)",
            "config": {"workload": f"k-means, {args.n}-point 1000 deg^2 cap, {npatch} patches, "
                                   f"{iters} iterations (tol 0), init tree",
                       "field": "NFieldSphere min_size 0, max_size inf, min_top 4, max_top 7"},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 24 * npatch,
                    "d2h_bytes_per_step": 24 * npatch},
            "gpu_launches": launches // max(args.steps, 1), "clocks": clk.summary(),
            "detail": {"build_s": build_s, "init_tree_s": init_s, "assign_s": assign_s,
                       "quick_assign_s": quick_s, "assign_equals_quick": bool(np.array_equal(pat, q)),
                       "patch_counts_min_max": [int(np.bincount(pat, minlength=npatch).min()),
                                                int(np.bincount(pat, minlength=npatch).max())]}}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        of = O.OracleField("N", "spherical", cat["x"], cat["y"], cat["z"], w=cat["w"],
                           min_size=0.0, max_size=np.inf, split_method="mean", min_top=4,
                           max_top=7)
        t0 = time.perf_counter()
        of.ntop()
        ob = time.perf_counter() - t0
        it_cpu = 2
        t0 = time.perf_counter()
        oc, _ = of.kmeans_run(c0, it_cpu, 0.0, False)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": args.n * it_cpu / dt, "unit": unit, "cores": 1,
                                "kind": "port",
                                "sample": f"{it_cpu} iterations of the same run ({dt:.1f} s; "
                                          f"tree build {ob:.1f} s excluded)"}
        c2 = c0.copy()
        f.KMeansRun(c2, npatch, it_cpu, 0.0, False)
        line["detail"]["max_center_diff_vs_port_2it"] = float(np.abs(c2 - oc).max())
    return line


def run_classes(args, rank, world):
    """The widened classes, one timed call each after a warm-up: 2-point NN and KK auto on
    the curved-sky catalog, NG and KG cross (its first half as the N / K field, the second
    half as the G field); 3-point LogMultipole cross12 GGG, NGG, GNN and NKK (1M vertex
    points, 1M pair points), NNG cross21 (ordered 3) and GGG three-field cross (ordered 4)
    on 1M-point catalogs of the multipole configuration's density and binning.  Each class
    is reported with its GPU rate and the oracle port's rate on a bounded sample."""
    import torch
    from treecorr_gb300 import _treecorr as T
    from oracle import oracle as O
    dev = torch.device("cuda", rank % max(torch.cuda.device_count(), 1))
    torch.cuda.set_device(dev)
    stream = torch.cuda.ExternalStream(T.stream_handle(), device=dev)
    nthreads = os.cpu_count() or 1
    e = np.array([])
    cat = curved_sky_catalog(args.n, seed=args.seed + rank)
    cat["k"] = np.random.default_rng(args.seed + 7).normal(0, 0.02, args.n)
    bins = binning(args.bin_slop)
    nb = bins["nbins"]
    half = args.n // 2

    def sub(c, lo, hi):
        return {k: np.ascontiguousarray(v[lo:hi]) for k, v in c.items()}

    def field2(L, c):
        cls = getattr(T, L + "FieldSphere")
        pay = [] if L == "N" else [c["k"]] if L == "K" else [c["g1"], c["g2"]]
        return cls(c["x"], c["y"], c["z"], *pay, c["w"], e, 0.0, 0.0, T.Mean, 0, False, 3, 10)

    def timed(fn):
        fn()                                  # warm-up
        barrier(world)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return allreduce_max(e0.elapsed_time(e1), world), r

    res = {}
    launches0 = T.launch_count()
    with ClockSampler(dev.index) as clk:
        for cls, (L1, L2) in (("NN", ("N", None)), ("KK", ("K", None)), ("NG", ("N", "G")),
                              ("KG", ("K", "G"))):
            def step():
                out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr",
                                                 "meanlogr", "weight", "npairs")}
                c = getattr(T, cls + "Corr")(
                    T.Log, bins["min_sep"], bins["max_sep"], nb, bins["bin_size"], bins["b"],
                    bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                    *[out[k] for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                       "weight", "npairs")])
                if L2 is None:
                    f = field2(L1, cat)
                    c.processAuto(f, False, False, T.Arc)
                else:
                    f, g = field2(L1, sub(cat, 0, half)), field2(L2, sub(cat, half, args.n))
                    c.processCross(f, g, False, False, T.Arc)
                return c.stats()["accepted"]
            ms, acc = timed(step)
            res[cls] = {"gpu_ms": ms, "pair_evals": acc, "gpu_rate": world * acc / (ms / 1e3),
                        "unit": UNIT, "n": args.n if L2 is None else [half, args.n - half]}
        B = ggg_bins()
        mb, mn = B["nbins"], B["max_n"]
        shape = (mb, mb, 2 * mn + 1)
        n3 = 1_000_000
        side = 600.0 * np.sqrt(2 * n3 / 2e6)
        cv = ggg_catalog(n3, args.seed + 11 + rank, side=side)
        cp = ggg_catalog(n3, args.seed + 12 + rank, side=side)
        for c3 in (cv, cp):
            c3["k"] = np.random.default_rng(args.seed + 13).normal(0, 0.02, n3)
        cw = ggg_catalog(n3, args.seed + 14 + rank, side=side)
        for cls in ("GGG", "NGG", "GNN", "NKK", "NNG_x21", "GGG_x3"):
            zk = {"GGG": 8, "NGG": 4, "GGG_x3": 8}.get(cls, 2)

            def step3():
                keys = [f"z{q}" for q in range(zk)] + [
                    "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3",
                    "meanu", "meanv", "weight", "weight_im", "ntri"]
                out = {k: np.zeros(shape) for k in keys}
                zeta = [out[f"z{q}"] for q in range(zk)] + [e] * (8 - zk)
                c = getattr(T, cls[:3] + "Corr")(
                    T.LogMultipole, B["min_sep"], B["max_sep"], mb, B["bin_size"], B["b"],
                    B["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0., -sys.float_info.max,
                    sys.float_info.max, 0., 0., 0., *zeta, *[out[k] for k in keys[zk:]])

                def fl(L, c3):
                    pay = [] if L == "N" else [c3["k"]] if L == "K" else [c3["g1"], c3["g2"]]
                    return getattr(T, L + "FieldFlat")(c3["x"], c3["y"], e, *pay, c3["w"], e,
                                                       B["min_size"], B["max_size"], T.Mean,
                                                       0, False, 3, 10)
                if cls == "NNG_x21":       # vertices 1 and 2 from the N catalog, 3 from G
                    c.processCross21(fl("N", cv), fl("G", cp), 3, False, False, T.Euclidean)
                elif cls == "GGG_x3":      # one vertex from each of three catalogs
                    c.processCross(fl("G", cv), fl("G", cp), fl("G", cw), 4, False, False,
                                   T.Euclidean)
                else:
                    c.processCross12(fl(cls[0], cv), fl(cls[1], cp), 1, False, False,
                                     T.Euclidean)
                return float(out["ntri"].sum())
            ms, ntri = timed(step3)
            key = cls if "_" in cls else cls + "_x12"
            res[key] = {"gpu_ms": ms, "triangles": ntri, "gpu_rate": world * ntri / (ms / 1e3),
                        "unit": "triangles/s", "n": [n3] * (3 if cls == "GGG_x3" else 2)}
    launches = T.launch_count() - launches0
    if rank == 0 and not args.no_cpu_baseline:
        # 2-point: auto classes over top-level rows of the same catalog, cross classes on
        # 1M + 1M points of it (the port's per-pair cost is what is compared).
        for cls in ("NN", "KK", "NG", "KG"):
            L1, L2 = cls[0], cls[1]
            t_budget = max(2.0, args.cpu_budget / 4)
            if cls in ("NN", "KK"):
                pay = {"N": (None, None), "K": (cat["k"], None)}[L1]
                f = O.OracleField(L1, "spherical", cat["x"], cat["y"], cat["z"], *pay, cat["w"],
                                  None, 0.0, 0.0, "mean", False, 3, 10)
                ntop = f.ntop()
                acc, spent, row, chunk = 0, 0.0, 0, 1
                while spent < t_budget and row < ntop:
                    r1 = min(ntop, row + chunk)
                    t0 = time.perf_counter()
                    o = O.process(cls, "Arc", bins, f, rows=(row, r1), nthreads=nthreads)
                    spent += time.perf_counter() - t0
                    acc += o["_accepted"]
                    row, chunk = r1, min(chunk * 2, 64)
                sample = f"top-level rows 0..{row} of {ntop} ({spent:.1f} s)"
            else:
                m = min(1_000_000, half)
                a, b = sub(cat, 0, m), sub(cat, half, half + m)
                pay1 = {"N": (None, None), "K": (a["k"], None)}[L1]
                f1 = O.OracleField(L1, "spherical", a["x"], a["y"], a["z"], *pay1, a["w"], None,
                                   0.0, 0.0, "mean", False, 3, 10)
                f2 = O.OracleField("G", "spherical", b["x"], b["y"], b["z"], b["g1"], b["g2"],
                                   b["w"], None, 0.0, 0.0, "mean", False, 3, 10)
                f1.ntop(); f2.ntop()
                t0 = time.perf_counter()
                o = O.process(cls, "Arc", bins, f1, f2, nthreads=nthreads)
                spent = time.perf_counter() - t0
                acc = o["_accepted"]
                sample = f"{m} + {m} points of the same catalog ({spent:.1f} s)"
            res[cls]["cpu_rate"] = acc / spent if spent > 0 else None
            res[cls]["cpu_sample"] = sample
        # 3-point: the oracle's cross12 on 50K + 50K points of the same density.
        ms_ = 50_000
        side_s = 600.0 * np.sqrt(2 * ms_ / 2e6)
        sv = ggg_catalog(ms_, args.seed + 21, side=side_s)
        sp = ggg_catalog(ms_, args.seed + 22, side=side_s)
        for c3 in (sv, sp):
            c3["k"] = np.random.default_rng(args.seed + 23).normal(0, 0.02, ms_)
        B = ggg_bins()
        sw = ggg_catalog(ms_, args.seed + 24, side=side_s)
        for cls in ("GGG", "NGG", "GNN", "NKK", "NNG_x21", "GGG_x3"):
            def of(L, c3, as_k):
                if as_k:    # the oracle's real-payload fields (NGG vertex / GNN pairs)
                    kv = c3["k"] if L == "K" else np.ones(len(c3["x"]))
                    return O.OracleField("K", "flat", c3["x"], c3["y"], None, kv, None,
                                         c3["w"], None, B["min_size"], B["max_size"], "mean",
                                         False, 3, 10)
                g1, g2 = (c3["g1"], c3["g2"]) if L == "G" else (0 * c3["w"], 0 * c3["w"])
                return O.OracleField("G", "flat", c3["x"], c3["y"], None, g1, g2, c3["w"],
                                     None, B["min_size"], B["max_size"], "mean", False, 3, 10)
            key = cls if "_" in cls else cls + "_x12"
            if cls == "NNG_x21":
                fn, fg = of("N", sv, True), of("G", sp, False)
                fn.ntop(); fg.ntop()
                t0 = time.perf_counter()
                o = O.multipole3("Euclidean", B, B["max_n"], fn, fn, fg, 4, nthreads=nthreads,
                                 mode=3)
            elif cls == "GGG_x3":
                fa, fb, fc = of("G", sv, False), of("G", sp, False), of("G", sw, False)
                fa.ntop(); fb.ntop(); fc.ntop()
                t0 = time.perf_counter()
                o = O.multipole3("Euclidean", B, B["max_n"], fa, fb, fc, 4, nthreads=nthreads)
            else:
                mode = 1 if cls == "NGG" else 2 if cls == "GNN" else 0
                f1 = of(cls[0], sv, mode == 1)
                f2 = of(cls[1], sp, mode == 2)
                f1.ntop(); f2.ntop()
                t0 = time.perf_counter()
                o = O.multipole("Euclidean", B, B["max_n"], f1, nthreads=nthreads, f2=f2,
                                mode=mode)
            spent = time.perf_counter() - t0
            res[key]["cpu_rate"] = float(o["ntri"].sum()) / spent
            res[key]["cpu_sample"] = f"{ms_}-point catalogs, same density ({spent:.1f} s)"
    ng = res["NG"]
    line = {
        "metric": "per-class throughput of the widened classes (value: NG cross pair-evals/s)",
        "value": ng["gpu_rate"], "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": ng["gpu_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded curved-sky catalog; seeded flat catalogs)",
        "config": {"workload": "classes: NN, KK auto and NG, KG cross on the 10M-point cap "
                               "(Arc, 30 Log bins 1-300', bin_slop 0.1); GGG, NGG, GNN, NKK "
                               "LogMultipole cross12, NNG cross21 and GGG three-field cross, "
                               "1M-point flat catalogs (20 bins 1-50', max_n 30)",
                   "n": args.n, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2; no flush"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "detail": {"classes": res, "cpu_cores": nthreads},
    }
    return line


def cpu_sample(cat, bins, args, budget_s=15.0):
    """The oracle port of the reference algorithm on the host cores, over top-level rows of
    the auto loop until about budget_s seconds of traversal have been timed."""
    from oracle import oracle as O
    nthreads = os.cpu_count() or 1
    f = O.OracleField("G", "spherical", cat["x"], cat["y"], cat["z"], cat["g1"], cat["g2"],
                      cat["w"], None, 0.0, 0.0, "mean", False, 3, 10)
    t0 = time.perf_counter()
    ntop = f.ntop()
    build_s = time.perf_counter() - t0
    acc, spent, row = 0, 0.0, 0
    chunk = 1
    while spent < budget_s and row < ntop:
        r1 = min(ntop, row + chunk)
        t0 = time.perf_counter()
        out = O.process("G", "Arc", bins, f, rows=(row, r1), nthreads=nthreads)
        dt = time.perf_counter() - t0
        acc += out["_accepted"]
        spent += dt
        row = r1
        chunk = min(chunk * 2, 64)
    return {"value": acc / spent if spent > 0 else None, "unit": UNIT, "cores": nthreads,
            "kind": "port",
            "sample": f"top-level rows 0..{row} of {ntop} of the same catalog "
                      f"({acc} pair evaluations, {spent:.1f} s traversal; "
                      f"tree build {build_s:.1f} s excluded)"}


def run_reference(args, rank, world):
    """The reference algorithm's CPU implementation (oracle port) on a bounded sample."""
    from oracle import oracle as O
    if rank != 0:
        return None
    cat = curved_sky_catalog(args.n, seed=args.seed)
    bins = binning(args.bin_slop)
    nthreads = os.cpu_count() or 1
    f = O.OracleField("G", "spherical", cat["x"], cat["y"], cat["z"], cat["g1"], cat["g2"],
                      cat["w"], None, 0.0, 0.0, "mean", False, 3, 10)
    ntop = f.ntop()
    # Size the per-step sample: a range of top-level rows with at least 4 rows per thread
    # (so that every core has work), grown until it takes ~cpu_budget/steps seconds.
    target = max(2.0, args.cpu_budget / max(args.steps, 1))
    rows = min(ntop, 4 * nthreads)
    while True:
        t0 = time.perf_counter()
        O.process("G", "Arc", bins, f, rows=(0, rows), nthreads=nthreads)
        dt = time.perf_counter() - t0
        if dt >= 0.5 * target or rows >= ntop:
            break
        rows = min(ntop, int(rows * max(1.5, min(4.0, target / max(dt, 1e-3)))))
    sample = (0, rows)
    for _ in range(args.warmup):
        O.process("G", "Arc", bins, f, rows=sample, nthreads=nthreads)
    acc, t = 0, 0.0
    for _ in range(args.steps):
        t1 = time.perf_counter()
        out = O.process("G", "Arc", bins, f, rows=sample, nthreads=nthreads)
        t += time.perf_counter() - t1
        acc += out["_accepted"]
    value = acc / t
    accurate = None
    if not args.no_exact:
        # The accurate entry's configuration (bin_slop 0, angle_slop 0): every pair is
        # evaluated, so even one top-level row of the 10M catalog is ~7e9 pairs; the sample is
        # the whole correlation of a 200,000-point random subsample of the same catalog.
        rng = np.random.default_rng(args.seed + 77)
        idx = np.sort(rng.choice(args.n, min(args.n, 200_000), replace=False))
        sub = {k: np.ascontiguousarray(cat[k][idx]) for k in ("x", "y", "z", "g1", "g2", "w")}
        bx = binning(0.0)
        bx["a"] = 0.0
        fx = O.OracleField("G", "spherical", sub["x"], sub["y"], sub["z"], sub["g1"], sub["g2"],
                           sub["w"], None, 0.0, 0.0, "mean", False, 3, 10)
        fx.ntop()
        t0 = time.perf_counter()
        outx = O.process("G", "Arc", bx, fx, nthreads=nthreads)
        dtx = time.perf_counter() - t0
        accurate = {"config": "bin_slop 0, angle_slop 0, same catalog and binning",
                    "value": outx["_accepted"] / dtx, "unit": UNIT, "cores": nthreads,
                    "kind": "port",
                    "sample": f"whole correlation of a {len(idx)}-point random subsample "
                              f"({outx['_accepted']} pair evaluations, {dtx:.1f} s; tree build "
                              "excluded)"}
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded curved-sky GRF catalog)", "impl": "reference",
            # The same configuration object as the GPU arm's line (the same catalog and
            # correlation; the l2 note describes the inputs' size).
            "config": {"workload": "GG auto, 10M-point 1000 deg^2 cap, Arc, 30 Log bins "
                                   f"1-300', bin_slop {args.bin_slop}, angle_slop 0.1",
                       "n": args.n, "nbins": 30, "bin_slop": args.bin_slop,
                       "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (480 MB columns + 1.3 GB tree); no flush"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"top-level rows 0..{rows} of {ntop} per step "
                                       "(tree build excluded)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "accurate": accurate}


# ----------------------------------------------------------------------------------------
# Multi-process plumbing (replicas: one independent full workload per GPU)

def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--workload", default="gg",
                   choices=["gg", "ggg", "learned", "patches", "kmeans", "classes", "exact"],
                   help="gg: the 2-point headline; ggg: the multipole 3-point configuration; "
                        "learned: the learned opening criterion against the plain rule; "
                        "patches: 150 patches, all pairs in one expansion + jackknife; "
                        "kmeans: k-means patches of the curved-sky catalog; "
                        "classes: the other 2-point and 3-point classes, one call each; "
                        "exact: one bin_slop 0 / angle_slop 0 correlation (--n, --area)")
    p.add_argument("--learned-threshold", type=float, default=-3.0)
    p.add_argument("--config5", action="store_true",
                   help="learned workload on 50M flat clumped points (40 bins 0.5-500')")
    p.add_argument("--n", type=int, default=10_000_000)
    p.add_argument("--area", type=float, default=1000.0,
                   help="cap area in deg^2 of the exact workload's catalog")
    p.add_argument("--bin-slop", type=float, default=0.1)
    p.add_argument("--seed", type=int, default=20261203)
    p.add_argument("--cpu-budget", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-exact", action="store_true",
                   help="skip the accurate (bin_slop 0, angle_slop 0) entry")
    p.add_argument("--exact-steps", type=int, default=2)
    p.add_argument("--fixed-order", type=int, default=1, choices=(0, 1),
                   help="1: fixed-order expansion (bit-identical repeats, the library's "
                        "default); 0: children appended in arrival order")
    p.add_argument("--tune-frac", type=float, default=0.02,
                   help="fraction of top-level pairs the autotuner times per trial in the "
                        "accurate entry (0: library defaults, no tuning)")
    p.add_argument("--traffic", type=float, default=None,
                   help="DRAM bytes per traversal launch from an ncu capture, if known")
    args = p.parse_args()
    rank, world = dist_init()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "ggg":
        line = run_gpu_ggg(args, rank, world)
    elif args.workload == "learned":
        line = run_learned(args, rank, world)
    elif args.workload == "patches":
        line = run_patches(args, rank, world)
    elif args.workload == "kmeans":
        line = run_kmeans(args, rank, world)
    elif args.workload == "classes":
        line = run_classes(args, rank, world)
    elif args.workload == "exact":
        line = run_exact(args, rank, world)
    else:
        line = run_gpu(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
