"""Throughput of the GB300 pixel-image likelihood (evaluations per second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl qlpix|reference]
                    [--config cfg5] [--batch B] [--precision mixed|fp64]

A step is one batch of B likelihood evaluations: B lens-parameter vectors are
drawn from the configuration's sampling region (for the default workload the
posterior region around the mock's parameters, where a sampler spends its
evaluations; the line's `draws` says which) and evaluated through the public
C ABI (qlp_eval_batch).  The default workload is the metric's own: the two-plane
subhalo configuration (300x300 pixels at 0.03", annulus 0.3"-3.5", 4x4 split,
31x31 Airy-like PSF; SIE + shear at z = 0.5, an elliptical NFW subhalo at
z = 0.8 given by its mass, 1e8-1e10 M_sun; source at z = 2), 1024 vectors per
step, each with its own source grid (side 32-64), on seeded synthetic data,
evaluated in mixed precision with the NFW deflection from the trained
surrogate (quadrature fallback).  `value` is evaluations per second of device
time (inputs resident: image, mask and PSF are uploaded once when the context
is created); `e2e` is the same metric through the public call with the step's
parameter vectors in pinned host memory and the results read back, timed on
the host.  After the timed region the same run evaluates a sample of the
timed vectors on the plain FP64 path (NFW by quadrature) and reports its
throughput, the ratio (`vs_plain_fp64`) and the largest |delta log L|
between the two paths on that sample (`accuracy`).  Under torchrun every rank
evaluates its own batches (replicas, weak scaling) and the slowest rank's
time counts.

--impl reference times the reference's CPU implementation of the same
workload (the oracle port of QLens's dense inversion, OpenMP over all host
cores) and prints the same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# one hardware work queue per concurrent evaluation slot (the default of 8
# would serialise streams beyond the eighth); must precede CUDA initialisation
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

METRIC = "pixel-likelihood evals/s on 1 GB300: batched+surrogate vs plain FP64 at |ΔlogL|<0.1"

# Useful FLOP of the surrogate network per ray on the tensor cores: its three
# 128 x 128 layers, each product counted once (the hi/lo split is not work).
MLP_FLOP_PER_RAY = 2 * 3 * 128 * 128
# DRAM bytes (read + written) of one evaluation's ray-shooting stage on the
# workload, from one ncu capture of its kernels (dram__bytes_read.sum +
# dram__bytes_write.sum of k_ray_pre and k_raytrace_sur<true>)
RAYSUR_TRAFFIC = {"cfg5": (255488 + 2560) + (22348032 + 24320)}
SYRK_TRAFFIC = {}
UNIT = "evals/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def reduce_over_ranks(values, dist, device="cuda"):
    """Slowest rank decides: element-wise max of the timing values over ranks."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_evals(batch, steps, world):
    """Evaluations of the whole job: every rank evaluates its own batches."""
    return batch * steps * world


def write_trace(pl, run_step, k, path):
    """One batched step (step k's parameters), kernel by kernel, under
    torch.profiler's CUPTI activity records; per kernel: launches, summed
    duration, and duration x min(1, CTAs / 152), a proxy for its share of the
    SMs while the evaluations' kernels overlap.  Untimed, after the measured
    region."""
    import collections
    import json
    import tempfile
    import torch
    from torch.profiler import ProfilerActivity, profile
    pl.set_graphs(False)                 # CUPTI reports kernels launched one by one
    ev = []
    for attempt in range(2):             # the first session of a process may come back empty
        torch.cuda.synchronize()
        with profile(activities=[ProfilerActivity.CUDA]) as prof:
            run_step(k)
            torch.cuda.synchronize()
        with tempfile.NamedTemporaryFile(suffix=".json", delete=False) as f:
            tmp = f.name
        prof.export_chrome_trace(tmp)
        ev = [e for e in json.load(open(tmp))["traceEvents"] if e.get("cat") == "kernel"]
        os.remove(tmp)
        if ev:
            break
    pl.set_graphs(True)
    if not ev:
        json.dump({"unavailable": "the profiler recorded no kernels"}, open(path, "w"))
        return
    t0 = min(e["ts"] for e in ev)
    t1 = max(e["ts"] + e["dur"] for e in ev)
    agg = collections.defaultdict(lambda: [0, 0.0, 0.0])
    for e in ev:
        g = e["args"].get("grid", [1, 1, 1])
        ctas = g[0] * g[1] * g[2]
        a = agg[e["name"].split("(")[0]]
        a[0] += 1
        a[1] += e["dur"]
        a[2] += e["dur"] * min(1.0, ctas / 152.0)
    tot = sum(a[2] for a in agg.values())
    rows = [{"kernel": n, "launches": a[0], "us": a[1], "sm_weighted_us": a[2], "sm_weighted_share": a[2] / tot}
            for n, a in sorted(agg.items(), key=lambda x: -x[1][2])]
    json.dump({"span_us": t1 - t0, "kernels": len(ev), "sm_weighted_us": tot, "rows": rows}, open(path, "w"),
              indent=1)


def make_context(wl, precision):
    from qlens_gb300 import PixelLikelihood, abi
    prec = abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64
    pl = PixelLikelihood(wl.xvals, wl.yvals, wl.data, wl.mask, wl.psf, covinv=None, bg_noise=wl.noise,
                         nsplit=wl.nsplit, src_npixels=wl.src_npixels, regparam=wl.regparam, precision=prec)
    pl.set_lens_model(wl.lenses, getattr(wl, "zfac", None), getattr(wl, "beta", None))
    return pl


def algorithmic_syrk_flops(res):
    """2 * N_pix * M(M+1)/2 per evaluation (the F = L'^T C^-1 L' contraction)."""
    tot = 0.0
    for r in res:
        N, M = r["n_active_pixels"], r["n_active_src"]
        tot += N * M * (M + 1.0)
    return tot


def instance_of(wl, inst, i):
    """(mask array, (src nx, src ny), lambda) of vector i of a batch drawn by
    wl.draw_instances (inst = its (mask ids, source sizes, lambdas)), or the
    workload's own for a batch without per-vector instances."""
    ids, sizes, lam = inst
    mask = wl.mask if ids is None or ids[i] < 0 else wl.instance_masks[ids[i]].reshape(wl.mask.shape)
    src = tuple(wl.src_npixels) if sizes is None else tuple(int(v) for v in sizes[i])
    reg = wl.regparam if lam is None else float(lam[i])
    return mask, src, reg


def cpu_port_eval(wl, params, inst=(None, None, None), i=0):
    """One evaluation of the oracle port (CPU, OpenMP over the host's cores)
    on vector i of a batch; returns (seconds, result)."""
    from oracle import oracle as O
    from qlens_gb300 import abi
    mask, src, reg = instance_of(wl, inst, i)
    img = abi.ImageBuffers(wl.xvals, wl.yvals, wl.data, mask, None, wl.noise)
    psf = abi.PSFBuffer(wl.psf)
    o = abi.srcgrid_defaults()
    o.nsplit = wl.nsplit
    o.npixels_x, o.npixels_y = src
    o.regparam = reg
    planes = abi.make_planes(getattr(wl, "zfac", None), getattr(wl, "beta", None))
    t = time.perf_counter()
    r = O.evaluate(img, psf, o, wl.lenses, lens_params=params, planes=planes)
    return time.perf_counter() - t, r


def draw_one(wl, rng):
    p = wl.draw(rng, 1)
    inst = wl.draw_instances(rng, 1) if wl.draw_instances is not None else (None, None, None)
    return p[0], inst


def cpu_sample(wl, rng, budget_s, max_n):
    """Evaluations of the oracle port on fresh draws of the workload, one at a
    time, until max_n are done or their time exceeds budget_s (at least one)."""
    times = []
    while len(times) < max_n:
        p, inst = draw_one(wl, rng)
        dt, _r = cpu_port_eval(wl, p, inst)
        times.append(dt)
        if sum(times) > budget_s:
            break
    return times


REF_BUDGET_S = 150.0     # wall-clock bound of the reference arm's timed evaluations
CPU_BUDGET_S = 30.0      # ... and of the cpu_baseline sample beside the GPU line


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from qlens_gb300 import synthetic
    from oracle import oracle as O
    O.build()
    wl = synthetic.CONFIGS[args.config]()
    rng = np.random.default_rng(4321)
    cores = O.threads()
    # one untimed warm-up evaluation (page-in, thread start-up); more would
    # only repeat it: the port keeps no state between evaluations
    cpu_port_eval(wl, *draw_one(wl, rng))
    times = cpu_sample(wl, rng, REF_BUDGET_S, max(1, args.steps))
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {**wl.describe(), "batch_per_step": 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d evaluations of fresh draws, one per step (steps stop once their time "
                                   "exceeds %.0f s), after 1 warm-up evaluation; OpenMP over %d host threads; "
                                   "median %.2f s" % (len(times), REF_BUDGET_S, cores, statistics.median(times))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def accuracy_of(fast, plain, has_nfw):
    """|delta log L| = |delta(-2 log evidence)| / 2 of the timed path against
    the plain FP64 path on the same vectors."""
    d = sorted(abs(a["m2logev"] - b["m2logev"]) / 2.0 for a, b in zip(fast, plain)
               if a["status"] == 0 and b["status"] == 0)
    if not d:
        return None
    return {"max_abs_dlogL": d[-1], "median_abs_dlogL": float(np.median(d)),
            "p90_abs_dlogL": float(np.quantile(d, 0.9)), "frac_within_bound": float(np.mean(np.array(d) < 0.1)),
            "n_draws": len(d), "vs": "plain FP64 path" + (" with NFW quadrature" if has_nfw else ""), "bound": 0.1}


def plain_fp64_arm(wl, params, inst, n, slots):
    """The plain FP64 path (FP64 SYRK, Cholesky and solves; the NFW deflection
    by quadrature) on the first n vectors of a timed batch: one warm-up batch
    (graph capture), then the n vectors as one batch; returns (evaluations per
    second of device time, results)."""
    pl = make_context(wl, "fp64")
    if wl.instance_masks is not None:
        pl.set_instance_masks(wl.instance_masks)
    pl.set_batch_slots(slots)
    pl.set_graphs(True)
    ids, sizes, lam = inst
    sl = lambda a, k: None if a is None else a[:k]   # noqa: E731
    k0 = min(n, slots)
    pl.eval_batch(params[:k0], regparams=sl(lam, k0), mask_ids=sl(ids, k0), src_sizes=sl(sizes, k0))
    res = pl.eval_batch(params[:n], regparams=sl(lam, n), mask_ids=sl(ids, n), src_sizes=sl(sizes, n))
    ms = pl.last_device_ms()
    pl.close()
    return n / (ms / 1e3), res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="qlpix", choices=["qlpix", "reference"])
    ap.add_argument("--config", default="cfg5", choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5", "cfg5_fixed"])
    ap.add_argument("--batch", type=int, default=0, help="evaluations per step (default: the workload's)")
    ap.add_argument("--slots", type=int, default=0, help="concurrent evaluation slots (default min(batch, 32))")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernel by kernel instead of replaying graphs")
    ap.add_argument("--precision", default=os.environ.get("QLPIX_BENCH_PRECISION", "mixed"),
                    choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-sample", type=int, default=32,
                    help="vectors of the first timed batch evaluated again on the plain FP64 path (0: skip)")
    ap.add_argument("--trace", default="",
                    help="after the measurement, record one more step's kernel timeline (launched kernel by kernel, "
                         "through torch.profiler) and write a per-kernel summary to this JSON file")
    ap.add_argument("--regopt", action="store_true",
                    help="choose lambda per evaluation by Brent's method (QLens 'optimize_regparam on')")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch schedule instead of tuning it on a sample batch first")
    ap.add_argument("--nfw", default="auto", choices=["auto", "surrogate", "quadrature"],
                    help="NFW deflection: trained MLP surrogate (quadrature fallback) or quadrature only; auto = "
                         "the surrogate, except on cfg4, where most rays' deflections are too large for its gate "
                         "(it saves nothing) and its prior-box draws on a sigma = 0.01 mock put the accepted rays' "
                         "errors far above the |delta log L| bound")
    ap.add_argument("--profile-step", action="store_true",
                    help="after the measurement, run one more step between cudaProfilerStart and cudaProfilerStop "
                         "(for ncu --profile-from-start off); untimed")
    ap.add_argument("--train-steps", type=int, default=0,
                    help="Adam steps of the surrogate's training (default: the library's; fewer only to shorten "
                         "profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)

    from qlens_gb300 import synthetic, abi
    wl = synthetic.CONFIGS[args.config]()
    precision = args.precision
    pl = make_context(wl, precision)
    pl.set_precision(abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64)
    probe = pl.invert_image_surface_brightness_map(wl.draw(np.random.default_rng(0), 1)[0])
    if probe["status"] != 0:
        raise RuntimeError("%s path status %d" % (precision, probe["status"]))
    # workloads with an elliptical NFW lens: train the deflection surrogate on
    # this GPU before the timed region (once per process), then ray-trace
    # through it with the default error gate
    nfw = None
    has_nfw = any(l["type"] in abi.NFW_TYPES for l in wl.lenses)
    if has_nfw:
        nfw = {"mode": "quadrature"}
        nfw_mode = args.nfw if args.nfw != "auto" else ("quadrature" if args.config == "cfg4" else "surrogate")
        if nfw_mode == "surrogate":
            from qlens_gb300 import pixlike
            rep = pixlike.train_nfw_surrogate(device=local_rank,
                                              **({"steps": args.train_steps} if args.train_steps > 0 else {}))
            pl.set_nfw_mode(abi.QLP_NFW_SURROGATE)
            nfw = {"mode": "surrogate", "threshold_arcsec": 2e-5, "train_ms": rep["train_ms"],
                   "val_mean_rel": rep["val_mean_rel"], "n_params": rep["n_params"]}
    if args.regopt:
        pl.set_regparam_optimization(True)
    uneven = wl.draw_instances is not None      # per-vector masks, source grids or lambdas
    if wl.instance_masks is not None:
        pl.set_instance_masks(wl.instance_masks)
    B = args.batch or wl.batch or (32 if precision == "mixed" else 4)
    pl.set_batch_slots(args.slots or min(B, 32))
    pl.set_graphs(not args.no_graphs)
    stream = torch.cuda.current_stream()
    pl.set_stream(stream.cuda_stream)

    rng = np.random.default_rng(1234 + rank)
    batches = [wl.draw(rng, B) for _ in range(args.warmup + args.steps)]
    pinned = [torch.from_numpy(b).pin_memory() for b in batches]
    insts = [wl.draw_instances(rng, B) if uneven else (None, None, None) for _ in batches]

    def run_step(k):
        ids, sizes, lam = insts[k]
        return pl.eval_batch(pinned[k].numpy(), regparams=lam, mask_ids=ids, src_sizes=sizes)

    # launch schedule: tuned on a sample of the first warm-up batch, before
    # the timed region (every schedule gives the same results)
    tune = None
    if not args.no_autotune:
        kk = min(B, 256)
        ids, sizes, lam = insts[0]
        t_tune = time.perf_counter()
        rep = pl.autotune(batches[0][:kk], regparams=None if lam is None else lam[:kk],
                          mask_ids=None if ids is None else ids[:kk], src_sizes=None if sizes is None else sizes[:kk],
                          reps=2)
        tune = {"sample": kk, "trials": rep["n_trials"], "start_ms": rep["start_ms"], "best_ms": rep["best_ms"],
                "wall_s": time.perf_counter() - t_tune}

    for k in range(args.warmup):
        run_step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    clocks = ClockSampler(local_rank)
    clocks.start()
    dev_ms = 0.0
    launches = 0
    h2d = d2h = 0
    results = []
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record(stream)
    for k in range(args.steps):
        res = run_step(args.warmup + k)
        dev_ms += pl.last_device_ms()
        launches += pl.last_launch_count()
        hb, db = pl.last_transfer_bytes()
        h2d += hb
        d2h += db
        results.extend(res)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    span_ms = e0.elapsed_time(e1)

    # slowest rank decides
    if dist:
        dev_ms, wall, span_ms = reduce_over_ranks([dev_ms, wall, span_ms], dist)

    n_evals = whole_job_evals(B, args.steps, world)
    value = n_evals / (dev_ms / 1e3)
    e2e = n_evals / wall
    bad = [r for r in results if r["status"] != 0]

    # Stage breakdown and the SYRK's own duration: a few evaluations after the
    # timed region, one at a time and launched kernel by kernel, with CUDA
    # events around each stage on the evaluation's stream (inside a batch the
    # stages of concurrent evaluations overlap, so they are not separable).
    iso = wl.draw(np.random.default_rng(777 + rank), 3)
    stage = np.zeros(6)
    iso_res = []
    for p in iso:
        iso_res.append(pl.invert_image_surface_brightness_map(p))
        stage += np.array(pl.stage_times())
    stage /= len(iso)

    # roofline of the tensor-core contraction F = L'^T C^-1 L'
    peaks = _peaks()
    syrk_ms = stage[3]
    flops = algorithmic_syrk_flops(iso_res) / len(iso)
    achieved = flops / (syrk_ms / 1e3) / 1e12 if syrk_ms > 0 else None
    if precision == "mixed":
        peak = peaks.get("bf16_tflops", 1900.0)
        peak_note = "measured bf16 burst (MEASURED_PEAKS.json)" if "bf16_tflops" in peaks else "fallback bf16"
        bound = "tensor"
    else:
        peak = 1.25
        peak_note = "nominal GB300 FP64 (no FP64 figure in MEASURED_PEAKS.json)"
        bound = "fp64"
    roofline_syrk = {"bound": bound, "kernel": "F = L'^T C^-1 L' (SYRK)", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": SYRK_TRAFFIC.get(args.config) if precision == "mixed" else None,
                     "peak_source": peak_note, "algorithmic_flops_per_launch": flops,
                     "timing": "CUDA events around the SYRK launch of single evaluations after the timed region"}
    if precision != "mixed":
        # k_syrk64 skips the 16-pixel steps where either tile of L' is zero
        # (the products it leaves out are zeros): the dense N M^2 count over
        # its time is a dense-equivalent rate, not a fraction of the pipe
        roofline_syrk["frac"] = None
        roofline_syrk["dense_equivalent_frac"] = (achieved / peak) if achieved else None
        roofline_syrk["note"] = ("achieved = the dense contraction's FLOP over the time of a kernel that skips L''s "
                                 "zero blocks: above the FP64 peak because most products are skipped")
    # the dominant kernel of the batch: the ray shooting on the NFW surrogate
    # workloads (k_raytrace_sur), else the factorisation of F
    roofline = roofline_syrk
    if precision == "mixed" and nfw and nfw["mode"] == "surrogate":
        ray_ms = stage[0]
        n_rays = wl.n_mask * wl.nsplit ** 2
        mlp = n_rays * MLP_FLOP_PER_RAY
        ach = mlp / (ray_ms / 1e3) / 1e12 if ray_ms > 0 else None
        roofline = {"bound": "tensor", "kernel": "ray shooting with the NFW surrogate (k_ray_pre + k_raytrace_sur)",
                    "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": (ach / peak) if ach else None,
                    "traffic": RAYSUR_TRAFFIC.get(args.config), "peak_source": peak_note,
                    "algorithmic_flops_per_launch": mlp,
                    "work": "the network's three 128x128 layers per ray (2 x 3 x 128^2 FLOP), %d rays" % n_rays,
                    "limiter": "the network's SIMT epilogues (tanh from the SFU's exp2 and reciprocal, F16 hi/lo "
                               "split, TMEM loads and stores) at 16 warps per SM: tensor pipe 29%, SFU 26%, FMA 20%, "
                               "FP64 7% in k_raytrace_sur, top stall the TMEM and ray loads; the FP64 lenses in "
                               "k_ray_pre at 85% of the FP64 pipe (one ncu capture)",
                    "timing": "CUDA events around the ray-shooting stage of single evaluations after the timed "
                              "region"}
    elif precision != "mixed":
        # the plain path's largest stage: the FP64 blocked Cholesky of F
        ch_flop = float(np.mean([r["n_active_src"] ** 3 / 3.0 for r in iso_res]))
        ach = ch_flop / (stage[4] / 1e3) / 1e12 if stage[4] > 0 else None
        roofline = {"bound": "fp64", "kernel": "FP64 Cholesky of F (k_potrf_t, k_trsm_inv_t, k_chol_update_t)",
                    "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": (ach / peak) if ach else None,
                    "traffic": None, "peak_source": peak_note, "algorithmic_flops_per_launch": ch_flop,
                    "work": "M^3/3 FLOP per factorisation",
                    "timing": "CUDA events around the factorisation stage of single evaluations after the timed "
                              "region"}
    elif precision == "mixed":
        ch_flop = float(np.mean([r["n_active_src"] ** 3 / 3.0 for r in iso_res]))
        ach = ch_flop / (stage[4] / 1e3) / 1e12 if stage[4] > 0 else None
        roofline = {"bound": "tensor", "kernel": "Cholesky of F (k_potrf128, k_chol_tile128, k_chol_upd16)",
                    "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": (ach / peak) if ach else None,
                    "traffic": None, "peak_source": peak_note, "algorithmic_flops_per_launch": ch_flop,
                    "work": "M^3/3 FLOP per factorisation",
                    "limiter": "the single-CTA pivot chain of M/128 steps per evaluation",
                    "timing": "CUDA events around the factorisation stage of single evaluations after the timed "
                              "region"}

    if args.trace and rank == 0:
        write_trace(pl, run_step, args.warmup, args.trace)
    if args.profile_step:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        run_step(args.warmup)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()

    # the plain FP64 path on the first vectors of the first timed batch: its
    # throughput, the ratio, and |delta log L| of the timed path against it
    plain = None
    accuracy = None
    if args.plain_sample > 0 and precision == "mixed":
        kfirst = args.warmup
        n = min(args.plain_sample, B)
        pv, pres = plain_fp64_arm(wl, batches[kfirst], insts[kfirst], n, slots=min(n, 8))
        plain = {"value": pv, "unit": UNIT, "sample": "the first %d vectors of the first timed batch" % n,
                 "path": "FP64 SYRK, Cholesky and solves" + ("; NFW deflection by quadrature" if has_nfw else ""),
                 "slots": min(n, 8)}
        accuracy = accuracy_of(results[:n], pres, has_nfw)

    # a second batch from the whole prior box (where the vectors above come
    # from a narrower region): its throughput and accuracy, untimed for the headline
    prior = None
    if wl.draw_prior is not None and precision == "mixed" and args.plain_sample > 0:
        rngp = np.random.default_rng(4242 + rank)
        Pp = wl.draw_prior(rngp, B)
        ip = wl.draw_instances(rngp, B) if uneven else (None, None, None)
        pl.eval_batch(Pp, regparams=ip[2], mask_ids=ip[0], src_sizes=ip[1])        # graphs already captured
        rp = pl.eval_batch(Pp, regparams=ip[2], mask_ids=ip[0], src_sizes=ip[1])
        pv_ms = pl.last_device_ms()
        n = min(args.plain_sample, B)
        _pv, pres = plain_fp64_arm(wl, Pp, ip, n, slots=min(n, 8))
        prior = {"value": B / (pv_ms / 1e3), "unit": UNIT, "batch": B,
                 "accuracy": accuracy_of(rp[:n], pres, has_nfw),
                 "median_chi2_per_pixel": float(np.median([r["chisq0"] / r["n_active_pixels"] for r in pres]))}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        times = cpu_sample(wl, np.random.default_rng(99), CPU_BUDGET_S, 5)
        cpu = {"value": 1.0 / statistics.median(times), "unit": UNIT, "cores": O.threads(), "kind": "port",
               "sample": "median of %d evaluations of fresh draws of the same workload by the oracle port of "
                         "QLens's dense inversion (stopped once their time exceeded %.0f s)" % (len(times),
                                                                                                CPU_BUDGET_S)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-tensor+f64" if precision == "mixed" else "f64",
            "data": "synthetic (seeded mock image; parameter vectors drawn as `draws` states)",
            "config": {**wl.describe(), "batch_per_step": B, "precision": precision,
                       "nfw": nfw["mode"] if nfw else None,
                       "schedule": pl.schedule(),
                       "autotune": tune,
                       "uneven": wl.uneven_note if uneven else None,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set (X, %.0f MB per evaluation) exceeds the 129 MB L2" % (
                           4e-6 * max(r["n_active_pixels"] for r in results) * max(r["n_active_src"] for r in results))},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d // args.steps),
                    "d2h_bytes_per_step": int(d2h // args.steps)},
            "vs_plain_fp64": (value / plain["value"]) if plain else None,
            "plain_fp64": plain,
            "accuracy": accuracy,
            "draws": wl.draws_note or "uniform over the configuration's prior box",
            "prior_draws": prior,
            "roofline": roofline,
            "roofline_syrk": roofline_syrk,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "launches_per_eval": launches / float(B * args.steps),
            "clocks": clk,
            "stage_ms_single_eval": [float(x) for x in stage],
            # the factorisation stage of one evaluation (stage 4: Cholesky of F and of R's band, the
            # triangular solves, the refinement): F's Cholesky is M^3/6 multiply-adds (M^3/3 FLOP),
            # over the stage's event time -- a pivot chain of M/128 steps, latency-bound for one
            # evaluation; the batch overlaps the slots' chains
            "cholesky_stage": {
                "ms": float(stage[4]),
                "algorithmic_tflop": float(np.mean([r["n_active_src"] ** 3 / 3.0 for r in iso_res])) / 1e12,
                "achieved_tflops": (float(np.mean([r["n_active_src"] ** 3 / 3.0 for r in iso_res]))
                                    / (stage[4] / 1e3) / 1e12) if stage[4] > 0 else None},
            "graphs": not args.no_graphs,
            "failed_evals": len(bad),
            "regopt": ({"lambda_trials_per_eval": float(np.mean([r["regopt_evals"] for r in results])),
                        "range_log10": [-3, 5], "tol": 0.01} if args.regopt else None),
            "nfw": (dict(nfw, fallback_rays_per_eval=float(np.mean([r["nfw_fallbacks"] for r in results])))
                    if nfw else None),
            "stream_span_ms": span_ms,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    pl.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
