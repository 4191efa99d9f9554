"""Throughput of the GB300 pixel-image likelihood (evaluations per second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl qlpix|reference]
                    [--config cfg2] [--batch B] [--precision mixed|fp64]

A step is one batch of B likelihood evaluations: B lens-parameter vectors are
drawn from the configuration's prior box and evaluated through the public C
ABI (qlp_eval_batch).  The default workload is the reference's larger
single-likelihood configuration (200x200 pixels at 0.04", annular mask,
4x4 split, 21x21 Airy-like PSF, 64x64 source grid, power-law lens + shear),
on seeded synthetic data.  `value` is evaluations per second of device time
(inputs resident: image, mask and PSF are uploaded once when the context is
created); `e2e` is the same metric through the public call with the step's
parameter vectors in pinned host memory and the results read back, timed on
the host.  Under torchrun every rank evaluates its own batches (replicas, weak
scaling) and the slowest rank's time counts.

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

# dram__bytes_read.sum + dram__bytes_write.sum of one k_syrk_tc launch on cfg2 (ncu, GB300)
SYRK_TC_DRAM_BYTES_CFG2 = 115.223e6 + 9.662e6

METRIC = "pixel-likelihood evals/s on 1 GB300: batched+surrogate vs plain FP64 at |ΔlogL|<0.1"
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


def cpu_port_eval(wl, params, threads=None):
    """One evaluation of the oracle port (CPU) on the workload; returns seconds."""
    from oracle import oracle as O
    from qlens_gb300 import abi
    img = abi.ImageBuffers(wl.xvals, wl.yvals, wl.data, wl.mask, None, wl.noise)
    psf = abi.PSFBuffer(wl.psf)
    o = abi.srcgrid_defaults()
    o.nsplit = wl.nsplit
    o.npixels_x, o.npixels_y = wl.src_npixels
    o.regparam = wl.regparam
    t = time.perf_counter()
    planes = abi.make_planes(getattr(wl, "zfac", None), getattr(wl, "beta", None))
    r = O.evaluate(img, psf, o, wl.lenses, lens_params=params, planes=planes)
    return time.perf_counter() - t, r


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from qlens_gb300 import synthetic
    from oracle import oracle as O
    O.build()
    wl = synthetic.CONFIGS[args.config]()
    rng = np.random.default_rng(4321)
    cores = O.threads()
    for _ in range(args.warmup):
        cpu_port_eval(wl, wl.draw(rng, 1)[0])
    times = []
    for _ in range(args.steps):
        dt, _r = cpu_port_eval(wl, wl.draw(rng, 1)[0])
        times.append(dt)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "batch_per_step": 1, **wl.describe()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d evaluations, one per step, OpenMP over %d host threads" % (args.steps, cores)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="qlpix", choices=["qlpix", "reference"])
    ap.add_argument("--config", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5"])
    ap.add_argument("--batch", type=int, default=0, help="evaluations per step (default per precision)")
    ap.add_argument("--slots", type=int, default=0, help="concurrent evaluation slots (default min(batch, 32))")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernel by kernel instead of replaying graphs")
    ap.add_argument("--precision", default=os.environ.get("QLPIX_BENCH_PRECISION", "mixed"),
                    choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--trace", default="",
                    help="after the measurement, record one more step's kernel timeline (launched kernel by kernel, "
                         "through torch.profiler) and write a per-kernel summary to this JSON file")
    ap.add_argument("--regopt", action="store_true",
                    help="choose lambda per evaluation by Brent's method (QLens 'optimize_regparam on')")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch schedule instead of tuning it on a sample batch first")
    ap.add_argument("--nfw", default="surrogate", choices=["surrogate", "quadrature"],
                    help="NFW deflection: trained MLP surrogate (quadrature fallback) or quadrature only")
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
    try:
        pl.set_precision(abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64)
        probe = pl.invert_image_surface_brightness_map(wl.draw(np.random.default_rng(0), 1)[0])
        if probe["status"] != 0:
            raise RuntimeError("mixed path status %d" % probe["status"])
    except Exception:
        precision = "fp64"
        pl.set_precision(abi.QLP_FP64)
    # workloads with an elliptical NFW lens: train the deflection surrogate on
    # this GPU before the timed region (once per process), then ray-trace
    # through it with the default error gate
    nfw = None
    if any(l["type"] == "nfw" for l in wl.lenses):
        nfw = {"mode": "quadrature"}
        if args.nfw == "surrogate":
            from qlens_gb300 import pixlike
            rep = pixlike.train_nfw_surrogate(device=local_rank)
            pl.set_nfw_mode(abi.QLP_NFW_SURROGATE)
            nfw = {"mode": "surrogate", "threshold_arcsec": 2e-5, "train_ms": rep["train_ms"],
                   "val_mean_rel": rep["val_mean_rel"], "n_params": rep["n_params"]}
    if args.regopt:
        pl.set_regparam_optimization(True)
    uneven = wl.draw_instances is not None      # per-instance masks, source grids and lambdas
    if uneven:
        pl.set_instance_masks(wl.instance_masks)
    B = args.batch or (4096 if uneven else 32 if precision == "mixed" else 4)
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

    # roofline of the dominant tensor-core kernel: the F = L'^T C^-1 L' contraction
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
    # DRAM bytes of one k_syrk_tc launch on cfg2 from one ncu capture (profiles/k_syrk_tc_cfg2.md)
    traffic = SYRK_TC_DRAM_BYTES_CFG2 if (precision == "mixed" and args.config == "cfg2") else None
    roofline = {"bound": bound, "kernel": "F = L'^T C^-1 L' (SYRK)", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "peak_source": peak_note, "algorithmic_flops_per_launch": flops,
                "timing": "CUDA events around the SYRK launch of single evaluations after the timed region"}

    if args.trace and rank == 0:
        write_trace(pl, run_step, args.warmup, args.trace)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, _r = cpu_port_eval(wl, wl.draw(np.random.default_rng(99), 1)[0])
        from oracle import oracle as O
        cpu = {"value": 1.0 / dt, "unit": UNIT, "cores": O.threads(), "kind": "port",
               "sample": "1 evaluation of the same workload by the oracle port of QLens's dense inversion"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-tensor+f64" if precision == "mixed" else "f64",
            "data": "synthetic (seeded mock image; parameters drawn from the prior box)",
            "config": {**wl.describe(), "batch_per_step": B, "precision": precision,
                       "schedule": pl.schedule(),
                       "autotune": tune,
                       "uneven": ("per vector: one of %d masks (r 1.5-3.0\"), source side 20-64, "
                                  "log10 lambda 0-2" % len(wl.instance_masks)) if uneven else None,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set (dense L' %.0f MB) exceeds the 129 MB L2" % (
                           8e-6 * max(r["n_active_pixels"] for r in results) * max(r["n_active_src"] for r in results))},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d // args.steps),
                    "d2h_bytes_per_step": int(d2h // args.steps)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "clocks": clk,
            "stage_ms_single_eval": [float(x) for x in stage],
            # the factorisation stage of one evaluation (stage 4: Cholesky of F and of R's band, the
            # triangular solves, the refinement): algorithmic M^3/3 multiply-adds of F's Cholesky
            # over the stage's event time -- a pivot chain of M/128 steps, latency-bound for one
            # evaluation; the batch overlaps 32 of them
            "cholesky_stage": {
                "ms": float(stage[4]),
                "algorithmic_tflop": float(np.mean([2.0 * r["n_active_src"] ** 3 / 3.0 for r in iso_res])) / 1e12,
                "achieved_tflops": (float(np.mean([2.0 * r["n_active_src"] ** 3 / 3.0 for r in iso_res]))
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
