#!/usr/bin/env python
"""LC2 similarity benchmark: evals/s at 256^3 on one GB300.

Workload (one "step"): one batched launch of K = 512 candidate affine
transforms of a 256^3 MR volume into a 256^3 US volume, 9^3 patches
(PatchSize 4), FP16 storage of both volumes, FP32 arithmetic with exact
64-bit fixed-point patch moments. The volumes are synthetic and seeded
(ellipsoid MR phantom, US synthesised from it with Rayleigh speckle, 10% of
the US replaced by constant 16^3 blocks).

Reported:
  value      batched evals/s, device-timed (CUDA events on the library's
             stream), inputs resident in HBM, L2 flushed between steps;
  e2e        the same through the public C ABI call lc2_evaluate_batch with
             host transforms in and host results out (H2D/D2H inside);
  plain      one evaluation per lc2_evaluate call (the reference's
             one-eval-per-objective form) on the same GPU;
  roofline   the moments kernel (the dominant one): algorithmic bytes
             (K*N*s_mov + N*s_fix per launch group) / its event-timed
             duration, against the measured HBM copy bandwidth;
  cpu_baseline  the FP64 oracle (a port of the reference formulas; the
             reference has no CPU LC2 path) on the host cores.

`--impl reference` times that CPU port alone on the same workload.
Multi-GPU: independent replicas (one process per GPU, no collective on the
data path); value = total evals / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LC2 evals/s at 256^3 (batched, 512 affines/launch, 9^3 patches, FP16 storage)"
UNIT = "evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--candidates", type=int, default=512)
    ap.add_argument("--patch", type=int, default=4)
    ap.add_argument("--storage", default="f16", choices=["f32", "f16", "bf16"])
    ap.add_argument("--plain-evals", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch options")
    ap.add_argument("--tile-rows", type=int, default=0,
                    help="with --no-autotune: tile height of the fused 3D kernel (8, 16, 24; "
                         "0 = the library's default)")
    ap.add_argument("--no-small", action="store_true", help="skip the 2D 256^2 / 3D 96^3 lines")
    ap.add_argument("--no-stack", action="store_true", help="skip the 2D-to-3D frame-stack line")
    ap.add_argument("--no-fixed", action="store_true",
                    help="skip the HighResolutionModality: Fixed lines")
    ap.add_argument("--no-mi", action="store_true", help="skip the mutual-information lines")
    ap.add_argument("--no-bf16", action="store_true", help="skip the bf16-storage line")
    ap.add_argument("--no-register", action="store_true",
                    help="skip the registration (recovered-parameter) lines")
    ap.add_argument("--stack-frames", type=int, default=64)
    ap.add_argument("--stack-poses", type=int, default=256)
    ap.add_argument("--serve-requests", type=int, default=200, help="requests per offered rate")
    ap.add_argument("--serve-rates", default="10,50,100,250,500",
                    help="offered Poisson arrival rates (requests/s), comma-separated")
    ap.add_argument("--serve-active", type=int, default=8)
    return ap.parse_args()


def workload(args):
    from lc2registration_gb300 import synth

    case = synth.case_3d(seed=2024, mr_size=args.size, us_size=args.size, r=args.patch,
                         constant_block_frac=0.1)
    import numpy as np

    from tests.helpers import perturbed

    mats = perturbed(case, np.random.default_rng(77), args.candidates, scale=1.0)
    return case, mats


def config_dict(args, case):
    return {
        "workload": f"3D affine, MR {args.size}^3 -> US {args.size}^3 at 1 mm, PatchSize "
                    f"{args.patch} ({2 * args.patch + 1}^3 patches), {args.candidates} candidate "
                    f"affines per launch, {args.storage} storage, 10% constant US blocks",
        "virtual_voxels": int(case.fixed_geom.n),
        "candidates_per_step": args.candidates,
        "patch_size": args.patch,
        "storage": args.storage,
        "l2": "flushed between steps (256 MiB write); per-step working set > L2",
        "parallelism": "replicas" if args.gpus > 1 else "single GPU",
    }


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_port(case, mats, seconds: float, storage: str):
    """FP64 oracle on the host cores over a bounded sample of candidates.
    Returns the rate, the count, the seconds and the oracle's LC2 values (in
    transform order), which the caller checks the GPU results against."""
    from tests.helpers import oracle_eval

    t0 = time.perf_counter()
    vals = []
    while True:
        vals.append(oracle_eval(case, mats[len(vals) % len(mats)], storage=storage))
        el = time.perf_counter() - t0
        if el >= seconds and len(vals) >= 2:
            break
    return len(vals) / el, len(vals), el, np.array(vals[: len(mats)])


def parity_vs_oracle(gpu_vals, oracle_vals, tol=1e-5):
    """Largest relative LC2 difference between the GPU's values and the FP64
    oracle's on the same transforms (the oracle fed the same storage-rounded
    volumes); raises when it exceeds tol, so a bench line is never printed
    for results that differ from the oracle."""
    g = np.asarray(gpu_vals[: len(oracle_vals)], dtype=np.float64)
    o = np.asarray(oracle_vals, dtype=np.float64)
    rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-300)
    worst = float(rel.max()) if len(rel) else None
    if worst is not None and not worst < tol:
        raise AssertionError(f"GPU vs FP64 oracle: max relative LC2 error {worst:.3e} > {tol}")
    return {"max_rel_err_vs_oracle": worst, "evaluations_checked": int(len(o)), "tolerance": tol}


def _registration(case, rng):
    """Registration settings of one served request: DIRECT on the translation,
    then two local rounds to xtol 1e-6, from a seeded start near identity."""
    c = case.fixed_geom.center()
    if case.mode == "2D":
        init = [rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(-2, 2), 1, 1, 0]
        lo = [-12, -12, -10, 0.9, 0.9, -0.06]
        hi = [12, 12, 10, 1.1, 1.1, 0.06]
    else:
        init = list(rng.uniform(-2, 2, 6)) + [1, 1, 1, 0, 0, 0]
        lo = [-12, -12, -12, -10, -10, -10, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05]
        hi = [12, 12, 12, 10, 10, 10, 1.1, 1.1, 1.1, 0.05, 0.05, 0.05]
    return dict(initial=init, lower=lo, upper=hi, center=c, direct_entries=["translation"],
                direct_maxeval=50, round_maxeval=400,
                rounds=[(["translation", "rotation"], 1e-6),
                        (["translation", "rotation", "scale", "shear"], 1e-6)])


def serve_sweep(args, main_case, device):
    """The serving leg at each offered rate of --serve-rates (requests/s),
    --serve-requests requests per rate."""
    rates = [float(r) for r in str(args.serve_rates).split(",") if r.strip()]
    rows = [serve_leg(args, main_case, device, rate, args.serve_requests) for rate in rates]
    return {"rates": rows,
            "note": "each rate: Poisson arrivals of the C5 mix on one server (merged launches "
                    "for 2D and 2D-to-3D steps); above about 2 requests/s of 256^3 "
                    "registrations the GPU is saturated and latency is queueing"}


def serve_leg(args, main_case, device, rate, nreq):
    """Serving: Poisson arrivals of whole registrations, mix 40% 2D 256^2,
    30% 3D 128^3 -> 96^3, 20% 3D 256^3 FP16 (the main workload's volumes),
    10% 2D-to-3D stacks of 16 uneven frames cut from the 256^3 MR. Returns the
    latency percentiles (submit -> result) and the request rate."""
    import numpy as np

    from lc2registration_gb300 import capi, synth

    rng = np.random.default_rng(4242)
    pools = {
        "2d_256": [synth.case_2d(seed=s, size=256, r=3) for s in (101, 102)],
        "3d_128_96": [synth.case_3d(seed=s, mr_size=128, us_size=96, r=3) for s in (103, 104)],
        "3d_256_f16": [main_case],
        "stack16": [synth.frame_stack(main_case.moving, main_case.moving_geom, 16, seed=105,
                                      spacing=0.5, r=3)],
    }
    kinds = rng.choice(list(pools), size=nreq, p=[0.4, 0.3, 0.2, 0.1])
    srv = capi.Server(budget_bytes=0, max_active=args.serve_active, device=device)

    def submit(case, storage):
        cfg = capi.make_config(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing,
                               case.r, case.hr_moving, storage, device=device)
        return srv.submit(cfg, case.fixed, case.moving, **_registration(case, rng))

    sent = []  # (kind, [tickets], submit time)
    t0 = time.perf_counter()
    for k in kinds:
        pool = pools[k]
        item = pool[int(rng.integers(len(pool)))]
        if k == "stack16":
            tickets = [("stack", srv.submit_stack(
                main_case.moving_geom, main_case.moving, 3, [(f.fixed_geom, f.fixed) for f in item],
                item[0].virt_spacing, [_registration(f, rng) for f in item], "f16"))]
        else:
            tickets = [("one", submit(item, "f16" if k == "3d_256_f16" else "f32"))]
        sent.append((k, tickets))
        time.sleep(rng.exponential(1.0 / rate))
    lat = {k: [] for k in pools}
    queue = {k: [] for k in pools}
    run = {k: [] for k in pools}
    evals = 0
    for k, tickets in sent:
        rs = []
        for kind, t in tickets:
            rs += srv.poll_stack(t) if kind == "stack" else [srv.poll(t)]
        for r in rs:
            assert r["status"] == 0, r["message"]
            evals += r["evaluations"]
        lat[k].append(max(r["total_ms"] for r in rs))
        queue[k].append(max(r["queue_ms"] for r in rs))
        run[k].append(max(r["run_ms"] for r in rs))
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    allv = np.array([v for vs in lat.values() for v in vs])

    def pct(v, q):
        return float(np.percentile(v, q, method="inverted_cdf")) if len(v) else None
    return {
        "requests": len(sent), "rate_offered": rate,
        "merged_launches": st["merged_launches"], "merged_steps": st["merged_steps"],
        "requests_per_s": len(sent) / wall, "evals_per_s": evals / wall,
        "p50_ms": pct(allv, 50), "p95_ms": pct(allv, 95), "p99_ms": pct(allv, 99),
        "by_kind_p50_ms": {k: pct(np.array(v), 50) for k, v in lat.items()},
        "by_kind_mean_queue_ms": {k: float(np.mean(v)) if v else None for k, v in queue.items()},
        "by_kind_mean_run_ms": {k: float(np.mean(v)) if v else None for k, v in run.items()},
        "by_kind_count": {k: len(v) for k, v in lat.items()},
        "max_active": args.serve_active, "peak_active": st["peak_active"],
        "peak_device_bytes": st["peak_bytes"],
        "mix": "40% 2D 256^2 r3, 30% 3D 128^3->96^3 r3, 20% 3D 256^3 f16 r4, 10% 2D-to-3D "
               "stacks of 16 frames (sides 128-512 at 0.5 mm, one stack request sharing one "
               "upload of the volume) r3; DIRECT + 2 rounds to xtol 1e-6",
    }


def replica_rate(units_local: float, seconds_local: float, dist=None, device=None) -> float:
    """Whole-job throughput of independent replicas: the units of every rank
    over the slowest rank's time (max over ranks, as the driver measures)."""
    if dist is None:
        return units_local / seconds_local
    import torch

    t = torch.tensor([seconds_local, units_local], dtype=torch.float64, device=device)
    tmax = t[:1].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    units = t[1:].clone()
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    return float(units.item()) / float(tmax.item())


def small_configs(device):
    """Batched vs plain on the small configurations (2D 256^2, 7x7 patches;
    3D 128^3 -> 96^3, 7^3 patches), where one evaluation does not fill the
    GPU: device-timed batches of 512 and 256 transforms, and one
    lc2_evaluate per transform through the public call (host in / host out)."""
    import numpy as np
    import torch

    from lc2registration_gb300 import capi, synth
    from tests.helpers import perturbed

    out = {}
    for name, case, K in (("2d_256_r3", synth.case_2d(seed=7, size=256, r=3), 512),
                          ("3d_128_96_r3", synth.case_3d(seed=8, mr_size=128, us_size=96, r=3), 256)):
        ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                           True, "f32", device=device)
        ctx.set_images(case.fixed, case.moving)
        mats = perturbed(case, np.random.default_rng(3), K)
        ctx.stage(mats)
        stream = torch.cuda.ExternalStream(ctx.stream())
        for _ in range(3):
            ctx.launch(K)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(5):
            ctx.launch(K)
        ev[1].record(stream)
        torch.cuda.synchronize()
        batched = 5 * K / (ev[0].elapsed_time(ev[1]) / 1e3)
        vals = ctx.fetch(K)
        for m in mats[:8]:
            ctx.evaluate(m)
        n = 200
        t0 = time.perf_counter()
        plain = [ctx.evaluate(m) for m in mats[:n % K or K][:n]]
        plain_eps = len(plain) / (time.perf_counter() - t0)
        assert np.array_equal(np.array(plain), vals[:len(plain)]), "plain != batched"
        nv = int(np.prod(ctx.virtual_dims()))
        # algorithmic bytes (f32): K N s_mov + N s_fix per batched launch, N (s_mov
        # + s_fix) per plain evaluation
        out[name] = {"batched_evals_per_s": batched, "plain_evals_per_s": plain_eps,
                     "plain_latency_ms": 1e3 / plain_eps,
                     "batched_over_plain": batched / plain_eps, "candidates_per_launch": K,
                     "virtual_voxels": nv, "storage": "f32",
                     "algorithmic_gbs_batched": (K * nv * 4 + nv * 4) * batched / K / 1e9,
                     "algorithmic_gbs_plain": nv * 8 * plain_eps / 1e9}
        ctx.close()
    return out


def bf16_leg(args, case, mats, device, flush):
    """The main workload with both volumes held in bf16 instead of f16: the
    same 512-transform launches, device-timed with L2 flushed between them,
    and two of the transforms checked against the FP64 oracle fed the same
    bf16-rounded volumes."""
    import torch

    from lc2registration_gb300 import capi
    from tests.helpers import oracle_eval

    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                       case.hr_moving, "bf16", device=device)
    ctx.set_images(case.fixed, case.moving)
    K = mats.shape[0]
    ctx.stage(mats)
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(2):
        ctx.launch(K)
    reps = 3
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(reps):
            flush.zero_()
            ev[i][0].record(stream)
            ctx.launch(K)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / reps
    vals = ctx.fetch(K)
    ctx.close()
    out = {"batched_evals_per_s": K / (ms / 1e3), "ms_per_launch": ms,
           "candidates_per_launch": K, "storage": "bf16"}
    if not args.no_cpu:
        ovals = [oracle_eval(case, mats[i], storage="bf16") for i in (0, K - 1)]
        out["parity"] = parity_vs_oracle(vals[[0, K - 1]], ovals)
    return out


def issue_roofline(ipv, voxels, kernel_ms, device, clk, source):
    """The bound the fused kernel actually meets: instruction issue. achieved =
    warp instructions of one launch (ncu's per-voxel count x voxels / 32) per
    second of the event-timed launch; peak = SMs x 4 schedulers x one warp
    instruction per cycle at the maximum SM clock sampled."""
    import torch

    if not ipv or not kernel_ms:
        return None
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = (clk.summary() or {}).get("sm_max_mhz") or 2070.0
    achieved = ipv * voxels / 32.0 / (kernel_ms / 1e3)
    peak = sms * 4 * mhz * 1e6
    return {"bound": "issue", "unit": "warp instructions/s", "achieved": achieved, "peak": peak,
            "frac": achieved / peak,
            "source": "instructions per voxel " + source + "; launch time measured in this run"}


def fixed_leg(args, main_case, device):
    """HighResolutionModality: Fixed (the reference's own configs use it): the
    MR/CT is the static high-resolution image on its own grid and the
    ultrasound is warped per transform. The same volumes with the roles
    swapped: device-timed batches through the fused kernel of this modality,
    the same batches through the generic kernels (LC2_OPTION_GENERIC), and one
    lc2_evaluate per transform."""
    import numpy as np
    import torch

    from lc2registration_gb300 import capi, synth
    from tests.helpers import perturbed

    def swapped(case):
        return synth.Case(case.mode, case.moving_geom, case.moving, case.fixed_geom, case.fixed,
                          list(case.moving_geom.spacing[: (2 if case.mode == "2D" else 3)]),
                          case.r, hr_moving=False, true_params={},
                          true_mat=np.linalg.inv(case.true_mat.astype(np.float64)).astype(np.float32))

    def timed(ctx, K, reps):
        stream = torch.cuda.ExternalStream(ctx.stream())
        for _ in range(2):
            ctx.launch(K)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(reps):
            ctx.launch(K)
        ev[1].record(stream)
        torch.cuda.synchronize()
        return reps * K / (ev[0].elapsed_time(ev[1]) / 1e3)

    out = {}
    for name, base, K, storage, plain_n in (
            (f"3d_{args.size}_r{args.patch}", main_case, 128, args.storage, 24),
            ("2d_256_r3", synth.case_2d(seed=7, size=256, r=3), 512, "f32", 200),
            ("3d_128_96_r3", synth.case_3d(seed=8, mr_size=128, us_size=96, r=3), 256, "f32", 100)):
        case = swapped(base)
        mats = np.linalg.inv(perturbed(base, np.random.default_rng(3), K).astype(np.float64))
        mats = mats.astype(np.float32)
        # max_batch 16: the generic path batches 16 transforms per group (its
        # scratch holds one warped image per transform); the fused path needs none
        ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                           False, storage, 16, device=device)
        ctx.set_images(case.fixed, case.moving)
        ctx.stage(mats)
        fused = timed(ctx, K, 5)
        vals = ctx.fetch(K)
        ctx.set_option(capi.OPTION_GENERIC, 1)
        generic = timed(ctx, K, 3)
        gvals = ctx.fetch(K)
        ctx.set_option(capi.OPTION_GENERIC, 0)
        for m in mats[:4]:
            ctx.evaluate(m)
        t0 = time.perf_counter()
        plain = [ctx.evaluate(m) for m in mats[:plain_n]]
        plain_eps = len(plain) / (time.perf_counter() - t0)
        assert np.array_equal(np.array(plain), vals[:len(plain)]), "plain != batched"
        out[name] = {"batched_evals_per_s": fused, "generic_batched_evals_per_s": generic,
                     "fused_over_generic": fused / generic, "plain_evals_per_s": plain_eps,
                     "max_rel_diff_fused_generic": float(np.max(np.abs(vals - gvals) /
                                                               np.maximum(np.abs(gvals), 1e-30))),
                     "candidates_per_launch": K, "virtual_voxels": int(np.prod(ctx.virtual_dims())),
                     "storage": storage}
        ctx.close()
    return out


def stack_leg(args, main_case, device):
    """2D-to-3D frame stack: frames of uneven sizes (sides 128-512 at 0.5 mm)
    cut from the 256^3 MR at seeded 6-DOF poses, `stack_poses` candidate
    poses per frame, all (frame, pose) pairs in one lc2_stack_evaluate call
    (one persistent launch, replayed from a CUDA graph after the first). The
    MR is held in f32 (the configuration's storage) and, second line, f16."""
    import numpy as np

    from lc2registration_gb300 import capi, synth
    from tests.helpers import perturbed

    frames = synth.frame_stack(main_case.moving, main_case.moving_geom, args.stack_frames,
                               seed=91, spacing=0.5, r=3)
    rng = np.random.default_rng(92)
    ids, mats = [], []
    for i, f in enumerate(frames):
        ids += [i] * args.stack_poses
        mats.append(perturbed(f, rng, args.stack_poses, scale=0.5))
    ids = np.array(ids, dtype=np.int32)
    mats = np.concatenate(mats)
    px = sum(int(f.fixed_geom.dim[0]) * int(f.fixed_geom.dim[1]) for f in frames)
    out = {"frames": len(frames), "poses_per_frame": args.stack_poses,
           "evaluations_per_call": int(len(ids)), "frame_pixels": px,
           "note": "end to end through lc2_stack_evaluate (host poses in, host LC2 out), "
                   "7x7 patches, one graph-replayed launch per call"}
    for storage in ("f32", "f16"):
        st = capi.Stack(main_case.moving_geom, 3, storage, device)
        st.set_moving(main_case.moving)
        for f in frames:
            st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed)
        st.evaluate(ids, mats)  # capture
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            vals = st.evaluate(ids, mats)
        el = (time.perf_counter() - t0) / reps
        assert np.all(np.isfinite(vals)) and vals.max() > 0
        st.close()
        s_mov = 4 if storage == "f32" else 2
        # algorithmic bytes: every frame pixel reads one moving element per pose
        # and one ultrasound element (f32) per call
        alg = px * args.stack_poses * s_mov + px * 4
        out[f"mr_{storage}"] = {"evals_per_s": len(ids) / el, "ms_per_call": el * 1e3,
                                "pixel_evals_per_s": px * args.stack_poses / el,
                                "algorithmic_gbs": alg / el / 1e9}
    return out


def mi_leg(args, main_case, device):
    """Normalised mutual information (PatchSize 0; cu_lc2_3d.cu:868-923,
    1196-1301): device-timed batches and one lc2_evaluate per transform, on
    the main 256^3 volumes (f16) and on the 128^3 -> 96^3 case (f32). NMI >= 1
    always; batched and plain values must agree bit for bit."""
    import numpy as np
    import torch

    from lc2registration_gb300 import capi, synth
    from tests.helpers import perturbed

    out = {}
    for name, case, storage, K in (
            ("3d_256_f16", main_case, "f16", 64),
            ("3d_128_96", synth.case_3d(seed=8, mr_size=128, us_size=96, r=3), "f32", 256)):
        ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, 0,
                           True, storage, device=device)
        ctx.set_images(case.fixed, case.moving)
        mats = perturbed(case, np.random.default_rng(5), K)
        ctx.stage(mats)
        stream = torch.cuda.ExternalStream(ctx.stream())
        for _ in range(2):
            ctx.launch(K)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        reps = 3
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(reps):
            ctx.launch(K)
        ev[1].record(stream)
        torch.cuda.synchronize()
        batched = reps * K / (ev[0].elapsed_time(ev[1]) / 1e3)
        vals = ctx.fetch(K)
        assert np.all(np.isfinite(vals)) and vals.min() >= 1.0, "NMI out of range"
        for m in mats[:4]:
            ctx.evaluate(m)
        n = 32
        t0 = time.perf_counter()
        plain = [ctx.evaluate(m) for m in mats[:n]]
        plain_eps = n / (time.perf_counter() - t0)
        assert np.array_equal(np.array(plain), vals[:n]), "plain != batched"
        nv = int(np.prod(ctx.virtual_dims()))
        out[name] = {"batched_evals_per_s": batched, "plain_evals_per_s": plain_eps,
                     "batched_over_plain": batched / plain_eps, "candidates_per_launch": K,
                     "virtual_voxels": nv, "voxel_evals_per_s": batched * nv,
                     "storage": storage}
        ctx.close()
    return out


def registration_leg(args, device):
    """Recovered parameters of the configured registrations, BOBYQA from the
    identity: 2D 256^2 at most 200 evaluations, 3D 128^3 -> 96^3 at most 500;
    each rigid (translation and rotation; scale and shear held at the
    generating values) and affine (all 6 / 12 parameters). The GPU run is
    timed end to end through lc2_register; the same driver with the FP64
    oracle objective gives the reference parameters (skipped with --no-cpu)."""
    import numpy as np

    from lc2registration_gb300 import capi, synth
    from tests.helpers import oracle_eval

    out = {}
    for cname, case, maxeval in (("2d_256", synth.case_2d(seed=7, size=256, r=3), 200),
                                 ("3d_128_96", synth.case_3d(seed=8, mr_size=128, us_size=96,
                                                             r=3), 500)):
        p = case.true_params
        if case.mode == "2D":
            truth = np.array(list(p["trans"]) + [p["rot"]] + list(p["scale"]) + [p["shear"]])
            nr = 3
            lo_a, hi_a = [-12, -12, -10, 0.9, 0.9, -0.06], [12, 12, 10, 1.1, 1.1, 0.06]
            init_a = [0, 0, 0, 1, 1, 0.0]
        else:
            truth = np.array(list(p["trans"]) + list(p["rot"]) + list(p["scale"]) +
                             list(p["shear"]))
            nr = 6
            lo_a, hi_a = [-12] * 6 + [0.9] * 3 + [-0.05] * 3, [12] * 6 + [1.1] * 3 + [0.05] * 3
            init_a = [0] * 6 + [1, 1, 1, 0, 0, 0.0]
        init_r = np.concatenate([np.zeros(nr), truth[nr:]])
        lo_r, hi_r = init_r.copy(), init_r.copy()
        lo_r[:nr], hi_r[:nr] = -12.0, 12.0
        for kind, init, lo, hi, entries in (
                ("rigid", init_r, lo_r, hi_r, ["translation", "rotation"]),
                ("affine", init_a, lo_a, hi_a, ["translation", "rotation", "scale", "shear"])):
            kw = dict(center=case.fixed_geom.center(), direct_entries=[],
                      rounds=[(entries, 1e-6)], round_maxeval=maxeval)
            ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing,
                               case.r, True, "f32", device=device)
            ctx.set_images(case.fixed, case.moving)
            t0 = time.perf_counter()
            gpu = capi.register(ctx, init, lo, hi, **kw)
            wall = time.perf_counter() - t0
            ctx.close()
            err = np.abs(gpu["params"] - truth)
            row = {"evaluations": gpu["evaluations"], "launches": gpu["launches"],
                   "wall_ms": wall * 1e3, "lc2": gpu["lc2"],
                   "max_err_vs_truth_mm_deg": float(err[:nr].max())}
            if kind == "affine":
                row["max_err_vs_truth_scale_shear"] = float(err[nr:].max())
            if not args.no_cpu:
                shape = (3, 3) if case.mode == "2D" else (4, 4)
                orc = capi.register(None, init, lo, hi, mode=case.mode,
                                    lc2_of_matrices=lambda M: np.array(
                                        [oracle_eval(case, m.reshape(shape)) for m in M]), **kw)
                d = np.abs(gpu["params"] - orc["params"])
                row.update({"oracle_evaluations": orc["evaluations"], "oracle_lc2": orc["lc2"],
                            "max_diff_vs_oracle_mm_deg": float(d[:nr].max()),
                            "lc2_rel_diff_vs_oracle": abs(gpu["lc2"] / orc["lc2"] - 1.0)})
                if kind == "affine":
                    row["max_diff_vs_oracle_scale_shear"] = float(d[nr:].max())
            out[f"{cname}_{kind}"] = row
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    case, mats = workload(args)
    cores = os.cpu_count() or 1
    from tests.helpers import oracle_eval

    for w in range(args.warmup):
        oracle_eval(case, mats[w % len(mats)], storage=args.storage)
    t0 = time.perf_counter()
    for s in range(args.steps):
        oracle_eval(case, mats[s % len(mats)], storage=args.storage)
    total = time.perf_counter() - t0
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_dict(args, case),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full {args.size}^3 evaluations (one per step) "
                                   "of the FP64 oracle, OpenMP over all host cores; the reference "
                                   "has no CPU LC2 implementation"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from lc2registration_gb300 import capi

    capi.load()
    case, mats = workload(args)
    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                       case.hr_moving, args.storage, device=local)
    ctx.set_images(case.fixed, case.moving)
    # tile height, kernel variant, z-chunk; timed on 64 transforms
    if args.no_autotune:
        if args.tile_rows:
            ctx.set_option(capi.OPTION_TILE_ROWS, args.tile_rows)
        tuned = (args.tile_rows or 24, 0)
    else:
        tuned = ctx.autotune(mats[:64])
    K = mats.shape[0]
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")

    ctx.stage(mats)
    for _ in range(args.warmup):
        ctx.launch(K)
    torch.cuda.synchronize()

    props = torch.cuda.get_device_properties(local)
    gpu_id = str(getattr(props, "uuid", local))
    if gpu_id and not gpu_id.startswith("GPU-") and len(gpu_id) > 8:
        gpu_id = "GPU-" + gpu_id
    # ---- timed region: K steps, device events per step, L2 flushed between ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    launches0 = ctx.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(gpu_id) as clk:
        with torch.cuda.stream(stream):
            for s in range(args.steps):
                flush.zero_()
                ev[s][0].record(stream)
                ctx.launch(K)
                ev[s][1].record(stream)
        torch.cuda.synchronize()
    launches = ctx.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    value = replica_rate(K * args.steps, total_ms / 1e3, dist, f"cuda:{local}")
    total_ms = world * K * args.steps / value * 1e3  # the slowest rank's time
    res = ctx.fetch(K)
    assert np.all(np.isfinite(res)) and res.max() > 0

    # ---- per-kernel timing of one step (roofline) ----
    ctx.enable_kernel_timing(True)
    ctx.launch(K)
    kt = ctx.kernel_times()
    ctx.enable_kernel_timing(False)
    n_vox = case.fixed_geom.n
    s_mov = 4 if args.storage == "f32" else 2
    s_fix = s_mov
    mom_ms, mom_launches = kt["moments"]
    alg_bytes = K * n_vox * s_mov + mom_launches * n_vox * s_fix
    achieved = alg_bytes / (mom_ms / 1e3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # the reference's own kernels on this GPU type, measured separately by
    # oracle/ref_golden/ref_gpu_time.py
    ref_gpu = None
    rfile = os.path.join(ROOT, "profiles", "reference_gpu_kernels.json")
    if os.path.exists(rfile):
        try:
            ref_rows = {w["workload"]: w for w in json.load(open(rfile))}
            row = ref_rows.get(f"3d_{args.size}_r{args.patch}")
            if row:
                ref_gpu = {"ms_per_eval": row["ms_per_eval"],
                           "evals_per_s": 1e3 / row["ms_per_eval"], "storage": "f32",
                           "lc2": row["lc2"],
                           "source": "from profiles/reference_gpu_kernels.json, not measured in "
                                     "this run (one plain evaluation of the reference's kernels "
                                     "by oracle/ref_golden/ref_gpu_time.py, CUDA events, same "
                                     "GPU type)"}
        except Exception:
            ref_gpu = None
    traffic = None
    ipv = None  # thread instructions per output voxel of the fused kernel (ncu)
    captured = None
    # the moments kernel of the tuned launch: 24-row tiles run k_fused_pt,
    # 8- and 16-row tiles k_fused_ps (presampled 3D form, radius <= 4)
    kname = "k_fused_pt" if tuned[0] == 24 else "k_fused_ps"
    tfile = os.path.join(ROOT, "profiles", "k_fused_traffic.json")
    if os.path.exists(tfile) and args.patch <= 4:
        try:
            tj = json.load(open(tfile))["kernels"][kname]
            # DRAM bytes of the moments pass over the step's launches: it reads
            # each transform's presampled image, so it scales with K
            traffic = int(tj["dram_bytes_per_transform"] * K)
            ipv = tj.get("thread_instructions_per_voxel")
            captured = tj.get("captured_at")
        except Exception:
            traffic = None
    from_profile = (f"from profiles/k_fused_traffic.json (ncu capture of {kname}"
                    + (f", {captured})" if captured else ")"))

    # ---- e2e through the public call, host buffers ----
    e2e_t = 0.0
    for s in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = ctx.evaluate_batch(mats)
        e2e_t += time.perf_counter() - t0
    e2e = replica_rate(K * args.steps, e2e_t, dist, f"cuda:{local}")
    assert np.array_equal(out, res), "batched results changed between runs"

    # ---- plain form: one evaluation per call ----
    P = min(args.plain_evals, K)
    for m in mats[:2]:
        ctx.evaluate(m)
    t0 = time.perf_counter()
    plain_vals = [ctx.evaluate(m) for m in mats[:P]]
    plain_t = time.perf_counter() - t0
    plain_eps = P / plain_t
    assert np.array_equal(np.array(plain_vals), res[:P]), "plain != batched"

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O

        O.build()
        eps, n, el, ovals = cpu_port(case, mats, args.cpu_seconds, args.storage)
        cpu = {"value": eps, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} full {args.size}^3 evaluations of the FP64 oracle over "
                         f"{el:.1f} s (OpenMP, all host cores); the reference has no CPU LC2 path"}
        parity = parity_vs_oracle(res, ovals)
        parity["note"] = (f"the first {len(ovals)} of the step's {K} transforms, GPU batch values "
                          f"vs the FP64 oracle on the same {args.storage}-rounded volumes")

    small = None
    if rank == 0 and not args.no_small:
        small = small_configs(local)
    bf16 = None
    if rank == 0 and not args.no_bf16 and args.storage == "f16":
        bf16 = bf16_leg(args, case, mats, local, flush)
    fixed = None
    if rank == 0 and not args.no_fixed:
        fixed = fixed_leg(args, case, local)
    stack = None
    if rank == 0 and not args.no_stack:
        stack = stack_leg(args, case, local)
    reg = None
    if rank == 0 and not args.no_register:
        reg = registration_leg(args, local)
    mi = None
    if rank == 0 and not args.no_mi:
        mi = mi_leg(args, case, local)
    serve = None
    if rank == 0 and not args.no_serve:
        serve = serve_sweep(args, case, local)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64", "data": "synthetic",
            "config": dict(config_dict(args, case), autotuned={"tile_rows": tuned[0],
                                                                  "zchunk": tuned[1]}),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": from_profile,
                         "kernel": f"{kname} (moments pass"
                                   + ("; the rows 24-row tiles leave over run on k_fused_ps"
                                      if kname == "k_fused_pt" else "")
                                   + "; the resample pass is kernels_ms_per_step.warp)",
                         "launches_per_step": mom_launches,
                         "kernel_ms_per_launch": mom_ms / max(1, mom_launches),
                         "scope": "achieved and traffic are totals of the step's moments launches",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
            "issue_roofline": issue_roofline(ipv, K * n_vox, mom_ms, local, clk, from_profile),
            "kernels_ms_per_step": {k: v[0] for k, v in kt.items()},
            "cpu_baseline": cpu,
            "parity": parity,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": K * 96,
                    "d2h_bytes_per_step": K * 8},
            "plain": {"value": plain_eps, "unit": UNIT, "evals": P,
                      "batched_over_plain": value / world / plain_eps},
            "reference_gpu_kernels": ref_gpu,
            "small_configs": small,
            "bf16_storage": bf16,
            "fixed_modality": fixed,
            "stack": stack,
            "mutual_information": mi,
            "registration": reg,
            "serve": serve,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "lc2_true_transform": float(ctx.evaluate(case.true_mat)),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
