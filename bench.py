#!/usr/bin/env python
"""Benchmark of the ICP registration hot path on GB300.

Workload (default): one 640x480 frame pair of the seeded planes+spheres
scene (fx = fy = 525, depth 0.5-4 m, sigma = 0.0012 z^2 noise, 5 % invalid
pixels, source offset by a random rigid motion up to 5 deg / 5 cm),
point-to-plane ICP with 10 Gauss-Newton iterations, distance threshold
0.1 m, normal-angle threshold 20 deg.  A step is one registration of that
pair (10 iterations + the final information matrix).

Metric: Gauss-Newton iterations per second (whole job, all ranks).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Secondary workloads (rank 0, N = 1, reported under "secondary"; skip with
--no-secondary):
  multiscale_hybrid_640x480  3 levels 640x480/320x240/160x120, iterations
      [10, 5, 3], geometric 1.0 + greyscale feature 0.1, one pair,
      MultiscaleRegistration and the one-pair batch kernel;
  loss_grad_32x640x480       PointToPlaneLoss forward + backward on 32 pairs
      at the poses of 5 Gauss-Newton iterations;
  batch_uneven_256           256 pairs with sizes drawn from 160x120 ...
      1280x720, 3 levels [10, 5, 3]: BatchRegistration (autotuned tile) vs
      the plain path (MultiscaleRegistration pair by pair, CUDA graph per
      level);
  feature_1080p_16ch_bf16    16 pairs 1920x1080, 16 BF16 feature channels,
      4 levels [10, 8, 5, 3], weights geometric 10 / feature 1 (the
      reference preset), BatchRegistration vs the plain path;
  bilateral_depth_filter     the depth bilateral filter on uint16 depth,
      640x480 and 1920x1080, widths 6 and 13;
  plain_kernels_larger_images  the plain path's association and reduction
      kernels at 1920x1080 and 3840x2160 (fraction of measured HBM);
  autograd_layer             ExpRtToMatrix forward + backward (1 M twists),
      the frame point-cloud matcher forward + backward (640x480, 3
      channels), one AutogradICP registration (320x240).

Under torchrun each rank registers its own pair (seeded by rank), no
collective touches the data path (weak scaling); a barrier and a max over
ranks bracket the timed region.
"""
import argparse
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "fusion-toolbox_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = ("ICP GN iters/s @640×480 (HBM % roofline); batched vs plain pairs/s "
          "at ≤1e-5 err")
UNIT = "GN iters/s"
ITERS = 10
DIST = 0.1
ANGLE = math.radians(20.0)
W, H = 640, 480
WORKLOAD = ("plain geometric point-to-plane ICP, 1 frame pair 640x480 per rank, "
            "10 GN iterations, d=0.1 m, 20 deg")
# Algorithmic bytes per pixel of the level per launch (packed element sizes):
# association = source xyz + normal + mask (25) + gathered target xyz +
# normal + mask (25) + correspondence-map init and update (16);
# reduction = source xyz + mask (13) + map (8) + target xyz + normal (24).
# The single-launch registration kernel runs ITERS associations and
# reductions, then the association at the final pose and the information
# pass (the map 8 + matched target xyz 12).
ALG_BYTES = {"association": 66, "reduction+solve": 45,
             "registration": ITERS * (66 + 45) + 66 + 20}
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--secondary-out", default=None,
                    help="write the full secondary results (JSON) to this file; the JSON "
                         "line carries their summary")
    ap.add_argument("--profile-case", choices=["batch", "loss", "feature"], default=None,
                    help="run only a small case of one secondary workload (for ncu captures)")
    ap.add_argument("--pairs", type=int, default=8, help="pairs of the --profile-case")
    ap.add_argument("--schedule", type=int, default=0,
                    help="batch schedule of the --profile-case (BatchRegistration.tile_config: "
                         "0..5 lock-step, 100 + g grouped with g groups)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, world, device=None):
    """The slowest rank's value (the timed region is bracketed by a barrier;
    the job's time is the maximum over ranks)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        peaks = json.loads(path.read_text())
        return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_inputs(seed, device):
    """The workload's frame pair prepared on the device by the product's
    own kernels (depth -> points, erosion, central-difference normals)."""
    import torch
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    p = synthetic.make_pair(seed, width=W, height=H)
    k = KCamera(p["kcam"])
    src = FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), device)
    tgt = FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), device)
    x = dict(kcam=torch.from_numpy(p["kcam"]).to(device),
             sp=src.points.reshape(-1, 3).contiguous(),
             sn=src.normals.reshape(-1, 3).contiguous(),
             sm=src.mask.reshape(-1).contiguous(),
             tp=tgt.points.contiguous(), tn=tgt.normals.contiguous(),
             tm=tgt.mask.contiguous())
    torch.cuda.synchronize(device)
    return x, p


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def mark(self, which):
        setattr(self, which, time.time())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        for line in out.strip().splitlines():
            cols = [c.strip() for c in line.split(",")]
            if len(cols) < 9:
                continue
            try:
                sm.append(float(cols[1]))
                smax.append(float(cols[2]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, cols[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def run_config():
    """The workload's config, the same on the GPU and reference arms."""
    return {"workload": WORKLOAD,
            "l2": "GPU arm: flushed (512 MB write) before every step; the pair (~18 MB) "
                  "stays L2-resident across its 10 iterations",
            "launch": "GPU arm: one cooperative kernel per registration (grid barriers "
                      "between its phases); reference arm: the CPU path on the host cores"}


def run_reference(args, rank, world):
    """CPU arm: the C/OpenMP restatement of the reference's CPU ICP path on
    the host cores, on the same workload; rank 0 only."""
    if rank != 0:
        return
    import numpy as np
    from oracle import frame_prep as fp
    from oracle import port
    from slamtb_gb300 import synthetic
    p = synthetic.make_pair(args.seed, width=W, height=H)
    src = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"])
    tgt = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"])
    threads = len(os.sched_getaffinity(0))

    def reg(iters):
        return port.icp_estimate(p["kcam"], src.points, src.normals, src.mask, tgt.points,
                                 tgt.normals, tgt.mask, num_iters=iters, geom_weight=1.0,
                                 feat_weight=0.0, distance_threshold=DIST,
                                 normals_angle_thresh=ANGLE, threads=threads)
    t = time.perf_counter()
    reg(ITERS)
    t_reg = time.perf_counter() - t
    # a step is one registration unless K of them would exceed ~2 minutes;
    # then a step is one Gauss-Newton iteration of it
    iters = ITERS if t_reg * (args.steps + args.warmup) < 120.0 else 1
    for _ in range(args.warmup):
        reg(iters)
    t = time.perf_counter()
    for _ in range(args.steps):
        reg(iters)
    total = time.perf_counter() - t
    value = args.steps * iters / total
    sample = (f"{args.steps} steps of {iters} Gauss-Newton iteration(s) of the 640x480 pair "
              f"(C/OpenMP restatement of the reference CPU path, {threads} threads)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": run_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


def cpu_baseline(x_host):
    """The C/OpenMP port on a bounded sample (~10 s) of the workload."""
    from oracle import frame_prep as fp
    from oracle import port
    p = x_host
    src = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"])
    tgt = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"])
    threads = len(os.sched_getaffinity(0))
    n = 0
    t = time.perf_counter()
    while True:
        port.icp_estimate(p["kcam"], src.points, src.normals, src.mask, tgt.points,
                          tgt.normals, tgt.mask, num_iters=ITERS, geom_weight=1.0,
                          feat_weight=0.0, distance_threshold=DIST, normals_angle_thresh=ANGLE,
                          threads=threads)
        n += 1
        el = time.perf_counter() - t
        if el > 10.0 or n >= 200:
            break
    return {"value": n * ITERS / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} registrations (10 GN iterations each) of the 640x480 pair, "
                      f"{el:.1f} s, C/OpenMP restatement of the reference CPU path"}

# ---------------------------------------------------------------------------
# secondary workloads
# ---------------------------------------------------------------------------

def device_pair(seed, w, h, device, feature_channels=None, feat_dtype=None, **kw):
    """A seeded pair rendered on the device and prepared by the product's
    kernels: (source FramePointCloud, target FramePointCloud, source feats,
    target feats, ground truth)."""
    import torch
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    p = synthetic.make_pair(seed, width=w, height=h, feature_channels=feature_channels,
                            device=device, **kw)
    k = KCamera(p["kcam"])
    src = FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), device)
    tgt = FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), device)
    src.normals, tgt.normals  # computed now, outside any timed region
    sf = tf = None
    if feature_channels is not None:
        dt = feat_dtype or torch.float32
        sf = torch.from_numpy(p["source_feats"]).to(device=device, dtype=dt)
        tf = torch.from_numpy(p["target_feats"]).to(device=device, dtype=dt)
    return src, tgt, sf, tf, p["gt"]


def _estimators(iters, scales, wg, wf):
    from slamtb_gb300.registration.icp import ICPOdometry
    return [(s, ICPOdometry(n, geom_weight=wg, feat_weight=wf, distance_threshold=DIST,
                            normals_angle_thresh=ANGLE, use_graph=True))
            for s, n in zip(scales, iters)]


def _pyramids(pairs, scales):
    from slamtb_gb300.processing import feature_pyramid
    out = []
    for src, tgt, sf, tf, _ in pairs:
        out.append((src.pyramid(scales), tgt.pyramid(scales),
                    None if sf is None else feature_pyramid(sf, scales),
                    None if tf is None else feature_pyramid(tf, scales)))
    return out


def _rel_pose(a, b):
    """||log(b^-1 a)|| over max(||log b||, 1e-3), by the rotation angle and
    translation of b^-1 a (no oracle involved)."""
    import numpy as np
    D = np.linalg.inv(b) @ a
    ang = math.acos(min(1.0, max(-1.0, (np.trace(D[:3, :3]) - 1.0) / 2.0)))
    Bb = b
    angb = math.acos(min(1.0, max(-1.0, (np.trace(Bb[:3, :3]) - 1.0) / 2.0)))
    return math.hypot(ang, np.linalg.norm(D[:3, 3])) / max(
        math.hypot(angb, np.linalg.norm(Bb[:3, 3])), 1e-3)


def _oracle_worker(job):
    """One pair's free-running FP64 oracle registration (run in a spawned
    process: numpy only).  job = (levels coarsest first, estimator keyword
    dicts finest first, channel mode).  Returns (final transform or None,
    condition number of the last successful step's J^T J)."""
    import numpy as np
    from oracle import icp_oracle as io
    levels, ests, mode = job
    res = io.multiscale_estimate(levels, [dict(e, channel_mode=mode) for e in ests])
    cond = float(np.linalg.cond(res.JtJ)) if res.JtJ is not None else None
    return (None if res.transform is None else np.asarray(res.transform)), cond


def _oracle_jobs(pyrs, iters, wg, wf, mode):
    """Host copies of device pyramids as oracle jobs (features as float32,
    what the oracle reads of BF16 maps)."""
    import torch
    jobs = []
    for spyr, tpyr, sfp, tfp in pyrs:
        levels = []
        for lv in range(len(spyr)):
            s, t = spyr[lv], tpyr[lv]
            d = dict(kcam=s.kcam.matrix.cpu().numpy() if torch.is_tensor(s.kcam.matrix)
                     else s.kcam.matrix,
                     src_points=s.points.cpu().numpy(), src_normals=s.normals.cpu().numpy(),
                     src_mask=s.mask.cpu().numpy(), tgt_points=t.points.cpu().numpy(),
                     tgt_normals=t.normals.cpu().numpy(), tgt_mask=t.mask.cpu().numpy())
            if sfp is not None and wf > 0:
                d["src_feats"] = sfp[lv].float().cpu().numpy().reshape(sfp[lv].size(0), -1)
                d["tgt_feats"] = tfp[lv].float().cpu().numpy()
            levels.append(d)
        ests = [dict(num_iters=n, geom_weight=wg, feat_weight=wf, distance_threshold=DIST,
                     normals_angle_thresh=ANGLE) for n in iters]
        jobs.append((levels, ests, mode))
    return jobs


def _oracle_runs(jobs, workers):
    """The FP64 oracle's free-running registration of every job, in spawned
    processes: [(final transform or None, cond(J^T J))]."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(workers) as pool:
        return list(pool.imap(_oracle_worker, jobs, chunksize=1))


def _error_table(transforms, outs):
    """Each pair's free-running final-pose error against the FP64 oracle's
    registration from the same start (||log(T_o^-1 T)|| over
    max(||log T_o||, 1e-3)), with the fractions within 1e-5 and 1e-3 and the
    three worst pairs with the condition number of their final J^T J.
    ``transforms``: 4x4 arrays or tensors (None for a failed pair), pair k
    against outs[k]."""
    import numpy as np
    errs = []
    for k, (T, (To, cond)) in enumerate(zip(transforms, outs)):
        if T is None or To is None:
            errs.append((k, None if (T is None) == (To is None) else math.inf, cond))
            continue
        errs.append((k, _rel_pose(np.asarray(T, dtype=np.float64), To), cond))
    vals = [e for _, e, _ in errs if e is not None]
    worst = sorted([x for x in errs if x[1] is not None], key=lambda x: -x[1])[:3]
    return {"pairs": len(errs), "both_failed": sum(1 for _, e, _ in errs if e is None),
            "max": max(vals) if vals else None,
            "median": statistics.median(vals) if vals else None,
            "within_1e-5": sum(1 for v in vals if v <= 1e-5) / max(len(vals), 1),
            "within_1e-3": sum(1 for v in vals if v <= 1e-3) / max(len(vals), 1),
            "worst": [{"pair": k, "err": e, "cond_JtJ": c} for k, e, c in worst],
            # every pair's error (None: both failed; inf: one of them failed)
            "per_pair": [None if e is None else float(f"{e:.3g}") for _, e, _ in errs]}


def _reference_arithmetic(jobs, outs, max_pairs):
    """The reference CPU path's own free-running accuracy on the first
    ``max_pairs`` jobs: the C/OpenMP port (float32 per-point partials in the
    reference's operation order, FP64 sums and solve) registers each pair
    from the same start, and its final pose is compared with the FP64
    oracle's as the GPU results are.  This is the floor a drop-in that
    reproduces the reference's float32 arithmetic starts from."""
    from oracle import port
    t0 = time.perf_counter()
    Ts = []
    for levels, ests, mode in jobs[:max_pairs]:
        r = port.multiscale_estimate(levels, [dict(e, channel_mode=mode) for e in ests])
        Ts.append(r["transform"])
    table = _error_table(Ts, outs[:max_pairs])
    table["wall_s"] = time.perf_counter() - t0
    table["threads"] = port.max_threads()
    return table


def _oracle_errors(results, jobs, workers):
    """_error_table of registration results (objects with .transform)
    against a fresh FP64 oracle run of the jobs."""
    return _error_table([r.transform for r in results], _oracle_runs(jobs, workers))


def _alg_bytes_batch(pyrs, iters, feat_bytes=0):
    """Algorithmic bytes of one batch run: per level and iteration, the
    association reads 66 B per source pixel and the reduction 45 B (+ the
    source and target feature bytes per pixel) per target pixel; the final
    information pass 66 + 33 B per finest pixel."""
    total = 0
    for spyr, tpyr, _, _ in pyrs:
        for lv, n in zip(range(len(spyr)), iters[::-1]):
            npx = spyr[lv].mask.numel()
            total += n * npx * (ALG_BYTES["association"] + ALG_BYTES["reduction+solve"]
                                + 2 * feat_bytes)
        total += spyr[-1].mask.numel() * (ALG_BYTES["association"] + 33)
    return total


def _time_plain(ms, pyrs, reps):
    """Plain path: MultiscaleRegistration.estimate_pyramid pair by pair (one
    CUDA graph per level, the result read back per level as the reference
    API returns it).  Returns (seconds per pass, transforms)."""
    import torch
    for spyr, tpyr, sfp, tfp in pyrs[:min(len(pyrs), 8)]:
        ms.estimate_pyramid(spyr, tpyr, sfp, tfp)
    torch.cuda.synchronize()
    best, Ts = None, None
    for _ in range(reps):
        t = time.perf_counter()
        Ts = [ms.estimate_pyramid(spyr, tpyr, sfp, tfp).transform for spyr, tpyr, sfp, tfp in pyrs]
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        best = el if best is None else min(best, el)
    return best, Ts


def _time_batch(br, plan, reps, device):
    """Seconds per BatchRegistration.run (CUDA graph replay), best of reps
    CUDA-event timings, as _time_plain takes the best of its passes."""
    import torch
    stream = torch.cuda.current_stream(device)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    for a, b in ev:
        a.record(stream)
        br.run(plan, graph=True)
        b.record(stream)
    torch.cuda.synchronize(device)
    ms = [a.elapsed_time(b) for a, b in ev]
    return min(ms) / 1e3


def _compare(batch_res, plain_T):
    """(max, median) relative pose difference between the batched and the
    plain registration of the same pairs (free-running loops: float32 sums
    in different orders drift apart where a pair's normal equations are
    ill-conditioned)."""
    diffs = [_rel_pose(r.transform.numpy(), T.numpy()) for r, T in zip(batch_res, plain_T)
             if r.transform is not None and T is not None]
    return (max(diffs), statistics.median(diffs)) if diffs else (None, None)


def _batch_vs_plain(name, pairs, iters, scales, wg, wf, device, reps_batch, reps_plain,
                    feat_bytes=0, mode="last", oracle_workers=0, reference_pairs=0):
    from slamtb_gb300.registration import BatchRegistration, MultiscaleRegistration
    ests = _estimators(iters, scales, wg, wf)
    pyrs = _pyramids(pairs, scales)
    feats = pyrs[0][2] is not None
    br = BatchRegistration(ests, feat_channel_mode=mode)
    plan = br.prepare([p[0] for p in pyrs], [p[1] for p in pyrs],
                      [p[2] for p in pyrs] if feats else None,
                      [p[3] for p in pyrs] if feats else None)
    tune = br.autotune(plan)
    t_batch = _time_batch(br, plan, reps_batch, device)
    res = br.results(plan)
    for _, est in ests:
        est.feat_channel_mode = mode
    t_plain, plain_T = _time_plain(MultiscaleRegistration(ests), pyrs, reps_plain)
    B = len(pairs)
    alg = _alg_bytes_batch(pyrs, iters, feat_bytes)
    peak, kind = measured_peak()
    gt_err = [_rel_pose(r.transform.numpy(), p[4]) if r.transform is not None else None
              for r, p in zip(res, pairs)]
    vs_oracle = plain_vs_oracle = ref_vs_oracle = None
    if oracle_workers:
        t0 = time.perf_counter()
        jobs = _oracle_jobs(pyrs, iters, wg, wf, mode)
        outs = _oracle_runs(jobs, oracle_workers)
        vs_oracle = _error_table([r.transform for r in res], outs)
        vs_oracle["wall_s"] = time.perf_counter() - t0
        plain_vs_oracle = _error_table(plain_T, outs)
        if reference_pairs:
            ref_vs_oracle = _reference_arithmetic(jobs, outs, reference_pairs)
    return {
        "workload": name, "pairs": B, "iters": iters, "scales": scales,
        "weights": {"geometric": wg, "feature": wf},
        "batch": {"pairs_per_s": B / t_batch, "ms_per_run": t_batch * 1e3,
                  "tile_config": br.tile_config,
                  "autotune_ms": {str(k): v for k, v in tune.items()},
                  "launches_per_run": 3},
        "plain": {"pairs_per_s": B / t_plain, "ms_per_pass": t_plain * 1e3,
                  "path": "MultiscaleRegistration.estimate_pyramid pair by pair"},
        "speedup_batch_vs_plain": t_plain / t_batch,
        "rel_pose_diff_batch_vs_plain": dict(zip(("max", "median"), _compare(res, plain_T))),
        "batch_vs_fp64_oracle": vs_oracle,
        "plain_vs_fp64_oracle": plain_vs_oracle,
        "reference_cpu_arithmetic_vs_fp64_oracle": ref_vs_oracle,
        "median_rel_pose_err_vs_ground_truth": statistics.median(
            [e for e in gt_err if e is not None]) if any(e is not None for e in gt_err) else None,
        "roofline": {"bound": "hbm", "kernel": "k_batch (whole run)",
                     "alg_bytes_per_run": alg, "achieved": alg / t_batch / 1e9,
                     "peak": peak, "peak_source": kind, "unit": "GB/s",
                     "frac": alg / t_batch / 1e9 / peak},
    }


def oracle_workers():
    """Processes of the FP64 oracle's accuracy runs (the host's cores, at
    most 16)."""
    return max(1, min(16, len(os.sched_getaffinity(0))))


def secondary_multiscale(device, seed):
    import torch
    from slamtb_gb300.registration import BatchRegistration, MultiscaleRegistration
    pair = device_pair(seed, 640, 480, device, feature_channels=0)
    iters, scales = [10, 5, 3], [1.0, 0.5, 0.5]
    ests = _estimators(iters, scales, 1.0, 0.1)
    pyrs = _pyramids([pair], scales)
    t_plain, Ts = _time_plain(MultiscaleRegistration(ests), pyrs * 50, 3)
    br = BatchRegistration(ests)
    plan = br.prepare([pyrs[0][0]], [pyrs[0][1]], [pyrs[0][2]], [pyrs[0][3]])
    br.autotune(plan)
    t_b = _time_batch(br, plan, 100, device)
    res = br.results(plan)
    # both paths' free-running results against the FP64 oracle's
    jobs = _oracle_jobs(pyrs, iters, 1.0, 0.1, "last")
    plain_res = MultiscaleRegistration(ests).estimate_pyramid(*pyrs[0])
    outs = _oracle_runs(jobs, 1)
    vs_oracle = {"plain": _error_table([plain_res.transform], outs),
                 "batch": _error_table([res[0].transform], outs),
                 "reference_cpu_arithmetic": _reference_arithmetic(jobs, outs, 1)}
    return {"workload": "multiscale hybrid ICP 640x480/320x240/160x120 [10, 5, 3], "
                        "geometric 1.0 + greyscale feature 0.1, 1 pair",
            "plain": {"registrations_per_s": 50 / t_plain,
                      "gn_iters_per_s": 50 * sum(iters) / t_plain,
                      "path": "MultiscaleRegistration (CUDA graph per level, result read "
                              "back per level)"},
            "batch_kernel_one_pair": {"registrations_per_s": 1.0 / t_b,
                                      "gn_iters_per_s": sum(iters) / t_b,
                                      "tile_config": br.tile_config},
            "max_rel_pose_diff_batch_vs_plain": _rel_pose(res[0].transform.numpy(),
                                                          Ts[0].numpy()),
            "rel_pose_err_vs_ground_truth": _rel_pose(res[0].transform.numpy(), pair[4]),
            "vs_fp64_oracle": vs_oracle}


def secondary_loss(device, seed, B=32):
    import torch
    from slamtb_gb300.registration import BatchRegistration, point_to_plane_loss
    pairs = [device_pair(seed + 100 + k, W, H, device) for k in range(B)]
    ests = _estimators([5], [1.0], 1.0, 0.0)
    br = BatchRegistration(ests)
    res = br.estimate_pyramids([[p[0]] for p in pairs], [[p[1]] for p in pairs])
    poses = torch.stack([r.transform.to(torch.float64) for r in res]).to(device)
    src_depth = torch.stack([p[0].points[..., 2] for p in pairs]).contiguous()
    sn = torch.stack([p[0].normals for p in pairs]).contiguous()
    sm = torch.stack([p[0].mask for p in pairs]).contiguous()
    tp = torch.stack([p[1].points for p in pairs]).contiguous()
    tn = torch.stack([p[1].normals for p in pairs]).contiguous()
    tm = torch.stack([p[1].mask for p in pairs]).contiguous()
    kcam = pairs[0][0].kcam.params()
    twist = torch.zeros(B, 6, dtype=torch.float64, device=device, requires_grad=True)
    depth = src_depth.clone().requires_grad_(True)

    def step():
        twist.grad = None
        depth.grad = None
        loss = point_to_plane_loss(twist, depth, sn, sm, tp, tn, tm, kcam, poses,
                                   DIST, ANGLE)
        loss.sum().backward()
    # the same step with the loss captured once as CUDA graphs (forward and
    # backward, torch.cuda.make_graphed_callables): the same kernels and
    # bytes, without the host's per-step launch and autograd overhead, which
    # otherwise sets the eager step's time
    def loss_fn(tw, z):
        return point_to_plane_loss(tw, z, sn, sm, tp, tn, tm, kcam, poses, DIST, ANGLE)

    graph_error = None
    try:
        graphed = torch.cuda.make_graphed_callables(loss_fn, (twist, depth))
    except Exception as exc:  # reported on the line, the eager timing stands in
        graphed, graph_error = None, f"{type(exc).__name__}: {exc}"

    def gstep():
        twist.grad = None
        depth.grad = None
        graphed(twist, depth).sum().backward()

    stream = torch.cuda.current_stream(device)
    reps = 50

    def timed(fn):
        for _ in range(3):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize(device)
        return a.elapsed_time(b) / 1e3 / reps

    t_eager = timed(step)
    t = timed(gstep) if graphed is not None else t_eager
    npx = B * H * W
    # forward: assoc 50 B/px (depth, normal, masks, target point+normal,
    # key) + key init 8 + the loss with its adjoint at a unit output
    # gradient 36 (key, winner depth, target point + normal) + the depth
    # adjoint's init 4; backward: the depth adjoint scaled, read 4 + write 4
    alg = npx * (50 + 8 + 36 + 4 + 8)
    peak, kind = measured_peak()
    return {"workload": f"point-to-plane loss forward + backward, {B} pairs 640x480 at the "
                        "poses of 5 GN iterations", "pairs": B,
            "pairs_per_s": B / t, "ms_per_step": t * 1e3,
            "path": ("PointToPlaneLoss under torch.cuda.make_graphed_callables (forward and "
                     "backward graphs)" if graphed is not None else
                     f"PointToPlaneLoss, eager (graph capture failed: {graph_error})"),
            "eager": {"pairs_per_s": B / t_eager, "ms_per_step": t_eager * 1e3},
            "launches_per_step": 8,
            "roofline": {"bound": "hbm", "alg_bytes_per_step": alg,
                         "achieved": alg / t / 1e9, "peak": peak, "peak_source": kind,
                         "unit": "GB/s", "frac": alg / t / 1e9 / peak}}


def secondary_batch_uneven(device, seed, B=256):
    import numpy as np
    rng = np.random.default_rng(seed + 7)
    sizes = [(160, 120), (320, 240), (640, 480), (848, 480), (1280, 720)]
    pick = rng.integers(0, len(sizes), size=B)
    pairs = [device_pair(seed + 1000 + k, *sizes[i], device) for k, i in enumerate(pick)]
    out = _batch_vs_plain("batched uneven ICP, 256 pairs from {160x120 ... 1280x720}, "
                          "3 levels [10, 5, 3], geometric", pairs, [10, 5, 3],
                          [1.0, 0.5, 0.5], 1.0, 0.0, device, 10, 2,
                          oracle_workers=oracle_workers(), reference_pairs=B)
    out["size_histogram"] = {f"{w}x{h}": int((pick == i).sum()) for i, (w, h) in enumerate(sizes)}
    return out


def secondary_feature_1080p(device, seed, B=16):
    import torch
    pairs = [device_pair(seed + 2000 + k, 1920, 1080, device, feature_channels=16,
                         feat_dtype=torch.bfloat16, max_rot_deg=10.0, max_trans=0.1)
             for k in range(B)]
    return _batch_vs_plain("high-resolution feature ICP, 16 pairs 1920x1080, 16 BF16 channels, "
                           "4 levels [10, 8, 5, 3]", pairs, [10, 8, 5, 3],
                           [1.0, 0.5, 0.5, 0.5], 10.0, 1.0, device, 5, 1, feat_bytes=32,
                           oracle_workers=oracle_workers(), reference_pairs=4)


def secondary_bilateral(device, seed, reps=200):
    """The depth bilateral filter on 16-bit millimetre depth images: per
    launch time from CUDA events over ``reps`` back-to-back launches (the
    input stays in L2: the kernel is bound by one exponential per tap, not
    by its 5 bytes per pixel), and the float32 oracle on one 640x480 image
    as the CPU side."""
    import numpy as np
    import torch
    from slamtb_gb300 import synthetic
    from slamtb_gb300.processing import BilateralDepthFilter
    out = {"workload": "bilateral depth filter, uint16 depth in mm (ElasticFusion sigmas "
                       "29.99 / 4.5)", "cases": {}}
    host = {}
    for w, h in ((640, 480), (1920, 1080)):
        z = synthetic.make_pair(seed + 3000, width=w, height=h)["source_depth"]
        host[(w, h)] = (z * 1000).astype(np.uint16)
        d = torch.from_numpy(host[(w, h)].astype(np.int32)).to(device).to(torch.uint16)
        m = d.view(torch.int16) != 0
        for width in (6, 13):
            filt = BilateralDepthFilter(filter_width=width)
            for _ in range(5):
                filt(d, m)
            st = torch.cuda.current_stream(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(device)
            e0.record(st)
            for _ in range(reps):
                filt(d, m)
            e1.record(st)
            torch.cuda.synchronize(device)
            s = e0.elapsed_time(e1) * 1e-3 / reps
            taps = (2 * (width // 2) + 1) ** 2
            out["cases"][f"{w}x{h}_width{width}"] = {
                "us_per_image": s * 1e6, "mpix_per_s": w * h / s / 1e6,
                "gtaps_per_s": w * h * taps / s / 1e9, "taps_per_pixel": taps}
    from oracle import frame_prep as fp
    z = host[(640, 480)].astype(np.int32)
    t = time.perf_counter()
    fp.bilateral_depth_filter(z, z > 0, 6)
    el = time.perf_counter() - t
    out["cpu_baseline"] = {"us_per_image": el * 1e6, "mpix_per_s": 640 * 480 / el / 1e6,
                           "cores": 1, "kind": "port",
                           "sample": "one 640x480 image, width 6, numpy float32 oracle"}
    return out


def secondary_plain_sizes(device, seed, reps=20):
    """The plain path at larger images (one pair, 10 iterations,
    geometric): the single-launch registration's time and fraction of the
    measured HBM bandwidth, and, for the multi-launch sequence, per-launch
    CUDA-event times of the association and of the reduction with its step
    (the profiled graph replay) with their fractions.  At 640x480 an
    iteration is a latency chain; these show how the kernels do when there
    are bytes enough to stream."""
    import torch
    from slamtb_gb300 import _native as N
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    from slamtb_gb300.registration.icp import ICPOdometry
    peak, kind = measured_peak()
    out = {"peak_gbs": peak, "peak_source": kind}
    for w, h in ((1920, 1080), (3840, 2160)):
        p = synthetic.make_pair(seed + 6000, width=w, height=h)
        k = KCamera(p["kcam"])
        src = FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), device)
        tgt = FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), device)
        kc = torch.from_numpy(p["kcam"]).to(device)
        args_ = (kc, src.points.reshape(-1, 3), src.normals.reshape(-1, 3), src.mask.reshape(-1))
        kw = dict(target_points=tgt.points, target_mask=tgt.mask, target_normals=tgt.normals)
        case = {}
        for launch in ("single", "multi"):
            icp = ICPOdometry(ITERS, geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
                              normals_angle_thresh=ANGLE, launch=launch)
            for _ in range(3):
                icp.launch(*args_, **kw)
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            for _ in range(reps):
                icp.launch(*args_, **kw)
            torch.cuda.synchronize(device)
            reg_ms = (time.perf_counter() - t0) * 1e3 / reps
            N.profile_enable(True)
            prof = {kk: [0.0, 0] for kk in N.PROFILE_KINDS}
            for _ in range(reps):
                icp.launch(*args_, **kw)
                torch.cuda.synchronize(device)
                for kk, (ms, cnt) in N.profile_read().items():
                    prof[kk][0] += ms
                    prof[kk][1] += cnt
            N.profile_enable(False)
            c = {"registration_ms": reg_ms, "gn_iters_per_s": ITERS / (reg_ms * 1e-3)}
            kinds = ("registration",) if launch == "single" else ("association",
                                                                  "reduction+solve")
            for kk in kinds:
                us = prof[kk][0] / max(prof[kk][1], 1) * 1e3
                gbs = ALG_BYTES[kk] * w * h / (us * 1e-6) / 1e9
                c[kk] = {"us_per_launch": us, "achieved_gbs": gbs, "frac": gbs / peak}
            case[launch] = c
        out[f"{w}x{h}"] = case
    return out


def secondary_autograd(device, seed, reps=50):
    """The differentiable registration layer: ExpRtToMatrix forward +
    backward on 1 M twists, the frame point-cloud matcher forward + backward
    on a 640x480 pair (3 feature channels; the forward includes its
    correspondence map), and one AutogradICP registration (depth only, 20
    BFGS iterations and 100 SGD steps, 320x240).  CUDA events for the
    kernels, wall clock for the optimiser (host-driven, as the
    reference's)."""
    import numpy as np
    import torch
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    from slamtb_gb300.registration import AutogradICP, ExpRtToMatrix
    from slamtb_gb300.spatial import FPCLMatcherOp
    st = torch.cuda.current_stream(device)

    def ev_time(fn, n):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        e0.record(st)
        for _ in range(n):
            fn()
        e1.record(st)
        torch.cuda.synchronize(device)
        return e0.elapsed_time(e1) * 1e-3 / n

    rng = np.random.default_rng(seed)
    x = torch.from_numpy(rng.normal(size=(1 << 20, 6)).astype(np.float32) * 0.3).to(device)
    x.requires_grad_(True)
    g = torch.randn(1 << 20, 3, 4, device=device)

    def exp_fb():
        ExpRtToMatrix.apply(x).backward(g)
    t_exp = ev_time(exp_fb, reps)
    p = synthetic.make_pair(seed + 5000, width=W, height=H, feature_channels=3)
    k = KCamera(p["kcam"])
    src = FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), device)
    tgt = FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), device)
    gt = torch.from_numpy(p["gt"]).float().to(device)
    m = src.mask.reshape(-1)
    sp = (src.points.reshape(-1, 3)[m] @ gt[:3, :3].T + gt[:3, 3]).contiguous()
    sn = (src.normals.reshape(-1, 3)[m] @ gt[:3, :3].T).contiguous()
    target = FPCLMatcherOp.Target(tgt.points, tgt.normals, tgt.mask,
                                  torch.from_numpy(p["target_feats"]).to(device), k, DIST,
                                  math.radians(30))
    spg = sp.clone().requires_grad_(True)
    dl = torch.randn(3, sp.size(0), device=device)

    def match_fb():
        FPCLMatcherOp.apply(spg, sn, target, FPCLMatcherOp.Match()).backward(dl)
    t_match = ev_time(match_fb, reps)
    p2 = synthetic.make_pair(seed + 5001, width=320, height=240, max_rot_deg=2.0,
                             max_trans=0.02)
    k2 = KCamera(p2["kcam"])
    s2 = FramePointCloud.from_frame(Frame(FrameInfo(k2), p2["source_depth"]), device)
    t2 = FramePointCloud.from_frame(Frame(FrameInfo(k2), p2["target_depth"]), device)
    icp = AutogradICP(20, geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
                      normals_angle_thresh=math.radians(30))
    args2 = (k2, s2.points.reshape(-1, 3), s2.normals.reshape(-1, 3), s2.mask.reshape(-1))
    kw2 = dict(target_points=t2.points, target_mask=t2.mask, target_normals=t2.normals)
    icp.estimate(*args2, **kw2)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    res = icp.estimate(*args2, **kw2)
    t_agicp = time.perf_counter() - t0
    return {"workload": "differentiable registration layer (AutogradICP)",
            "exp_rt_to_matrix_fwd_bwd": {"twists": 1 << 20, "us": t_exp * 1e6,
                                         "mtwists_per_s": (1 << 20) / t_exp / 1e6},
            "fpcl_matcher_fwd_bwd_640x480": {"points": int(sp.size(0)), "channels": 3,
                                            "us": t_match * 1e6,
                                            "mpoints_per_s": sp.size(0) / t_match / 1e6},
            "autograd_icp_320x240": {"seconds": t_agicp, "bfgs_iters": 20, "sgd_steps": 100,
                                     "rel_pose_err_vs_ground_truth": _rel_pose(
                                         res.transform.numpy(), p2["gt"])}}


def profile_case(args, device):
    """A small case of one secondary workload, --steps runs after --warmup,
    for profiler captures (prints one JSON line; not a bench result)."""
    import numpy as np
    import torch
    from slamtb_gb300.registration import BatchRegistration, point_to_plane_loss
    B = args.pairs
    if args.profile_case in ("batch", "feature"):
        if args.profile_case == "batch":
            rng = np.random.default_rng(args.seed + 7)
            sizes = [(160, 120), (320, 240), (640, 480), (848, 480), (1280, 720)]
            pairs = [device_pair(args.seed + 1000 + k, *sizes[i], device)
                     for k, i in enumerate(rng.integers(0, len(sizes), size=B))]
            iters, scales, wg, wf, feats = [10, 5, 3], [1.0, 0.5, 0.5], 1.0, 0.0, False
        else:
            pairs = [device_pair(args.seed + 2000 + k, 1920, 1080, device, feature_channels=16,
                                 feat_dtype=torch.bfloat16, max_rot_deg=10.0, max_trans=0.1)
                     for k in range(B)]
            iters, scales, wg, wf, feats = [10, 8, 5, 3], [1.0, 0.5, 0.5, 0.5], 10.0, 1.0, True
        pyrs = _pyramids(pairs, scales)
        br = BatchRegistration(_estimators(iters, scales, wg, wf))
        br.tile_config = args.schedule
        plan = br.prepare([p[0] for p in pyrs], [p[1] for p in pyrs],
                          [p[2] for p in pyrs] if feats else None,
                          [p[3] for p in pyrs] if feats else None)
        run = lambda: br.run(plan)  # noqa: E731
    else:
        pairs = [device_pair(args.seed + 100 + k, W, H, device) for k in range(B)]
        br = BatchRegistration(_estimators([5], [1.0], 1.0, 0.0))
        res = br.estimate_pyramids([[p[0]] for p in pairs], [[p[1]] for p in pairs])
        poses = torch.stack([r.transform.to(torch.float64) for r in res]).to(device)
        st = lambda f: torch.stack([f(p) for p in pairs]).contiguous()  # noqa: E731
        depth = st(lambda p: p[0].points[..., 2]).requires_grad_(True)
        sn, sm = st(lambda p: p[0].normals), st(lambda p: p[0].mask)
        tp, tn, tm = st(lambda p: p[1].points), st(lambda p: p[1].normals), st(lambda p: p[1].mask)
        twist = torch.zeros(B, 6, dtype=torch.float64, device=device, requires_grad=True)
        kcam = pairs[0][0].kcam.params()

        def run():
            loss = point_to_plane_loss(twist, depth, sn, sm, tp, tn, tm, kcam, poses, DIST, ANGLE)
            loss.sum().backward()
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize(device)
    t = time.perf_counter()
    for _ in range(args.steps):
        run()
    torch.cuda.synchronize(device)
    print(json.dumps({"profile_case": args.profile_case, "pairs": B, "steps": args.steps,
                      "ms_per_step": 1e3 * (time.perf_counter() - t) / args.steps}))


def _r(x, nd=4):
    """x rounded to nd significant digits (None stays None)."""
    if x is None or isinstance(x, (str, bool)):
        return x
    if isinstance(x, int):
        return x
    return float(f"{x:.{nd}g}")


def summarize(sec):
    """The compact per-workload summary carried on the JSON line: rates,
    speed-ups, roofline fractions and accuracy against the FP64 oracle."""
    out = {}
    for name, d in sec.items():
        if "error" in d:
            out[name] = {"error": d["error"]}
            continue
        if name == "multiscale_hybrid_640x480":
            vo = d.get("vs_fp64_oracle") or {}
            out[name] = {"plain_regs_per_s": _r(d["plain"]["registrations_per_s"]),
                         "batch_regs_per_s": _r(d["batch_kernel_one_pair"]["registrations_per_s"]),
                         "err_vs_fp64_oracle": {k: _r(v["max"]) for k, v in vo.items()},
                         "err_vs_ground_truth": _r(d["rel_pose_err_vs_ground_truth"])}
        elif name in ("batch_uneven_256", "feature_1080p_16ch_bf16"):
            vo = d.get("batch_vs_fp64_oracle") or {}
            out[name] = {"pairs": d["pairs"],
                         "batch_pairs_per_s": _r(d["batch"]["pairs_per_s"]),
                         "plain_pairs_per_s": _r(d["plain"]["pairs_per_s"]),
                         "speedup": _r(d["speedup_batch_vs_plain"]),
                         "frac": _r(d["roofline"]["frac"]),
                         "batch_vs_plain": {k: _r(v) for k, v in
                                            d["rel_pose_diff_batch_vs_plain"].items()},
                         "vs_fp64_oracle": {
                             "pairs": vo.get("pairs"), "max": _r(vo.get("max")),
                             "median": _r(vo.get("median")),
                             "within_1e-5": _r(vo.get("within_1e-5")),
                             "within_1e-3": _r(vo.get("within_1e-3")),
                             "worst": [{k: _r(v) for k, v in w.items()}
                                       for w in vo.get("worst", [])]} if vo else None}
            # the same table, max / median / within 1e-5, for the plain path
            # and for the reference CPU path's arithmetic (the port)
            for key, src in (("plain_vs_fp64_oracle", "plain_vs_fp64_oracle"),
                             ("reference_arith_vs_fp64_oracle",
                              "reference_cpu_arithmetic_vs_fp64_oracle")):
                t = d.get(src)
                out[name][key] = {"pairs": t["pairs"], "max": _r(t["max"]),
                                  "median": _r(t["median"]),
                                  "within_1e-5": _r(t["within_1e-5"])} if t else None
        elif name == "loss_grad_32x640x480":
            out[name] = {"pairs_per_s": _r(d["pairs_per_s"]), "frac": _r(d["roofline"]["frac"]),
                         "eager_pairs_per_s": _r(d["eager"]["pairs_per_s"])}
        elif name == "plain_kernels_larger_images":
            out[name] = {size: {launch: {"gn_iters_per_s": _r(c["gn_iters_per_s"]),
                                         **{k: _r(v["frac"]) for k, v in c.items()
                                            if isinstance(v, dict)}}
                                for launch, c in case.items()}
                         for size, case in d.items() if "x" in size}
        elif name == "bilateral_depth_filter":
            out[name] = {k: _r(v["us_per_image"]) for k, v in d["cases"].items()}
        elif name == "autograd_layer":
            out[name] = {"exp_rt_mtwists_per_s": _r(d["exp_rt_to_matrix_fwd_bwd"]["mtwists_per_s"]),
                         "matcher_mpoints_per_s":
                             _r(d["fpcl_matcher_fwd_bwd_640x480"]["mpoints_per_s"])}
    return out


def run_secondary(device, seed):
    out = {}
    for name, fn in (("multiscale_hybrid_640x480", secondary_multiscale),
                     ("loss_grad_32x640x480", secondary_loss),
                     ("batch_uneven_256", secondary_batch_uneven),
                     ("feature_1080p_16ch_bf16", secondary_feature_1080p),
                     ("bilateral_depth_filter", secondary_bilateral),
                     ("autograd_layer", secondary_autograd),
                     ("plain_kernels_larger_images", secondary_plain_sizes)):
        t = time.perf_counter()
        try:
            out[name] = fn(device, seed)
        except Exception as exc:  # reported, never hidden
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
        out[name]["wall_s"] = time.perf_counter() - t
    return out



def main():
    args = parse()
    rank, world, local = dist_env()
    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if world > 1:
            dist.destroy_process_group()
        return

    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration.icp import ICPOdometry
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if args.profile_case:
        profile_case(args, device)
        return
    x, host = make_inputs(args.seed + rank, device)
    icp = ICPOdometry(ITERS, geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
                      normals_angle_thresh=ANGLE, use_graph=True)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    def step():
        icp.launch(x["kcam"], x["sp"], x["sn"], x["sm"], target_points=x["tp"],
                   target_mask=x["tm"], target_normals=x["tn"])

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(device)

    def timed(k, fn, between=None):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(k)]
        for a, b in evs:
            flush.zero_()  # L2 flush between steps, outside the events
            a.record(stream)
            fn()
            b.record(stream)
            if between:
                between()
        torch.cuda.synchronize(device)
        return [a.elapsed_time(b) for a, b in evs]

    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        step()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    clocks.mark("t0")
    step_ms = timed(args.steps, step)
    barrier()
    clocks.mark("t1")
    clock_info = clocks.stop()
    total_ms = max_over_ranks(sum(step_ms), world, device)
    value = world * args.steps * ITERS / (total_ms / 1e3)

    # per-kernel times: the same steps with CUDA events around every kernel
    N.profile_enable(True)
    for _ in range(3):
        step()
    prof = {k: [0.0, 0] for k in N.PROFILE_KINDS}

    def read():
        torch.cuda.synchronize(device)
        for k, (ms, cnt) in N.profile_read().items():
            prof[k][0] += ms
            prof[k][1] += cnt
    prof_steps = min(args.steps, 200)
    timed(prof_steps, step, between=read)
    N.profile_enable(False)
    npix = H * W
    dom = max(ALG_BYTES, key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / max(prof[dom][1], 1)
    alg = ALG_BYTES[dom] * npix
    achieved = alg / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = None
    tpath = ROOT / "profiles" / "traffic.json"
    if tpath.exists():
        traffic = json.loads(tpath.read_text()).get(f"plain640/{dom}")

    # end to end through the public API: host (pinned) inputs copied in,
    # the result read back, every step.  The frame pair sits in one pinned
    # host buffer (the inputs packed back to back, each 256-byte aligned), so
    # a step's upload is one copy; the device views into it are what
    # ICPOdometry.estimate receives.
    names = ("kcam", "sp", "sn", "sm", "tp", "tn", "tm")
    offs, total = {}, 0
    for k in names:
        nb = x[k].numel() * x[k].element_size()
        offs[k] = (total, nb)
        total += (nb + 255) // 256 * 256
    host_pack = torch.empty(total, dtype=torch.uint8).pin_memory()
    dev_pack = torch.empty(total, dtype=torch.uint8, device=device)
    for k in names:
        o, nb = offs[k]
        host_pack[o:o + nb].copy_(x[k].reshape(-1).view(torch.uint8).cpu())
    dev_bufs = {k: dev_pack[offs[k][0]:offs[k][0] + offs[k][1]].view(x[k].dtype).view(x[k].shape)
                for k in names}
    h2d = sum(nb for _, nb in offs.values())

    def e2e_step():
        dev_pack.copy_(host_pack, non_blocking=True)
        icp.estimate(dev_bufs["kcam"], dev_bufs["sp"], dev_bufs["sn"], dev_bufs["sm"],
                     target_points=dev_bufs["tp"], target_mask=dev_bufs["tm"],
                     target_normals=dev_bufs["tn"])
    for _ in range(3):
        e2e_step()
    barrier()
    e2e_steps = min(args.steps, 500)
    sync_ms = max_over_ranks(sum(timed(e2e_steps, e2e_step)), world, device)
    sync_value = world * e2e_steps * ITERS / (sync_ms / 1e3)

    # The same end to end, double-buffered as a tracker runs it: two device
    # copies of the pair; the upload of step k + 1 (on a copy stream) runs
    # while step k registers, and step k's result is read back while step
    # k + 1 runs.  Every step still uploads its 15.4 MB and reads back its
    # result; wall clock over all steps, both ends synchronised.
    n_src = x["sp"].size(0)
    dev_packs = [dev_pack, torch.empty_like(dev_pack)]
    views = [dev_bufs, {k: dev_packs[1][offs[k][0]:offs[k][0] + offs[k][1]].view(x[k].dtype)
                           .view(x[k].shape) for k in names}]
    copy_stream = torch.cuda.Stream(device)
    host_res = [torch.empty(N.RES_SIZE, dtype=torch.float64).pin_memory() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]

    def pipelined(n):
        with torch.cuda.stream(copy_stream):
            dev_packs[0].copy_(host_pack, non_blocking=True)
            copied[0].record(copy_stream)
        results = []
        for k in range(n):
            b = k & 1
            stream.wait_event(copied[b])
            v = views[b]
            res = icp.launch(v["kcam"], v["sp"], v["sn"], v["sm"], target_points=v["tp"],
                             target_mask=v["tm"], target_normals=v["tn"])[0]
            host_res[b].copy_(res, non_blocking=True)
            done[b].record(stream)
            if k + 1 < n:
                with torch.cuda.stream(copy_stream):
                    if k >= 1:  # step k - 1 has finished reading that buffer
                        copy_stream.wait_event(done[1 - b])
                    dev_packs[1 - b].copy_(host_pack, non_blocking=True)
                    copied[1 - b].record(copy_stream)
            if k >= 1:
                done[1 - b].synchronize()
                results.append(ICPOdometry._result(host_res[1 - b], n_src, torch.float32))
        done[(n - 1) & 1].synchronize()
        results.append(ICPOdometry._result(host_res[(n - 1) & 1], n_src, torch.float32))
        return results

    pipelined(5)
    barrier()
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    out = pipelined(e2e_steps)
    torch.cuda.synchronize(device)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3, world, device)
    assert len(out) == e2e_steps and out[-1].transform is not None
    e2e_value = world * e2e_steps * ITERS / (e2e_ms / 1e3)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(host)
    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        secondary = run_secondary(device, args.seed)

    if rank == 0:
        launches_per_step = sum(v[1] for v in prof.values()) / max(prof_steps, 1)
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": run_config(),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "alg_bytes_per_launch": alg, "avg_launch_us": avg_ms * 1e3,
                         "kernels": {k: {"ms": v[0], "launches": v[1]}
                                     for k, v in prof.items()}},
            "cpu_baseline": base,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": N.RES_SIZE * 8, "steps": e2e_steps,
                    "mode": "double-buffered: upload of step k+1 overlaps step k; wall clock",
                    "one_call_at_a_time": {"value": sync_value, "unit": UNIT,
                                           "ms_per_step": sync_ms / e2e_steps}},
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "clocks": clock_info,
            "secondary_summary": summarize(secondary) if secondary else None,
        }))
        if secondary and args.secondary_out:
            pathlib.Path(args.secondary_out).write_text(json.dumps(secondary, indent=1) + "\n")
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
