"""Benchmark: batched GJK/EPA contact pairs/s on one GB300.

Workload: 1,048,576 mixed convex pairs (Ball, Cuboid, Capsule, Cone and
ConvexHull with 8..1024 points, seeded synthetic data), query::contact with
prediction 0 in the PRECISE tolerance set, inputs resident in HBM (1.5 GB,
larger than L2).  One step = one contact_batch over the whole batch.
`--dispatch query` (default) routes Ball pairs as query::contact does;
`--dispatch support_map` sends every pair through GJK/EPA; the line reports
the other dispatch's throughput too.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is device-resident throughput; `e2e` is the
same metric through the library's host entry point with host<->device copies
inside the timed region; `cpu_baseline` times the CPU restatement of the
reference path (the oracle, f32) on the host cores; `roofline` describes the
dominant kernel.  With torchrun (N > 1) every rank processes its own batch
(weak scaling, no collective on the data path).
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

METRIC = "GJK/EPA contact pairs/s on 1 GB300: warm-started vs plain at ≤1e-5 rel err"
N_PAIRS = 1 << 20
SEED = 1
# Algorithmic FP32 operations per unit of work, counted from the restated
# reference: a quaternion rotation is 30 flops and each support call rotates
# twice (66 flops with the CSO difference), a hull point costs 5 flops in the
# arg-max (3 mul + 2 add), a GJK sub-solve ~300 and an EPA face ~150.
FLOPS_SUPPORT, FLOPS_HULL_POINT, FLOPS_SUBSOLVE, FLOPS_FACE = 66.0, 5.0, 300.0, 150.0


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_workload(rank, n_pairs=N_PAIRS):
    from ncollide_gb300 import workloads as W
    return W.mixed_convex(n_pairs, seed=SEED + rank)


def algorithmic(batch, counters):
    """Bytes and FP32 flops per pair (inputs read once, outputs written once)."""
    n = batch.n_pairs
    kinds = batch.shapes["kind"]
    hull_bytes = 16.0 * (batch.shapes["hull_n"][batch.g1].astype(np.float64) +
                         batch.shapes["hull_n"][batch.g2].astype(np.float64))
    in_bytes = 2 * 32 + 2 * 32 + 2 * 4 + hull_bytes.mean()
    out_bytes = 40 + 1 + 12 + 4
    c = counters.astype(np.float64)
    flops = (c[:, 2] * FLOPS_SUPPORT + c[:, 3] * FLOPS_HULL_POINT + (c[:, 7].astype(np.uint32) & 0xffffff) *
             FLOPS_SUBSOLVE + c[:, 4] * FLOPS_FACE).mean()
    del kinds
    return in_bytes + out_bytes, in_bytes, out_bytes, flops


def err_table(c, has, r64, scale, curved, ballball):
    """Depth, normal and witness-point errors of contacts c (n x 10: world1,
    world2, normal, depth) against the f64 oracle, per class of pair."""
    both = (has == 1) & (r64.tag == 1) & (r64.value > 0) & ~ballball
    dd = np.abs(c[:, 9] - r64.value) / np.maximum(np.abs(r64.value), scale)
    dn = np.linalg.norm(c[:, 6:9] - r64.dir, axis=1)
    dp = np.maximum(np.linalg.norm(c[:, 0:3] - r64.p1, axis=1), np.linalg.norm(c[:, 3:6] - r64.p2, axis=1)) / scale

    def pct(x, m):
        return {"p50": float(np.percentile(x[m], 50)), "p99": float(np.percentile(x[m], 99)),
                "max": float(x[m].max()), "frac_gt_1e-5": float((x[m] > 1e-5).mean()), "n": int(m.sum())} \
            if m.any() else None
    return {"depth": {"polytope_pairs": pct(dd, both & ~curved), "curved_pairs": pct(dd, both & curved)},
            "normal": {"polytope_pairs": pct(dn, both & ~curved), "curved_pairs": pct(dn, both & curved)},
            "witness_points": {"polytope_pairs": pct(dp, both & ~curved), "curved_pairs": pct(dp, both & curved)}}


def oracle_contacts(r):
    """An oracle result as the GPU's (n x 10) contact layout."""
    return np.concatenate([r.p1, r.p2, r.dir, r.value[:, None]], 1)


def mixed_parity(batch, query, param, tolerance, gpu, distance=None, policy=None, r=None):
    """Bit-exact check of a whole batch's GPU outputs against the oracle: the
    mixed-precision instantiation (the kernels' default arithmetic split) or,
    with policy F32, the reference's f32 path (NCG_ARITH_F32).  Counts the
    pairs whose tag, status or any output float differs (NaN equal to NaN).
    gpu: contact outputs (has_contact, contact n x 10, dir, status); distance:
    distance outputs (distance, status); r: the oracle's result when already
    computed."""
    from oracle import oracle as O
    policy = O.MIXED if policy is None else policy
    eps, epa_tol = (-1.0, 1e-6) if tolerance == "precise" else (0.0, 0.0)
    t0 = time.perf_counter()
    if r is None:
        r = O.query(batch, query, policy, param=float(np.float32(param)), eps=eps, epa_tol=epa_tol)

    def differ(a, b):
        a, b = np.asarray(a), np.asarray(b)
        bad = (a != b) & ~(np.isnan(a) & np.isnan(b)) if np.issubdtype(a.dtype, np.floating) else a != b
        return bad.reshape(len(a), -1).any(1)
    out = {"pairs": int(batch.n_pairs), "tolerance": tolerance,
           "oracle": "MIXED (f32 support points, double-word sub-solve)" if policy == O.MIXED else
                     "F32 (the reference's f32 path: f32 sub-solve, Rust heap order)"}
    if distance is None:
        m = r.tag == 1
        want = oracle_contacts(r).astype(np.float32)
        got = gpu["contact"]
        out["has_contact_mismatches"] = int(differ(gpu["has_contact"], r.tag).sum())
        out["contact_mismatches"] = int((differ(np.where(m[:, None], got, 0), np.where(m[:, None], want, 0))).sum())
        out["dir_mismatches"] = int(differ(gpu["dir"], r.dir.astype(np.float32)).sum())
        out["status_mismatches"] = int(differ(gpu["status"].view(np.uint32), r.status).sum())
    else:
        out["distance_mismatches"] = int(differ(distance["distance"], r.value.astype(np.float32)).sum())
        out["status_mismatches"] = int(differ(distance["status"].view(np.uint32), r.status).sum())
    out["bit_exact"] = all(v == 0 for k, v in out.items() if k.endswith("_mismatches"))
    out["oracle_seconds"] = time.perf_counter() - t0
    return out


def accuracy_report(batch, gpu_out, sample, query):
    """Errors of the GPU contacts against the oracle built with f64 (the error
    oracle) on the first `sample` pairs, beside the same errors of the
    reference's f32 path; the contact classification (Some / None) against the
    f32 reference path and against f64, outside a +-1e-6 band around touching
    (the band is on the f64 signed gap: -depth when penetrating, else the
    distance)."""
    from oracle import oracle as O
    sub = batch.subset(np.arange(sample))
    r64 = O.query(sub, query, O.F64, param=0.0)
    r32 = O.query(sub, query, O.F32, param=0.0)
    d64 = O.query(sub, O.DISTANCE, O.F64)
    has = gpu_out["has_contact"][:sample]
    c = gpu_out["contact"][:sample].astype(np.float64)
    k1, k2 = sub.kinds()
    curved = np.isin(k1, [0, 2, 3]) | np.isin(k2, [0, 2, 3])
    ballball = (k1 == 0) & (k2 == 0)
    gap = np.where(r64.tag == 1, -r64.value, d64.value)
    band = np.abs(gap) <= 1e-6
    gpu_cls, ref_cls, f64_cls = has == 1, r32.tag == 1, r64.tag == 1
    return {
        "sample_pairs": int(sample),
        "relative_to": "max(|f64 value|, rA+rB); normals absolute",
        "gpu_vs_f64": err_table(c, has, r64, sub.scale, curved, ballball),
        "f32_reference_path_vs_f64": err_table(oracle_contacts(r32), r32.tag, r64, sub.scale, curved, ballball),
        "classification_outside_band": {
            "pairs_outside_band": int((~band).sum()),
            "gpu_vs_f32_reference_mismatches": int(((gpu_cls != ref_cls) & ~band).sum()),
            "gpu_vs_f64_mismatches": int(((gpu_cls != f64_cls) & ~band).sum()),
            "f32_reference_vs_f64_mismatches": int(((ref_cls != f64_cls) & ~band).sum())},
        "ball_ball_pairs_excluded_from_errors": int(ballball.sum()),
    }


def _quat_mul_t(a, b):
    import torch
    ai, aj, ak, aw = a.unbind(1)
    bi, bj, bk, bw = b.unbind(1)
    return torch.stack([aw * bi + ai * bw + aj * bk - ak * bj, aw * bj - ai * bk + aj * bw + ak * bi,
                        aw * bk + ai * bj - aj * bi + ak * bw, aw * bw - ai * bi - aj * bj - ak * bk], 1)


def _advance_poses_t(m, gen, sigma_t=0.01, sigma_r=0.02):
    """One frame of coherent motion on the device (the workload generator's
    advance_frame): translation += N(0, sigma_t^2) per axis, rotation about a
    random axis by N(0, sigma_r^2) rad."""
    import torch
    n = m.shape[0]
    ax = torch.randn((n, 3), generator=gen, device=m.device, dtype=torch.float64)
    ax = ax / ax.norm(dim=1, keepdim=True)
    ang = torch.randn(n, generator=gen, device=m.device, dtype=torch.float64) * sigma_r
    dq = torch.cat([ax * torch.sin(ang / 2)[:, None], torch.cos(ang / 2)[:, None]], 1)
    q = _quat_mul_t(dq, m[:, :4].double())
    q = q / q.norm(dim=1, keepdim=True)
    out = m.clone()
    out[:, :4] = q.float()
    out[:, 4:7] += (torch.randn((n, 3), generator=gen, device=m.device, dtype=torch.float64) * sigma_t).float()
    return out


def coherent_warm_start(args, local, tolerance, peak_hbm, peak_fp32, mlp_params=None):
    """Large coherent batch: ConvexHull-ConvexHull pairs over a pool of shared
    hulls, stepped over 8 frames; plain GJK vs previous-frame direction reuse,
    each frame one replay of a captured CUDA graph."""
    import torch
    from ncollide_gb300 import _native as Nn
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n, frames = args.coherent_pairs, 8
    b0 = W.coherent_hull_pairs(n, seed=5, pool=1 << 16)
    db = Q.DeviceBatch.from_host(b0, device=f"cuda:{local}")
    gen = torch.Generator(device=f"cuda:{local}")
    gen.manual_seed(5)
    poses = [(db.m1.clone(), db.m2.clone())]
    for _ in range(frames - 1):
        poses.append((_advance_poses_t(poses[-1][0], gen), _advance_poses_t(poses[-1][1], gen)))
    ctx = Q.Context(local, tolerance=tolerance, dispatch="support_map")
    if args.only == "coherent":  # a profiling run of this leg alone takes the command line's overrides
        for kv in args.tune:
            k, v = kv.split("=", 1)
            ctx.set_tuning(k, int(v))
    dirs = torch.empty((n, 3), dtype=torch.float32, device=db.m1.device)
    g_plain = Q.ContactGraph(ctx, db, 0.0)
    g_mlp = None
    strategies = ["plain", "previous_frame_dir"]
    if mlp_params is not None:
        ctx.set_mlp_params(mlp_params)
        ctx.set_warm_start(Nn.WARM_MLP)
        g_mlp = Q.ContactGraph(ctx, db, 0.0)
        ctx.set_warm_start(Nn.WARM_NONE)
        strategies.append("mlp")
    res = {}
    for strategy in strategies:
        if strategy == "previous_frame_dir":
            ctx.set_warm_start(Nn.WARM_NONE)
        times, iters = [], []
        g_warm = None
        for f in range(frames):
            db.m1.copy_(poses[f][0])
            db.m2.copy_(poses[f][1])
            if strategy == "previous_frame_dir" and f == 1:
                ctx.set_warm_start(Nn.WARM_INIT_DIR)
                g_warm = Q.ContactGraph(ctx, db.with_init_dir(dirs), 0.0, reuse_dir=True)
            g = g_warm if (strategy == "previous_frame_dir" and f >= 1) else g_plain
            if strategy == "mlp":
                g = g_mlp
            if f == frames - 1:  # the start directions of the last frame, for the accuracy check
                if strategy == "previous_frame_dir":
                    init_last = dirs[:4096].cpu().numpy()
                elif strategy == "mlp":
                    from ncollide_gb300 import warm_mlp as M
                    init_last = M.infer(db, mlp_params)[:4096].cpu().numpy()
                else:
                    init_last = None
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            out = g.launch()
            e1.record()
            torch.cuda.synchronize()
            if strategy == "previous_frame_dir" and f == 0:
                dirs.copy_(out["dir"])
            st = ctx.stats()
            if f >= 1:
                times.append(e0.elapsed_time(e1))
                iters.append(st["gjk_iters"] / n)
        last = {k: (None if v is None else v[:4096].cpu().numpy()) for k, v in out.items()}
        if strategy == "plain":  # the last frame's first 65,536 pairs, for the bit-exact check
            parity_last = {k: out[k][:65536].cpu().numpy() for k in ("contact", "has_contact", "dir", "status")}
        ms = sum(times) / len(times)
        res[strategy] = {"pairs_per_s": n / (ms / 1e3), "ms_per_frame": ms,
                         "gjk_iters_per_pair": sum(iters) / len(iters), "frames_timed": len(times),
                         "_last": last, "_init": init_last}
        if g_warm is not None:
            g_warm.close()
    ctx.set_warm_start(Nn.WARM_NONE)
    # algorithmic bytes / flops (plain-path counts from the oracle on a sample of frame 0)
    sample = b0.subset(np.arange(16384))
    rs = O.query(sample, O.CONTACT, O.MIXED, param=0.0, eps=-1.0 if tolerance == "precise" else 0.0,
                 epa_tol=1e-6 if tolerance == "precise" else 0.0)
    bytes_pp, _, _, flops_pp = algorithmic(sample, rs.counters)
    # accuracy of the last frame (first 4096 pairs) against the f64 oracle
    lastb = b0.subset(np.arange(4096))
    lastb = type(lastb)(lastb.shapes, lastb.hull_points, poses[-1][0][:4096].cpu().numpy(), lastb.g1,
                        poses[-1][1][:4096].cpu().numpy(), lastb.g2, None, lastb.scale, dict(lastb.meta))
    r64 = O.query(lastb, O.CONTACT, O.F64, param=0.0)

    def rel_err(last, ref):
        m = (last["has_contact"] == 1) & (ref.tag == 1)
        rel = np.abs(last["contact"][:, 9].astype(np.float64) - ref.value) / np.maximum(np.abs(ref.value),
                                                                                      lastb.scale)
        return {"p99": float(np.percentile(rel[m], 99)) if m.any() else None,
                "max": float(rel[m].max()) if m.any() else None,
                "frac_gt_1e-5": float((rel[m] > 1e-5).mean()) if m.any() else None}
    both_ok = True
    for strategy, r in res.items():
        last = r.pop("_last")
        init = r.pop("_init")
        # against the f64 reference started like the plain method, and started
        # from the same directions (the same algorithm and inputs in f64)
        r["depth_rel_err_vs_f64_plain_start"] = rel_err(last, r64)
        r64s = r64 if init is None else O.query(lastb.with_init_dir(init), O.CONTACT, O.F64, param=0.0)
        r["depth_rel_err_vs_f64_same_start"] = rel_err(last, r64s)
        r["classification_mismatch_vs_f64"] = int((last["has_contact"] != r64s.tag).sum())
        r["hbm_gbs"] = r["pairs_per_s"] * bytes_pp / 1e9
        r["hbm_frac"] = r["hbm_gbs"] / peak_hbm
        r["fp32_frac"] = r["pairs_per_s"] * flops_pp / 1e12 / peak_fp32
        both_ok &= r["classification_mismatch_vs_f64"] >= 0
    # the plain method's last frame, bit for bit against the oracle on its
    # first 65,536 pairs (run inside the whole batch, sorted by hull locality)
    kp = 65536
    pb = b0.subset(np.arange(kp))
    pb = type(pb)(pb.shapes, pb.hull_points, poses[-1][0][:kp].cpu().numpy(), pb.g1,
                  poses[-1][1][:kp].cpu().numpy(), pb.g2, None, pb.scale, dict(pb.meta))
    parity = mixed_parity(pb, O.CONTACT, 0.0, tolerance, parity_last)
    g_plain.close()
    if g_mlp is not None:
        g_mlp.close()
    ctx.close()
    out = {"workload": f"coherent_hull_pairs: {n} ConvexHull-ConvexHull pairs, 32-1024 points, pool of 65536 "
                       f"shared hulls, 8 frames (sigma_t 0.01, sigma_r 0.02), seed 5; frames 1-7 timed",
           "strategies": res,
           "speedup_previous_frame_vs_plain": res["previous_frame_dir"]["pairs_per_s"] / res["plain"]["pairs_per_s"],
           "speedup_mlp_vs_plain": (res["mlp"]["pairs_per_s"] / res["plain"]["pairs_per_s"]) if "mlp" in res else None,
           "bytes_per_pair": bytes_pp, "flops_per_pair": flops_pp,
           "accuracy_sample": "first 4096 pairs of the last frame",
           "parity_vs_oracle_last_frame_first_65536": parity}
    return out


def learned_warm_start(args, local, tolerance, dispatch, headline_db, headline_batch, headline_tuning=None):
    """Trains the warm-start network on plain-GJK labels (20 epochs, batch 8192,
    4,194,304 pairs of the mixed distribution over a pool of shared shapes),
    evaluates it on 4,194,304 held-out pairs (other seed, other pool) and times
    the warm-started contact against plain on the headline batch (with the
    headline's launch tuning)."""
    import torch
    from ncollide_gb300 import _native as Nn
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import warm_mlp as M
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    dev = f"cuda:{local}"
    ctx = Q.Context(local, tolerance=tolerance, dispatch="support_map")
    t0 = time.perf_counter()
    train_b = W.mixed_convex_pooled(args.mlp_pairs, seed=3, pool=1 << 17)
    held_b = W.mixed_convex_pooled(args.mlp_pairs, seed=4, pool=1 << 17)
    gen_s = time.perf_counter() - t0
    dtr = Q.DeviceBatch.from_host(train_b, device=dev)
    dhe = Q.DeviceBatch.from_host(held_b, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, Xtr = M.features(dtr)
    Ytr = M.labels(ctx, dtr)
    torch.cuda.synchronize()
    label_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    params, hist = M.train(Xtr, Ytr, epochs=args.mlp_epochs, batch_size=8192, lr=2e-3, seed=0)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    _, Xhe = M.features(dhe)
    Yhe = M.labels(ctx, dhe)
    held_loss = M.evaluate(Xhe, Yhe, params)
    ctx.set_mlp_params(params)
    ctx.set_dispatch(dispatch)

    def run(db, warm, steps):
        ctx.set_warm_start(warm)
        for _ in range(2):
            Q.contact_batch(ctx, db, 0.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            o = Q.contact_batch(ctx, db, 0.0, with_iters=True)
        e1.record()
        torch.cuda.synchronize()
        it = o["iters"].cpu().numpy().view(np.uint32)
        g = (it & 0xffff).astype(np.float64)
        e = (it >> 16).astype(np.float64)
        return {"pairs_per_s": db.n_pairs * steps / (e0.elapsed_time(e1) / 1e3),
                "ms_per_step": e0.elapsed_time(e1) / steps,
                "gjk_iters_mean": float(g.mean()), "gjk_iters_p99": float(np.percentile(g, 99)),
                "epa_iters_mean": float(e.mean()), "flags": ctx.stats()["flags"]}, o

    held = {"plain": run(dhe, Nn.WARM_NONE, 3)[0], "mlp": run(dhe, Nn.WARM_MLP, 3)[0]}

    def run_closest(db, warm, steps):
        # closest points with prediction 0.1: GJK refines to convergence there,
        # so the start direction changes its iteration count
        ctx.set_warm_start(warm)
        for _ in range(2):
            Q.closest_points_batch(ctx, db, 0.1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            o = Q.closest_points_batch(ctx, db, 0.1, with_iters=True)
        e1.record()
        torch.cuda.synchronize()
        g = (o["iters"].cpu().numpy().view(np.uint32) & 0xffff).astype(np.float64)
        return {"pairs_per_s": db.n_pairs * steps / (e0.elapsed_time(e1) / 1e3), "ms_per_step": e0.elapsed_time(e1) / steps,
                "gjk_iters_mean": float(g.mean()), "gjk_iters_p99": float(np.percentile(g, 99))}
    closest = {"plain": run_closest(dhe, Nn.WARM_NONE, 3), "mlp": run_closest(dhe, Nn.WARM_MLP, 3)}
    closest["gjk_iteration_reduction"] = 1.0 - closest["mlp"]["gjk_iters_mean"] / closest["plain"]["gjk_iters_mean"]
    closest["speedup_mlp_vs_plain"] = closest["mlp"]["pairs_per_s"] / closest["plain"]["pairs_per_s"]
    if headline_tuning:
        ctx.apply_tuning(headline_tuning)
    head_plain, op = run(headline_db, Nn.WARM_NONE, args.steps)
    head_mlp, om = run(headline_db, Nn.WARM_MLP, args.steps)
    ctx.set_warm_start(Nn.WARM_NONE)
    # accuracy of both against the f64 oracle on the first 4096 headline pairs
    k = 4096
    sub = headline_batch.subset(np.arange(k))
    q = O.CONTACT_QUERY if dispatch == "query" else O.CONTACT
    r64 = O.query(sub, q, O.F64, param=0.0)
    acc = {}
    for name, o in (("plain", op), ("mlp", om)):
        has = o["has_contact"][:k].cpu().numpy()
        c = o["contact"][:k].cpu().numpy().astype(np.float64)
        m = (has == 1) & (r64.tag == 1)
        rel = np.abs(c[:, 9] - r64.value) / np.maximum(np.abs(r64.value), sub.scale)
        acc[name] = {"depth_rel_err_p99": float(np.percentile(rel[m], 99)) if m.any() else None,
                     "depth_rel_err_max": float(rel[m].max()) if m.any() else None,
                     "frac_gt_1e-5": float((rel[m] > 1e-5).mean()) if m.any() else None,
                     "has_contact_mismatch_vs_f64": int((has != r64.tag).sum())}
    ctx.close()
    return params, {"train": {"pairs": train_b.n_pairs, "epochs": args.mlp_epochs, "batch": 8192,
                      "optimizer": "Adam lr 2e-3", "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1],
                      "seconds_generate_host": gen_s, "seconds_label_gpu": label_s, "seconds_train_gpu": train_s,
                      "data": "mixed_convex over a pool of 131072 shapes, seed 3 (train) / 4 (held out)"},
            "held_out": {"pairs": held_b.n_pairs, "loss": held_loss, **held,
                         "closest_points_prediction_0.1": closest},
            "headline_batch": {"plain": head_plain, "mlp": head_mlp,
                               "speedup_mlp_vs_plain": head_mlp["pairs_per_s"] / head_plain["pairs_per_s"],
                               "accuracy_vs_f64_first_4096": acc}}


def near_touching(batch, seed=2, newton=3):
    """Places every pair at a signed gap +-g, g log-uniform in [1e-7, 1e-1] (sign
    50/50), by Newton steps on the f64 oracle's signed distance along the
    centre line (the contact query with prediction 1: -depth, normal A->B).
    Returns the batch with the moved second poses and the target gaps."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed + 1000)
    n = batch.n_pairs
    target = np.exp(rng.uniform(np.log(1e-7), np.log(1e-1), n)) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    c1 = batch.m1[:, 4:7].astype(np.float64)
    d = batch.m2[:, 4:7].astype(np.float64) - c1
    t = np.linalg.norm(d, axis=1)
    u = d / np.maximum(t, 1e-30)[:, None]
    b = batch
    for _ in range(newton):
        r = O.query(b, O.CONTACT, O.F64, param=1.0)
        ok = r.tag == 1
        s_now = np.where(ok, -r.value, 1.0)
        slope = np.maximum((r.dir * u).sum(1), 0.05)
        t = np.maximum(t + np.where(ok, (target - s_now) / slope, -0.5 * t), 0.0)
        m2 = b.m2.copy()
        m2[:, 4:7] = (c1 + t[:, None] * u).astype(np.float32)
        b = type(b)(b.shapes, b.hull_points, b.m1, b.g1, m2, b.g2, None, b.scale, dict(b.meta))
    return b, target


def precision_stress(args, local, tolerance):
    """Thin shapes (one axis scaled by logU[1e-3, 1]) placed near touching; the
    GPU's contact and distance against the f64 oracle on the same f32 inputs
    (beside the reference f32 path's own errors), the intersect classification
    against the f32 reference path and f64 outside a +-1e-6 band around
    touching, and the whole batch bit for bit against the oracle's
    mixed-precision instantiation."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    t0 = time.perf_counter()
    base = W.mixed_convex(args.stress_pairs, seed=2, thin=True)
    b, target = near_touching(base)
    prep_s = time.perf_counter() - t0
    db = Q.DeviceBatch.from_host(b, device=f"cuda:{local}")
    ctx = Q.Context(local, tolerance=tolerance, dispatch="support_map")
    oc = Q.contact_batch(ctx, db, 0.0)
    od = Q.distance_batch(ctx, db)
    torch.cuda.synchronize()
    gpu_c = {k: v.cpu().numpy() for k, v in oc.items() if v is not None}
    gpu_d = {k: v.cpu().numpy() for k, v in od.items() if v is not None}
    has = gpu_c["has_contact"]
    dist = gpu_d["distance"].astype(np.float64)
    ctx.close()
    # the reference's f32 path on the GPU (NCG_ARITH_F32, reference tolerances)
    ctx32 = Q.Context(local, tolerance="reference", dispatch="support_map", arithmetic="f32")
    o32 = Q.contact_batch(ctx32, db, 0.0)
    torch.cuda.synchronize()
    gpu32 = {k: v.cpu().numpy() for k, v in o32.items() if v is not None}
    ctx32.close()
    r64c = O.query(b, O.CONTACT, O.F64, param=0.0)
    r64d = O.query(b, O.DISTANCE, O.F64)
    r32c = O.query(b, O.CONTACT, O.F32, param=0.0)
    r32d = O.query(b, O.DISTANCE, O.F32)
    scale = b.scale
    k1, k2 = b.kinds()
    ballball = (k1 == 0) & (k2 == 0)
    gap = np.where(r64c.tag == 1, -r64c.value, r64d.value)  # true signed gap of the f32 inputs
    band = np.abs(gap) <= 1e-6
    curved = np.isin(k1, [0, 2, 3]) | np.isin(k2, [0, 2, 3])

    def dist_stats(x, m):
        if not m.any():
            return None
        return {"n": int(m.sum()), "p50": float(np.percentile(x[m], 50)), "p99": float(np.percentile(x[m], 99)),
                "max": float(x[m].max()), "frac_gt_1e-5": float((x[m] > 1e-5).mean())}
    sep = (r64d.value > 0) & ~ballball

    def dist_errs(d):
        e = np.abs(d - r64d.value) / scale
        return {"all": dist_stats(e, sep), "polytope": dist_stats(e, sep & ~curved), "curved": dist_stats(e, sep & curved)}
    gpu_int, ref_int, f64_int = has == 1, r32c.tag == 1, r64c.tag == 1
    return {"workload": f"{b.n_pairs} mixed pairs (seed 2), thin shapes (one axis x logU[1e-3,1]), signed gap "
                        "+-logU[1e-7,1e-1] set by 3 Newton steps of the f64 oracle; errors relative to rA+rB",
            "seconds_prepare_host": prep_s,
            "achieved_gap_minus_target_p50": float(np.percentile(np.abs(gap - target), 50)),
            "gpu_distance_error": dist_errs(dist),
            "f32_reference_distance_error": dist_errs(r32d.value),
            "gpu_contact_error": err_table(gpu_c["contact"].astype(np.float64), has, r64c, scale, curved, ballball),
            "f32_reference_contact_error": err_table(oracle_contacts(r32c), r32c.tag, r64c, scale, curved, ballball),
            "classification_outside_band": {
                "pairs_outside_band": int((~band).sum()),
                "gpu_vs_f32_reference_mismatches": int(((gpu_int != ref_int) & ~band).sum()),
                "gpu_vs_f64_mismatches": int(((gpu_int != f64_int) & ~band).sum()),
                "f32_reference_vs_f64_mismatches": int(((ref_int != f64_int) & ~band).sum())},
            "parity_vs_oracle_contact": mixed_parity(b, O.CONTACT, 0.0, tolerance, gpu_c),
            "parity_vs_oracle_distance": mixed_parity(b, O.DISTANCE, 0.0, tolerance, None, gpu_d),
            "f32_arithmetic": {
                "classification_vs_f32_reference_mismatches_outside_band":
                    int(((gpu32["has_contact"] == 1) != ref_int)[~band].sum()),
                "parity_vs_f32_reference_path": mixed_parity(b, O.CONTACT, 0.0, "reference", gpu32, policy=O.F32,
                                                             r=r32c)},
            "ball_ball_pairs_excluded": int(ballball.sum())}


def cuboid_small(args, local, tolerance):
    """65,536 Cuboid-Cuboid pairs, query::contact with prediction 0: GPU
    throughput (inputs resident, and through the host entry point), the CPU
    reference path on the same pairs, classification outside the +-1e-6 band,
    and the whole batch bit for bit against the oracle."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    b = W.cuboid_pairs(65536, seed=0)
    db = Q.DeviceBatch.from_host(b, device=f"cuda:{local}")
    ctx = Q.Context(local, tolerance=tolerance, dispatch="query")
    for _ in range(3):
        Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        o = Q.contact_batch(ctx, db, 0.0)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 20
    gpu = {k: v.cpu().numpy() for k, v in o.items() if v is not None}
    has = gpu["has_contact"]
    # through the host entry point: pinned inputs copied in, outputs copied out
    for _ in range(3):
        Q.contact_batch_host(ctx, b, 0.0)
    t0 = time.perf_counter()
    for _ in range(20):
        Q.contact_batch_host(ctx, b, 0.0)
    host_s = (time.perf_counter() - t0) / 20
    ctx.close()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r32 = O.query(b, O.CONTACT_QUERY, O.F32, param=0.0, threads=threads)
    cpu_s = time.perf_counter() - t0
    r64 = O.query(b, O.CONTACT_QUERY, O.F64, param=0.0)
    d64 = O.query(b, O.DISTANCE, O.F64)
    gap = np.where(r64.tag == 1, -r64.value, d64.value)
    band = np.abs(gap) <= 1e-6
    k1, k2 = b.kinds()
    none = np.zeros(b.n_pairs, bool)
    pk = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    bytes_pp = 2 * 32 + 2 * 32 + 2 * 4 + 40 + 1 + 12 + 4
    return {"workload": "65536 Cuboid-Cuboid pairs, seed 0, query::contact prediction 0",
            "pairs_per_s": 65536 / (ms / 1e3), "ms_per_step": ms,
            "host_entry_pairs_per_s": 65536 / host_s,
            "roofline_hbm": {"bytes_per_pair": bytes_pp, "achieved_gbs": 65536 * bytes_pp / (ms / 1e3) / 1e9,
                             "peak_gbs": hbm, "frac": 65536 * bytes_pp / (ms / 1e3) / 1e9 / hbm,
                             "note": "the whole call (inputs fit in L2; launch-bound at this size)"},
            "cpu_reference_path_pairs_per_s": 65536 / cpu_s, "cpu_cores": threads,
            "classification_outside_band": {
                "pairs_outside_band": int((~band).sum()),
                "gpu_vs_f32_reference_mismatches": int(((has != r32.tag) & ~band).sum()),
                "gpu_vs_f64_mismatches": int(((has != r64.tag) & ~band).sum()),
                "f32_reference_vs_f64_mismatches": int(((r32.tag != r64.tag) & ~band).sum())},
            "gpu_contact_error": err_table(gpu["contact"].astype(np.float64), has, r64, b.scale, none, none),
            "f32_reference_contact_error": err_table(oracle_contacts(r32), r32.tag, r64, b.scale, none, none),
            "parity_vs_oracle": mixed_parity(b, O.CONTACT_QUERY, 0.0, tolerance, gpu)}


def time_of_impact_report(args, local, tolerance, dispatch):
    """query::time_of_impact over 2^20 linear sweeps (toi_sweeps, seed 7):
    GPU throughput with inputs resident, the CPU reference path (oracle, f32)
    on a 65,536-sweep sample with every host core, and agreement with f64."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n = args.toi_pairs
    b, v1, v2 = W.toi_sweeps(n, seed=7)
    dev = f"cuda:{local}"
    db = Q.DeviceBatch.from_host(b, device=dev)
    tv1, tv2 = torch.from_numpy(v1).to(dev), torch.from_numpy(v2).to(dev)
    ctx = Q.Context(local, tolerance=tolerance, dispatch=dispatch)
    for _ in range(3):
        o = Q.time_of_impact_batch(ctx, db, tv1, tv2, with_iters=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        o = Q.time_of_impact_batch(ctx, db, tv1, tv2, with_iters=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    has = o["has_toi"].cpu().numpy()
    toi = o["toi"].cpu().numpy()
    iters = o["iters"].cpu().numpy()
    ctx.close()
    sample = min(65536, n)
    idx = np.arange(sample)
    sb = b.subset(idx)
    threads = os.cpu_count() or 1
    qd = 1 if dispatch == "query" else 0
    t0 = time.perf_counter()
    r32 = O.toi(sb, v1[idx], v2[idx], O.F32, dispatch=qd, threads=threads)
    cpu_s = time.perf_counter() - t0
    r64 = O.toi(sb, v1[idx], v2[idx], O.F64, dispatch=qd, threads=threads)
    m = (has[idx] == 1) & (r64["some"] == 1)
    rel = np.abs(toi[idx][m] - r64["toi"][m]) / np.maximum(np.abs(r64["toi"][m]), 1e-30)
    m32 = (r32["some"] == 1) & (r64["some"] == 1)
    rel32 = np.abs(r32["toi"][m32] - r64["toi"][m32]) / np.maximum(np.abs(r64["toi"][m32]), 1e-30)
    return {"workload": f"toi_sweeps {n} pairs, seed 7, max_toi inf, target_distance 0", "dispatch": dispatch,
            "pairs_per_s": n / (ms / 1e3), "ms_per_step": ms, "some_fraction": float(has.mean()),
            "ray_cast_iters_per_pair": float(iters.astype(np.float64).mean()),
            "cpu_reference_path_pairs_per_s": sample / cpu_s, "cpu_cores": threads,
            "cpu_sample": f"first {sample} sweeps, f32 reference path (oracle)",
            "some_mismatch_vs_f64": int((has[idx] != r64["some"]).sum()),
            "some_mismatch_f32_reference_vs_f64": int((r32["some"] != r64["some"]).sum()),
            "toi_rel_err_vs_f64_p50_p99": [float(np.percentile(rel, 50)), float(np.percentile(rel, 99))] if rel.size else None,
            "toi_rel_err_f32_reference_vs_f64_p50_p99":
                [float(np.percentile(rel32, 50)), float(np.percentile(rel32, 99))] if rel32.size else None}


def ray_cast_report(args, local, tolerance):
    """RayCast::toi_and_normal_with_ray (GJK ray cast) for 2^20 rays
    (ray_casts, seed 9; solid): GPU throughput with inputs resident, the CPU
    reference path (oracle, f32) on a 65,536-ray sample with every host core,
    and agreement with f64."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n = args.ray_count
    b, rays = W.ray_casts(n, seed=9)
    dev = f"cuda:{local}"
    db = Q.DeviceBatch.from_host(b, device=dev)
    tr = torch.from_numpy(rays).to(dev)
    ctx = Q.Context(local, tolerance=tolerance)
    for _ in range(3):
        o = Q.ray_cast_batch(ctx, db, tr, with_iters=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        o = Q.ray_cast_batch(ctx, db, tr, with_iters=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    hit = o["has_hit"].cpu().numpy()
    toi = o["toi"].cpu().numpy()
    iters = o["iters"].cpu().numpy()
    ctx.close()
    sample = min(65536, n)
    idx = np.arange(sample)
    sb = b.subset(idx)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r32 = O.ray_cast(sb, rays[idx], O.F32, threads=threads)
    cpu_s = time.perf_counter() - t0
    r64 = O.ray_cast(sb, rays[idx], O.F64, threads=threads)
    m = (hit[idx] == 1) & (r64["hit"] == 1)
    rel = np.abs(toi[idx][m] - r64["toi"][m]) / np.maximum(np.abs(r64["toi"][m]), 1e-30)
    return {"workload": f"ray_casts {n} rays, seed 9, solid, max_toi inf", "rays_per_s": n / (ms / 1e3),
            "ms_per_step": ms, "hit_fraction": float(hit.mean()),
            "ray_cast_iters_per_ray": float(iters.astype(np.float64).mean()),
            "cpu_reference_path_rays_per_s": sample / cpu_s, "cpu_cores": threads,
            "cpu_sample": f"first {sample} rays, f32 reference path (oracle)",
            "hit_mismatch_vs_f64": int((hit[idx] != r64["hit"]).sum()),
            "hit_mismatch_f32_reference_vs_f64": int((r32["hit"] != r64["hit"]).sum()),
            "toi_rel_err_vs_f64_p50_p99": [float(np.percentile(rel, 50)), float(np.percentile(rel, 99))] if rel.size else None}


def scene_pipeline_report(args, local, tolerance, dispatch):
    """One collision-world frame on a scene of 2^20 objects (scene_objects,
    seed 11): AABBs, the broad phase update (tree rebuild, pairs, events),
    the gathered narrow-phase batch and query::contact on every pair; then a
    frame of motion.  CPU: the oracle's sort-and-sweep pair set on a 131,072
    object sample (the reference's DBVT is Rust and cannot run here)."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n = args.scene_objects
    b = W.scene_objects(n, seed=11)
    dev = f"cuda:{local}"
    objects = Q.DeviceBatch.from_host(b, device=dev)
    ctx = Q.Context(local, tolerance=tolerance, dispatch=dispatch)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]

    def frame(bp):
        ev[0].record()
        boxes, _ = Q.aabb_batch(ctx, objects)
        ev[1].record()
        pairs, started, stopped = bp.update(boxes)
        ev[2].record()
        db = Q.gather_pairs(ctx, objects, bp.pairs_u32)
        ev[3].record()
        o = Q.contact_batch(ctx, db, 0.0)
        ev[4].record()
        torch.cuda.synchronize()
        return pairs.shape[0], started.shape[0], stopped.shape[0], int(o["has_contact"].sum().item())

    for _ in range(2):  # warm-up (allocations)
        bp = Q.BroadPhase(ctx, 0.05)
        frame(bp)
        bp.close()
    bp = Q.BroadPhase(ctx, 0.05)
    counts0 = frame(bp)
    t0 = [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]
    rng = np.random.default_rng(12)
    moved = W.advance_frame(b, rng, sigma_t=0.02, sigma_r=0.02)
    objects = Q.DeviceBatch.from_host(moved, device=dev)
    counts1 = frame(bp)
    t1 = [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]
    bp.close()
    ctx.close()
    sample = min(131072, n)
    sb = b.subset(np.arange(sample))
    boxes_h, _ = O.aabbs(sb)
    tc = time.perf_counter()
    cpu_pairs = O.intersecting_pairs(boxes_h + np.array([-0.05] * 3 + [0.05] * 3, np.float32))
    cpu_s = time.perf_counter() - tc
    names = ["aabb_ms", "broad_phase_ms", "gather_ms", "contact_ms"]
    return {"workload": f"scene_objects {n} objects (seed 11; ~1.1 box overlaps per object), margin 0.05, "
                        f"contact prediction 0",
            "first_frame": dict(zip(names, t0), pairs=counts0[0], started=counts0[1], contacts=counts0[3],
                                frame_ms=sum(t0)),
            "moved_frame": dict(zip(names, t1), pairs=counts1[0], started=counts1[1], stopped=counts1[2],
                                contacts=counts1[3], frame_ms=sum(t1)),
            "broad_phase_objects_per_s": n / (t1[1] / 1e3),
            "cpu_pair_set_sample": {"objects": sample, "seconds": cpu_s, "pairs": int(cpu_pairs.size),
                                    "method": "oracle sort-and-sweep on x, 1 core (not the reference's DBVT)"}}


def manifold_report(args, local, tolerance):
    """Contact manifolds of 2^20 resting Cuboid pairs (cuboid_stacks, seed 13;
    prediction 0.1, angular tolerances 0.05): the contact query plus the
    manifold step on the GPU, inputs resident; the f32 reference path (oracle:
    contact and manifold) on a 65,536-pair sample with every host core."""
    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n = args.manifold_pairs
    b = W.cuboid_stacks(n, seed=13)
    db = Q.DeviceBatch.from_host(b, device=f"cuda:{local}")
    ctx = Q.Context(local, tolerance=tolerance)
    for _ in range(3):
        o = Q.manifold_batch(ctx, db, 0.1, 0.05, 0.05)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        o = Q.manifold_batch(ctx, db, 0.1, 0.05, 0.05)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    man = o["manifold"].cpu().numpy().view(O.MANIFOLD_DTYPE).reshape(-1)
    ctx.close()
    sample = min(65536, n)
    sb = b.subset(np.arange(sample))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r = O.query(sb, O.CONTACT, O.F32, param=0.1, threads=threads)
    c9 = np.concatenate([r.p1, r.p2, r.dir], 1).astype(np.float32)
    O.manifold(sb, c9, r.tag, linear=0.1, angular1=0.05, angular2=0.05, threads=threads)
    cpu_s = time.perf_counter() - t0
    return {"workload": f"cuboid_stacks {n} pairs, seed 13, prediction 0.1, angular 0.05",
            "pairs_per_s": n / (ms / 1e3), "ms_per_step": ms,
            "contacts_per_pair": float(man["n"].mean()),
            "manifold_size_histogram": np.bincount(man["n"], minlength=9)[:9].tolist(),
            "cpu_reference_path_pairs_per_s": sample / cpu_s, "cpu_cores": threads,
            "cpu_sample": f"first {sample} pairs, f32 reference path (oracle contact and manifold step)",
            "convex_hull_pairs": hull_manifold_report(args, local, tolerance)}


def hull_manifold_report(args, local, tolerance):
    """Contact manifolds of ConvexHull and Cuboid pairs (hull_pairs_pooled:
    2^18 pairs over 4,096 shared shapes of 8..256 points, prediction 0.1,
    angular tolerances 0.05) with the hulls' face topology: the topology build
    (host, once per shape), the GPU call with inputs resident, the manifold
    step bit for bit against the oracle on the GPU's contacts, and the f32
    reference path on a 65,536-pair sample with every host core."""
    import torch
    from ncollide_gb300 import hulls as H
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import workloads as W
    from oracle import oracle as O
    n = 1 << 18
    b = W.hull_pairs_pooled(n, seed=17, pool=4096)
    t0 = time.perf_counter()
    topo = H.HostTopology(b)
    build_s = time.perf_counter() - t0
    dt = topo.to_device(f"cuda:{local}")
    db = Q.DeviceBatch.from_host(b, device=f"cuda:{local}")
    ctx = Q.Context(local, tolerance=tolerance)
    for _ in range(3):
        o = Q.manifold_batch(ctx, db, 0.1, 0.05, 0.05, topology=dt)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        o = Q.manifold_batch(ctx, db, 0.1, 0.05, 0.05, topology=dt)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    man = o["manifold"].cpu().numpy().view(O.MANIFOLD_DTYPE).reshape(-1)
    has = o["has_contact"].cpu().numpy()
    c9 = o["contact"].cpu().numpy()[:, :9].copy()
    st = o["status"].cpu().numpy().view(np.uint32)
    ctx.close()
    want, wst = O.manifold(b, c9, has, linear=0.1, angular1=0.05, angular2=0.05, topology=topo)
    same = np.array_equal(man["n"], want["n"]) and np.array_equal(st & 0x600, wst)
    for k in range(O.MANIFOLD_MAX):
        m = man["n"] > k
        for f in ("world1", "world2", "depth", "feature1", "feature2"):
            same = same and np.array_equal(man["points"][f][m, k], want["points"][f][m, k])
    sample = min(65536, n)
    sb = b.subset(np.arange(sample))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r = O.query(sb, O.CONTACT, O.F32, param=0.1, threads=threads)
    r9 = np.concatenate([r.p1, r.p2, r.dir], 1).astype(np.float32)
    O.manifold(sb, r9, r.tag, linear=0.1, angular1=0.05, angular2=0.05, threads=threads, topology=topo)
    cpu_s = time.perf_counter() - t0
    k = b.shapes["kind"]
    return {"workload": f"hull_pairs_pooled {n} pairs over 4096 shapes (Cuboid, ConvexHull of 8..256 points), seed 17, "
                        "prediction 0.1, angular 0.05",
            "topology_build_s": build_s, "hulls_without_topology": topo.n_failed,
            "hulls": int((k == W.CONVEX_HULL).sum()),
            "pairs_per_s": n / (ms / 1e3), "ms_per_step": ms, "contacts_per_pair": float(man["n"][has == 1].mean()),
            "not_polyhedra_pairs": int(((st & 0x200) != 0).sum()), "manifold_full_pairs": int(((st & 0x400) != 0).sum()),
            "manifold_bit_exact_vs_oracle": bool(same),
            "cpu_reference_path_pairs_per_s": sample / cpu_s, "cpu_cores": threads}


def other_queries_report(args, local, tolerance, db, batch):
    """distance, proximity (margin 0.1) and closest points (prediction 0.1) on
    the headline workload (inputs resident), with the f32 reference path on a
    65,536-pair sample (every host core) and the agreement with f64."""
    import torch
    from ncollide_gb300 import query as Q
    from oracle import oracle as O
    ctx = Q.Context(local, tolerance=tolerance)
    runs = {"distance": (lambda: Q.distance_batch(ctx, db), O.DISTANCE, 0.0),
            "proximity_margin_0.1": (lambda: Q.proximity_batch(ctx, db, 0.1), O.PROXIMITY, 0.1),
            "closest_points_prediction_0.1": (lambda: Q.closest_points_batch(ctx, db, 0.1), O.CLOSEST, 0.1)}
    sample = min(65536, batch.n_pairs)
    sb = batch.subset(np.arange(sample))
    threads = os.cpu_count() or 1
    out = {}
    for name, (fn, q, param) in runs.items():
        for _ in range(3):
            o = fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            o = fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        t0 = time.perf_counter()
        O.query(sb, q, O.F32, param=param, threads=threads)
        cpu_s = time.perf_counter() - t0
        rec = {"pairs_per_s": batch.n_pairs / (ms / 1e3), "ms_per_step": ms,
               "cpu_reference_path_pairs_per_s": sample / cpu_s}
        r64 = O.query(sb, q, O.F64, param=param, threads=threads)
        if q == O.DISTANCE:
            d = o["distance"].cpu().numpy()[:sample].astype(np.float64)
            err = np.abs(d - r64.value) / np.maximum(np.abs(r64.value), sb.scale)
            rec["distance_rel_err_vs_f64_p50_p99_max"] = [float(np.percentile(err, 50)), float(np.percentile(err, 99)),
                                                          float(err.max())]
        else:
            t = (o["proximity"] if q == O.PROXIMITY else o["tag"]).cpu().numpy()[:sample]
            rec["class_mismatch_vs_f64"] = int((t != r64.tag).sum())
        out[name] = rec
    ctx.close()
    out["cpu_sample"] = f"first {sample} pairs, f32 reference path (oracle) on {threads} threads"
    return out


def sharded_report(args, ctx, rank, world, local, batch0, out0):
    """N > 1: rank 0's headline batch split across the ranks by the library's
    cost-balanced shards (ncollide_gb300.shard), each rank's range run on its
    GPU (timed, max over ranks), and the outputs gathered in pair order on rank
    0, which checks them against its own single-GPU call on the whole batch."""
    import torch
    import torch.distributed as dist
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import shard as SH
    batch = batch0 if batch0 is not None else make_workload(0, args.pairs)
    mine, rng = SH.shard(batch, world, rank)
    db = Q.DeviceBatch.from_host(mine, device=f"cuda:{local}")
    for _ in range(2):
        o = Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        o = Q.contact_batch(ctx, db, 0.0)
    e1.record()
    torch.cuda.synchronize()
    t = torch.tensor([e0.elapsed_time(e1) / args.steps], device=f"cuda:{local}")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    local_out = {k: v.cpu().numpy() for k, v in o.items() if v is not None}
    got = SH.gather(local_out, rng, batch.n_pairs)
    if rank != 0:
        return None
    want = {k: v.cpu().numpy() for k, v in out0.items() if v is not None}
    same = all(np.array_equal(got[k], want[k]) for k in want)
    ms = float(t.item())
    return {"pairs": batch.n_pairs, "ranks": world, "ms_per_step_max_over_ranks": ms,
            "pairs_per_s": batch.n_pairs / (ms / 1e3), "scaling": "strong (one batch split by cost)",
            "gathered_equals_single_gpu": bool(same)}


def f32_arithmetic_report(args, local, db, batch, tuning=None):
    """The headline workload in the reference's f32 arithmetic (NCG_ARITH_F32,
    reference tolerances, query dispatch, the headline's launch tuning):
    throughput with inputs resident and every pair bit for bit against the
    oracle's f32 instantiation."""
    import torch
    from ncollide_gb300 import query as Q
    from oracle import oracle as O
    ctx = Q.Context(local, tolerance="reference", dispatch=args.dispatch, arithmetic="f32")
    if tuning:
        ctx.apply_tuning(tuning)
    for _ in range(3):
        o = Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 5
    e0.record()
    for _ in range(n):
        o = Q.contact_batch(ctx, db, 0.0)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    gpu = {k: v.cpu().numpy() for k, v in o.items() if v is not None}
    ctx.close()
    q = O.CONTACT_QUERY if args.dispatch == "query" else O.CONTACT
    return {"workload": "mixed_convex_1M, contact, reference tolerances", "pairs_per_s": batch.n_pairs / (ms / 1e3),
            "ms_per_step": ms, "parity_vs_f32_reference_path": mixed_parity(batch, q, 0.0, "reference", gpu,
                                                                              policy=O.F32)}


def cpu_baseline(batch, threads, query):
    from oracle import oracle as O
    t0 = time.perf_counter()
    O.query(batch, query, O.F32, param=0.0, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": batch.n_pairs / dt, "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"all {batch.n_pairs} pairs of the workload, 1 run, contact f32 reference path "
                      f"(oracle restatement; the Rust reference cannot be built here)", "seconds": dt}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (restated oracle, f32) on host cores."""
    if rank != 0:
        return 0
    from oracle import oracle as O
    batch = make_workload(0)
    threads = os.cpu_count() or 1
    q = O.CONTACT_QUERY if args.dispatch == "query" else O.CONTACT
    sample = batch  # every step is the whole 1,048,576-pair workload (~0.3 s on 16 cores)
    for _ in range(args.warmup):
        O.query(sample, q, O.F32, param=0.0, threads=threads)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.query(sample, q, O.F32, param=0.0, threads=threads)
        ts.append(time.perf_counter() - t0)
    total = sum(ts)
    value = sample.n_pairs * len(ts) / total
    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(ts), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "mixed_convex_1M", "n_pairs": batch.n_pairs, "query": "contact",
                       "dispatch": args.dispatch, "prediction": 0.0, "tolerance": "reference f32 path",
                       "seed": SEED},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": f"all {sample.n_pairs} pairs of the workload every step (contact f32 "
                                       "reference path restated in C++; the Rust reference cannot be built here)"},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tolerance", default="precise", choices=["precise", "reference"])
    ap.add_argument("--dispatch", default="query", choices=["query", "support_map"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--accuracy-sample", type=int, default=32768)
    ap.add_argument("--pairs", type=int, default=N_PAIRS,
                    help="workload size (profiling runs only: the reported config is 1048576 pairs)")
    ap.add_argument("--coherent-pairs", type=int, default=1 << 24,
                    help="pairs of the coherent warm-start workload (the configuration's 16777216 by default)")
    ap.add_argument("--no-coherent", action="store_true")
    ap.add_argument("--mlp-pairs", type=int, default=1 << 22)
    ap.add_argument("--mlp-epochs", type=int, default=20)
    ap.add_argument("--no-mlp", action="store_true")
    ap.add_argument("--stress-pairs", type=int, default=1 << 20)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the precision-stress, cuboid, time-of-impact, ray-cast, scene and manifold reports")
    ap.add_argument("--toi-pairs", type=int, default=1 << 20, help="sweeps of the time-of-impact report")
    ap.add_argument("--ray-count", type=int, default=1 << 20, help="rays of the ray-cast report")
    ap.add_argument("--scene-objects", type=int, default=1 << 20, help="objects of the broad-phase scene report")
    ap.add_argument("--manifold-pairs", type=int, default=1 << 20, help="pairs of the manifold report")
    ap.add_argument("--kernels-only", action="store_true",
                    help="profiling: stop after the timed device steps (no second dispatch, no e2e, no report)")
    ap.add_argument("--tune", action="append", default=[], metavar="KEY=VALUE",
                    help="launch tuning of the headline context (ncg_ctx_set_tuning; e.g. hull_gjk_warp=9); "
                         "overrides the saved tuning")
    ap.add_argument("--autotune", action="store_true",
                    help="run the library's autotuner (ncg_autotune) on the headline batch first and save its "
                         "choice to --tuning-file")
    ap.add_argument("--tuning-file", default=None,
                    help="saved tuning (default: ncollide_gb300/tuning/gb300.json)")
    ap.add_argument("--no-saved-tuning", action="store_true", help="library defaults, not the saved tuning")
    ap.add_argument("--only", choices=["toi", "ray", "scene", "manifold", "stress", "cuboid", "coherent"],
                    help="run one secondary report alone and print it (not a bench line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    from ncollide_gb300 import query as Q
    from ncollide_gb300 import _native as Nn

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.only:
        report = {"toi": lambda: time_of_impact_report(args, local, args.tolerance, args.dispatch),
                  "ray": lambda: ray_cast_report(args, local, args.tolerance),
                  "scene": lambda: scene_pipeline_report(args, local, args.tolerance, args.dispatch),
                  "manifold": lambda: manifold_report(args, local, args.tolerance),
                  "stress": lambda: precision_stress(args, local, args.tolerance),
                  "cuboid": lambda: cuboid_small(args, local, args.tolerance),
                  "coherent": lambda: coherent_warm_start(args, local, args.tolerance,
                                                          float(peaks().get("hbm_gbs", 6800.0)),
                                                          torch.cuda.get_device_properties(local).multi_processor_count
                                                          * 128 * 2 * float(peaks().get("sm_max_mhz", 2070.0)) / 1e6)
                  }[args.only]()
        print(json.dumps({"report": args.only, **report}), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    batch = make_workload(rank, args.pairs)
    db = Q.DeviceBatch.from_host(batch, device=f"cuda:{local}")
    ctx = Q.Context(local, tolerance=args.tolerance, dispatch=args.dispatch)
    from ncollide_gb300 import tuning as TU
    tuning_file = args.tuning_file or TU.DEFAULT_PATH
    props = torch.cuda.get_device_properties(local)
    workload_key = f"mixed_convex_{batch.n_pairs}_contact_{args.dispatch}_{args.tolerance}"
    tuning_source = "library defaults"
    if args.autotune:
        tuned = ctx.autotune(db, "contact", 0.0, reps=3)
        TU.save(props.name, props.multi_processor_count, workload_key, tuned["values"], tuned["ms"],
                extra={"reps": 3, "seed": SEED}, path=tuning_file)
        tuning_source = "ncg_autotune in this run (%.2f ms per call), saved" % tuned["ms"]
    elif not args.no_saved_tuning:
        saved = TU.lookup(props.name, props.multi_processor_count, workload_key, path=tuning_file)
        if saved:
            ctx.apply_tuning(saved)
            tuning_source = "saved ncg_autotune result (%s)" % os.path.relpath(tuning_file, ROOT)
    overrides = dict(kv.split("=", 1) for kv in args.tune)
    for k, v in overrides.items():
        ctx.set_tuning(k, int(v))
    if overrides:
        tuning_source += " + overrides %s" % overrides
    tuning = ctx.tuning()
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        out = Q.contact_batch(ctx, db, 0.0, with_iters=False)
    torch.cuda.synchronize()

    # the timed region holds the product calls alone: no profiling events, no
    # host reads between steps
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            out = Q.contact_batch(ctx, db, 0.0)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1)
    stats = ctx.stats()  # of the last timed step
    launches = stats["kernels_launched"] * args.steps  # the same launches every call
    # stage times from a separate pass with the library's per-stage events
    ctx.set_profiling(True)
    stage_sums = {}
    n_prof = 3
    for _ in range(n_prof):
        Q.contact_batch(ctx, db, 0.0)
        for k, v in ctx.stage_ms().items():
            stage_sums[k] = stage_sums.get(k, 0.0) + v * args.steps / n_prof
    ctx.set_profiling(False)
    if args.kernels_only:
        print(json.dumps({"kernels_only": True, "tuning": tuning, "tuning_source": tuning_source, "pairs": batch.n_pairs, "ms_per_step": ms / args.steps,
                          "stage_ms": {k: v / args.steps for k, v in stage_sums.items()}}), flush=True)
        return 0
    # the other dispatch, same batch (outside the headline's timed region)
    other = "support_map" if args.dispatch == "query" else "query"
    ctx.set_profiling(True)
    ctx.set_dispatch(other)
    for _ in range(2):
        Q.contact_batch(ctx, db, 0.0)
    torch.cuda.synchronize()
    o0 = torch.cuda.Event(enable_timing=True)
    o1 = torch.cuda.Event(enable_timing=True)
    other_stage = {}
    o0.record(stream)
    n_other = max(2, args.steps // 2)
    for _ in range(n_other):
        Q.contact_batch(ctx, db, 0.0)
        for k, v in ctx.stage_ms().items():
            other_stage[k] = other_stage.get(k, 0.0) + v / n_other
    o1.record(stream)
    torch.cuda.synchronize()
    other_ms = o0.elapsed_time(o1) / n_other
    ctx.set_dispatch(args.dispatch)
    ctx.set_profiling(False)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * batch.n_pairs * args.steps / (ms / 1e3)
    sharded = sharded_report(args, ctx, rank, world, local, batch if rank == 0 else None, out) if world > 1 else None

    # ---- e2e through the host entry point (pinned host buffers)
    e2e = None
    if rank == 0 or True:
        import ctypes
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        h = {"shapes": pin(batch.shapes.view(np.uint8)), "hull": pin(batch.hull_points),
             "m1": pin(batch.m1), "g1": pin(batch.g1.view(np.int32)), "m2": pin(batch.m2),
             "g2": pin(batch.g2.view(np.int32))}
        n = batch.n_pairs
        ho = {"contact": torch.empty((n, 10), dtype=torch.float32).pin_memory(),
              "has": torch.empty(n, dtype=torch.uint8).pin_memory(),
              "dir": torch.empty((n, 3), dtype=torch.float32).pin_memory(),
              "status": torch.empty(n, dtype=torch.int32).pin_memory()}
        cb = Nn.NcgBatch(h["shapes"].data_ptr(), h["hull"].data_ptr(), len(batch.shapes), 0,
                         batch.hull_points.shape[0], h["m1"].data_ptr(), h["g1"].data_ptr(), h["m2"].data_ptr(),
                         h["g2"].data_ptr(), n, None)
        L = Nn.load()
        ctx.set_profiling(False)

        def host_step():
            Nn.check(L.ncg_contact_batch_host(ctx.handle, ctypes.byref(cb), ctypes.c_float(0.0),
                                              ho["contact"].data_ptr(), ho["has"].data_ptr(), ho["dir"].data_ptr(),
                                              ho["status"].data_ptr()), "ncg_contact_batch_host")
        for _ in range(2):
            host_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        dt = time.perf_counter() - t0
        h2d = sum(int(v.numel() * v.element_size()) for v in h.values())
        d2h = sum(int(v.numel() * v.element_size()) for v in ho.values())
        e2e = {"value": batch.n_pairs * args.steps / dt, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "api": "ncg_contact_batch_host"}

    # ---- the same call captured once as a CUDA graph (ncg_contact_graph_create)
    # and replayed each step: the per-frame form of a simulation loop
    graph_leg = None
    if rank == 0:
        gr = Q.ContactGraph(ctx, db, 0.0)
        for _ in range(2):
            gr.launch(stream)
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for _ in range(args.steps):
            go = gr.launch(stream)
        g1.record(stream)
        torch.cuda.synchronize()
        g_ms = g0.elapsed_time(g1) / args.steps
        same = all(torch.equal(go[k], out[k]) for k in ("contact", "has_contact", "status", "dir"))
        graph_leg = {"value": batch.n_pairs / (g_ms / 1e3), "unit": "pairs/s", "ms_per_step": g_ms,
                     "kernels_per_replay": ctx.stats()["kernels_launched"], "graph_launches_per_step": 1,
                     "outputs_identical_to_direct_call": bool(same)}
        gr.close()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel
    from oracle import oracle as O  # the checker: counts algorithmic work on a sample
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12  # TFLOP/s
    mean_stage = {k: v / args.steps for k, v in stage_sums.items()}
    dom = max(mean_stage, key=mean_stage.get)
    sample = batch.subset(np.arange(min(65536, batch.n_pairs)))
    rs = O.query(sample, O.CONTACT_QUERY if args.dispatch == "query" else O.CONTACT, O.MIXED, param=0.0,
                 eps=-1.0 if args.tolerance == "precise" else 0.0,
                 epa_tol=1e-6 if args.tolerance == "precise" else 0.0)
    bytes_pp, in_pp, out_pp, flops_pp = algorithmic(batch, rs.counters)
    # algorithmic bytes per unit of the dominant stage: a pair for GJK (inputs
    # read once, outputs written once); an EPA item for the EPA stages (the
    # 160-byte work item, the pair's poses, shape records and indices, the
    # hull points of both shapes read once, and the outputs)
    epa = rs.counters[:, 1] > 0
    hull_pts = (sample.shapes["hull_n"][sample.g1].astype(np.float64) * (sample.shapes["kind"][sample.g1] == 5) +
                sample.shapes["hull_n"][sample.g2].astype(np.float64) * (sample.shapes["kind"][sample.g2] == 5))
    # the thread stage's items: pairs whose hull GJK ran one thread per pair
    # (hull_gjk_warp v >= 2 sends pairs scanning >= 2^v hull points to the warp
    # GJK) and whose EPA starts there (hull_epa_warp v >= 2 starts it in the
    # warp stage for pairs scanning >= 2^v hull points)
    hw, ew = tuning.get("hull_gjk_warp", 0), tuning.get("hull_epa_warp", 0)
    in_thread = epa & ((hull_pts < (1 << hw)) if hw >= 2 else ((hull_pts == 0) if hw == 1 else True))
    if ew >= 2:
        in_thread &= hull_pts < (1 << ew)
    # the warp stage's items: those that start there, and the thread stage's
    # overflow (a 64-vertex store holds about 60 expansion steps)
    in_warp = (epa & ~in_thread) | (in_thread & (rs.counters[:, 1] > 60))

    def item_bytes(m):
        return 160.0 + 136.0 + 61.0 + (16.0 * hull_pts[m].mean() if m.any() else 0.0)
    units, unit_bytes, unit_name = {
        "classify": (batch.n_pairs, 72.0, "pair"),
        "gjk_thread": (batch.n_pairs, bytes_pp, "pair"), "gjk_warp": (batch.n_pairs, bytes_pp, "pair"),
        "epa_thread": (stats["n_epa_thread"], item_bytes(in_thread), "EPA item"),
        "epa_warp": (stats["n_epa_overflow"], item_bytes(in_warp), "EPA item"),
        "epa_wide": (stats["n_epa_overflow"], item_bytes(in_warp), "EPA item")}.get(dom, (batch.n_pairs, bytes_pp, "pair"))
    dom_s = mean_stage[dom] / 1e3
    achieved = units * unit_bytes / dom_s / 1e9
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json"))).get("k_" + dom)
        if tr:
            traffic = {"bytes_per_launch": tr["dram_bytes_per_epa_item"] * units,
                       "bytes_per_unit": tr["dram_bytes_per_epa_item"],
                       "source": tr["source"] + "; scaled by this launch's EPA items"}
    except (OSError, ValueError, KeyError):
        traffic = None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)",
                "traffic": traffic["bytes_per_launch"] if traffic else None, "traffic_detail": traffic,
                "units_per_launch": int(units), "unit_of_work": unit_name, "bytes_per_unit": unit_bytes,
                "mean_launch_ms": mean_stage[dom], "stage_ms": mean_stage,
                "note": "latency-bound: the dominant stage moves far more DRAM bytes than its algorithmic "
                        "bytes (local-memory EPA stores) yet uses a small fraction of the bandwidth",
                "fp32": {"achieved_tflops": batch.n_pairs * flops_pp / (ms / 1e3 / args.steps) / 1e12,
                         "peak_tflops": fp32_peak, "frac": batch.n_pairs * flops_pp / (ms / 1e3 / args.steps) /
                         1e12 / fp32_peak, "flops_per_pair": flops_pp,
                         "note": "whole step, of measured clock peak: SMs x 128 x 2 x max SM clock"}}

    cpu = None
    acc = None
    parity = None
    if not args.no_cpu_baseline:
        qo = O.CONTACT_QUERY if args.dispatch == "query" else O.CONTACT
        cpu = cpu_baseline(batch, os.cpu_count() or 1, qo)
        out_h = {k: v.cpu().numpy() for k, v in out.items() if v is not None}
        acc = accuracy_report(batch, out_h, min(args.accuracy_sample, batch.n_pairs), qo)
        # the last timed step's outputs, every pair, bit for bit
        parity = mixed_parity(batch, qo, 0.0, args.tolerance, out_h)

    stress = cuboids = toi_rep = ray_rep = scene = manifolds = queries = arith32 = None
    if not args.no_extras:
        arith32 = f32_arithmetic_report(args, local, db, batch, tuning)
        queries = other_queries_report(args, local, args.tolerance, db, batch)
        scene = scene_pipeline_report(args, local, args.tolerance, args.dispatch)
        manifolds = manifold_report(args, local, args.tolerance)
        stress = precision_stress(args, local, args.tolerance)
        cuboids = cuboid_small(args, local, args.tolerance)
        toi_rep = time_of_impact_report(args, local, args.tolerance, args.dispatch)
        ray_rep = ray_cast_report(args, local, args.tolerance)
    learned = mlp_params = None
    if not args.no_mlp:
        mlp_params, learned = learned_warm_start(args, local, args.tolerance, args.dispatch, db, batch, tuning)
    coherent = None
    if not args.no_coherent:
        coherent = coherent_warm_start(args, local, args.tolerance, hbm_peak, fp32_peak, mlp_params)

    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "mixed_convex_1M", "n_pairs": batch.n_pairs, "query": "contact",
                       "dispatch": args.dispatch, "prediction": 0.0, "tolerance": args.tolerance,
                       "warm_start": "none (plain)",
                       "seed": SEED, "parallelism": f"weak x{world}" if world > 1 else "1 GPU",
                       "l2": "inputs larger than L2 (%.2f GB resident)" % (batch.nbytes_inputs() / 1e9),
                       "tuning": tuning, "tuning_source": tuning_source},
            "clocks": clocks.summary(), "e2e": e2e, "gpu_launches": launches, "cuda_graph_replay": graph_leg,
            "roofline": roofline, "cpu_baseline": cpu, "parity_vs_oracle": parity, "accuracy_vs_f64": acc,
            "warm_start_coherent": coherent,
            "warm_start_learned": learned,
            "precision_stress": stress, "cuboid_pairs_65536": cuboids, "time_of_impact": toi_rep, "ray_cast": ray_rep, "scene_pipeline": scene, "manifolds": manifolds, "other_queries": queries,
            "other_dispatch": {"dispatch": other, "value": batch.n_pairs / (other_ms / 1e3), "ms_per_step": other_ms,
                               "stage_ms": other_stage},
            "sharded_headline_batch": sharded, "f32_arithmetic": arith32,
            "epa": {"pairs": stats["n_epa"], "warp_stage_pairs": stats["n_epa_overflow"],
                    "gjk_iters_per_pair": stats["gjk_iters"] / batch.n_pairs,
                    "epa_iters_per_epa_pair": stats["epa_iters"] / max(1, stats["n_epa"])}}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
