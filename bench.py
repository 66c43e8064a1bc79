"""E-step throughput benchmark on synthetic particles.

One step = one local particle-filter phase over a batch of particles at the
production configuration (256^3 map, 1.1 A/px, 200 blobs, cutoff 80 Fourier
pixels -> K = 9,930, padding 2, 1,000 rotations x 100 translations per
particle): projection of every particle's rotations, phase-shifted weighted
data, likelihood of every hypothesis, marginal weights, and narrowing +
systematic resampling of the rotation and translation sets.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|bf16x3]
  python bench.py --impl reference ...   # the CPU path timed on the host cores

Prints one JSON line (rank 0).  Under torchrun each rank drives its own GPU
with its own particles (weak scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "thunder-refactor-expectation_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "E-step particles/sec, box 256: learned+BF16 vs plain FP32 GPU at equal pose error"
UNIT = "particles/s"
WORKLOAD = dict(box=256, pixel_size=1.1, n_blobs=200, sigma_a=(1.5, 3.0), radius_px=80.0,
                shift=8.0, snr=0.03, rU=80, pf=2, nR=1000, nT=100, kappa=200.0,
                n_classes=1, shared=1.0)
# the same local phase with 3 classes whose maps share 70 % of their blobs
# (the other 30 % re-drawn per class, particles split 1:1:1) at cutoff 120
WORKLOAD_C3 = dict(WORKLOAD, rU=120, n_classes=3, shared=0.7)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


# ---------------------------------------------------------------- clocks ----
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- workload ---
def make_workload(torch, dev, nP, n_batches, seed, box=None, W0=None):
    """Synthetic class maps + particle batches, generated on the GPU."""
    from tg3 import synth
    W = dict(WORKLOAD if W0 is None else W0)
    if box is not None:          # reduced case for profiling captures
        scale = box / W["box"]
        W.update(box=box, rU=max(8, int(W["rU"] * scale)), radius_px=W["radius_px"] * scale)
    rng = np.random.default_rng(seed)
    maps = synth.class_maps(rng, W["n_classes"], W["shared"], W["n_blobs"], W["sigma_a"],
                            W["pixel_size"], W["radius_px"])
    vols = [synth.padded_volume(bm, W["box"], W["pf"], device=dev, dtype=torch.float32)
            for bm in maps]
    rL = synth.config_rL(W["box"], W["pixel_size"])
    n = nP * n_batches
    st = synth.make_stack(seed + 1, maps, W["box"], W["pixel_size"], W["pf"], W["rU"], rL, n,
                          W["shift"], W["snr"], device=dev)
    qc, tc = synth.perturb_poses(rng, st.quat_true, st.trans_true, 3.0, 1.0)
    qs, ts = synth.local_hypotheses(rng, qc, tc, W["nR"], W["nT"], W["kappa"], 2.0)
    nR, nT = W["nR"], W["nT"]
    batches = []
    for b in range(n_batches):
        sl = slice(b * nP, (b + 1) * nP)
        perm_r = np.stack([rng.permutation(nR) for _ in range(nP)]).astype(np.int32)
        perm_t = np.stack([rng.permutation(nT) for _ in range(nP)]).astype(np.int32)
        host = dict(
            dat=np.ascontiguousarray(st.dat[sl].astype(np.complex64)),
            ctf=np.ascontiguousarray(st.ctf[sl].astype(np.float32)),
            sig=np.ascontiguousarray(st.sigRcp[sl].astype(np.float32)),
            quat=np.ascontiguousarray(qs[sl]), trans=np.ascontiguousarray(ts[sl]),
            pwR=np.full((nP, nR), 1.0 / nR), pwT=np.full((nP, nT), 1.0 / nT), pwC=np.ones(nP),
            cls=np.ascontiguousarray(st.cls_true[sl].astype(np.int32)),
            q_true=np.ascontiguousarray(st.quat_true[sl]),
            perm_r=perm_r, perm_t=perm_t,
            u0_r=rng.random(nP) / nR, u0_t=rng.random(nP) / nT,
            peak_r=np.full(nP, np.nan), peak_t=np.zeros(nP))
        batches.append(host)
    return W, vols, st, batches


def to_dev(torch, dev, host):
    return {k: torch.as_tensor(v).to(dev).contiguous() for k, v in host.items()}


def pin(torch, host):
    out = {}
    for k, v in host.items():
        t = torch.as_tensor(v)
        out[k] = t.pin_memory() if torch.cuda.is_available() else t
    return out


# ---------------------------------------------------------------- tg3 arm ---
def fp32_sgemm_peak(torch, dev):
    """cuBLAS FP32 SGEMM (TF32 off) throughput, the CUDA-core denominator."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, device=dev)
    b = torch.randn(8192, 8192, device=dev)
    for _ in range(3):
        a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e9
    for _ in range(5):
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = prev
    return 2 * 8192 ** 3 / (best * 1e-3) / 1e12


def run_tg3(args, rank, world, local_rank):
    import torch
    import tg3

    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    nP = args.batch
    W0 = WORKLOAD_C3 if args.workload == "local256c3" else WORKLOAD
    W, vols, st, batches = make_workload(torch, dev, nP, args.batches, rank_seed(1001, rank),
                                         box=args.box, W0=W0)
    nR, nT, K = W["nR"], W["nT"], st.K
    ctx = tg3.Context(local_rank)
    ctx.set_option(tg3.OPT_LOCAL_BK, args.local_bk)
    ctx.set_option(tg3.OPT_PROJECT_FORM, args.project_form)
    ctx.set_option(tg3.OPT_PROJECT_GROUP, args.project_group)
    if args.fused:
        ctx.set_option(tg3.OPT_FUSED, 1)
    for c, v in enumerate(vols):
        ctx.set_volume(c, v, W["pf"])
    ctx.set_pixels(st.iCol, st.iRow, W["box"])
    del vols
    dbat = [to_dev(torch, dev, b) for b in batches]
    out = dict(wC=torch.empty(nP, dtype=torch.float64, device=dev),
               wR=torch.empty((nP, nR), dtype=torch.float64, device=dev),
               wT=torch.empty((nP, nT), dtype=torch.float64, device=dev),
               base=torch.empty(nP, dtype=torch.float64, device=dev),
               src_r=torch.empty((nP, nR), dtype=torch.int32, device=dev),
               src_t=torch.empty((nP, nT), dtype=torch.int32, device=dev),
               w_r=torch.empty((nP, nR), dtype=torch.float64, device=dev),
               w_t=torch.empty((nP, nT), dtype=torch.float64, device=dev),
               top=torch.empty(nP, dtype=torch.int32, device=dev))
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step(i, prec):
        b = dbat[i % len(dbat)]
        ctx.local_phase(nP, nR, nT, b["dat"], b["ctf"], b["sig"], b["quat"], b["trans"],
                        b["pwR"], b["pwT"], b["pwC"], b["cls"], out["wC"], out["wR"], out["wT"],
                        out["base"], None, prec)
        ctx.resample(nP, nR, out["wR"], b["pwR"], b["perm_r"], b["u0_r"], b["peak_r"], nR,
                     out["src_r"], out["w_r"], out["top"])
        ctx.resample(nP, nT, out["wT"], b["pwT"], b["perm_t"], b["u0_t"], b["peak_t"], nT,
                     out["src_t"], out["w_t"], out["top"])

    def timed(prec):
        """W warm-up steps, then exactly K timed steps between barriers and
        device synchronisations, CUDA events on the library's stream."""
        for i in range(args.warmup):
            step(i, prec)
        ctx.sync()
        barrier(world)
        torch.cuda.synchronize()
        clk = ClockSampler(local_rank)
        clk.start()
        ctx.set_timing(True)
        ctx.stage_times(reset=True)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for i in range(args.steps):
                step(i, prec)
            ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        barrier(world)
        clocks = clk.stop()
        stages = ctx.stage_times(reset=True)
        ctx.set_timing(False)
        ctx.sync()
        return reduce_max(world, ev0.elapsed_time(ev1)), stages, clocks

    def best_rotations(prec_):
        """Best rotation (argmax of the marginal wR) of every particle of
        batch 0, and its angle to the particle's true pose in degrees."""
        step(0, prec_)
        ctx.sync()
        best = out["wR"].argmax(1).cpu().numpy()
        q = batches[0]["quat"][np.arange(nP), best]
        dot = np.abs((q * batches[0]["q_true"]).sum(1)).clip(0.0, 1.0)
        return best, np.degrees(2.0 * np.arccos(dot))

    prec = tg3.SCORE_BF16X3 if args.precision == "bf16x3" else tg3.SCORE_FP32
    ms, stages, clocks = timed(prec)
    plain = None
    if prec != tg3.SCORE_FP32 and not args.no_compare:
        ms_p, stages_p, clocks_p = timed(tg3.SCORE_FP32)
        plain = (ms_p, stages_p, clocks_p)
    best_m, ang_m = best_rotations(prec)
    pose = {"particles": nP, f"median_deg_{args.precision}": round(float(np.median(ang_m)), 4)}
    if prec != tg3.SCORE_FP32:
        best_p, ang_p = best_rotations(tg3.SCORE_FP32)
        pose.update(median_deg_fp32=round(float(np.median(ang_p)), 4),
                    same_best_rotation=round(float(np.mean(best_m == best_p)), 4))
    pose["note"] = ("best local rotation (argmax of the marginal weights) against the true pose "
                    "of the synthetic particle")

    # ---- insertion of every particle's best pose (MKB kernel), timed alone
    ctx.insert_begin(W["pf"] * W["box"], W["pf"])
    ins_w = torch.ones(nP, dtype=torch.float32, device=dev)
    zero2 = torch.zeros((nP, 2), dtype=torch.float64, device=dev)
    ins_q = [b["quat"][:, 0, :].contiguous() for b in dbat]
    ins_t = [b["trans"][:, 0, :].contiguous() for b in dbat]

    def time_insert(gather):
        # pixel-order scatter form (the default) or the voxel gather form
        ctx.set_option(tg3.OPT_INSERT_GATHER, gather)
        for i in range(2):
            ctx.insert(nP, dbat[i % len(dbat)]["dat"], dbat[i % len(dbat)]["ctf"],
                       ins_q[i % len(dbat)], ins_t[i % len(dbat)], zero2, ins_w, tg3.KERNEL_MKB)
        ctx.sync()
        ctx.set_timing(True)
        ctx.stage_times(reset=True)
        for i in range(args.steps):
            ctx.insert(nP, dbat[i % len(dbat)]["dat"], dbat[i % len(dbat)]["ctf"],
                       ins_q[i % len(dbat)], ins_t[i % len(dbat)], zero2, ins_w, tg3.KERNEL_MKB)
        stage = ctx.stage_times(reset=True)["insert"]
        ctx.set_timing(False)
        ctx.sync()
        ctx.set_option(tg3.OPT_INSERT_GATHER, 0)
        return stage

    ins_stage = time_insert(0)
    ins_gather = time_insert(1)

    # ---- end to end: host buffers, copies inside the timed region
    hbat = [pin(torch, b) for b in batches]
    hout = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in out.items()}
    inputs = ("dat", "ctf", "sig", "quat", "trans", "pwR", "pwT", "pwC", "cls")
    h2d = sum(hbat[0][k].numel() * hbat[0][k].element_size() for k in inputs)
    h2d += sum(hbat[0][k].numel() * hbat[0][k].element_size()
               for k in ("perm_r", "perm_t", "u0_r", "u0_t", "peak_r", "peak_t", "pwR", "pwT"))
    d2h = sum(hout[k].numel() * hout[k].element_size()
              for k in ("wC", "wR", "wT", "base", "src_r", "src_t", "w_r", "w_t", "top"))

    def e2e_step(i):
        b = hbat[i % len(hbat)]
        ctx.local_phase_host(nP, nR, nT, b["dat"], b["ctf"], b["sig"], b["quat"], b["trans"],
                             b["pwR"], b["pwT"], b["pwC"], b["cls"], hout["wC"], hout["wR"],
                             hout["wT"], hout["base"], None, prec)
        tg3.check(tg3.lib().tg3_resample(nP, nR, tg3.ptr(hout["wR"]), tg3.ptr(b["pwR"]),
                                         tg3.ptr(b["perm_r"]), tg3.ptr(b["u0_r"]),
                                         tg3.ptr(b["peak_r"]), nR, tg3.ptr(hout["src_r"]),
                                         tg3.ptr(hout["w_r"]), tg3.ptr(hout["top"])))
        tg3.check(tg3.lib().tg3_resample(nP, nT, tg3.ptr(hout["wT"]), tg3.ptr(b["pwT"]),
                                         tg3.ptr(b["perm_t"]), tg3.ptr(b["u0_t"]),
                                         tg3.ptr(b["peak_t"]), nT, tg3.ptr(hout["src_t"]),
                                         tg3.ptr(hout["w_t"]), tg3.ptr(hout["top"])))

    for i in range(2):
        e2e_step(i)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.e2e_steps):
        e2e_step(i)
    torch.cuda.synchronize()
    e2e_s = reduce_max(world, time.perf_counter() - t0)
    barrier(world)

    hbm, bf16, kind = peaks()
    fp32_peak = fp32_sgemm_peak(torch, dev)

    def per_launch(st_, name):
        t, n = st_[name]
        return t / max(n, 1)

    flop = 4.0 * K * nR * nT * nP          # real part of the complex cross term
    proj_bytes = 72.0 * nR * K * nP        # 8 corners x 8 B read + 8 B written per sample

    def cross_roof(st_, p_):
        ach = flop / (per_launch(st_, "cross") * 1e-3) / 1e12
        if p_ == tg3.SCORE_FP32:
            pk, note = fp32_peak, "cuBLAS FP32 SGEMM (TF32 off) measured live in this run"
        else:
            pk, note = bf16, f"bf16 dense tensor burst, {kind} (MEASURED_PEAKS.json)"
        return {"kernel": "k_gemm_nt_fp32" if p_ == tg3.SCORE_FP32 else "k_gemm_bf16x3 (tcgen05)",
                "bound": "tensor", "achieved": round(ach, 2), "peak": round(pk, 1),
                "unit": "TFLOP/s", "frac": round(ach / pk, 4), "peak_source": note,
                "traffic": traffic("cross_bf16x3" if p_ != tg3.SCORE_FP32 else "cross_fp32",
                                   W["box"], nP),
                "algorithmic_flop_per_launch": flop,
                "executed_bf16_flop_per_launch": 3 * flop if p_ != tg3.SCORE_FP32 else None}

    def proj_roof(st_):
        ach = proj_bytes / (per_launch(st_, "project") * 1e-3) / 1e9
        return {"kernel": "k_project", "bound": "hbm", "achieved": round(ach, 1),
                "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
                "peak_source": f"hbm_gbs, {kind} (MEASURED_PEAKS.json)",
                "traffic": traffic("project", W["box"], nP),
                "traffic_note": "DRAM bytes per launch (ncu); below the algorithmic bytes "
                                "because L2 serves the volume blocks a pixel band reuses",
                "algorithmic_bytes_per_launch": proj_bytes}

    def fused_roof(st_):
        """k_fused_bf16x3: the gather bound (64 B of corners per sample, no
        slice written), with the tensor rate of the same launch beside it."""
        t = per_launch(st_, "fused") * 1e-3
        fb = 64.0 * nR * K * nP
        ach = fb / t / 1e9
        return {"kernel": "k_fused_bf16x3 (gather + tcgen05)", "bound": "hbm",
                "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(ach / hbm, 4),
                "peak_source": f"hbm_gbs, {kind} (MEASURED_PEAKS.json)",
                "traffic": traffic("fused", W["box"], nP),
                "algorithmic_bytes_per_launch": fb,
                "tensor": {"achieved_tflops": round(flop / t / 1e12, 2), "peak": round(bf16, 1),
                           "frac": round(flop / t / 1e12 / bf16, 4),
                           "algorithmic_flop_per_launch": flop,
                           "executed_bf16_flop_per_launch": 3 * flop}}

    fused = stages.get("fused", (0.0, 0))[1] > 0
    if fused:
        roof = fused_roof(stages)
    else:
        dominant = max(("project", "cross"), key=lambda k: per_launch(stages, k))
        roof = proj_roof(stages) if dominant == "project" else cross_roof(stages, prec)
    # kernels of one step: shift, x0, rotation matrices, 2 x resample, weights, plus
    # fused: descriptors + the fused kernel; else: projection, norm sum, cross term
    launches_per_step = 8 if fused else 9
    ins_ms = ins_stage[0] / max(ins_stage[1], 1)
    ins_ga_ms = ins_gather[0] / max(ins_gather[1], 1)
    ins_bytes = 705.5 * K * nP             # 16 B in + 28.7 voxel updates x 24 B per pixel
    value = job_rate(nP * args.steps, ms, world)
    res = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32" if prec == tg3.SCORE_FP32 else "bf16x3 cross term, fp32 elsewhere",
        "data": "synthetic (seeded Gaussian-blob map and particles, generated on the GPU)",
        "config": {"workload": f"local particle-filter phase, box {W['box']}, K={K}, "
                               f"{nR} rotations x {nT} translations per particle"
                               + (f", {W['n_classes']} classes sharing "
                                  f"{round(100 * W['shared'])} % of their blobs, particles "
                                  "split evenly" if W["n_classes"] > 1 else ""),
                   "box": W["box"], "pf": W["pf"], "K": K, "nR": nR, "nT": nT,
                   "classes": W["n_classes"], "particles_per_step": nP,
                   "precision": args.precision, "projection_form": args.project_form,
                   "projection_group": args.project_group,
                   "l2": "inputs larger than L2: the projection bank alone is "
                         f"{nP * nR * ctx_kp(K) * 4 / 1e9:.1f} GB per step"},
        "clocks": clocks,
        "e2e": {"value": round(job_rate(nP * args.e2e_steps, e2e_s * 1e3, world), 2), "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "wall_s": round(e2e_s, 3)},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roof,
        "roofline_cross_term": None if fused else cross_roof(stages, prec),
        "roofline_projection": None if fused else proj_roof(stages),
        "stages": {k: {"ms_per_launch": round(v[0] / max(v[1], 1), 4), "launches": v[1]}
                   for k, v in stages.items() if v[1]},
        "insertion": {"kernel": "k_insert (MKB, a = 1.9, alpha = 15)",
                      "particles": nP,
                      "ms_per_launch": round(ins_ms, 4),
                      "particles_per_s": round(nP / (ins_ms * 1e-3), 1),
                      "achieved_gbs": round(ins_bytes / (ins_ms * 1e-3) / 1e9, 1),
                      "peak_gbs": hbm, "frac": round(ins_bytes / (ins_ms * 1e-3) / 1e9 / hbm, 4),
                      "algorithmic_bytes": "705.5 B per inserted pixel (16 B in + 28.73 "
                                           "voxel updates x 24 B)",
                      "gather_form": {"kernel": "k_insert_stage + k_insert_gather",
                                      "ms_per_launch": round(ins_ga_ms, 4),
                                      "particles_per_s": round(nP / (ins_ga_ms * 1e-3), 1)}},
        "hypotheses_per_s": round(value * nR * nT, 1),
        "pose": pose,
    }
    if plain is not None:
        ms_p, stages_p, clocks_p = plain
        v_p = job_rate(nP * args.steps, ms_p, world)
        res["plain_fp32"] = {"value": round(v_p, 2), "ms_per_step": round(ms_p / args.steps, 4),
                             "stages": {k: round(v[0] / max(v[1], 1), 4)
                                        for k, v in stages_p.items() if v[1]},
                             "roofline_cross_term": cross_roof(stages_p, tg3.SCORE_FP32),
                             "clocks": clocks_p}
        res["speedup_vs_plain_fp32"] = round(value / v_p, 3)
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(st, batches[0], W, args.cpu_sample)
    ctx.close()
    return res


def run_global(args, rank, world, local_rank):
    """Global scan of the CPU-runnable configuration: 64^3 map, 1.5 A/px, 40
    blobs, 2,000 particles, 6,912 rotations (HEALPix nside 4 x 36 in-plane) x
    49 translations (7 x 7, 1 px), cutoff 16 -> K = 375."""
    import torch
    import tg3
    from tg3 import synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    box, px, pf, rU, n = 64, 1.5, 2, 16, args.global_particles
    rng = np.random.default_rng(rank_seed(1000, rank))
    bm = synth.blob_map(rng, 40, (2.0, 4.0), px, 20.0)
    vol = synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32)
    st = synth.make_stack(rank_seed(1001, rank), [bm], box, px, pf, rU, synth.config_rL(box, px), n,
                          3.0, 0.05, device=dev)
    quats = synth.global_rotations(4, 36)
    mats = torch.as_tensor(synth.quat_to_mat(quats).reshape(-1, 9)).to(dev)
    trans = torch.as_tensor(synth.global_translations(3, 1.0)).to(dev)
    nR, nT, K = len(quats), 49, st.K
    ctx = tg3.Context(local_rank)
    ctx.set_volume(0, vol, pf)
    ctx.set_pixels(st.iCol, st.iRow, box)
    d = dict(dat=torch.as_tensor(st.dat.astype(np.complex64)).to(dev),
             ctf=torch.as_tensor(st.ctf.astype(np.float32)).to(dev),
             sig=torch.as_tensor(st.sigRcp.astype(np.float32)).to(dev),
             pR=torch.full((nR,), 1.0 / nR, dtype=torch.float64, device=dev),
             pT=torch.full((nT,), 1.0 / nT, dtype=torch.float64, device=dev))
    o = dict(wC=torch.empty(n, dtype=torch.float64, device=dev),
             wR=torch.empty((n, nR), dtype=torch.float64, device=dev),
             wT=torch.empty((n, nT), dtype=torch.float64, device=dev),
             base=torch.empty(n, dtype=torch.float64, device=dev))
    prec = tg3.SCORE_BF16X3 if args.precision == "bf16x3" else tg3.SCORE_FP32

    def step():
        ctx.global_scan(0, n, nR, nT, d["dat"], d["ctf"], d["sig"], mats, trans, d["pR"], d["pT"],
                        o["wC"], o["wR"], o["wT"], o["base"], None, prec)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    clk = ClockSampler(local_rank)
    clk.start()
    ctx.set_timing(True)
    ctx.stage_times(reset=True)
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    clocks = clk.stop()
    stages = ctx.stage_times(reset=True)
    ms = reduce_max(world, e0.elapsed_time(e1)) / args.steps
    cross = stages["cross"][0] / max(stages["cross"][1], 1)
    flop = 4.0 * K * nR * nT * n
    hbm, bf16, kind = peaks()
    res = {"metric": "global scan particles/s, box 64, 6912 rotations x 49 translations, K=375",
           "value": round(job_rate(n, ms, world), 1), "unit": UNIT, "ms_per_step": round(ms, 3),
           "n_gpus": world, "scaling": "weak",
           "particles": n, "precision": args.precision, "clocks": clocks,
           "hypotheses_per_s": round(job_rate(n * nR * nT, ms, world), 1),
           "stages": {k: round(v[0] / max(v[1], 1), 4) for k, v in stages.items() if v[1]},
           "cross_term": {"achieved_tflops": round(flop / (cross * 1e-3) / 1e12, 1),
                          "note": "algorithmic 4 K FLOP per hypothesis; the stage also "
                                  "holds the per-image norm GEMM"}}
    ctx.close()
    return res


CLASS2D = dict(box=128, pixel_size=1.4, pf=2, rU=24, n_classes=16, n_blobs=80,
               sigma_a=(1.5, 3.0), radius_px=40.0, nR=72, half_t=3, snr=0.1)


def run_class2d(args, rank, world, local_rank):
    """2-D classification's global search (ExpectGlobal2D, Optimiser's 2-D
    expectation): 16 class images (box 128, padded 2x, central sections of
    blob maps), 2,000 particles per step, 72 in-plane rotations (5 degrees)
    x 49 translations (7 x 7, 1 px), cutoff 24 px; all classes scored in one
    pass and merged, each particle's class read from the merged weights."""
    import torch
    import tg3
    from tg3 import synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    W = CLASS2D
    box, px, pf, n, nK, nR = W["box"], W["pixel_size"], W["pf"], args.global_particles, \
        W["n_classes"], W["nR"]
    rng = np.random.default_rng(rank_seed(3000, rank))
    maps = [synth.blob_map(rng, W["n_blobs"], W["sigma_a"], px, W["radius_px"]) for _ in range(nK)]
    imgs = synth.class_images_2d(maps, box, pf, device=dev)
    iCol, iRow = synth.pixel_index(box, W["rU"], synth.config_rL(box, px))[:2]
    K = len(iCol)
    ang = np.arange(nR) * (2 * np.pi / nR)
    rot_np = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    trans_np = np.ascontiguousarray(synth.global_translations(W["half_t"], 1.0))
    nT = len(trans_np)
    rot, trans = torch.as_tensor(rot_np).to(dev), torch.as_tensor(trans_np).to(dev)
    # particles: class, rotation and translation drawn from the grids, CTF, noise
    kt = torch.as_tensor(rng.integers(0, nK, n)).to(dev)
    rt, tt = rng.integers(0, nR, n), rng.integers(0, nT, n)
    attr = synth.ctf_attrs(rng, n)
    ctf_np = synth.ctf_values(attr, px, box, iCol, iRow).astype(np.float32)
    clean = synth.sample_2d(imgs, kt, rot[torch.as_tensor(rt).to(dev)], iCol, iRow, pf)
    clean = clean * torch.as_tensor(synth.phase_shift(trans_np[tt], box, iCol, iRow)).to(dev) \
        .to(torch.complex64) * torch.as_tensor(ctf_np).to(dev)
    s2 = float((clean.abs() ** 2).mean()) / W["snr"] / 2
    gen = torch.Generator(device=dev).manual_seed(rank_seed(3001, rank))
    noise = torch.complex(torch.randn(clean.shape, generator=gen, device=dev),
                          torch.randn(clean.shape, generator=gen, device=dev)) * math.sqrt(s2)
    dat = (clean + noise).contiguous()
    ctf = torch.as_tensor(ctf_np).to(dev)
    sig = torch.full((n, K), -1.0 / (2 * s2), dtype=torch.float32, device=dev)
    pR = torch.full((nR,), 1.0 / nR, dtype=torch.float64, device=dev)
    pT = torch.full((nT,), 1.0 / nT, dtype=torch.float64, device=dev)
    o = dict(wC=torch.empty((n, nK), dtype=torch.float32, device=dev),
             wR=torch.empty((n, nK, nR), dtype=torch.float32, device=dev),
             wT=torch.empty((n, nK, nT), dtype=torch.float32, device=dev),
             base=torch.empty(n, dtype=torch.float32, device=dev))
    ctx = tg3.Context(local_rank)
    ctx.set_pixels(iCol, iRow, box)
    prec = tg3.SCORE_BF16X3 if args.precision == "bf16x3" else tg3.SCORE_FP32

    def step(p=prec):
        # every class in one pass, merged over the classes (ExpectGlobal2D's outputs)
        ctx.global_scan2d_classes(imgs, pf, n, nR, nT, dat, ctf, sig, rot, trans, pR, pT,
                                  o["wC"], o["wR"], o["wT"], o["base"], p)

    stream = torch.cuda.ExternalStream(ctx.stream)

    def timed(fn, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        barrier(world)
        return reduce_max(world, e0.elapsed_time(e1)) / steps

    for _ in range(args.warmup):
        step()
    ctx.sync()
    clk = ClockSampler(local_rank)
    clk.start()
    ctx.set_timing(True)
    ctx.stage_times(reset=True)
    ms = timed(step, args.steps)
    stages = ctx.stage_times(reset=True)
    ctx.set_timing(False)
    clocks = clk.stop()
    # each particle's class: the one with the largest merged class weight
    best = o["wC"].argmax(1)
    recovered = float((best == kt).float().mean())
    ms_fp32 = None
    if prec != tg3.SCORE_FP32 and not args.no_compare:
        step(tg3.SCORE_FP32)
        ctx.sync()
        ms_fp32 = timed(lambda: step(tg3.SCORE_FP32), max(3, args.steps // 4))
    # end to end through the reference-shaped entry (ExpectGlobal2D; FP32
    # scoring, host buffers, all classes in one pass per batch of 1,024):
    # class images, particles and weights cross the host link every call
    host = dict(vol=imgs.cpu().numpy(), dat=dat.cpu().numpy(), ctf=ctf_np,
                sig=sig.cpu().numpy())
    host = {k: np.ascontiguousarray(v) for k, v in host.items()}
    wCh = np.zeros(n * nK, np.float32)
    wRh = np.zeros(n * nK * nR, np.float32)
    wTh = np.zeros(n * nK * nT, np.float32)
    pRh, pTh = np.full(nR, 1.0 / nR), np.full(nT, 1.0 / nT)
    ic, ir = np.ascontiguousarray(iCol, np.int32), np.ascontiguousarray(iRow, np.int32)

    def e2e():
        tg3.check(tg3.lib().tg3_ExpectGlobal2D(
            tg3.ptr(host["vol"]), tg3.ptr(host["dat"]), tg3.ptr(host["ctf"]), tg3.ptr(host["sig"]),
            tg3.ptr(trans_np), tg3.ptr(wCh), tg3.ptr(wRh), tg3.ptr(wTh), tg3.ptr(pRh),
            tg3.ptr(pTh), tg3.ptr(rot_np), tg3.ptr(ic), tg3.ptr(ir), nK, nR, nT, pf, 1, box,
            pf * box, K, n))

    e2e()
    barrier(world)
    t0 = time.perf_counter()
    e2e_steps = max(1, args.e2e_steps // 2)
    for _ in range(e2e_steps):
        e2e()
    e2e_ms = reduce_max(world, (time.perf_counter() - t0) * 1e3) / e2e_steps
    e2e_rec = float((wCh.reshape(n, nK).argmax(1) == kt.cpu().numpy()).mean())
    # 2-D insertion through the reference-shaped entry (InsertI2D): every
    # particle's best (class, rotation, translation) into its class's
    # accumulators, host volumes in and out, as the reference's call
    best_k = wCh.reshape(n, nK).argmax(1).astype(np.int32)
    wRb = wRh.reshape(n, nK, nR)[np.arange(n), best_k]
    wTb = wTh.reshape(n, nK, nT)[np.arange(n), best_k]
    nRd = np.ascontiguousarray(rot_np[wRb.argmax(1)])
    nTd = np.ascontiguousarray(trans_np[wTb.argmax(1)])
    vdim = pf * box
    F2 = np.zeros((nK, vdim, vdim // 2 + 1), np.complex64)
    T2 = np.zeros((nK, vdim, vdim // 2 + 1), np.float32)
    O2 = np.zeros((nK, 2))
    cnt = np.zeros(nK, np.int32)
    wl = np.ones(n, np.float32)
    offS = np.zeros((n, 2))
    icp, irp = np.ascontiguousarray(ic * pf), np.ascontiguousarray(ir * pf)

    def insert2d():
        tg3.check(tg3.lib().tg3_InsertI2D(
            tg3.ptr(F2), tg3.ptr(T2), tg3.ptr(O2), tg3.ptr(cnt), tg3.ptr(host["dat"]),
            tg3.ptr(host["ctf"]), tg3.ptr(host["sig"]), tg3.ptr(wl), tg3.ptr(offS),
            tg3.ptr(best_k), tg3.ptr(nRd), tg3.ptr(nTd), None, None, tg3.ptr(icp), tg3.ptr(irp),
            px, 0, nK, pf, K, 1, box, vdim, n))

    insert2d()
    t0 = time.perf_counter()
    for _ in range(3):
        insert2d()
    ins_ms = (time.perf_counter() - t0) * 1e3 / 3
    # roofline of the scoring GEMM (the "cross" stage: 4 K FLOP per hypothesis)
    cross = stages["cross"][0] / max(stages["cross"][1], 1)
    flop = 4.0 * K * nK * nR * nT * n
    hbm, bf16, kind = peaks()
    achieved = flop / (cross * 1e-3) / 1e12
    res = {"metric": "2-D classification global search particles/s, box 128, 16 classes x "
                     "72 rotations x 49 translations, K=%d" % K,
           "value": round(job_rate(n, ms, world), 1), "unit": UNIT, "ms_per_step": round(ms, 3),
           "n_gpus": world, "scaling": "weak", "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "dtype": "f32" if prec == tg3.SCORE_FP32 else "bf16x3",
           "data": "synthetic: central sections of blob maps, CTF, Gaussian noise",
           "config": {"workload": "class2d128", "particles": n, "classes": nK, "nR": nR,
                      "nT": nT, "K": K, "l2": "inputs stay resident (scored once per class)"},
           "precision": args.precision, "clocks": clocks,
           "class_recovered": round(recovered, 4),
           "hypotheses_per_s": round(job_rate(n * nK * nR * nT, ms, world), 1),
           "fp32_value": None if ms_fp32 is None else round(job_rate(n, ms_fp32, world), 1),
           "stages": {k: round(v[0] / max(v[1], 1), 4) for k, v in stages.items() if v[1]},
           "roofline": {"bound": "tensor", "kernel": "cross-term GEMM",
                        "achieved": round(achieved, 1), "peak": bf16, "unit": "TFLOP/s",
                        "frac": round(achieved / bf16, 4), "peak_kind": kind, "traffic": None},
           "e2e": {"value": round(job_rate(n, e2e_ms, world), 1), "unit": UNIT,
                   "path": "tg3_ExpectGlobal2D, FP32 scoring, host buffers",
                   "h2d_bytes_per_step": int(host["vol"].nbytes + host["dat"].nbytes +
                                             host["ctf"].nbytes + host["sig"].nbytes),
                   "d2h_bytes_per_step": int(wCh.nbytes + wRh.nbytes + wTh.nbytes),
                   "class_recovered": round(e2e_rec, 4)},
           "insert2d": {"path": "tg3_InsertI2D, host volumes in and out, 16 classes",
                        "images_per_s": round(n / (ins_ms * 1e-3), 1),
                        "ms_per_call": round(ins_ms, 3)}}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        m = 16
        sel = np.arange(m)
        rotP = O.project2d(host["vol"][0].astype(np.complex128), rot_np, iCol, iRow, pf)
        traP = O.translate(trans_np, box, iCol, iRow)
        t0 = time.perf_counter()
        O.score_global(rotP, traP, host["dat"][sel].astype(np.complex128),
                       host["ctf"][sel].astype(np.float64), host["sig"][sel].astype(np.float64),
                       pRh, pTh, want_dvp=False)
        secs = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": round(m / (secs * nK), 3), "unit": UNIT, "cores": 1,
                               "kind": "port",
                               "sample": f"{m} particles x 1 of {nK} classes (projection and "
                                         f"shift banks precomputed), scaled to {nK} classes "
                                         f"({secs:.2f} s measured); double-precision oracle, "
                                         "one core"}
    ctx.close()
    return res


def run_prep(args, rank, world, local_rank):
    """Input preprocessing of box-256 particle images (Optimiser::initImg and
    allocPreCal): 4,096 real-space images per step to the pixel data of the
    production cutoff (K = 9,930): background normalisation, zero soft mask
    (radius 100 px), transform, gather.  e2e: the MRC stack read from a file
    by the library, copied in, preprocessed and the pixel data copied out."""
    import tempfile
    import torch
    import tg3
    from tg3 import io, synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    N, n, r, px = 256, 4096, 100.0, 1.1
    rng = np.random.default_rng(rank_seed(4000, rank))
    c = np.arange(N) - N // 2
    ii, jj = np.meshgrid(c, c)
    gen = torch.Generator(device=dev).manual_seed(rank_seed(4001, rank))
    imgs = 2.0 + torch.randn((n, N, N), generator=gen, device=dev)
    blob = torch.as_tensor(np.exp(-(ii ** 2 + jj ** 2) / (2 * 30.0 ** 2)), dtype=torch.float32,
                           device=dev)
    imgs += 3.0 * blob
    iCol, iRow = synth.pixel_index(N, 80, synth.config_rL(N, px))[:2]
    K = len(iCol)
    ctx = tg3.Context(local_rank)
    ctx.set_pixels(iCol, iRow, N)
    dat = torch.empty((n, K), dtype=torch.complex64, device=dev)

    def step():
        ctx.prepare_images(imgs, r, dat, mask=True)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    clk = ClockSampler(local_rank)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    clocks = clk.stop()
    ms = reduce_max(world, e0.elapsed_time(e1)) / args.steps
    # algorithmic bytes: every image read once, its pixel data written once
    alg = n * (N * N * 4 + K * 8)
    hbm, bf16, kind = peaks()
    achieved = alg / (ms * 1e-3) / 1e9
    # end to end: an MRC stack of 512 images on local disk through the library
    m = 512
    host = imgs[:m].cpu().numpy()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "particles.mrcs")
        io.write_mrc(path, host, pixel_size=px)
        pin = torch.empty((m, N, N), dtype=torch.float32).pin_memory()
        out = torch.empty((m, K), dtype=torch.complex64).pin_memory()
        dimg = torch.empty((m, N, N), dtype=torch.float32, device=dev)
        ddat = torch.empty((m, K), dtype=torch.complex64, device=dev)

        def e2e():
            # copies on torch's stream (its pinned-memory allocator keeps
            # events on the stream a copy ran on), the preprocessing on the
            # library's
            tg3.check(tg3.lib().tg3_mrc_read(path.encode(), 0, m, pin.data_ptr()))
            dimg.copy_(pin, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            ctx.prepare_images(dimg, r, ddat, mask=True)
            ctx.sync()
            out.copy_(ddat, non_blocking=True)
            torch.cuda.current_stream().synchronize()

        e2e()
        t0 = time.perf_counter()
        for _ in range(max(1, args.e2e_steps)):
            e2e()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.e2e_steps)
    res = {"metric": "image preprocessing images/s, box 256, K=%d" % K,
           "value": round(job_rate(n, ms, world), 1), "unit": "images/s",
           "ms_per_step": round(ms, 3), "n_gpus": world, "scaling": "weak",
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic: a Gaussian blob on unit-variance noise",
           "config": {"workload": "prep256", "images": n, "box": N, "mask_radius_px": r, "K": K,
                      "l2": "inputs (1.07 GB) larger than L2"},
           "clocks": clocks,
           "roofline": {"bound": "hbm", "kernel": "whole preprocessing step",
                        "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(achieved / hbm, 4), "peak_kind": kind,
                        "algorithmic_bytes_per_image": N * N * 4 + K * 8, "traffic": None},
           "e2e": {"value": round(m / (e2e_ms * 1e-3) * world, 1), "unit": "images/s",
                   "path": "tg3_mrc_read from a local file, pinned copies, tg3_prepare_images_d",
                   "h2d_bytes_per_step": m * N * N * 4, "d2h_bytes_per_step": m * K * 8}}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import preprocess as PP
        k = 32
        t0 = time.perf_counter()
        PP.preprocess(host[:k], r, iCol, iRow, mask=True)
        secs = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": round(k / secs, 1), "unit": "images/s", "cores": 1,
                               "kind": "port",
                               "sample": f"{k} images through the numpy oracle ({secs:.2f} s)"}
    ctx.close()
    return res


# the rescoring cross term's kernel under each TG3_OPT_BANK_GATHER value
BANK_KERNELS = {0: "k_gemm_bank_cp (bank rows gathered by cp.async)",
                1: "k_gemm_bf16x3 (rows copied out of the banks first)",
                2: "k_gemm_bank_bf16x3 (bank rows gathered by TMA)"}


def run_bank(args, rank, world, local_rank):
    """The learned E-step's rescoring on its own: one box-256 class (200-blob
    map, cutoff 80, K = 9,930), its projection bank at the 6,912 global
    rotations, and args.batch particles with 256 proposed bank rows x 25
    translations each (rows drawn near each particle's true rotation: the
    512 nearest bank rotations, 256 of them at random).  One step = the
    split-bf16 bank-row phase (shift bank, cross term, weights) over the
    batch; timed with the cross term reading the proposed rows from the bank
    and with the rows copied out first (TG3_OPT_BANK_GATHER).  A small,
    self-contained case for profiling the rescoring kernels."""
    import torch
    import tg3
    from tg3 import learned, synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    # --box: a smaller map for profiling captures (cutoff scaled with it)
    box = args.box or 256
    px, pf, rU = 1.1, 2, 80 * box // 256
    nP, nR, nT = args.batch, 256, 25
    f64 = dict(dtype=torch.float64, device=dev)
    rng = np.random.default_rng(rank_seed(6000, rank))
    bm = synth.blob_map(rng, 200, (1.5, 3.0), px, 80.0)
    rL = synth.config_rL(box, px)
    nv = synth.signal_power([bm], box, px, rU, rL, device=dev) / 0.03 / 2.0
    ps = synth.particle_set_dev(rank_seed(6001, rank), [bm], np.zeros(nP, np.int64), box, px,
                                rU, rL, 3.0, nv, device=dev)
    ctx = tg3.Context(local_rank)
    ctx.set_volume(0, synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32), pf)
    ctx.set_pixels(ps.iCol, ps.iRow, box)
    qg = synth.global_rotations(4, 36)
    ctx.set_bank(0, torch.as_tensor(qg, **f64), len(qg))
    # proposals: 256 of the 512 bank rotations nearest each particle's own
    near = np.argsort(-np.abs(ps.quat_true @ qg.T), axis=1)[:, :512]
    idx = np.stack([rng.choice(near[l], nR, replace=False) for l in range(nP)]).astype(np.int32)
    idx_d = torch.as_tensor(idx, device=dev)
    trans = torch.as_tensor(ps.trans_true[:, None, :] + rng.normal(0, 1.0, (nP, nT, 2)), **f64)
    cls = torch.zeros(nP, dtype=torch.int32, device=dev)
    o = dict(wC=torch.empty(nP, **f64), wR=torch.empty((nP, nR), **f64),
             wT=torch.empty((nP, nT), **f64), base=torch.empty(nP, **f64))
    pR = torch.full((nP, nR), 1.0 / nR, **f64)
    pT = torch.full((nP, nT), 1.0 / nT, **f64)
    pC = torch.ones(nP, **f64)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step():
        ctx.local_phase_bank(nP, nR, nT, ps.dat, ps.ctf, ps.sigRcp, idx_d, trans, pR, pT, pC,
                             cls, o["wC"], o["wR"], o["wT"], o["base"], None, tg3.SCORE_BF16X3)

    ctx.set_option(tg3.OPT_BANK_SHAPE, args.bank_shape)

    def timed(form, order):
        ctx.set_option(tg3.OPT_BANK_GATHER, int(form))
        ctx.set_option(tg3.OPT_BANK_ORDER, int(order))
        for _ in range(args.warmup):
            step()
        ctx.sync()
        ctx.set_timing(True)
        ctx.stage_times(reset=True)
        clk = ClockSampler(local_rank)
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
        clocks = clk.stop()
        st = ctx.stage_times(reset=True)
        ctx.set_timing(False)
        ctx.sync()
        best = o["wR"].argmax(1).cpu().numpy()
        return reduce_max(world, e0.elapsed_time(e1)) / args.steps, st, clocks, best

    # every form, the headline one (--bank-form, --bank-order) last
    main = (args.bank_form, args.bank_order)
    others = {}
    for form, order in ((1, 0), (2, 0), (2, 1), (0, 0), (0, 1)):
        if (form, order) != main:
            others[(form, order)] = timed(form, order)
    ms, st, clocks, best = timed(*main)
    K, Kp = len(ps.iCol), ctx_kp(len(ps.iCol))
    hbm, bf16, kind = peaks()
    cross_ms = st["cross"][0] / max(st["cross"][1], 1)
    algo = float(nP) * (nR * 4.0 * Kp + nT * 4.0 * Kp + nR * nT * 4.0)
    ach = algo / (cross_ms * 1e-3) / 1e9
    err = learned.angle_deg(qg[idx[np.arange(nP), best]], ps.quat_true)
    res = {"metric": "rescoring particles/s (learned E-step, bank-row local phase), box 256",
           "value": round(job_rate(nP, ms, world), 1), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16x3", "data": "synthetic",
           "config": {"workload": f"{nP} particles x {nR} bank rows x {nT} translations, one "
                                  f"box-{box} class, bank of {len(qg)} rotations, K = {K}",
                      "l2": "inputs larger than L2 (bank 0.55 GB)"},
           "clocks": clocks,
           "roofline": {"kernel": BANK_KERNELS[main[0]], "bound": "hbm",
                        "achieved": round(ach, 1),
                        "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
                        "peak_source": f"hbm_gbs, {kind} (MEASURED_PEAKS.json)",
                        "traffic": None, "algorithmic_bytes_per_launch": algo,
                        "ms_per_launch": round(cross_ms, 4),
                        "tflops_algorithmic": round(4.0 * K * nP * nR * nT / (cross_ms * 1e-3)
                                                    / 1e12, 2)},
           "stages": {k: round(v[0] / max(v[1], 1), 4) for k, v in st.items() if v[1]},
           "bank_form": {"form": main[0], "order": main[1], "shape": args.bank_shape,
                         "what": "TG3_OPT_BANK_GATHER (0: cp.async gathers in the cross term, "
                                 "1: rows copied out then the GEMM, 2: TMA gathers in the cross "
                                 "term) and TG3_OPT_BANK_ORDER (particles sorted by first "
                                 "proposed row)"},
           "other_forms": {f"form{f}_order{r}": {
               "ms_per_step": round(v[0], 4),
               "stages": {k: round(x[0] / max(x[1], 1), 4) for k, x in v[1].items() if x[1]},
               "same_best_rotation": round(float(np.mean(best == v[3])), 4)}
               for (f, r), v in others.items()},
           "speedup_vs_copy_form": round(others[(1, 0)][0] / ms, 3) if (1, 0) in others else 1.0,
           "median_error_best_deg": round(float(np.median(err)), 3),
           "gpu_launches": (5 if main[0] == 1 else 4 + main[1]) * args.steps}
    ctx.close()
    return res


def run_fallback(args, rank, world, local_rank):
    """The learned E-step's fallback search on its own: the global search of a
    few particles of one class (args.batch, default 70, about one class's
    share of the fallback particles of a 2,000-particle step) over the
    class's bank of 6,912 rotations x 49 translations, split-bf16, at box 256
    (cutoff 80, K = 9,930; --box for a smaller profiling case).  One step =
    one search of the batch; stages timed by the library (the norm term, the
    cross term, the weights)."""
    import torch
    import tg3
    from tg3 import synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    box = args.box or 256
    px, pf, rU = 1.1, 2, 80 * box // 256
    nP = args.batch if args.batch != 128 else 70
    f64 = dict(dtype=torch.float64, device=dev)
    rng = np.random.default_rng(rank_seed(7000, rank))
    bm = synth.blob_map(rng, 200, (1.5, 3.0), px, 80.0)
    rL = synth.config_rL(box, px)
    nv = synth.signal_power([bm], box, px, rU, rL, device=dev) / 0.03 / 2.0
    ps = synth.particle_set_dev(rank_seed(7001, rank), [bm], np.zeros(nP, np.int64), box, px,
                                rU, rL, 3.0, nv, device=dev)
    ctx = tg3.Context(local_rank)
    ctx.set_option(tg3.OPT_SCAN_PAIR, args.scan_pair)
    ctx.set_option(tg3.OPT_SCAN_BK, args.scan_bk)
    ctx.set_option(tg3.OPT_PROJECT_FORM, args.project_form)
    ctx.set_volume(0, synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32), pf)
    ctx.set_pixels(ps.iCol, ps.iRow, box)
    qg = synth.global_rotations(4, 36)
    R = torch.as_tensor(synth.quat_to_mat(qg).reshape(-1, 9)).to(dev).contiguous()
    tr = torch.as_tensor(synth.global_translations(3, 1.0), **f64).contiguous()
    nR, nT = len(qg), len(tr)
    pR = torch.full((nR,), 1.0 / nR, **f64)
    pT = torch.full((nT,), 1.0 / nT, **f64)
    o = dict(wC=torch.empty(nP, **f64), wR=torch.empty((nP, nR), **f64),
             wT=torch.empty((nP, nT), **f64), base=torch.empty(nP, **f64))
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step():
        ctx.global_scan(0, nP, nR, nT, ps.dat, ps.ctf, ps.sigRcp, R, tr, pR, pT, o["wC"], o["wR"],
                        o["wT"], o["base"], None, tg3.SCORE_BF16X3)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    ctx.set_timing(True)
    ctx.stage_times(reset=True)
    clk = ClockSampler(local_rank)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    clocks = clk.stop()
    st = ctx.stage_times(reset=True)
    ctx.set_timing(False)
    ms = reduce_max(world, e0.elapsed_time(e1)) / args.steps
    K = len(ps.iCol)
    hbm, bf16, kind = peaks()
    cross_ms = st["cross"][0] / max(st["cross"][1], 1)
    flop = 4.0 * K * nP * nR * nT
    res = {"metric": "fallback global search particles/s (learned E-step), box 256",
           "value": round(job_rate(nP, ms, world), 1), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16x3", "data": "synthetic",
           "config": {"workload": f"{nP} particles of one box-{box} class x {nR} rotations x "
                                  f"{nT} translations, K = {K}",
                      "scan_pair": args.scan_pair, "scan_bk": args.scan_bk},
           "clocks": clocks,
           "roofline": {"kernel": "k_gemm_bf16x3 (cross term; the norm term is stage norm)",
                        "bound": "tensor",
                        "achieved": round(flop / (cross_ms * 1e-3) / 1e12, 2), "peak": bf16,
                        "unit": "TFLOP/s",
                        "frac": round(flop / (cross_ms * 1e-3) / 1e12 / bf16, 4),
                        "executed_bf16_tflops": round(3 * flop / (cross_ms * 1e-3) / 1e12, 1),
                        "peak_source": f"bf16_tflops, {kind} (MEASURED_PEAKS.json)",
                        "traffic": None, "ms_per_launch": round(cross_ms, 4)},
           "stages": {k: round(v[0] / max(v[1], 1), 4) for k, v in st.items() if v[1]},
           "gpu_launches": 13 * args.steps}
    ctx.close()
    return res


def run_reco(args, rank, world, local_rank):
    """Reconstruction of a box-256 map from its insertion accumulators
    (Reconstructor::reconstruct): padded grid 512^3 (pf 2), Wiener filter from
    an FSC curve, grid correction by balancing against the MKB kernel, the
    inverse transform and gridding correction.  F: the padded transform of a
    200-blob map; T: a smooth radial weight.  One step = one map."""
    import torch
    import tg3
    from tg3 import synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    N, pf, px, maxR = 256, 2, 1.1, 120
    vdim = N * pf
    rng = np.random.default_rng(rank_seed(5000, rank))
    bm = synth.blob_map(rng, 200, (1.5, 3.0), px, 80.0)
    F = synth.padded_volume(bm, N, pf, device=dev, dtype=torch.float32)
    q = torch.fft.fftfreq(vdim, 1.0 / vdim, device=dev)
    kz, ky, kx = torch.meshgrid(q, q, torch.arange(vdim // 2 + 1, device=dev, dtype=q.dtype),
                                indexing="ij")
    T = (50.0 * torch.exp(-torch.sqrt(kx * kx + ky * ky + kz * kz) / (0.4 * vdim)) + 0.5).float()
    F = (F * T).contiguous()
    del kx, ky, kz
    fsc = torch.as_tensor(np.clip(1.05 - np.arange(N // 2 + 1) / (N / 2), 0, 1)).to(dev)
    ctx = tg3.Context(local_rank)
    ctx.insert_begin(vdim, pf)
    vol = torch.empty((N, N, N), dtype=torch.float32, device=dev)

    def step():
        ctx.insert_load(F, T)
        return ctx.reconstruct(vol, maxR, fsc=fsc, join_half=True, grid_corr=True,
                               kernel=tg3.KERNEL_MKB)

    for _ in range(args.warmup):
        rounds = step()
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    clk = ClockSampler(local_rank)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 10))
    barrier(world)
    e0.record(stream)
    for _ in range(steps):
        rounds = step()
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    clocks = clk.stop()
    ms = reduce_max(world, e0.elapsed_time(e1)) / steps
    nh = vdim * vdim * (vdim // 2 + 1)
    nr = vdim ** 3
    # algorithmic bytes of one balancing round: T, W read and C written
    # (C = T W), C read and the real map written (inverse), the map read and
    # written (kernel product), read and C written (forward), C read and W
    # read and written (update) -- each array once per pass
    per_round = 4 * nh * 2 + 8 * nh + 8 * nh + 4 * nr + 8 * nr + 4 * nr + 8 * nh + 8 * nh + 8 * nh
    alg = rounds * per_round + 16 * nh + 8 * nh + 4 * nr + 4 * N ** 3
    hbm, bf16, kind = peaks()
    achieved = alg / (ms * 1e-3) / 1e9
    ctx.close()
    return {"metric": "reconstruction maps/s, box 256 (512^3 padded), grid correction",
            "value": round(job_rate(1, ms, world), 3), "unit": "maps/s", "ms_per_step": round(ms, 3),
            "n_gpus": world, "scaling": "weak", "steps": steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f32",
            "data": "synthetic: padded transform of a 200-blob map, radial T",
            "config": {"workload": "reco256", "box": N, "pf": pf, "max_radius": maxR,
                       "balancing_rounds": rounds, "l2": "arrays (2.7 GB) larger than L2"},
            "clocks": clocks,
            "roofline": {"bound": "hbm", "kernel": "whole reconstruction (cuFFT-dominated)",
                         "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "peak_kind": kind, "traffic": None}}


UNEVEN = dict(box=192, pixel_size=1.3, n_blobs=150, sigma_a=(1.5, 3.0), radius_px=60.0,
              cutoffs=(40, 56, 72, 96), pf=2, shift=8.0, snr=0.03, kappa=200.0,
              nR=(200, 8000), nT=(9, 81))


def run_uneven(args, rank, world, local_rank):
    """Uneven batches: 192^3 maps, 1.3 A/px, 4 classes of 150-blob maps with
    cutoffs 40 / 56 / 72 / 96 (K = 2,452 / 4,844 / 8,026 / 14,324); every
    particle keeps log-uniform [200, 8,000] rotations x [9, 81] translations,
    as after narrowing.  A step is one ragged plan over the batch (waves of
    similar particles, replayed as one captured CUDA graph, autotuned wave
    budget); the same particles scored one at a time (three calls each) are
    timed beside it on a bounded sample."""
    import torch
    import tg3
    from tg3 import synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    U = UNEVEN
    nP = args.batch_uneven
    rng = np.random.default_rng(rank_seed(3000, rank))
    box, px, pf = U["box"], U["pixel_size"], U["pf"]
    nC = len(U["cutoffs"])
    maps = [synth.blob_map(rng, U["n_blobs"], U["sigma_a"], px, U["radius_px"]) for _ in range(nC)]
    ctx = tg3.Context(local_rank)
    for c, bm in enumerate(maps):
        ctx.set_volume(c, synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32), pf)
    rL = synth.config_rL(box, px)
    cls = np.arange(nP) % nC
    lo_r, hi_r = U["nR"]
    lo_t, hi_t = U["nT"]
    nR = np.round(np.exp(rng.uniform(np.log(lo_r), np.log(hi_r), nP))).astype(np.int32)
    nT = np.round(np.exp(rng.uniform(np.log(lo_t), np.log(hi_t), nP))).astype(np.int32)
    stacks, Ks = [], []
    for c, rU in enumerate(U["cutoffs"]):
        n_c = int(np.sum(cls == c))
        st = synth.make_stack(rank_seed(3100 + c, rank), [maps[c]], box, px, pf, rU, rL, n_c,
                              U["shift"], U["snr"], device=dev)
        ctx.set_pixels_slot(c, st.iCol, st.iRow, box)
        stacks.append(st)
        Ks.append(st.K)
    # particle l is particle l // nC of its class's stack
    row = np.arange(nP) // nC
    qtrue = np.stack([stacks[cls[l]].quat_true[row[l]] for l in range(nP)])
    ttrue = np.stack([stacks[cls[l]].trans_true[row[l]] for l in range(nP)])
    qc, tc = synth.perturb_poses(rng, qtrue, ttrue, 3.0, 1.0)
    quat = synth.vmf_quaternions_many(rng, qc, U["kappa"], nR)
    trans = np.repeat(tc, nT, axis=0) + 2.0 * rng.standard_normal((int(nT.sum()), 2))
    cat = lambda f: np.concatenate([f(l) for l in range(nP)])
    host = dict(
        dat=cat(lambda l: stacks[cls[l]].dat[row[l]]).astype(np.complex64),
        ctf=cat(lambda l: stacks[cls[l]].ctf[row[l]]).astype(np.float32),
        sig=cat(lambda l: stacks[cls[l]].sigRcp[row[l]]).astype(np.float32),
        quat=quat, trans=trans,
        pwR=np.repeat(1.0 / nR, nR), pwT=np.repeat(1.0 / nT, nT), pwC=np.ones(nP),
        permR=cat(lambda l: rng.permutation(int(nR[l]))).astype(np.int32),
        u0R=rng.random(nP) / nR, peakR=np.full(nP, np.nan),
        permT=cat(lambda l: rng.permutation(int(nT[l]))).astype(np.int32),
        u0T=rng.random(nP) / nT, peakT=np.zeros(nP))
    inp = {k: torch.as_tensor(np.ascontiguousarray(v)).to(dev) for k, v in host.items()}
    R, T = int(nR.sum()), int(nT.sum())
    f64 = dict(dtype=torch.float64, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    out = dict(wC=torch.empty(nP, **f64), base=torch.empty(nP, **f64), wR=torch.empty(R, **f64),
               wT=torch.empty(T, **f64), srcR=torch.empty(R, **i32), wOutR=torch.empty(R, **f64),
               srcT=torch.empty(T, **i32), wOutT=torch.empty(T, **f64),
               topR=torch.empty(nP, **i32), topT=torch.empty(nP, **i32))
    prec = tg3.SCORE_BF16X3 if args.precision == "bf16x3" else tg3.SCORE_FP32
    t0 = time.perf_counter()
    plan = tg3.RaggedPlan(ctx, cls, nR, nT, inp, out, prec, budget=0, graph=True)
    plan_s = time.perf_counter() - t0
    waves, budget = plan.info()
    kblock = plan.kblock()
    pgroup = plan.project_group()
    for _ in range(args.warmup):
        plan.run()
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream)
    torch.cuda.synchronize()
    clk = ClockSampler(local_rank)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    e0.record(stream)
    for _ in range(args.steps):
        plan.run()
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    clocks = clk.stop()
    ctx.sync()
    ms = reduce_max(world, e0.elapsed_time(e1)) / args.steps
    # the same particles one at a time (local phase + two resamplings each)
    ns = min(nP, args.per_particle_sample)
    pref = dict(po=np.concatenate([[0], np.cumsum([Ks[c] for c in cls])]),
                ro=np.concatenate([[0], np.cumsum(nR)]), to=np.concatenate([[0], np.cumsum(nT)]))
    cl1 = [torch.tensor([c], dtype=torch.int32, device=dev) for c in range(nC)]
    tmp = {k: torch.empty_like(v) for k, v in out.items()}

    def one(l):
        K, r, t = Ks[cls[l]], int(nR[l]), int(nT[l])
        po, ro, to = int(pref["po"][l]), int(pref["ro"][l]), int(pref["to"][l])
        ctx.use_pixels(int(cls[l]))
        ctx.local_phase(1, r, t, inp["dat"][po:po + K], inp["ctf"][po:po + K],
                        inp["sig"][po:po + K], inp["quat"][ro:ro + r], inp["trans"][to:to + t],
                        inp["pwR"][ro:ro + r], inp["pwT"][to:to + t], inp["pwC"][l:l + 1],
                        cl1[cls[l]], tmp["wC"][l:l + 1], tmp["wR"][ro:ro + r],
                        tmp["wT"][to:to + t], tmp["base"][l:l + 1], None, prec)
        ctx.resample(1, r, tmp["wR"][ro:ro + r], inp["pwR"][ro:ro + r], inp["permR"][ro:ro + r],
                     inp["u0R"][l:l + 1], inp["peakR"][l:l + 1], r, tmp["srcR"][ro:ro + r],
                     tmp["wOutR"][ro:ro + r], tmp["topR"][l:l + 1])
        ctx.resample(1, t, tmp["wT"][to:to + t], inp["pwT"][to:to + t], inp["permT"][to:to + t],
                     inp["u0T"][l:l + 1], inp["peakT"][l:l + 1], t, tmp["srcT"][to:to + t],
                     tmp["wOutT"][to:to + t], tmp["topT"][l:l + 1])

    for l in range(min(ns, 8)):
        one(l)
    ctx.sync()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for l in range(ns):
        one(l)
    e3.record(stream)
    e3.synchronize()
    ctx.sync()
    pp_ms = e2.elapsed_time(e3)
    # per-particle work of the sample, to scale its time to the whole batch
    work = lambda idx: float(np.sum(nR[idx].astype(np.float64) * np.array(Ks)[cls[idx]]))
    pp_batch_ms = pp_ms * work(np.arange(nP)) / work(np.arange(ns))
    samples = work(np.arange(nP))
    hyps = float(np.sum(nR.astype(np.float64) * nT))
    flop = 4.0 * float(np.sum(nR.astype(np.float64) * nT * np.array(Ks)[cls]))
    res = {"metric": "uneven-batch E-step particles/s, box 192, 4 classes, ragged hypothesis sets",
           "value": round(job_rate(nP, ms, world), 1), "unit": UNIT, "ms_per_step": round(ms, 3),
           "n_gpus": world, "scaling": "weak",
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "precision": args.precision, "clocks": clocks,
           "config": {"workload": "ragged plan: 4 classes, cutoffs 40/56/72/96 (K = "
                                  + "/".join(str(k) for k in Ks) + "), rotations log-uniform "
                                  "[200, 8000] x translations log-uniform [9, 81] per particle",
                      "particles_per_step": nP, "rotations_total": R, "translations_total": T,
                      "plan_waves": waves, "wave_budget_bytes": budget,
                      "cross_term_k_block": kblock, "projection_group": pgroup,
                      "plan_create_s": round(plan_s, 2)},
           "hypotheses_per_s": round(job_rate(hyps, ms, world), 1),
           "samples_per_s": round(job_rate(samples, ms, world), 1),
           "cross_term_tflops": round(job_rate(flop, ms, world) / 1e12, 1),
           "per_particle_launches": {
               "value": round(nP / (pp_batch_ms * 1e-3), 1), "unit": UNIT,
               "sample": f"first {ns} particles one at a time (local phase + 2 resamplings "
                         f"each, {pp_ms:.1f} ms), scaled to the batch by rotations x pixels"},
           "speedup_vs_per_particle": round(pp_batch_ms / ms, 2)}
    plan.close()
    ctx.close()
    return res


# the same comparison at box 256: maps, cutoff and noise model of the
# production configuration (256^3, 1.1 A/px, 200 blobs; cutoff 80, K = 9,930;
# SNR 0.03 over the likelihood's pixels), shifts within the global search's
# 7 x 7 translation grid
LEARNED256 = dict(box=256, pixel_size=1.1, n_blobs=200, sigma_a=(1.5, 3.0), radius_px=80.0,
                  n_maps=16, n_train_maps=12, rU=80, pf=2, shift=3.0, snr_lik=0.03,
                  n_rot=256, n_trans=25)
LEARNED = dict(box=128, pixel_size=1.4, n_blobs=120, sigma_a=(1.5, 3.0), radius_px=40.0,
               n_maps=16, n_train_maps=12, rU=32, pf=2, shift=3.0, snr_lik=0.05,
               n_rot=256, n_trans=25)


def reconstruction_resolution(tg3, torch, ctx, ps, maps, quat, trans, box, pf, px, rU, dev):
    """Mean over the set's maps of the FSC-0.143 resolution (A) of the map
    reconstructed from its particles at the given poses."""
    vdim = pf * box
    n_shell = int(pf * rU) + 1
    shape = (vdim, vdim, vdim // 2 + 1)
    ctx.set_pixels(ps.iCol, ps.iRow, box)
    out = []
    for c in np.unique(ps.cls):
        g = np.nonzero(ps.cls == c)[0]

        def d(x):
            if torch.is_tensor(x):
                return x[torch.as_tensor(g, device=x.device)].contiguous()
            return torch.as_tensor(np.ascontiguousarray(np.asarray(x)[g])).to(dev)
        ctx.insert_begin(vdim, pf)
        ctx.insert(len(g), d(ps.dat), d(ps.ctf), d(np.asarray(quat, np.float64)),
                   d(np.asarray(trans, np.float64)), None,
                   torch.ones(len(g), dtype=torch.float32, device=dev), tg3.KERNEL_MKB)
        F = torch.empty(shape + (2,), dtype=torch.float32, device=dev)
        T = torch.empty(shape, dtype=torch.float32, device=dev)
        V = torch.empty(shape, dtype=torch.complex64, device=dev)
        ctx.insert_read(F, T)
        ctx.sync()
        floor = 0.01 * float(T[T > 0].mean())
        ctx.insert_ratio(V, floor)
        ctx.sync()
        truth = synth_padded(maps[int(c)], box, pf, dev)
        f = tg3.fsc(V, truth, n_shell).cpu().numpy()
        u = n_shell - 1.0
        for k in range(2, n_shell):
            if f[k] < 0.143:
                u = (k - 1) + (f[k - 1] - 0.143) / max(f[k - 1] - f[k], 1e-12)
                break
        out.append(pf * box * px / u)
        del F, T, V
    return round(float(np.mean(out)), 3)


_TRUTH = {}


def synth_padded(bm, box, pf, dev):
    """The map's exact padded transform (kept: every pose source is compared
    with the same maps)."""
    import torch
    from tg3 import synth
    key = (id(bm), box, pf)
    if key not in _TRUTH:
        _TRUTH[key] = synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32)
    return _TRUTH[key]


def run_learned(args, rank, world, local_rank):
    """The headline: the learned E-step (pose-network proposals rescored by
    the exact split-bf16 likelihood, global search as the fallback) against
    the plain FP32 global search, at box 256 (learned256) or 128 (learned128).

    16 blob maps; 12 give the training particles, 4 are held out.  The
    training labels are the plain method's converged poses (the global
    search over 6,912 rotations x 49 translations, then three narrowing local
    phases of 1,000 x 100; scored in split-bf16 by default, whose argmax
    equals the FP64 oracle's on the population tests, so that the whole
    line, training included, finishes in under five minutes).  The network (matching mode, trained on the GPU by
    the library's kernels) proposes 256 rotations x 25 translations per
    particle; the fallback threshold is calibrated on held-out particles of
    the training maps against the plain method's poses.  The timed step is
    one E-step over the particles of the 4 held-out maps; after it both
    methods' poses are refined by one local phase of 1,000 x 100 and compared
    (median error against the true pose, FSC-0.143 of the maps
    reconstructed from them)."""
    import torch
    import tg3
    from tg3 import learned, synth
    torch.cuda.set_device(local_rank)
    dev = f"cuda:{local_rank}"
    L = LEARNED256 if args.workload == "learned256" else LEARNED
    box, px, pf, rU = L["box"], L["pixel_size"], L["pf"], L["rU"]
    nTr, nMaps = L["n_train_maps"], L["n_maps"]
    nRot, nTrans = L["n_rot"], L["n_trans"]
    prec = tg3.SCORE_BF16X3 if args.precision == "bf16x3" else tg3.SCORE_FP32
    lab_prec = tg3.SCORE_FP32 if args.label_precision == "fp32" else tg3.SCORE_BF16X3
    f64 = dict(dtype=torch.float64, device=dev)
    rng = np.random.default_rng(4000)
    maps = [synth.blob_map(rng, L["n_blobs"], L["sigma_a"], px, L["radius_px"])
            for _ in range(nMaps)]
    rL = synth.config_rL(box, px)
    iCol, iRow, _, _ = synth.pixel_index(box, rU, rL)
    K = len(iCol)
    noise_var = synth.signal_power(maps[:nTr], box, px, rU, rL, device=dev) / L["snr_lik"] / 2.0
    ctx = tg3.Context(local_rank)
    ctx.set_option(tg3.OPT_BANK_GATHER, args.bank_form)
    ctx.set_option(tg3.OPT_BANK_SHAPE, args.bank_shape)
    ctx.set_option(tg3.OPT_BANK_ORDER, args.bank_order)
    ctx.set_option(tg3.OPT_SCAN_PAIR, args.scan_pair)
    ctx.set_option(tg3.OPT_SCAN_BK, args.scan_bk)
    ctx.set_option(tg3.OPT_PROJECT_FORM, args.project_form)
    for c, bm in enumerate(maps):
        ctx.set_volume(c, synth.padded_volume(bm, box, pf, device=dev, dtype=torch.float32), pf)
    ctx.set_pixels(iCol, iRow, box)
    quats_g = synth.global_rotations(4, 36)
    nRg = len(quats_g)
    quats_g_dev = torch.as_tensor(quats_g, **f64)
    mats_g = torch.as_tensor(synth.quat_to_mat(quats_g).reshape(-1, 9), **f64)
    trans_g = torch.as_tensor(synth.global_translations(3, 1.0), **f64)
    nTg = int(trans_g.shape[0])
    gen = torch.Generator(device=dev)
    gen.manual_seed(rank_seed(7100, rank))
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if args.verbose else (lambda m: None)

    # ---- 1. training particles of the 12 training maps, labelled with the
    # plain method's converged poses
    t0 = time.perf_counter()
    imgs, q_lab, t_lab, q_tru, cls_tr, moves = [], [], [], [], [], []
    chunk = 10000
    n_train = 0 if args.load_net else args.train_particles
    for s0 in range(0, n_train, chunk):
        m = min(chunk, args.train_particles - s0)
        ps = synth.particle_set_dev(4100 + s0, maps, (s0 + np.arange(m)) % nTr, box, px, rU, rL,
                                    L["shift"], noise_var, device=dev)
        ql, tl, mv = learned.plain_method_poses(ctx, ps, quats_g, mats_g, trans_g, lab_prec, gen)
        imgs.append(ps.images)
        q_lab.append(ql)
        t_lab.append(tl)
        q_tru.append(ps.quat_true)
        cls_tr.append(ps.cls)
        moves.append(mv)
        del ps
        log(f"labels {s0 + m}/{args.train_particles}: phase moves {mv}")
    net = tg3.Cnn(local_rank, seed=4242)
    if args.load_net:
        # a network trained by an earlier run of this workload (profiling runs)
        net.set_params(np.load(args.load_net)["params"])
        label_s = train_s = 0.0
        restarts = 0
        label_err, moves, losses = np.zeros(1), [[0.0, 0.0, 0.0]], []
    else:
        images = torch.cat(imgs)
        del imgs
        q_lab, t_lab = np.concatenate(q_lab), np.concatenate(t_lab)
        q_tru, cls_tr = np.concatenate(q_tru), np.concatenate(cls_tr)
        torch.cuda.synchronize()
        label_s = time.perf_counter() - t0
        label_err = learned.angle_deg(q_lab, q_tru)

        # ---- 2. training (matching mode): references at the label rotations
        refs = torch.empty_like(images)
        for c in range(nTr):
            sel = np.nonzero(cls_tr == c)[0]
            refs[torch.as_tensor(sel, device=dev)] = learned.render_references(ctx, c, q_lab[sel],
                                                                               box)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        # a run that stays on the loss's starting plateau through its first
        # epoch starts again from another initialisation (at most twice)
        restarts = 0
        while True:
            try:
                losses = learned.train_match(net, images, refs, torch.as_tensor(t_lab, **f64),
                                             cls_tr, args.epochs, 256, args.learned_lr,
                                             tau=args.learned_tau, seed=7 + restarts,
                                             stall_check=restarts < 2)
                break
            except learned.TrainingStalled as ex:
                log(f"training stalled ({ex}); new initialisation")
                restarts += 1
                net.close()
                net = tg3.Cnn(local_rank, seed=4242 + restarts)
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t1
        del refs, images
        log(f"trained: losses {losses}")
        if args.save_net:
            np.savez(args.save_net, params=net.params())

    # ---- 3. evaluation particles: held-out particles of the training maps
    # (calibration) and particles of the 4 held-out maps (the timed batch)
    nSeen, nUn = args.eval_particles_seen, args.eval_particles_unseen
    seen = synth.particle_set_dev(rank_seed(5001, rank), maps, np.arange(nSeen) % nTr, box, px,
                                  rU, rL, L["shift"], noise_var, device=dev)
    unseen = synth.particle_set_dev(rank_seed(5002, rank), maps,
                                    nTr + np.arange(nUn) % (nMaps - nTr), box, px, rU, rL,
                                    L["shift"], noise_var, device=dev)

    # ---- 4. per map, once: the 6,912 references rendered and embedded, the
    # projection bank at the same rotations, the references attached to it
    classes = sorted(set(int(c) for c in seen.cls) | set(int(c) for c in unseen.cls))
    emb, embed_ms, bank_ms = {}, {}, {}
    for c in classes:
        torch.cuda.synchronize()
        ta = time.perf_counter()
        emb[c] = learned.reference_embeddings(net, learned.render_references(ctx, c, quats_g, box))
        torch.cuda.synchronize()
        embed_ms[c] = (time.perf_counter() - ta) * 1e3
    ctx.set_pixels(iCol, iRow, box)          # the particles' pixel set, for the banks
    for c in classes:
        ctx.sync()
        ta = time.perf_counter()
        ctx.set_bank(c, quats_g_dev, nRg)
        ctx.set_references(c, emb[c])
        ctx.sync()
        bank_ms[c] = (time.perf_counter() - ta) * 1e3
    held = [c for c in classes if c >= nTr]
    map_ms = float(np.mean([embed_ms[c] + bank_ms[c] for c in held]))
    per_map_particles = 50000
    map_ms_pp = map_ms / per_map_particles

    # ---- 5. the plain method run to convergence on the evaluation particles:
    # the plain method's converged poses: what the proposals' errors are
    # measured against (and the poses the calibration trusts)
    conv_seen, _, _ = learned.plain_method_poses(ctx, seen, quats_g, mats_g, trans_g,
                                                  tg3.SCORE_FP32, gen)
    conv_un, conv_un_t, _ = learned.plain_method_poses(ctx, unseen, quats_g, mats_g, trans_g,
                                                         tg3.SCORE_FP32, gen)

    def outputs(n, full=True):
        o = dict(bestQuat=torch.empty((n, 4), **f64), bestTrans=torch.empty((n, 2), **f64),
                 baseL=torch.empty(n, **f64),
                 peak=torch.empty(n, dtype=torch.float32, device=dev),
                 fellBack=torch.empty(n, dtype=torch.int32, device=dev))
        if full:
            o.update(propIdx=torch.empty((n, nRot), dtype=torch.int32, device=dev),
                     propQuat=torch.empty((n, nRot, 4), **f64),
                     propTrans=torch.empty((n, nTrans, 2), **f64),
                     propWR=torch.empty((n, nRot), **f64), propWT=torch.empty((n, nTrans), **f64),
                     propBase=torch.empty(n, **f64),
                     propDvp=torch.empty((n, nRot, nTrans), dtype=torch.float32, device=dev))
        return o

    def expect(ps, peak_min, out, precision=prec):
        ctx.learned_expect(net, ps.images, ps.dat, ps.ctf, ps.sigRcp,
                           torch.as_tensor(ps.cls.astype(np.int32), device=dev), nRot, nTrans, 99,
                           trans_g, peak_min, precision, out)

    # ---- 6. fallback threshold: 95 % of the held-out particles of the
    # training maps whose proposal lies within 10 degrees of the plain
    # method's converged pose pass it
    o_seen = outputs(nSeen, full=False)
    expect(seen, float("-inf"), o_seen)
    err_seen = learned.angle_deg(o_seen["bestQuat"].cpu().numpy(), conv_seen)
    pk_seen = o_seen["peak"].cpu().numpy()
    good = err_seen < 10.0
    tau = float(np.quantile(pk_seen[good], 0.05)) if good.any() else float("inf")
    del o_seen

    # ---- 7. the timed E-steps over the particles of the held-out maps
    n = nUn
    cls_un = torch.as_tensor(unseen.cls.astype(np.int32), device=dev)
    out = outputs(n)
    stream = torch.cuda.ExternalStream(ctx.stream)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def learned_step():
        ctx.learned_expect(net, unseen.images, unseen.dat, unseen.ctf, unseen.sigRcp, cls_un,
                           nRot, nTrans, 99, trans_g, tau, prec, out)

    for _ in range(args.warmup):
        learned_step()
    barrier(world)
    torch.cuda.synchronize()
    ctx.set_timing(True)
    ctx.stage_times(reset=True)
    clk = ClockSampler(local_rank)
    clk.start()
    e0, e1 = ev(), ev()
    # an NVTX range around the timed steps: profilers select its kernels
    # (ncu --nvtx --nvtx-include "learned_step/")
    torch.cuda.nvtx.range_push("learned_step")
    e0.record(stream)
    for _ in range(args.steps):
        learned_step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    clocks = clk.stop()
    torch.cuda.synchronize()
    barrier(world)
    tl_ms = reduce_max(world, e0.elapsed_time(e1))
    st_l = ctx.stage_times(reset=True)
    ctx.set_timing(False)
    # the other rescoring form on the same step, stage-timed (not the headline)
    ab = {"timed_form": {"bank_form": args.bank_form, "bank_order": args.bank_order,
                         "ms_per_step": round((st_l["project"][0] if "project" in st_l else 0.0)
                                              / args.steps + st_l["cross"][0] / args.steps, 4)},
          "note": "rescoring of the same step, slices copied out of the banks then the cross "
                  "term (TG3_OPT_BANK_GATHER 1) and the cross term reading the proposed bank "
                  "rows itself (0: cp.async gathers, 2: TMA gathers; TG3_OPT_BANK_ORDER: "
                  "particles sorted by first proposed row); project + cross stages"}
    for form, order in ((1, 0), (0, 0), (0, 1), (2, 1)):
        if (form, order) == (args.bank_form, args.bank_order):
            continue
        ctx.set_option(tg3.OPT_BANK_GATHER, form)
        ctx.set_option(tg3.OPT_BANK_ORDER, order)
        learned_step()
        ctx.set_timing(True)
        ctx.stage_times(reset=True)
        for _ in range(2):
            learned_step()
        st_g = ctx.stage_times(reset=True)
        ctx.set_timing(False)
        ab[f"form{form}_order{order}_ms_per_step"] = round(
            ((st_g["project"][0] if "project" in st_g else 0.0) + st_g["cross"][0]) / 2, 4)
    ctx.set_option(tg3.OPT_BANK_GATHER, args.bank_form)
    ctx.set_option(tg3.OPT_BANK_SHAPE, args.bank_shape)
    ctx.set_option(tg3.OPT_BANK_ORDER, args.bank_order)
    fb = out["fellBack"].cpu().numpy().astype(bool)
    q_l = out["bestQuat"].cpu().numpy()
    t_l = out["bestTrans"].cpu().numpy()
    base_l = out["baseL"].cpu().numpy()
    prop_q = out["propQuat"].cpu().numpy()
    prop_base = out["propBase"].cpu().numpy()
    peak_un = out["peak"].cpu().numpy()
    idx_un = out["propIdx"].cpu().numpy()
    ptr_un = out["propTrans"].cpu().numpy()
    dvp_un = out["propDvp"].cpu().numpy()
    q_prop_best = prop_q[np.arange(n), out["propWR"].argmax(1).cpu().numpy()]

    # the plain FP32 global search on the same particles (per map)
    groups = [(int(c), torch.as_tensor(np.nonzero(unseen.cls == c)[0], device=dev))
              for c in np.unique(unseen.cls)]
    sub = []
    for c, idx in groups:
        m = len(idx)
        sub.append((c, m, unseen.dat[idx].contiguous(), unseen.ctf[idx].contiguous(),
                    unseen.sigRcp[idx].contiguous(),
                    dict(wC=torch.empty(m, **f64), wR=torch.empty((m, nRg), **f64),
                         wT=torch.empty((m, nTg), **f64), base=torch.empty(m, **f64))))
    pRg = torch.full((nRg,), 1.0 / nRg, **f64)
    pTg = torch.full((nTg,), 1.0 / nTg, **f64)

    def plain_step(precision=tg3.SCORE_FP32):
        for c, m, dd, cc, ss, o in sub:
            ctx.global_scan(c, m, nRg, nTg, dd, cc, ss, mats_g, trans_g, pRg, pTg, o["wC"],
                            o["wR"], o["wT"], o["base"], None, precision)
        ctx.sync()

    plain_step()
    plain_steps = max(1, min(args.steps, args.plain_steps))
    clk_p = ClockSampler(local_rank)
    clk_p.start()
    barrier(world)
    torch.cuda.nvtx.range_push("plain_step")
    e0.record(stream)
    for _ in range(plain_steps):
        plain_step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    clocks_p = clk_p.stop()
    tp_ms = reduce_max(world, e0.elapsed_time(e1))
    q_p = np.empty((n, 4))
    t_p = np.empty((n, 2))
    base_p = np.empty(n)
    for (c, idx), (_, m, _, _, _, o) in zip(groups, sub):
        g = idx.cpu().numpy()
        q_p[g] = quats_g[o["wR"].argmax(1).cpu().numpy()]
        t_p[g] = trans_g.cpu().numpy()[o["wT"].argmax(1).cpu().numpy()]
        base_p[g] = o["base"].cpu().numpy()

    # ---- 8. end to end through the host-buffer C ABI (page-locked inputs
    # copied in, poses copied out, inside the timed calls)
    hin = dict(images=unseen.images.cpu().pin_memory(), dat=unseen.dat.cpu().pin_memory(),
               ctf=unseen.ctf.cpu().pin_memory(), sig=unseen.sigRcp.cpu().pin_memory(),
               cls=cls_un.cpu().pin_memory(), gt=trans_g.cpu().pin_memory())
    hout = dict(q=torch.empty((n, 4), dtype=torch.float64).pin_memory(),
                t=torch.empty((n, 2), dtype=torch.float64).pin_memory(),
                b=torch.empty(n, dtype=torch.float64).pin_memory(),
                pk=torch.empty(n, dtype=torch.float32).pin_memory(),
                fb=torch.empty(n, dtype=torch.int32).pin_memory())

    def e2e_step():
        ctx.learned_expect_host(net, hin["images"], hin["dat"], hin["ctf"], hin["sig"],
                                hin["cls"], nRot, nTrans, 99, hin["gt"], tau, prec, hout["q"],
                                hout["t"], hout["b"], hout["pk"], hout["fb"])

    e2e_step()
    barrier(world)
    te = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    e2e_s = reduce_max(world, time.perf_counter() - te)
    e2e_same = bool(np.array_equal(hout["q"].numpy(), q_l))
    h2d = sum(int(v.numel() * v.element_size()) for v in hin.values())
    d2h = sum(int(v.numel() * v.element_size()) for v in hout.values())

    # ---- 9. the fallback by likelihood, measured beside the threshold: the
    # global search on every particle, its pose taken where its best
    # likelihood beats the proposal's
    o_all = outputs(n, full=False)
    expect(unseen, float("inf"), o_all)          # every particle through the global search
    torch.cuda.synchronize()
    tb = time.perf_counter()
    expect(unseen, float("inf"), o_all)
    t_all_ms = reduce_max(world, (time.perf_counter() - tb) * 1e3)
    base_gs = o_all["baseL"].cpu().numpy()
    q_gs = o_all["bestQuat"].cpu().numpy()
    t_gs = o_all["bestTrans"].cpu().numpy()
    ruleB = base_gs > prop_base
    t_prop_best = ptr_un[np.arange(n), out["propWT"].argmax(1).cpu().numpy()]
    q_B = np.where(ruleB[:, None], q_gs, q_prop_best)
    t_B = np.where(ruleB[:, None], t_gs, t_prop_best)
    del o_all

    # ---- 10. one local refinement phase about each method's pose
    # (1,000 vMF rotations, kappa 200, x 100 translations, deviation 2 px)
    def refine(q, t, precision):
        torch.cuda.synchronize()
        ta = time.perf_counter()
        qn, tn, _ = learned.local_refine(ctx, unseen, torch.as_tensor(q, **f64),
                                         torch.as_tensor(t, **f64), 200.0, 2.0, precision, gen)
        torch.cuda.synchronize()
        return qn.cpu().numpy(), tn.cpu().numpy(), (time.perf_counter() - ta) * 1e3

    q_p_r, t_p_r, tr_p_ms = refine(q_p, t_p, tg3.SCORE_FP32)
    q_l_r, t_l_r, tr_l_ms = refine(q_l, t_l, prec)
    q_B_r, t_B_r, _ = refine(q_B, t_B, prec)
    qt = unseen.quat_true
    err = lambda q: learned.angle_deg(q, qt)
    med = lambda x: round(float(np.median(x)), 3)

    # ---- 11. FSC-0.143 of the held-out maps reconstructed from each method's
    # refined poses (and from the true poses)
    poses = {"true_poses": (qt, unseen.trans_true),
             "plain_fp32_refined": (q_p_r, t_p_r),
             "learned_refined": (q_l_r, t_l_r),
             "plain_fp32_e_step": (q_p, t_p),
             "learned_e_step": (q_l, t_l)}
    fsc_res = {k: reconstruction_resolution(tg3, torch, ctx, unseen, maps, q, t, box, pf, px, rU,
                                            dev)
               for k, (q, t) in poses.items()}

    # ---- 12. the FP64 oracle on the proposals of >= 1,000 held-out
    # particles: the same argmax among the proposals, and the error of the
    # log-likelihood differences L - max L
    parity = None
    if args.check_particles > 0 and rank == 0:
        parity = proposal_parity_fp64(ctx, maps, unseen, idx_un, ptr_un, dvp_un, quats_g, box, pf,
                                      args.check_particles, dev)

    # ---- 13. rates, roofline, baselines
    stages = {k: {"ms_per_step": round(v[0] / args.steps, 4), "launches": v[1]}
              for k, v in st_l.items() if v[1]}
    ms_step = tl_ms / args.steps
    v_l = job_rate(n, ms_step + n * map_ms_pp, world)
    v_p = job_rate(n, tp_ms / plain_steps, world)
    # the learned step's kernels against their rooflines; the dominant one
    # is the line's roofline
    dom, roofs = learned_rooflines(st_l, args.steps, n, nRot, nTrans, K, ctx_kp(K),
                                   int(fb.sum()), nRg, nTg, args.bank_form, ms_step)
    roof = dict(roofs[dom]) if dom else {"kernel": None, "note": "no stage timed"}
    res = {
        "metric": METRIC, "value": round(v_l, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3 (split-bf16 cross term, FP32 accumulate)" if prec == tg3.SCORE_BF16X3
                 else "fp32",
        "data": "synthetic (seeded blob maps and particles; no dataset is named)",
        "config": {"workload": f"learned E-step, box {box}: 16 blob maps {box}^3 "
                               f"({L['n_blobs']} blobs, {px} A/px), 12 for training, 4 held out; "
                               f"{n} particles of the held-out maps per step; proposals "
                               f"{nRot} rotations x {nTrans} translations rescored exactly, "
                               f"fallback {nRg} x {nTg} global search; cutoff {rU}, K = {K}",
                   "snr": f"{L['snr_lik']} over the likelihood's pixels",
                   "train_particles": 0 if args.load_net else args.train_particles,
                   "epochs": args.epochs, "network": ("loaded: " + args.load_net) if args.load_net
                   else "trained in this run",
                   "labels": "the plain method's converged poses: the global search, then "
                             "three local phases of 1,000 x 100 (kappa 200 / 1,000 / 5,000, "
                             "translation deviation 2 / 0.7 / 0.3 px), scored in "
                             + ("FP32" if lab_prec == tg3.SCORE_FP32 else "split-bf16"),
                   "l2": "inputs larger than L2 (pixel data 159 MB, banks 0.55 GB per map)",
                   "per_map_work": f"references and bank once per map ({map_ms:.1f} ms), "
                                   f"charged over {per_map_particles} particles per map"},
        "clocks": clocks,
        "e2e": {"value": round(job_rate(n * args.e2e_steps, e2e_s * 1e3 + n * args.e2e_steps
                                        * map_ms_pp, world), 1),
                "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "wall_s": round(e2e_s, 3), "entry": "tg3_ExpectLearned3D (host buffers)",
                "same_poses_as_device_entry": e2e_same},
        "gpu_launches": learned_launches(fb, unseen.cls, args.bank_form != 1,
                                         args.bank_order and args.bank_form != 1) * args.steps,
        "roofline": roof,
        "roofline_kernels": roofs,
        "rescoring_forms": ab,
        "stages": stages,
        "plain_fp32": {"value": round(v_p, 1), "ms_per_step": round(tp_ms / plain_steps, 3),
                       "steps": plain_steps, "clocks": clocks_p,
                       "what": f"FP32 global search, {nRg} x {nTg} hypotheses per particle"},
        "speedup_vs_plain_fp32": round(v_l / v_p, 2),
        "hypotheses_per_s": round(v_l * (nRot * nTrans + fb.mean() * nRg * nTg), 1),
        "pose": {
            "median_error_deg": {"plain_fp32_e_step": med(err(q_p)),
                                 "learned_e_step": med(err(q_l)),
                                 "plain_fp32_refined": med(err(q_p_r)),
                                 "learned_refined": med(err(q_l_r)),
                                 "global_wins_rule_refined": med(err(q_B_r)),
                                 "plain_method_converged": med(err(conv_un))},
            "refined_gap_deg": round(float(np.median(err(q_l_r)) - np.median(err(q_p_r))), 3),
            "within_5deg_of_plain_converged": round(float(np.mean(
                learned.angle_deg(q_l_r, conv_un) < 5.0)), 4),
            "note": "error = angle between the method's best rotation and the true one; "
                    "refined = after one local phase of 1,000 x 100 about the method's pose "
                    "(plain in FP32, learned in its own precision)"},
        "fsc_0143_resolution_A": fsc_res,
        "fsc_gap_refined_A": round(fsc_res["learned_refined"] - fsc_res["plain_fp32_refined"], 3),
        "fallback": {
            "rule": "peak score (best - median) / (1.4826 MAD) of the rescored proposals below "
                    "a threshold; threshold = 5 % quantile of the peaks of the held-out "
                    "particles of the training maps whose proposal is within 10 degrees of "
                    "the plain method's converged pose",
            "threshold": round(tau, 4), "fraction": round(float(fb.mean()), 4),
            "global_wins_rule": {
                "rule": "global search on every particle; its pose where its best likelihood "
                        "beats the proposal's",
                "fraction": round(float(ruleB.mean()), 4),
                "particles_per_s": round(job_rate(n, t_all_ms + n * map_ms_pp, world), 1),
                "median_error_refined_deg": med(err(q_B_r))}},
        "with_refinement": {
            "plain_fp32_particles_per_s": round(job_rate(n, tp_ms / plain_steps + tr_p_ms,
                                                         world), 1),
            "learned_particles_per_s": round(job_rate(n, ms_step + n * map_ms_pp + tr_l_ms,
                                                      world), 1),
            "refine_ms": {"plain_fp32": round(tr_p_ms, 2), "learned": round(tr_l_ms, 2)}},
        "training": {"label_s": round(label_s, 1), "train_s": round(train_s, 1),
                     "restarts": restarts,
                     "label_median_error_deg": med(label_err),
                     "label_phase_moves_deg": [round(float(x), 3) for x in
                                               np.median(np.asarray(moves), 0)],
                     "loss_per_epoch": [round(x, 4) for x in losses]},
        "reference_maps": {"embed_ms_per_map": round(float(np.mean([embed_ms[c] for c in held])), 2),
                           "bank_ms_per_map": round(float(np.mean([bank_ms[c] for c in held])), 2)},
    }
    if parity is not None:
        res["parity_vs_fp64"] = parity
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline_global(ctx, maps[nTr], unseen, quats_g, box, pf,
                                                  args.cpu_sample_global, 1)
    net.close()
    ctx.close()
    return res


def learned_rooflines(st, steps, n, nRot, nTrans, K, Kp, nfb, nRg, nTg, bank_form, step_ms):
    """Rooflines of the learned step's kernels, from the stage times of the
    timed steps (CUDA events on the library's stream), and the dominant one.
    - rescoring slice gather (TG3_OPT_BANK_GATHER form): per proposed row its
      hi and lo bf16 rows (4 Kp bytes) and |P|^2 row (4 K) in, the operand
      rows (4 Kp) out;
    - rescoring cross term (every form): per launch the proposed rows' planes
      (4 Kp bytes a row), the shifted data (4 Kp a translation) and the
      log-likelihoods (4 bytes a hypothesis): HBM-bound (4 K FLOP per
      hypothesis, 3x that in bf16, is far below the tensor cores' rate);
    - fallback cross term (the global search of the fallback particles):
      4 K FLOP per hypothesis, nRg x nTg per fallback particle."""
    hbm, bf16, src = peaks()
    out = {}
    tot = lambda k: st[k][0] if st.get(k, (0, 0))[1] else 0.0
    if tot("project") > 0:
        algo = float(n) * nRot * (8.0 * Kp + 4.0 * K + 4.0) * steps
        ach = algo / (tot("project") * 1e-3) / 1e9
        out["rescoring_gather"] = {
            "kernel": "k_bank_gather (rescoring slices copied from the banks)", "bound": "hbm",
            "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
            "traffic": None, "algorithmic_bytes_per_launch": algo / steps}
    if tot("cross") > 0:
        # every form streams the proposed rows' planes: HBM-bound
        algo = (float(n) * nRot * 4.0 * Kp + float(n) * nTrans * 4.0 * Kp
                + float(n) * nRot * nTrans * 4.0) * steps
        ach = algo / (tot("cross") * 1e-3) / 1e9
        out["rescoring_cross"] = {
            "kernel": BANK_KERNELS[bank_form], "bound": "hbm", "achieved": round(ach, 1),
            "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4), "traffic": None,
            "algorithmic_bytes_per_launch": algo / steps,
            "tflops_algorithmic": round(4.0 * K * n * nRot * nTrans * steps
                                        / (tot("cross") * 1e-3) / 1e12, 2)}
    if tot("fallback_cross") > 0 and nfb > 0:
        flop = 4.0 * K * nfb * nRg * nTg * steps
        ach = flop / (tot("fallback_cross") * 1e-3) / 1e12
        out["fallback_cross"] = {
            "kernel": "k_gemm_bf16x3 (global search of the fallback particles)",
            "bound": "tensor", "achieved": round(ach, 2), "peak": bf16, "unit": "TFLOP/s",
            "frac": round(ach / bf16, 4), "traffic": None,
            "algorithmic_flop_per_step": flop / steps,
            "executed_bf16_flop_per_step": 3 * flop / steps}
    for k, v in out.items():
        stage = {"rescoring_gather": "project", "rescoring_cross": "cross",
                 "fallback_cross": "fallback_cross"}[k]
        v["ms_per_step"] = round(tot(stage) / steps, 4)
        v["share_of_step"] = round(tot(stage) / steps / step_ms, 4)
        v["peak_source"] = f"{'hbm_gbs' if v['bound'] == 'hbm' else 'bf16_tflops'}, {src} " \
                           "(MEASURED_PEAKS.json)"
    dom = max(out, key=lambda k: out[k]["ms_per_step"]) if out else None
    return dom, out


def learned_launches(fb, cls, bank_gemm, order=False):
    """Kernels of one learned E-step (this library's own): network 17 (8
    weight repacks, the first convolution, 6 tensor-core layers, the split-K
    sum, the output layer), matching 1, priors 3, rescoring 4 with the
    bank-row cross term (shift bank, |X|^2, cross term, weights; 5 with the
    slice gather or with the particles' visiting order sorted first),
    confidence and best pose 2; per class with fallback
    particles 13 (3 gathers, priors, |P|^2, translations, shift bank, |X|^2,
    norm operand, norm GEMM, cross term, weights, best pose) and 1 for the
    translation priors."""
    k = len(np.unique(np.asarray(cls)[np.asarray(fb, bool)]))
    return 17 + 1 + 3 + (4 + int(bool(order)) if bank_gemm else 5) + 2 + (13 * k + 1 if k else 0)


def _fp64_bank_rows(job):
    """Worker: FP64 oracle projections of rows [r0, r1) of one map's bank,
    written into the shared output file."""
    import sys as _s
    for p in job["paths"]:
        if p not in _s.path:
            _s.path.insert(0, p)
    from oracle import oracle as O
    vol = np.load(job["vol"], mmap_mode="r")
    out = np.load(job["out"], mmap_mode="r+")
    out[job["r0"]:job["r1"]] = O.project(np.asarray(vol), job["mats"], job["iCol"], job["iRow"],
                                         job["pf"])
    out.flush()
    return job["r1"] - job["r0"]


def proposal_parity_fp64(ctx, maps, ps, idx, trans, dvp, quats_g, box, pf, n_check, dev):
    """The FP64 oracle's log-likelihoods of the proposals of n_check
    particles (the first of every held-out map in turn): projections of the
    bank rotations by the oracle (a spawn pool over the host's cores),
    L(r, t) = sum_p sigRcp |X - c S_t P_r|^2 expanded as
    x0 + sum sigRcp c^2 |P_r|^2 - 2 Re sum sigRcp c conj(X) S_t P_r, checked
    against the oracle's logDataVSPrior on a sample.  Reports the fraction of
    particles whose best proposal (argmax over rotation x translation) is
    the oracle's, and the largest error of L - max L."""
    import multiprocessing as mp
    import tempfile
    import torch
    from tg3 import synth
    from oracle import oracle as O
    n = len(ps.cls)
    order = []
    per = {int(c): list(np.nonzero(ps.cls == c)[0]) for c in np.unique(ps.cls)}
    while len(order) < min(n_check, n):
        for c in per:
            if per[c] and len(order) < n_check:
                order.append(per[c].pop(0))
    order = np.asarray(order)
    iCol, iRow = ps.iCol, ps.iRow
    mats = synth.quat_to_mat(quats_g).reshape(-1, 9)
    workers = max(1, min(16, os.cpu_count() or 1))
    tmp = tempfile.mkdtemp()
    dat = ps.dat[torch.as_tensor(order, device=dev)].cpu().numpy().astype(np.complex128)
    ctf = ps.ctf[torch.as_tensor(order, device=dev)].cpu().numpy().astype(np.float64)
    sig = ps.sigRcp[torch.as_tensor(order, device=dev)].cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    same, max_err, max_err_near, checked = 0, 0.0, 0.0, 0
    spot = []
    ctxp = mp.get_context("spawn")
    with ctxp.Pool(workers) as pool:
        for c in sorted(set(int(x) for x in ps.cls[order])):
            vol = synth.padded_volume(maps[c], box, pf, device=dev,
                                      dtype=torch.float64).cpu().numpy()
            vpath = os.path.join(tmp, "vol.npy")
            opath = os.path.join(tmp, "bank.npy")
            np.save(vpath, vol)
            del vol
            bank = np.lib.format.open_memmap(opath, mode="w+", dtype=np.complex128,
                                             shape=(len(mats), len(iCol)))
            del bank
            step = (len(mats) + workers - 1) // workers
            jobs = [dict(vol=vpath, out=opath, r0=r0, r1=min(len(mats), r0 + step),
                         mats=mats[r0:r0 + step], iCol=iCol, iRow=iRow, pf=pf,
                         paths=[str(ROOT), str(PKG)]) for r0 in range(0, len(mats), step)]
            pool.map(_fp64_bank_rows, jobs)
            bank = np.load(opath, mmap_mode="r")
            for j in np.nonzero(ps.cls[order] == c)[0]:
                l = order[j]
                P = np.asarray(bank[idx[l]])                       # [nRot][K]
                S = O.translate(trans[l], box, iCol, iRow)         # [nTrans][K]
                X, cc, ss = dat[j], ctf[j], sig[j]
                x0 = float(np.sum(ss * np.abs(X) ** 2))
                nrm = (np.abs(P) ** 2) @ (ss * cc * cc)
                A = (ss * cc * np.conj(X))[None, :] * S
                cross = np.real(A @ P.T)                          # [nTrans][nRot]
                L64 = x0 + nrm[:, None] - 2.0 * cross.T           # [nRot][nTrans]
                if len(spot) < 8:
                    r, t = len(spot) % L64.shape[0], len(spot) % L64.shape[1]
                    ref = O.logdvp(X, S[t] * P[r], cc, ss)
                    spot.append(abs(ref - L64[r, t]) / abs(ref))
                d64 = L64 - L64.max()
                g = dvp[l].astype(np.float64)
                dg = g - g.max()
                same += int(np.argmax(L64) == np.argmax(g))
                e = np.abs(dg - d64)
                max_err = max(max_err, float(e.max()))
                near = d64 > -30.0
                max_err_near = max(max_err_near, float(e[near].max()))
                checked += 1
            del bank
            os.unlink(opath)
            os.unlink(vpath)
    os.rmdir(tmp)
    return {"particles": checked, "same_argmax": round(same / max(checked, 1), 5),
            "max_abs_err_dL": round(max_err, 5),
            "max_abs_err_dL_within_30": round(max_err_near, 5),
            "expansion_check_rel": float(max(spot)) if spot else None,
            "oracle_s": round(time.perf_counter() - t0, 1),
            "what": "the learned step's rescored proposals (split-bf16) against the FP64 "
                    "oracle: argmax over rotation x translation, and |(L - max L) - "
                    "(L64 - max L64)| over all hypotheses and over those within 30 of the "
                    "best (the ones with weight)"}


def cpu_baseline_global(ctx, bm, ps, quats_g, box, pf, n_rot, workers):
    """The oracle port of the reference's CPU global search (doGlobalSearch:
    projections of the rotations, then every image against every rotation x
    translation) on a bounded sample: one particle x n_rot of the 6,912
    rotations x 49 translations, scaled to a full particle (the projections
    are shared by all particles of an E-step and not charged)."""
    import torch
    from tg3 import synth
    from oracle import oracle as O
    vol = synth.padded_volume(bm, box, pf, device=ps.dat.device,
                              dtype=torch.float32).cpu().numpy().astype(np.complex128)
    sel = np.linspace(0, len(quats_g) - 1, n_rot).astype(int)
    mats = synth.quat_to_mat(quats_g[sel]).reshape(-1, 9)
    P = O.project(vol, mats, ps.iCol, ps.iRow, pf)
    trans = synth.global_translations(3, 1.0)
    S = O.translate(trans, box, ps.iCol, ps.iRow)
    l = int(np.nonzero(ps.cls == ps.cls[0])[0][0])
    X = ps.dat[l:l + 1].cpu().numpy().astype(np.complex128)
    c = ps.ctf[l:l + 1].cpu().numpy().astype(np.float64)
    s = ps.sigRcp[l:l + 1].cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    O.score_global(P, S, X, c, s, np.full(n_rot, 1.0 / n_rot), np.full(len(trans), 1.0 / len(trans)),
                   want_dvp=False)
    secs = time.perf_counter() - t0
    per_particle = secs * len(quats_g) / n_rot
    return {"value": round(1.0 / per_particle, 6), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"1 particle x {n_rot} of the {len(quats_g)} global rotations x "
                      f"{len(trans)} translations, K={len(ps.iCol)}, scaled to a full particle "
                      f"({secs:.2f} s measured); double-precision oracle port of the "
                      "reference's CPU global search (doGlobalSearch), one core"}


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per particle of a
# launch, box 256 local workload: one 1-pass ncu capture of a 64-particle
# launch (k_project 13.36 GB read + 5.09 GB written; k_gemm_bf16x3 5.62 GB +
# 0.02 GB), divided by 64.  Both grow in proportion to the particles of a
# launch (every particle's volume footprint and operand planes are its own).
TRAFFIC_PER_PARTICLE_BOX256 = {"project": 18.45e9 / 64, "cross_bf16x3": 5.643e9 / 64}


def traffic(key, box, nP):
    per = TRAFFIC_PER_PARTICLE_BOX256.get(key) if box == 256 else None
    return None if per is None else round(per * nP)


def ctx_kp(K):
    return int(math.ceil(2 * K / 64) * 64)


# --------------------------------------------------------------- CPU path ---
def _cpu_worker(job):
    """Score `job` particles with the oracle port (one process per core)."""
    import sys as _s
    for p in job["paths"]:
        if p not in _s.path:
            _s.path.insert(0, p)
    from oracle import oracle as O
    vol = job["vol"]
    if isinstance(vol, str):
        vol = np.load(vol, mmap_mode="r")
    out = []
    for d in job["items"]:
        r = O.score_local(vol, job["pf"], job["iCol"], job["iRow"], job["box"], d["dat"],
                          d["ctf"], d["sig"], d["quat"], d["trans"], d["pwR"], d["pwT"], 1.0,
                          want_dvp=False)
        src, w, top = O.resample(r["wR"], d["pwR"], d["perm_r"], d["u0_r"],
                                 O.peak_factor_r(r["wR"]), len(d["pwR"]))
        src, w, top = O.resample(r["wT"], d["pwT"], d["perm_t"], d["u0_t"], 0.0, len(d["pwT"]))
        out.append(r["base"])
    return out


def cpu_time(vol_np, st, host, W, n_particles, n_rot, workers):
    """Time the CPU path on a bounded sample: n_particles particles with n_rot
    of their rotations each (all translations), over `workers` processes."""
    import multiprocessing as mp
    items = []
    for l in range(n_particles):
        items.append(dict(dat=host["dat"][l].astype(np.complex128),
                          ctf=host["ctf"][l].astype(np.float64),
                          sig=host["sig"][l].astype(np.float64),
                          quat=host["quat"][l][:n_rot], trans=host["trans"][l],
                          pwR=host["pwR"][l][:n_rot] * (len(host["pwR"][l]) / n_rot),
                          pwT=host["pwT"][l], perm_r=np.random.default_rng(l).permutation(n_rot).astype(np.int32),
                          perm_t=host["perm_t"][l], u0_r=float(host["u0_r"][l]), u0_t=float(host["u0_t"][l])))
    paths = [str(ROOT), str(PKG)]
    if workers == 1:
        job = dict(items=items, vol=vol_np, pf=W["pf"], iCol=st.iCol, iRow=st.iRow,
                   box=W["box"], paths=paths)
        t0 = time.perf_counter()
        _cpu_worker(job)
        return time.perf_counter() - t0
    # the volume reaches the workers through one memory-mapped file
    import tempfile
    fd, vpath = tempfile.mkstemp(suffix=".npy")
    os.close(fd)
    np.save(vpath, np.ascontiguousarray(vol_np))
    try:
        jobs = [dict(items=items[i::workers], vol=vpath, pf=W["pf"], iCol=st.iCol,
                     iRow=st.iRow, box=W["box"], paths=paths) for i in range(workers)]
        jobs = [j for j in jobs if j["items"]]
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(jobs)) as pool:
            pool.map(_cpu_worker, jobs[:1])          # start-up and page-in, untimed
            t0 = time.perf_counter()
            pool.map(_cpu_worker, jobs)
            return time.perf_counter() - t0
    finally:
        os.unlink(vpath)


def cpu_baseline(st, host, W, sample_rot):
    """The oracle port of the reference CPU E-step, timed on this host."""
    from tg3 import synth
    import torch
    rng = np.random.default_rng(1001)
    bm = synth.blob_map(rng, W["n_blobs"], W["sigma_a"], W["pixel_size"], W["radius_px"])
    vol = synth.padded_volume(bm, W["box"], W["pf"], device="cuda" if torch.cuda.is_available() else "cpu",
                              dtype=torch.float32).cpu().numpy().astype(np.complex128)
    secs = cpu_time(vol, st, host, W, 1, sample_rot, 1)
    per_particle = secs * W["nR"] / sample_rot
    return {"value": round(1.0 / per_particle, 6), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"1 particle x {sample_rot} of its {W['nR']} rotations x {W['nT']} "
                      f"translations, K={st.K}, scaled to a full particle ({secs:.1f} s measured); "
                      "double-precision oracle port, one core"}


def _cpu_global_worker(job):
    """Score one particle against the shared projections (oracle port)."""
    import sys as _s
    for p in job["paths"]:
        if p not in _s.path:
            _s.path.insert(0, p)
    from oracle import oracle as O
    O.score_global(job["P"], job["S"], job["X"], job["c"], job["s"], job["pR"], job["pT"],
                   want_dvp=False)
    return 0


# a pool worker's copy of the reference arm's inputs, sent once at start-up
_CPU_JOBS = None


def _cpu_init(jobs):
    global _CPU_JOBS
    _CPU_JOBS = jobs


def _cpu_global_task(i):
    """Particle i of the inputs the worker received at start-up: only the
    index crosses the process boundary inside the timed steps."""
    return _cpu_global_worker(_CPU_JOBS[i])


def run_reference_learned(args, rank, world):
    """The reference's CPU E-step that the learned E-step replaces: the
    global search (doGlobalSearch, src/Optimiser.cpp:633-1136) of the
    held-out maps' particles over 6,912 rotations x 49 translations, as the
    oracle port on every host core (one particle per core), each step a
    bounded sample of the rotations scaled to full particles."""
    if rank != 0:
        return None
    import multiprocessing as mp
    import torch
    from tg3 import synth
    from oracle import oracle as O
    L = LEARNED256 if args.workload == "learned256" else LEARNED
    box, px, pf, rU = L["box"], L["pixel_size"], L["pf"], L["rU"]
    rng = np.random.default_rng(4000)
    maps = [synth.blob_map(rng, L["n_blobs"], L["sigma_a"], px, L["radius_px"])
            for _ in range(L["n_maps"])]
    rL = synth.config_rL(box, px)
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    cores = os.cpu_count() or 1
    nTr = L["n_train_maps"]
    noise_var = synth.signal_power(maps[:nTr], box, px, rU, rL, device=dev) / L["snr_lik"] / 2.0
    ps = synth.particle_set_dev(rank_seed(5002, rank), maps, np.full(cores, nTr), box, px, rU,
                                rL, L["shift"], noise_var, device=dev)
    vol = synth.padded_volume(maps[nTr], box, pf, device=dev,
                              dtype=torch.float32).cpu().numpy().astype(np.complex128)
    quats_g = synth.global_rotations(4, 36)
    n_rot = args.cpu_sample_global
    sel = np.linspace(0, len(quats_g) - 1, n_rot).astype(int)
    P = O.project(vol, synth.quat_to_mat(quats_g[sel]).reshape(-1, 9), ps.iCol, ps.iRow, pf)
    trans = synth.global_translations(3, 1.0)
    S = O.translate(trans, box, ps.iCol, ps.iRow)
    del vol
    X = ps.dat.cpu().numpy().astype(np.complex128)
    c = ps.ctf.cpu().numpy().astype(np.float64)
    s = ps.sigRcp.cpu().numpy().astype(np.float64)
    jobs = [dict(P=P, S=S, X=X[i:i + 1], c=c[i:i + 1], s=s[i:i + 1],
                 pR=np.full(n_rot, 1.0 / n_rot), pT=np.full(len(trans), 1.0 / len(trans)),
                 paths=[str(ROOT), str(PKG)]) for i in range(cores)]
    times = []
    # the inputs go to every worker once, at start-up (untimed); a step sends
    # each worker one particle index
    with mp.get_context("spawn").Pool(cores, initializer=_cpu_init, initargs=(jobs,)) as pool:
        pool.map(_cpu_global_task, range(cores), chunksize=1)   # start-up and page-in
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_cpu_global_task, range(cores), chunksize=1)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    value = cores * (n_rot / len(quats_g)) / per_step
    sample = (f"{cores} particles of a held-out map (one per core) x {n_rot} of the "
              f"{len(quats_g)} global rotations x {len(trans)} translations per step, K = "
              f"{len(ps.iCol)}, scaled to full particles (the projections, shared by every "
              "particle of an E-step, are made once and not timed); double-precision oracle "
              "port of doGlobalSearch (the reference's sources are not on this machine)")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(per_step * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic", "config": {"workload": f"E-step of the held-out maps' "
                                            f"particles, box {box}: global search "
                                            f"{len(quats_g)} x {len(trans)}, cutoff {rU}, "
                                            f"K = {len(ps.iCol)}",
                                            "sample_rotations": n_rot,
                                            "particles_per_step": cores},
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def run_reference(args, rank, world):
    """The CPU implementation of the path on all host cores (rank 0 only)."""
    if args.workload in ("learned128", "learned256"):
        return run_reference_learned(args, rank, world)
    if rank != 0:
        return None
    import torch
    from tg3 import synth
    W = dict(WORKLOAD)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(1001)
    bm = synth.blob_map(rng, W["n_blobs"], W["sigma_a"], W["pixel_size"], W["radius_px"])
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    vol = synth.padded_volume(bm, W["box"], W["pf"], device=dev,
                              dtype=torch.float32).cpu().numpy().astype(np.complex128)
    n = cores
    rL = synth.config_rL(W["box"], W["pixel_size"])
    st = synth.make_stack(1002, [bm], W["box"], W["pixel_size"], W["pf"], W["rU"], rL, n,
                          W["shift"], W["snr"], device=dev)
    qc, tc = synth.perturb_poses(rng, st.quat_true, st.trans_true, 3.0, 1.0)
    qs, ts = synth.local_hypotheses(rng, qc, tc, W["nR"], W["nT"], W["kappa"], 2.0)
    host = dict(dat=st.dat, ctf=st.ctf, sig=st.sigRcp, quat=qs, trans=ts,
                pwR=np.full((n, W["nR"]), 1.0 / W["nR"]), pwT=np.full((n, W["nT"]), 1.0 / W["nT"]),
                perm_t=np.stack([rng.permutation(W["nT"]) for _ in range(n)]).astype(np.int32),
                u0_r=rng.random(n) / W["nR"], u0_t=rng.random(n) / W["nT"])
    n_rot = args.cpu_sample
    times = []
    for i in range(args.warmup + args.steps):
        secs = cpu_time(vol, st, host, W, n, n_rot, cores)
        if i >= args.warmup:
            times.append(secs)
    per_step = float(np.mean(times))
    value = n * n_rot / W["nR"] / per_step
    return {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(per_step * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic", "config": {"workload": "local particle-filter phase, box 256, "
                                            "K=9930, 1000 rotations x 100 translations",
                                            "sample_rotations": n_rot, "particles_per_step": n},
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n} particles (one per core) x {n_rot} of 1000 rotations "
                                       "x 100 translations per step, scaled to full particles; "
                                       "double-precision oracle port (the reference sources are "
                                       "not present on this machine)"},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


# ------------------------------------------------------------ distributed ---
_pg = None


def init_dist():
    global _pg
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        _pg = dist
    return rank, world, local


def barrier(world):
    if world > 1 and _pg is not None:
        _pg.barrier()


def reduce_max(world, x: float) -> float:
    if world > 1 and _pg is not None:
        import torch
        t = torch.tensor([float(x)])
        _pg.all_reduce(t, op=_pg.ReduceOp.MAX)
        return float(t.item())
    return float(x)


def rank_seed(base: int, rank: int) -> int:
    """Seed of one rank's particles: every rank scores its own particles (the
    E-step shards over particles with no exchange), so the sets differ."""
    return base + 97 * rank


def job_rate(units_per_rank: float, ms: float, world: int) -> float:
    """Whole-job throughput (units/s): the units all ranks processed over the
    slowest rank's time; `ms` is already the max over ranks."""
    return units_per_rank * world / (ms * 1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tg3", choices=["tg3", "reference"])
    ap.add_argument("--precision", default="bf16x3", choices=["fp32", "bf16x3"])
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain FP32 measurement beside a bf16x3 run")
    ap.add_argument("--batch", type=int, default=128, help="particles per step")
    ap.add_argument("--batches", type=int, default=3, help="distinct particle batches cycled")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-sample", type=int, default=40,
                    help="rotations per particle in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fused", action="store_true",
                    help="split-bf16 path through the fused projection + tcgen05 kernel")
    ap.add_argument("--box", type=int, default=None, help="reduced box (profiling only)")
    ap.add_argument("--workload", default="learned256",
                    choices=["local256", "local256c3", "global64", "uneven192", "learned128",
                             "learned256", "class2d128", "prep256", "reco256", "bank256",
                             "fallback256"])
    ap.add_argument("--train-particles", type=int, default=150000)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--learned-snr", type=float, default=1.0,
                    help="noise level of the learned-proposal particles (signal / noise power)")
    ap.add_argument("--learned-lr", type=float, default=2e-3)
    ap.add_argument("--learned-mode", default="match", choices=["match", "regress"],
                    help="learned proposal: embedding match against the map's reference "
                         "projections, or pose regression")
    ap.add_argument("--learned-tau", type=float, default=0.1,
                    help="temperature of the matching loss")
    ap.add_argument("--eval-particles-seen", type=int, default=1200)
    ap.add_argument("--eval-particles-unseen", type=int, default=2000)
    ap.add_argument("--batch-uneven", type=int, default=4096,
                    help="particles per ragged plan (uneven192)")
    ap.add_argument("--per-particle-sample", type=int, default=256,
                    help="particles timed one at a time beside the plan (uneven192)")
    ap.add_argument("--global-particles", type=int, default=2000)
    ap.add_argument("--label-precision", default="bf16x3", choices=["fp32", "bf16x3"],
                    help="precision of the plain method that labels the training particles")
    ap.add_argument("--plain-steps", type=int, default=20,
                    help="timed steps of the plain FP32 global search beside the learned step")
    ap.add_argument("--check-particles", type=int, default=1000,
                    help="particles whose proposals are checked against the FP64 oracle")
    ap.add_argument("--cpu-sample-global", type=int, default=96,
                    help="rotations per particle in the CPU global-search sample")
    ap.add_argument("--bank-form", type=int, default=0, choices=[0, 1, 2],
                    help="rescoring form (TG3_OPT_BANK_GATHER): 0 cross term gathers the bank "
                         "rows with cp.async, 1 rows copied out first, 2 TMA gathers")
    ap.add_argument("--scan-pair", type=int, default=0, choices=[0, 1],
                    help="TG3_OPT_SCAN_PAIR: the global search's cross term on CTA pairs that "
                         "share each column tile by TMA multicast")
    ap.add_argument("--local-bk", type=int, default=64, choices=[32, 64],
                    help="TG3_OPT_LOCAL_BK: K block of the local phase's split cross term")
    ap.add_argument("--bank-shape", type=int, default=3, choices=[0, 1, 2, 3],
                    help="TG3_OPT_BANK_SHAPE: the cp.async bank cross term's K block and "
                         "CTAs per SM (0: 64, one; 1: 32, twice the stages; 2: 32, two; "
                         "3: as 0 with 16 gather warps)")
    ap.add_argument("--project-group", type=int, default=8, choices=[4, 8, 16],
                    help="TG3_OPT_PROJECT_GROUP: rotations per projection CTA (forms 3, 4)")
    ap.add_argument("--project-form", type=int, default=4, choices=[0, 1, 2, 3, 4],
                    help="TG3_OPT_PROJECT_FORM: 0 a lane pair per pixel, 1 one lane per pixel, "
                         "2 one lane per pixel with the block index computed, 3/4 lane pairs "
                         "sharing whole-block loads (index looked up / computed)")
    ap.add_argument("--scan-bk", type=int, default=32, choices=[32, 64],
                    help="TG3_OPT_SCAN_BK: K block of the global search's cross-term stages")
    ap.add_argument("--bank-order", type=int, default=1, choices=[0, 1],
                    help="TG3_OPT_BANK_ORDER: particles visited sorted by first proposed row")
    ap.add_argument("--no-local", action="store_true",
                    help="learned workloads: skip the local-phase measurement beside them")
    ap.add_argument("--save-net", default=None,
                    help="learned workloads: save the trained network's parameters (.npz)")
    ap.add_argument("--load-net", default=None,
                    help="learned workloads: use saved parameters instead of labelling and "
                         "training (profiling runs)")
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args()
    rank, world, local = init_dist()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    elif args.workload == "global64":
        res = run_global(args, rank, world, local)
    elif args.workload == "uneven192":
        res = run_uneven(args, rank, world, local)
    elif args.workload == "class2d128":
        res = run_class2d(args, rank, world, local)
    elif args.workload == "prep256":
        res = run_prep(args, rank, world, local)
    elif args.workload == "reco256":
        res = run_reco(args, rank, world, local)
    elif args.workload == "bank256":
        res = run_bank(args, rank, world, local)
    elif args.workload == "fallback256":
        res = run_fallback(args, rank, world, local)
    elif args.workload in ("learned128", "learned256"):
        res = run_learned(args, rank, world, local)
        if args.workload == "learned256" and not args.no_local:
            # the local particle-filter phase at box 256 (1,000 x 100 per
            # particle), split-bf16 beside plain FP32, kept beside the headline
            import torch
            torch.cuda.empty_cache()
            loc = run_tg3(args, rank, world, local)
            if res is not None and loc is not None:
                res["local_phase_box256"] = {k: v for k, v in loc.items()
                                             if k not in ("metric", "n_gpus", "higher_is_better",
                                                          "scaling", "vs_baseline", "data")}
    else:
        res = run_tg3(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1 and _pg is not None:
        _pg.destroy_process_group()


if __name__ == "__main__":
    main()
