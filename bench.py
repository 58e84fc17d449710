#!/usr/bin/env python
"""Benchmark of the reconstruction path on one workload.

Default workload (rytov_1024): 600 synthetic off-axis holograms, 1024 x 1024
uint16 (12-bit), NXMAX 128 (256 x 256 fields), Rytov fields with Volkov
unwrapping and aberration correction, mapped into a 512^3 spectrum and
inverted.  One step reconstructs one volume from its 600 holograms.

  value  volumes/s with the holograms already in HBM (device buffers)
  e2e    volumes/s through the C ABI with pinned host holograms and host
         outputs (index, absorption, OTF mask), copies inside the timed region:
         consecutive volumes queued with tdm_pipeline_async (a volume's
         downloads overlap the next one's uploads and kernels); sync_value is
         the same with one blocking tdm_pipeline call per volume

Multi-GPU (torchrun): independent replicas, one volume per rank per step,
no data-path collective; value is the whole-job volumes/s.

--impl reference times the FP64 CPU restatement of the reference (the
reference's programs link FFTW3, OpenCV and libtiff, none of which the GPU
host has) on the host cores, each step a bounded sample of the same
workload, with the value credited scipy's FFT where that beats the oracle's.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "512³ volumes/s (600 holos): plain vs batched/TV-adjoint; rel-L2≤1e-4 vs FP64"
UNIT = "volumes/s"
E2E_TRIALS = 5
SCHEDULE = (16, 4)  # angles per chunk, chunks in flight (tdm_set_schedule)

# Algorithmic bytes per launch unit: the compulsory input and output bytes of
# each kernel (what it must read and write at least once, wherever it lives).
def algorithmic_bytes(name, acq, hits_per_angle, band):
    H, F, D = acq.ccd_roix, 2 * acq.nxmax, acq.dim_final
    per_angle = {
        "extract_rows": H * H * 2 + H * F * 8,
        "extract_cols": H * F * 8 + F * F * 8,
        "argmax": F * F * 8,
        "field_rows": F * F * 8 * 2,
        "field_cols": F * F * 8 + F * F * 4 * 2,
        # phasor in, gx out
        "volkov_rows": F * F * 8 + F * F * 4,
        # phasor and gx in; the columns' DCT-II of gx and DST-II of gy out
        "volkov_cols": F * F * 8 + F * F * 4 + F * F * 8,
        # those in, one real row of the Poisson solve's DCT-III along x out
        "volkov_integ_rows": F * F * 8 + F * F * 4,
        # that in, the unwrapped phase out
        "volkov_integ_cols": F * F * 4 * 2,
        "aber_fit": 2 * F * F * 4,
        "form": 3 * F * F * 4 + F * F * 8,
        "cap_rows": 2 * F * F * 8,
        "cap_cols": F * F * 8 + F * F * 10,
    }
    per_volume = {
        # the gather with the z pass: cap cells in, the z-transformed spectrum and the OTF out
        "gather": hits_per_angle * acq.nb_holo * 10 + D ** 3 * 8 + D ** 3,
        "ypass": 2 * D ** 3 * 8,
        "xpass": D ** 3 * 8 + 2 * D ** 3 * 4,
    }
    return per_angle, per_volume


# Algorithmic bytes per stage of the path, compulsory input plus output of the
# stage as a whole (the intermediates between a stage's kernels are not
# counted; hits = NA-disc bins per angle):
#   extraction   per hologram  H^2 2 (uint16) + F^2 8 (complex crop)
#   fields       per angle     F^2 8 + F^2 8
#   cap mapping  per angle     F^2 8 + hits (8 + 4) 2
#   volume       per volume    D^3 12 (zeroing) + D^3 12 (normalise, 3D IFFT) + D^3 8 (two f32 volumes)
# Each stage's time is the sum of its kernels' event times (one chunk in
# flight).  The fields' last step (forming the field from the unwrapped phase
# and the fits) runs fused into the cap mapping's row pass, and is timed there.
STAGE_KERNELS = {
    "extraction": ("extract_rows", "extract_cols", "argmax"),
    "fields": ("field_rows", "field_cols", "volkov_rows", "volkov_cols", "volkov_integ_rows",
               "volkov_integ_cols", "aber_fit", "form"),
    "cap_mapping": ("cap_rows", "cap_cols"),
    "volume": ("gather", "ypass", "xpass"),
}


# Stage of each kernel, for the dominant kernel's roofline: its achieved
# bandwidth is the stage's per-unit algorithmic bytes (above) times the units
# its launches process, over its own launch time.
KERNEL_STAGE = {k: st for st, ks in STAGE_KERNELS.items() for k in ks}


def stage_bytes(acq, hits_per_angle):
    H, F, D, M = acq.ccd_roix, 2 * acq.nxmax, acq.dim_final, acq.nb_holo
    return {
        "extraction": M * (H * H * 2 + F * F * 8),
        "fields": M * (F * F * 8 * 2),
        "cap_mapping": M * (F * F * 8 + hits_per_angle * (8 + 4) * 2),
        "volume": D ** 3 * (12 + 12 + 8),
    }


def stage_roofline(acq, hits_per_angle, kern_ms, step_ms, peak):
    """Achieved GB/s and fraction of the HBM peak per stage (from the per-kernel
    event times kern_ms, ms per step), and for the whole path over the live
    step time step_ms."""
    b = stage_bytes(acq, hits_per_angle)
    out = {}
    for st, ks in STAGE_KERNELS.items():
        t = sum(kern_ms.get(k, 0.0) for k in ks)
        if t > 0:
            gbs = b[st] / (t / 1e3) / 1e9
            out[st] = {"bytes_per_step": int(b[st]), "ms_per_step": round(t, 4), "achieved_gbs": round(gbs, 1),
                       "frac": round(gbs / peak, 4)}
    tot = sum(b.values())
    if step_ms > 0:
        gbs = tot / (step_ms / 1e3) / 1e9
        out["whole_path_live"] = {"bytes_per_step": int(tot), "ms_per_step": round(step_ms, 4),
                                  "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    return out


# DRAM bytes (read + write) per launch from the committed ncu capture of
# the kernel on this code (the file named in the returned source), as
# (bytes that do not depend on the angle count, bytes per 600 angles): the
# row pass on the 64-hologram case (a launch processes 16 holograms), the
# gather on the 600-angle workload (its record reads grow with the angles;
# its volume and OTF writes do not).  None where no capture of this
# workload's kernel is committed.
NCU_TRAFFIC = {
    "extract_rows": (33.616128e6 + 0.341504e6, 0.0, "profiles/k_extract_rows_rytov_1024_64holos.md"),
    "gather": (1083.210e6, 393.620e6, "profiles/k_gather_z_rytov_1024.md"),
}


def ncu_traffic_per_launch(name, acq):
    if acq.ccd_roix != 1024 or acq.nxmax != 128 or acq.dim_final != 512 or name not in NCU_TRAFFIC:
        return None, None
    fixed, per600, src = NCU_TRAFFIC[name]
    return fixed + per600 * acq.nb_holo / 600, src


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark(self) -> int:
        """Index of the next sample: samples from a mark on fall in the timed region."""
        return len(self.lines)

    def stop(self, first: int = 0, last: int = None) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines[first:last]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def schedule_for(angles: int):
    """SCHEDULE, with its chunks in flight limited to the context's scratch
    capacity (min(128, angles rounded up to 16) angles)."""
    cap = min(128, (angles + 15) // 16 * 16)
    return SCHEDULE[0], max(1, min(SCHEDULE[1], cap // SCHEDULE[0]))


def max_over_ranks(values, world: int, device):
    """Element-wise maximum of per-rank timings over the job's ranks (the
    slowest rank sets the whole job's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), device=device, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def host_link_probe(h_in, d_in, pairs_out, reps: int = 3, chunk: int = 128 << 20):
    """Copy throughput of the host link with the step's own pinned buffers:
    h_in -> d_in alone, the (device, host) pairs_out device -> host alone, and
    both at once on two streams; 128 MB copies, about the size of the
    pipeline's grouped uploads (four 16-hologram chunks), best of reps.
    GB/s (1e9 bytes/s)."""
    import torch
    src = h_in.view(-1).view(torch.uint8)
    dst = d_in.view(-1).view(torch.uint8)
    outs = [(d.view(-1).view(torch.uint8), h.view(-1).view(torch.uint8)) for d, h in pairs_out]
    n_in = src.numel()
    n_out = sum(d.numel() for d, _ in outs)
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()

    def up():
        with torch.cuda.stream(s_in):
            for o in range(0, n_in, chunk):
                dst[o:o + chunk].copy_(src[o:o + chunk], non_blocking=True)

    def down():
        with torch.cuda.stream(s_out):
            for d, h in outs:
                for o in range(0, d.numel(), chunk):
                    h[o:o + chunk].copy_(d[o:o + chunk], non_blocking=True)

    def best(*fns):
        t_best = 1e9
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            for f in fns:
                f()
            torch.cuda.synchronize()
            t_best = min(t_best, time.perf_counter() - t)
        return t_best

    t_up, t_down, t_both = best(up), best(down), best(up, down)
    return {"h2d_gbs": round(n_in / t_up / 1e9, 1), "d2h_gbs": round(n_out / t_down / 1e9, 1),
            "both_gbs": round((n_in + n_out) / t_both / 1e9, 1), "both_ms": round(1e3 * t_both, 3)}


def whole_job_rate(world: int, steps: int, seconds: float) -> float:
    """Units per second of the whole job: each of the `world` replicas
    processed `steps` units in at most `seconds`."""
    return world * steps / seconds


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(acq, ph, seed, sample_angles: int, threads: int):
    """FP64 oracle on a bounded sample: `sample_angles` holograms through
    extraction, field formation and cap mapping, plus one full volume stage;
    extrapolated to the workload's angle count."""
    import numpy as np

    import oracle
    from tests import simul
    from tests.helpers import oracle_cfg
    oracle.set_threads(threads)
    cfg = oracle_cfg(acq)
    d = simul.holograms(acq, ph, M=sample_angles, seed=seed)
    holos = d["holos"].numpy().astype(np.float64)
    t0 = time.perf_counter()
    spec = oracle.extract_stack(holos, cfg)
    t1 = time.perf_counter()
    fields, pos = oracle.fields(spec, cfg, d["mask"].numpy())
    t2 = time.perf_counter()
    r = oracle.reconstruction(fields, pos, cfg, want_counts=False, want_otf=False)
    loop_s, vol_s = float(r["seconds"][0]), float(r["seconds"][1])
    per_angle = (t1 - t0 + t2 - t1 + loop_s) / sample_angles
    total = per_angle * acq.nb_holo + vol_s
    return {"per_angle_s": per_angle, "volume_s": vol_s, "seconds_per_volume": total,
            "sample_wall_s": time.perf_counter() - t0}


def fft_check(acq, threads: int):
    """The oracle's FFT against scipy.fft (workers = threads) on the transform
    sizes of one volume: the hologram (H^2), the field (F^2), the Volkov mirror
    ((2F)^2) and the volume (D^3), complex128, ms per transform.  Returns the
    timings and the CPU seconds per volume that scipy's FFT would save where it
    is faster: per hologram one H^2, per angle two F^2 and nine (2F)^2
    transforms, and one D^3 transform."""
    import numpy as np
    import scipy.fft

    import oracle
    oracle.set_threads(threads)
    rng = np.random.default_rng(0)
    H, F, D, M = acq.ccd_roix, 2 * acq.nxmax, acq.dim_final, acq.nb_holo
    out = {}
    for name, shape, reps in (("hologram", (H, H), 3), ("field", (F, F), 10), ("mirror", (2 * F, 2 * F), 5),
                              ("volume", (D, D, D), 1)):
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        ofn = oracle.fft3d if len(shape) == 3 else oracle.fft2d
        ofn(a)
        t0 = time.perf_counter()
        for _ in range(reps):
            ofn(a)
        t_o = (time.perf_counter() - t0) / reps
        scipy.fft.fftn(a, workers=threads)
        t0 = time.perf_counter()
        for _ in range(reps):
            scipy.fft.fftn(a, workers=threads)
        t_s = (time.perf_counter() - t0) / reps
        out[name] = {"shape": list(shape), "oracle_ms": round(1e3 * t_o, 3), "scipy_ms": round(1e3 * t_s, 3)}
    gain = lambda k: max(0.0, out[k]["oracle_ms"] - out[k]["scipy_ms"]) / 1e3  # noqa: E731
    saved = M * (gain("hologram") + 2 * gain("field") + 9 * gain("mirror")) + gain("volume")
    return out, saved


def run_reference(args, acq, ph, seed):
    """The reference arm: the FP64 oracle port on all host threads.  Each step
    is a bounded sample of the workload, `--ref-sample` holograms through
    extraction, fields and cap mapping plus one full volume stage, and
    `ms_per_step` is that sample's wall time.  The value extrapolates the
    timed steps to the workload's hologram count, less the time that scipy's
    FFT would save over the oracle's own on every transform of a volume
    (measured once in warm-up), so the figure favours the reference."""
    threads = os.cpu_count() or 1
    import oracle
    oracle.build()
    S = args.ref_sample
    saved, per, vol, wall = None, [], [], []
    for i in range(args.warmup + args.steps):
        if i == 0:
            _, saved = fft_check(acq, threads)
        t0 = time.perf_counter()
        r = cpu_baseline(acq, ph, seed + i, S, threads)
        if i >= args.warmup:
            wall.append(time.perf_counter() - t0)
            per.append(r["per_angle_s"])
            vol.append(r["volume_s"])
    spv_port = statistics.mean(per) * acq.nb_holo + statistics.mean(vol)
    spv = max(spv_port - saved, 1e-9)
    value = 1.0 / spv
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(wall),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(acq, args),
        "seconds_per_volume": spv, "seconds_per_volume_oracle_fft": spv_port,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: {S} of {acq.nb_holo} holograms through extraction, fields and cap "
                                   f"mapping plus one {acq.dim_final}^3 volume stage; value = the steps' per-hologram "
                                   f"time x {acq.nb_holo} + the volume stage, less {saved:.1f} s per volume that "
                                   f"scipy's FFT saves over the oracle's ({1.0 / spv_port:.4f} volumes/s without)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def tv_form(iterations: int = 50, segment: int = 5):
    """Regularised reconstruction form: forward-operator data of a missing-cone
    phantom (two touching cells, dn 0.03) on 256^3 from 400 caps of 128^2,
    single-pass reconstruction against projected gradient with positivity and
    TV 1e-3.  The iterations run in segments of `segment`, each resuming from
    the previous segment's saved iterate, with the error to the phantom read
    between segments."""
    from dataclasses import replace

    import numpy as np
    import torch

    from mtd_transmission_gb300 import Context, Geometry
    from tests import simul
    acq, _, _ = simul.workload("plain_512_born")
    M = 400
    acq = replace(acq, nb_holo=M)
    N, D = acq.nxmax, acq.dim_final
    t = simul.spiral_tilts(M, N)
    pos = torch.from_numpy(np.concatenate([N + t[:, 0], N + t[:, 1]]).astype(np.int32)).cuda()
    z, y, x = torch.meshgrid(*(torch.arange(D, device="cuda", dtype=torch.float32) - D / 2,) * 3, indexing="ij")
    truth = torch.zeros((D, D, D), device="cuda")
    for cx in (-0.12 * D, 0.12 * D):
        truth[(x - cx) ** 2 + y ** 2 + (z / 0.8) ** 2 < (0.12 * D) ** 2] = 0.03
    del x, y, z

    def err(v):
        return float(torch.linalg.vector_norm(v - truth) / torch.linalg.vector_norm(truth))

    opts = dict(step=1.0, tv_weight=1e-3, tv_eps=1e-3, index_min=0.0, index_max=0.1)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        caps = torch.empty((M, 2 * N, 2 * N, 2), device="cuda")
        ctx.forward(truth, None, n=M, posspec=pos, caps_out=caps)
        born = torch.empty_like(truth)
        ctx.tv_reconstruct(born, caps=caps, n=M, posspec=pos, iterations=0, init=1)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.tv_reconstruct(born, caps=caps, n=M, posspec=pos, iterations=0, init=1)
        torch.cuda.synchronize()
        born_s = time.perf_counter() - t0
        e_born = err(born)
        xv = torch.empty_like(truth)
        tol = 0.5 * e_born
        dev_s, done, trace, t_tol = 0.0, 0, [], None
        while done < iterations:
            k = min(segment, iterations - done)
            rep = ctx.tv_reconstruct(xv, caps=caps, n=M, posspec=pos, iterations=k, init=1 if done == 0 else 0,
                                     **opts)
            dev_s += rep["seconds"]
            done += k
            e = err(xv)
            trace.append([done, round(e, 4)])
            if t_tol is None and e <= tol:
                t_tol = dev_s
    return {"workload": f"two touching cells dn 0.03 in {D}^3, {M} Ewald caps of {2 * N}^2 (forward-operator data)",
            "single_pass_rel_l2": round(e_born, 4), "single_pass_s": round(born_s, 5),
            "regularised_rel_l2": trace[-1][1], "iterations": iterations,
            "ms_per_iteration": round(1e3 * dev_s / iterations, 3),
            "tolerance": f"rel-L2 <= {tol:.4f} (half the single-pass error)",
            "time_to_tolerance_s": round(t_tol, 5) if t_tol is not None else None,
            "rel_l2_trace": trace, "options": opts}


def batched_form(count: int = 8, seed: int = 2, rounds: int = 3):
    """Batched form: `count` acquisitions of uneven size (holograms of 256^2 to
    2048^2, 50-800 angles, volumes 128^3-512^3 matched to the crop, random
    bead/ellipsoid phantoms with dn 0.005-0.05; the stacks are synthesised on
    the device and held in HBM), reconstructed one by one (one tdm_pipeline
    call each) and as one CUDA-graph launch (tdm_batch)."""
    import numpy as np
    import torch

    from mtd_transmission_gb300 import Batch, Context, Geometry
    from tests import simul
    rng = np.random.default_rng(seed)
    specs, stacks, ctxs = [], [], []
    for i in range(count):
        H = int(rng.choice([256, 512, 1024, 2048]))
        N = int(rng.choice([n for n in (32, 64, 128) if n <= H // 4]))
        M = int(rng.integers(50, 801))
        acq = simul.Acquisition(ccd_roix=H, nxmax=N, circle_cx=H // 4, circle_cy=H // 4, dim_final=4 * N,
                                nb_holo=M, born=int(rng.integers(0, 2)))
        objs = [simul.Ellipsoid(tuple(rng.uniform(-0.2, 0.2, 3)), tuple(rng.uniform(0.04, 0.15, 3)),
                                float(rng.uniform(0.005, 0.05)), smooth=bool(rng.integers(0, 2)))
                for _ in range(int(rng.integers(1, 5)))]
        ph = simul.Phantom(objs, phase_max=None if acq.born else 20.0)
        d = simul.holograms(acq, ph, seed=seed * 100 + i, device="cuda")
        ctx = Context(Geometry.from_acquisition(acq), M)
        ctxs.append(ctx)
        ctx.set_mask(np.ascontiguousarray(d["mask"].cpu().numpy()))
        D = acq.dim_final
        holos = d["holos"].contiguous()
        re = torch.empty((D, D, D), device="cuda")
        im = torch.empty_like(re)
        otf = torch.empty((D, D, D), dtype=torch.uint8, device="cuda")
        stacks.append((ctx, holos, re, im, otf))
        specs.append([H, M, D])
        del d
    holos_total = sum(m for _, m, _ in specs)

    def one_by_one():
        for ctx, holos, re, im, otf in stacks:
            ctx.pipeline(holos, indice=re, absorption=im, otf=otf)
        for ctx in ctxs:
            ctx.synchronize()

    one_by_one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(rounds):
        one_by_one()
    seq_s = (time.perf_counter() - t0) / rounds
    with Batch(stacks) as b:
        st = torch.cuda.current_stream()
        b.launch(st.cuda_stream)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(st)
        for _ in range(rounds):
            b.launch(st.cuda_stream)
        ev1.record(st)
        torch.cuda.synchronize()
        graph_s = ev0.elapsed_time(ev1) / 1e3 / rounds
    for ctx in ctxs:
        ctx.close()
    return {"stacks": [{"hologram_px": h, "holograms": m, "volume": d} for h, m, d in specs],
            "holograms": holos_total,
            "one_by_one": {"holograms_per_s": round(holos_total / seq_s, 1), "volumes_per_s": round(count / seq_s, 3),
                           "s": round(seq_s, 5)},
            "graph": {"holograms_per_s": round(holos_total / graph_s, 1), "volumes_per_s": round(count / graph_s, 3),
                      "s": round(graph_s, 5)},
            "note": "holograms resident in HBM; one CUDA graph with the stacks as independent branches"}


def cufft_reference(acq, kern):
    """cuFFT (through torch.fft) on the transforms of the hand-written passes,
    timed with CUDA events on the same device, as a reference point: the
    hologram row and column FFTs of one 16-hologram chunk (full 1024-point
    complex transforms of the packed rows and of the band's columns), the
    256^2 field transforms of 16 angles, and the 512^3 inverse 3D FFT."""
    import torch
    H, F, D = acq.ccd_roix, 2 * acq.nxmax, acq.dim_final

    def t(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    rows = torch.randn(16 * H // 2, H, dtype=torch.complex64, device="cuda")
    cols = torch.randn(16 * F, H, dtype=torch.complex64, device="cuda")
    fld = torch.randn(16, F, F, dtype=torch.complex64, device="cuda")
    vol = torch.randn(D, D, D, dtype=torch.complex64, device="cuda")
    out = {"hologram_rows_16": round(t(lambda: torch.fft.fft(rows, dim=-1)), 4),
           "hologram_cols_16": round(t(lambda: torch.fft.fft(cols, dim=-1)), 4),
           "fields_2d_16": round(t(lambda: torch.fft.ifft2(fld)), 4),
           "volume_3d": round(t(lambda: torch.fft.ifftn(vol), reps=5), 4)}
    del rows, cols, fld, vol
    n_chunks = (acq.nb_holo + 15) // 16

    def ours(*names):
        return round(sum(kern.get(n, (0.0, 0))[0] for n in names), 4)

    return {"unit": "ms", "cufft": out,
            "hand_written_per_launch": {
                "hologram_rows_16": round(ours("extract_rows") / n_chunks, 4),
                "hologram_cols_16": round(ours("extract_cols") / n_chunks, 4),
                "fields_2d_16": round(ours("field_rows", "field_cols") / n_chunks, 4),
                "volume_3d": ours("gather", "ypass", "xpass")},
            "note": "the hand-written passes include their fused work (Tukey window, row packing and band "
                    "separation, crop, recentring, atan2/phasor, shifts, scaling and the index/absorption split; "
                    "the volume's z pass runs inside the cap gather, so volume_3d includes the gather); "
                    "the cuFFT calls are bare transforms"}


def workload_config(acq, args):
    return {"workload": f"{args.workload}: {acq.nb_holo} x {acq.ccd_roix}^2 uint16 12-bit holograms, "
                        f"NXMAX {acq.nxmax} ({2 * acq.nxmax}^2 fields), {'Born' if acq.born else 'Rytov'}, "
                        f"{'Volkov' if acq.volkov else 'Herraez'} + aberration correction, {acq.dim_final}^3 volume",
            "holograms": acq.nb_holo, "hologram_px": acq.ccd_roix, "field_px": 2 * acq.nxmax,
            "volume": acq.dim_final, "parallelism": f"replicas x{args.gpus}",
            "schedule": {"chunk": schedule_for(acq.nb_holo)[0], "lanes": schedule_for(acq.nb_holo)[1]},
            "l2": f"inputs larger than L2: {acq.nb_holo * acq.ccd_roix ** 2 * 2 / 1e9:.2f} GB of holograms per step "
                  "(no flush needed)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rytov_1024")
    ap.add_argument("--e2e-steps", type=int, default=24)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=12)
    ap.add_argument("--ref-sample", type=int, default=8)
    ap.add_argument("--profile-out", default=None)
    ap.add_argument("--no-profile-pass", action="store_true", help="skip the per-kernel event pass")
    ap.add_argument("--holograms", type=int, default=None, help="override the workload's hologram count")
    ap.add_argument("--herraez", action="store_true", help="unwrap with Herraez's method (VOLKOV 0) instead of Volkov's")
    ap.add_argument("--no-forms", action="store_true", help="skip the regularised-reconstruction form")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    from dataclasses import replace

    from tests import simul
    acq, ph, seed = simul.workload(args.workload)
    if args.holograms:
        acq = replace(acq, nb_holo=args.holograms)
    if args.herraez:
        acq = replace(acq, volkov=0)
    world, rank, local = dist_setup()

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, acq, ph, seed)
        return

    import numpy as np
    import torch
    import torch.distributed as dist

    from mtd_transmission_gb300 import Context, Geometry
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    # synthetic stack on the device (seeded per rank)
    data = simul.holograms(acq, ph, seed=seed + rank, device="cuda")
    holos = data["holos"].contiguous()
    mask = np.ascontiguousarray(data["mask"].cpu().numpy())
    del data
    torch.cuda.empty_cache()
    M, D = acq.nb_holo, acq.dim_final
    ctx = Context(Geometry.from_acquisition(acq), M)
    ctx.set_mask(mask)
    sched = schedule_for(M)
    ctx.set_schedule(*sched)
    re = torch.empty((D, D, D), dtype=torch.float32, device="cuda")
    im = torch.empty_like(re)
    otf = torch.empty((D, D, D), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream)

    for _ in range(args.warmup):
        ctx.pipeline(holos, indice=re, absorption=im, otf=otf)
    ctx.synchronize()
    barrier()
    torch.cuda.synchronize()

    # timed region: K steps, device-resident inputs
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = ctx.launch_count
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    s_first = sampler.mark()
    ev0.record(stream)
    t_enq = time.perf_counter()
    for _ in range(args.steps):
        ctx.pipeline(holos, indice=re, absorption=im, otf=otf)
    t_enq = time.perf_counter() - t_enq  # host time to enqueue the K steps
    ctx.join()  # the last volume stages run on the context's second stream
    ev1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    s_last = sampler.mark()
    ms = ev0.elapsed_time(ev1)
    launches = ctx.launch_count - launches0
    clocks = sampler.stop(s_first, s_last)
    # per-kernel device times: the same K steps again with CUDA events around
    # every launch, one chunk in flight and each volume stage joined before the
    # next call (launches that share the GPU would have overlapping durations)
    prof, prof_ms = {}, 0.0
    if not args.no_profile_pass:
        ctx.set_schedule(sched[0], 1)
        ctx.profile(True)
        ev0.record(stream)
        for _ in range(args.steps):
            ctx.pipeline(holos, indice=re, absorption=im, otf=otf)
            ctx.join()
        ev1.record(stream)
        ctx.synchronize()
        prof_ms = ev0.elapsed_time(ev1)
        prof = ctx.profile_read()
        ctx.profile(False)
        ctx.set_schedule(*sched)
    ms_max = max_over_ranks([ms], world, "cuda")[0]
    value = whole_job_rate(world, args.steps, ms_max / 1e3)

    # end to end: pinned host holograms and outputs through the C ABI.  Sync:
    # tdm_pipeline per step (returns with the volume in host memory).
    # Pipelined: tdm_pipeline_async per step into alternating host output
    # sets and one tdm_synchronize, so that a step's downloads overlap the
    # next step's uploads and kernels; every step's upload and download is
    # inside the timed region either way.
    h_holos = torch.empty(holos.shape, dtype=holos.dtype, pin_memory=True)
    h_holos.copy_(holos)
    h_outs = [(torch.empty((D, D, D), dtype=torch.float32, pin_memory=True),
               torch.empty((D, D, D), dtype=torch.float32, pin_memory=True),
               torch.empty((D, D, D), dtype=torch.uint8, pin_memory=True)) for _ in range(2)]
    # Host-link throughput varies from run to run (trials of the same schedule
    # have differed by tens of percent), so the pipelined figure is taken over
    # E2E_TRIALS trials of e2e_steps volumes and the median trial is reported
    # (every trial is listed in the line).
    e2e_trials_s = []
    e2e_enqueue_s = []
    e2e_sync_s = 0.0
    if args.e2e_steps > 0:
        h_re, h_im, h_otf = h_outs[0]
        ctx.pipeline(h_holos, indice=h_re, absorption=h_im, otf=h_otf)  # warm-up of the host path
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            ctx.pipeline(h_holos, indice=h_re, absorption=h_im, otf=h_otf)
        e2e_sync_s = time.perf_counter() - t0
        for k in range(2):  # warm-up of the pipelined path (both output sets), untimed
            h_re, h_im, h_otf = h_outs[k % 2]
            ctx.pipeline_async(h_holos, indice=h_re, absorption=h_im, otf=h_otf)
        ctx.synchronize()
        for _ in range(E2E_TRIALS):
            barrier()
            t0 = time.perf_counter()
            for k in range(args.e2e_steps):
                h_re, h_im, h_otf = h_outs[k % 2]
                ctx.pipeline_async(h_holos, indice=h_re, absorption=h_im, otf=h_otf)
            e2e_enqueue_s.append(time.perf_counter() - t0)
            ctx.synchronize()
            e2e_trials_s.append(time.perf_counter() - t0)
    t_e = max_over_ranks(e2e_trials_s + [e2e_sync_s], world, "cuda")
    e2e_trials = [whole_job_rate(world, args.e2e_steps, s) for s in t_e[:-1]]
    e2e_value = statistics.median(e2e_trials) if e2e_trials else None
    e2e_sync = whole_job_rate(world, args.e2e_steps, t_e[-1]) if args.e2e_steps > 0 else None
    h2d = int(h_holos.numel() * h_holos.element_size())
    d2h = int(2 * D ** 3 * 4 + D ** 3)
    # the host link on this machine with these buffers: one step's upload and
    # download at once bound the end-to-end rate
    link = None
    if args.e2e_steps > 0:
        link = host_link_probe(h_holos, holos, [(re, h_outs[0][0]), (im, h_outs[0][1]), (otf, h_outs[0][2])])
        link["bound_per_s"] = round(1e3 / link["both_ms"], 3)

    if rank == 0:
        # roofline of the dominant kernel
        hits = float((np.arange(-acq.nxmax, acq.nxmax)[:, None] ** 2 +
                      np.arange(-acq.nxmax, acq.nxmax)[None, :] ** 2 < acq.nxmax ** 2).sum())
        per_angle, per_volume = algorithmic_bytes(None, acq, hits, ctx.cap_planes[1])
        peak, peak_kind = measured_peaks()
        kern = {k: (t / args.steps, n / args.steps) for k, (t, n) in prof.items()}
        dom = max(kern, key=lambda k: kern[k][0]) if kern else None
        roof = None
        if dom:
            t_step_ms, n_launch = kern[dom]
            stage = KERNEL_STAGE.get(dom)
            bytes_step = stage_bytes(acq, hits)[stage] if stage else 0
            achieved = bytes_step / (t_step_ms / 1e3) / 1e9
            traffic, traffic_src = ncu_traffic_per_launch(dom, acq)
            roof = {"kernel": dom, "stage": stage, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                    "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "traffic": round(traffic / 1e6, 3) if traffic else None,
                    "traffic_unit": "MB per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                    "traffic_source": traffic_src,
                    "algorithmic_bytes": "the stage's per-unit bytes (extraction: H^2 2 + F^2 8 per hologram; "
                                         "fields: 2 F^2 8 per angle; cap mapping: F^2 8 + 24 hits per angle; "
                                         "volume: 32 D^3) times the units of the kernel's launches",
                    "algorithmic_bytes_per_launch_mb": round(bytes_step / max(n_launch, 1) / 1e6, 3),
                    "peak_source": f"{peak_kind} hbm_gbs (of measured)" if peak_kind == "measured"
                    else f"{peak_kind} (of fallback)",
                    "launches_per_step": n_launch, "ms_per_step": round(t_step_ms, 4),
                    "algorithmic_bytes_per_step": int(bytes_step)}
        # every kernel with algorithmic bytes: achieved GB/s and fraction of the HBM peak
        roof_all = {}
        for k, (t_ms, _) in kern.items():
            b = per_angle[k] * M if k in per_angle else per_volume.get(k)
            if b and t_ms > 0:
                gbs = b / (t_ms / 1e3) / 1e9
                roof_all[k] = {"achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            r = cpu_baseline(acq, ph, seed, args.cpu_sample, threads)
            cpu = {"value": 1.0 / r["seconds_per_volume"], "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"{args.cpu_sample} of {acq.nb_holo} holograms through extraction, fields and cap "
                             f"mapping ({r['per_angle_s']:.3f} s/angle), extrapolated, plus one full "
                             f"{acq.dim_final}^3 volume stage ({r['volume_s']:.1f} s)"}
            # the reference's default thread count (recon.txt NB_THREADS 4)
            r4 = cpu_baseline(acq, ph, seed, max(2, args.cpu_sample // 3), 4)
            cpu["nb_threads_4"] = {"value": 1.0 / r4["seconds_per_volume"], "cores": 4,
                                   "sample": f"{max(2, args.cpu_sample // 3)} holograms, extrapolated, plus one "
                                             f"volume stage ({r4['volume_s']:.1f} s)"}
            # the oracle's FFT against scipy.fft on the same sizes: the baseline
            # with the faster of the two (a conservative speed-up)
            fft, saved = fft_check(acq, threads)
            cpu["fft_check"] = fft
            cpu["value_with_faster_fft"] = 1.0 / max(r["seconds_per_volume"] - saved, 1e-9)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT,
            "holograms_per_s": round(value * acq.nb_holo, 1), "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(acq, args),
            "e2e": {"value": round(e2e_value, 3) if e2e_value else None, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "mode": "pipelined: tdm_pipeline_async per step (pinned host holograms in, pinned host "
                            "volumes out, alternating output sets), one tdm_synchronize at the end; median of "
                            f"{E2E_TRIALS} trials of {args.e2e_steps} volumes",
                    "trials": [round(v, 3) for v in e2e_trials],
                    # host time spent inside the pipeline_async calls of each trial, per volume
                    # (including time blocked on full launch queues while the GPU catches up)
                    "enqueue_ms_per_step": [round(1e3 * s / args.e2e_steps, 3) for s in e2e_enqueue_s],
                    "sync_value": round(e2e_sync, 3) if e2e_sync else None,
                    # copy throughput of the host link measured after the trials with the same pinned
                    # buffers (one step's upload and download), and the rate it bounds
                    "link": link,
                    "sync_mode": "tdm_pipeline per step, each call returns with the volume in host memory"},
            "gpu_launches": int(launches),
            # host time spent inside the K pipeline calls, per step: the calls queue work and return,
            # but block while launch queues are full, so this is an upper bound on the host cost
            "enqueue_ms_per_step": round(1e3 * t_enq / args.steps, 3),
            "roofline": roof,
            "roofline_all": roof_all,
            "roofline_stages": stage_roofline(acq, hits, {k: v[0] for k, v in kern.items()}, ms_max / args.steps,
                                              peak),
            "cpu_baseline": cpu,
            "clocks": clocks,
            "kernels_ms_per_step": {k: round(v[0], 4) for k, v in sorted(kern.items(), key=lambda x: -x[1][0])},
            "profiled_ms_per_step": round(prof_ms / args.steps, 3),
            "profile_schedule": {"chunk": sched[0], "lanes": 1},
        }
        if not args.no_forms:
            ctx.close()
            line["forms"] = {"tv_adjoint": tv_form(), "batched": batched_form()}
            line["cufft_reference"] = cufft_reference(acq, kern)
        if args.profile_out:
            with open(args.profile_out, "w") as f:
                json.dump(line, f, indent=1)
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
