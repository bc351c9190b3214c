"""Benchmark of the streaming FBP chain on the full-rate streaming workload.

Workload (one step): 2 detector planes x 2000 frames = 4000 slices of
1000 fan projections x 1152 detectors (uint16, Poisson counts, 1% seeded
defective detector columns) -> defect repair -> attenuation -> rebinning to
1024 angles x 1024 rays -> Shepp-Logan filter (zero padded to 2048) ->
backprojection to 512 x 512 FP32 images with the circular mask.

  value  slices/s of the whole job with the raw frames resident in HBM, the job
         replayed as one captured CUDA graph (batched path)
  e2e    slices/s through the host-buffer entry point risa_gb_fbp_run_host:
         pinned host frames in, pinned host images out, copies overlapped with
         compute, all inside the timed region
  plain  slices/s of the per-stage path (one frame per launch, a stream sync
         after every stage, as the reference's stage threads do)

`python bench.py --impl reference` times the FP64 CPU oracle FBP on the host
cores instead (the reference has no CPU implementation of the chain).
"""
from __future__ import annotations

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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = dict(n_planes=2, n_fan_det=1152, n_fan_proj=1000, n_par_proj=1024, n_par_det=1024, n_pixels=512,
                source_offset=0.0, detector_diameter=480.0, image_width=200.0, source_diameter=[430.0, 430.0],
                delta_x=[0.0, 0.0], delta_z=[1417.0, 1430.0], source_angle=[360.0, 360.0])
FRAMES_PER_PLANE = 2000
FLOPS_PER_UPDATE = 6  # ray coordinate FMA (2) + weight add (1) + interpolation FMA (2) + accumulate (1)
SMEM_BYTES_PER_UPDATE = 8  # one FP32 (midpoint, difference) pair per pixel x angle and slice
SMEM_BYTES_PER_CLK_SM = 128  # nominal shared-memory bandwidth per SM
# dram__bytes_read.sum + dram__bytes_write.sum of a 64-slice launch of the autotuned
# backprojection variant (staged_cp_s4_a8_p4, profiles/bp_staged_fbp512_ncu.txt):
# the pair records read once and the images written, both proportional to the
# slices, so a launch of B slices moves B/64 of it
BP_DRAM_BYTES_PER_SLICE = 722.1e6 / 64
WORKLOAD_NAME = ("full-rate streaming: 2 planes x 2000 frames of 1000x1152 uint16 fan sinograms, 1% defective "
                 "detectors -> 1024x1024 parallel (pad 2048, Shepp-Logan) -> 512^2 FP32, circular mask")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--frames", type=int, default=FRAMES_PER_PLANE, help="frames per plane")
    ap.add_argument("--batch", type=int, default=512, help="frames per engine chunk (multiple of 2)")
    ap.add_argument("--distinct", type=int, default=8, help="distinct synthetic frames per plane")
    ap.add_argument("--no-extras", action="store_true", help="skip plain/e2e/roofline/cpu legs")
    ap.add_argument("--scaling", choices=["weak", "strong"], default="weak",
                    help="under torchrun: weak = every rank reconstructs the whole job; strong = the job's "
                         "frames are split over the ranks (replicas.shard_indices) and the images gathered")
    ap.add_argument("--bp-variant", type=int, default=-1,
                    help="backprojection variant to use instead of autotuning (for profiling one kernel)")
    ap.add_argument("--only", choices=["precision", "differentiation", "sweep"], default=None,
                    help="run one of the other scope-table workloads alone and print its JSON (no headline)")
    return ap.parse_args()


def make_oracle_geom():
    class G:
        pass

    g = G()
    g.__dict__.update(WORKLOAD, image_center_x=0.0, image_center_y=0.0, rotation_offset=0.0)
    return g


def synthetic_scan(frames_per_plane: int, distinct: int):
    from risa_gb300 import phantom

    w = WORKLOAD
    return phantom.make_scan(frames_per_plane, w["n_planes"], w["n_fan_proj"], w["n_fan_det"],
                             w["source_diameter"][0] / 2.0, w["detector_diameter"] / 2.0, seed=2026,
                             defect_fraction=0.01, distinct=distinct)


def oracle_fbp_sample(sc, n_slices: int, threads: int):
    """FP64 CPU oracle on the first n_slices frames; returns (images, seconds)."""
    import oracle

    og = make_oracle_geom()
    op = oracle.make_params(quirk=oracle.QUIRK_NONE, filter_type="sheppLogan", defects=True, masking=True)
    ref, dark = oracle.attenuation_init(sc.ref, sc.dark, WORKLOAD["n_planes"], 0.67, 1.5, True, oracle.QUIRK_NONE)
    rec = oracle.f2p_records(og, oracle.QUIRK_NONE)
    t0 = time.perf_counter()
    out = oracle.fbp(og, op, rec, ref, dark, sc.raw[:n_slices], sc.planes[:n_slices], n_threads=threads)
    return out, time.perf_counter() - t0, (ref, dark, rec, op, og)


# --------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        power = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(power) if power else None}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------------------- reference arm
def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sc = synthetic_scan(max(1, cores // 2 + 1), 2)
    n = min(sc.raw.shape[0], max(2, cores))
    times = []
    for i in range(args.warmup + args.steps):
        _, dt, _ = oracle_fbp_sample(sc, n, cores)
        if i >= args.warmup:
            times.append(dt)
    sec = sum(times) / len(times)
    value = n / sec
    line = {
        "impl": "reference", "metric": "FBP slices/s @512^2", "value": value, "unit": "slices/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD_NAME, "sample_slices_per_step": n},
        "cpu_baseline": {"value": value, "unit": "slices/s", "cores": cores, "kind": "port",
                         "sample": f"{n} slices of the workload per step (FP64 C oracle, {cores} threads)"},
        "e2e": {"value": value, "unit": "slices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- our arm
def run_ours(args, rank: int, world: int, local_rank: int):
    import torch
    import torch.distributed as dist

    import risa_gb300 as rg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    L = WORKLOAD["n_planes"]
    g = rg.make_geometry(**WORKLOAD)
    p = rg.make_params(filter_type="sheppLogan", defects=True, masking=True)
    sc = synthetic_scan(args.frames, args.distinct)
    n_job = sc.raw.shape[0]
    strong = args.scaling == "strong" and world > 1
    if strong:  # this rank's plane groups of the job, dealt round robin
        import dataclasses

        from risa_gb300 import replicas

        mine = replicas.shard_indices(n_job, rank, world, L)
        sc = dataclasses.replace(sc, raw=np.ascontiguousarray(sc.raw[mine]), planes=sc.planes[mine])
    n = sc.raw.shape[0]
    # frames all ranks reconstruct per step
    job_frames = n_job if strong else world * n
    # a chunk never holds more frames than the job (every enqueue below reads B frames)
    B = min(args.batch, n)
    B -= B % L
    if B < L:
        raise SystemExit("bench.py: --batch and --frames leave no whole plane group per chunk")
    Pf, Df, N = WORKLOAD["n_fan_proj"], WORKLOAD["n_fan_det"], WORKLOAD["n_pixels"]
    Pp, Dp = WORKLOAD["n_par_proj"], WORKLOAD["n_par_det"]
    fbp = rg.FBP(g, p, sc.ref, 1, sc.dark, 1, max_batch=B)
    raw = torch.from_numpy(sc.raw.view(np.int16)).to(dev)
    img = torch.empty((n, N, N), dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    # autotune the backprojection tile shape on this geometry, then capture the job
    fan_buf, par_buf = fbp.intermediates()
    with torch.cuda.stream(stream):
        fbp.enqueue(raw[:B], img[:B], rg.PLANES_INTERLEAVED, B, stream)
    stream.synchronize()
    bp = fbp.backprojection()
    if args.bp_variant >= 0:
        bp.set_variant(args.bp_variant)
        variant = args.bp_variant
    else:
        variant = bp.autotune(par_buf, img.data_ptr(), B, stream)
    graph = fbp.graph_capture(raw, img, rg.PLANES_INTERLEAVED, n, stream)
    launches_per_step = graph.kernel_count

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        graph.replay(stream)
    stream.synchronize()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local_rank) as clk:
        torch.cuda.synchronize()
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            graph.replay(stream)
        e1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = job_frames / (ms / 1e3)
    clocks = clk.summary()

    gathered = None
    if strong:
        # every rank's images, reduced to one checksum per frame, collected on
        # rank 0 in frame order; frames cycle through `distinct` source frames
        # per plane, so equal sources must give equal checksums
        from risa_gb300 import replicas

        sums = img.double().sum(dim=(1, 2)).cpu().numpy()[:, None]
        allsums = replicas.gather_images(sums, n_job, L)
        if rank == 0:
            period = args.distinct * L
            gathered = {"frames": int(allsums.shape[0]),
                        "frame_order_check": bool(np.array_equal(allsums[:, 0],
                                                                 allsums[np.arange(n_job) % period, 0]))}
    extras = {}
    if not args.no_extras:
        # end to end through the host-buffer entry point, on every rank
        t_e2e, e2e_runs = measure_e2e(args, sc, fbp, torch, rg)
        if world > 1:
            t = torch.tensor([t_e2e], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            t_e2e = float(t.item())
        extras["e2e"] = {"value": job_frames / t_e2e, "unit": "slices/s",
                         "h2d_bytes_per_step": int(job_frames * Pf * Df * 2),
                         "d2h_bytes_per_step": int(job_frames * N * N * 4), "entry_point": "risa_gb_fbp_run_host",
                         "statistic": "median of %d steps (max over ranks)" % len(e2e_runs),
                         "rank0_step_ms": [round(x * 1e3, 2) for x in e2e_runs]}
    if rank == 0 and not args.no_extras:
        extras.update(measure_extras(args, sc, fbp, raw, img, stream, B, variant, torch, rg, g, p))
    if rank != 0:
        return
    peaks = measured_peaks()
    line = {
        "metric": "FBP slices/s @512^2", "value": value, "unit": "slices/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "strong" if strong else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantoms, Poisson uint16 counts; "
                f"{args.distinct} distinct frames per plane cycled)",
        "config": {"workload": WORKLOAD_NAME, "frames_per_plane": args.frames, "slices_per_step": job_frames,
                   "slices_per_rank": n,
                   "batch": B, "bp_variant": variant,
                   "graph": "one CUDA graph per step, the stages of each chunk in sequence (one lane)",
                   "l2": "inputs larger than L2 (%.1f GB raw per step)" % (sc.raw.nbytes / 1e9),
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    if gathered is not None:
        line["gathered"] = gathered
    line.update(extras)
    if "plain" in line:
        line["speedup_vs_plain"] = value / world / line["plain"]["value"]
    if line.get("plain_reference", {}).get("value"):
        line["speedup_vs_plain_reference"] = value / world / line["plain_reference"]["value"]
        line["e2e_speedup_vs_plain_reference"] = line["e2e"]["value"] / world / line["plain_reference"]["value"]
    if "roofline" in line and peaks:
        line["roofline"]["peaks_file"] = {k: peaks.get(k) for k in ("hbm_gbs", "sm_max_mhz")}
    print(json.dumps(line), flush=True)


def timed(torch, stream, fn, reps: int) -> float:
    """Average ms of fn() on `stream` over reps, after one warm-up call."""
    fn()
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def measure_e2e(args, sc, fbp, torch, rg):
    """Seconds per step through risa_gb_fbp_run_host: pinned host frames in,
    pinned host images out, the copies inside the timed region. Each step is
    timed on its own (host clock around the call, which returns once the
    images are in host memory); the median of the steps is the figure, since
    the host link is shared with the machine's other tenants and one step
    slowed by their traffic would otherwise set it. Returns (median, all)."""
    n, N = sc.raw.shape[0], WORKLOAD["n_pixels"]
    hraw = torch.from_numpy(sc.raw.view(np.int16)).pin_memory()
    himg = torch.empty((n, N, N), dtype=torch.float32).pin_memory()
    fbp.run_host(hraw, himg, n, rg.PLANES_INTERLEAVED)  # warm-up (captures the slot graphs)
    e2e_steps = max(1, min(args.steps, 5))
    ts = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        fbp.run_host(hraw, himg, n, rg.PLANES_INTERLEAVED)
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), ts


def measure_extras(args, sc, fbp, raw, img, stream, B, variant, torch, rg, g, p):
    out = {}
    dev = raw.device
    n = sc.raw.shape[0]
    L = WORKLOAD["n_planes"]
    Pf, Df, N = WORKLOAD["n_fan_proj"], WORKLOAD["n_fan_det"], WORKLOAD["n_pixels"]
    Pp, Dp = WORKLOAD["n_par_proj"], WORKLOAD["n_par_det"]
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 2.0 * 128 * sms * sm_mhz * 1e6 / 1e12  # TFLOP/s
    hbm = float(peaks.get("hbm_gbs", 6800.0))

    # ---- per-stage timings on one chunk (isolated kernels, CUDA events on the launch stream)
    fan_buf, par_buf = fbp.intermediates()
    att = rg.Attenuation(g, p, sc.ref, 1, sc.dark, 1)
    f2p = rg.Fan2Para(g, p)
    filt = rg.Filter(g, p)
    bp = fbp.backprojection()
    reps = 5
    # the engine's own kernels on one chunk, CUDA events between them on the launch stream
    es = fbp.time_stages(raw[:B], img[:B], rg.PLANES_INTERLEAVED, B, reps, stream)
    t_def, t_att, t_f2p, t_filt = es["defect_detect"], es["attenuation_repair"], es["rebinning"], es["filter"]
    t_stage, t_kern = es["bp_staging"], es["bp_kernel"]
    t_bp = t_stage + t_kern
    fs, ps = Pf * Df, Pp * Dp
    att_bytes = B * fs * (2 + 4) + L * fs * 4
    f2p_bytes = B * (fs * 4 + ps * 4) + L * ps * 4 * 12
    # the filter reads the rebinned sinogram; fused with the staging pass it
    # writes the padded pair records (8 B per window bin, angle and slice)
    win_lo, win_len = bp.window(True)
    # with a staged variant the filter writes the pair records itself and no
    # staging pass runs (its event interval is then only the events' own
    # overhead, a few microseconds against ~1 ms for a real staging pass)
    prefilled = t_stage < 0.05 * t_filt
    filt_bytes = B * ps * 4 + (B * Pp * win_len * 8 if prefilled else B * ps * 4)
    yy, xx = np.mgrid[:N, :N]
    inside = int(((xx - (N - 1) / 2) ** 2 + (yy - (N - 1) / 2) ** 2 <= N * N / 4).sum())
    updates = B * inside * Pp
    # The backprojection kernel is bound by shared-memory bandwidth: every
    # update reads one FP32 (midpoint, difference) pair of its slice (8 B).
    # Denominators measured on this GPU (risa_gb_measure_peak), nominal beside.
    smem_meas = rg.measure_peak(rg.PEAK_SMEM_READ, 5, stream)
    fma_meas = rg.measure_peak(rg.PEAK_FP32_FMA, 5, stream)
    smem_nominal = SMEM_BYTES_PER_CLK_SM * sms * sm_mhz * 1e6 / 1e9  # GB/s
    smem_peak = smem_meas["value"]
    fp32_peak_meas = fma_meas["value"]
    smem_gbs = updates * SMEM_BYTES_PER_UPDATE / (t_kern / 1e3) / 1e9
    bp_tflops = updates * FLOPS_PER_UPDATE / (t_kern / 1e3) / 1e12
    out["roofline"] = {
        "kernel": f"bp_linear_async ({rg.Backprojection.variant_name(variant)})", "bound": "smem",
        "achieved": smem_gbs, "peak": smem_peak, "unit": "GB/s", "frac": smem_gbs / smem_peak,
        "traffic": BP_DRAM_BYTES_PER_SLICE * B,
        "traffic_source": "ncu capture of a 64-slice launch, scaled by slices per launch",
        "work": f"{SMEM_BYTES_PER_UPDATE} B of shared-memory reads per pixel x angle update and slice, "
                f"{inside} in-circle pixels x {Pp} angles x {B} slices per launch",
        "peak_source": "measured: risa_gb_measure_peak(RISA_GB_PEAK_SMEM_READ), conflict-free 128-bit "
                       f"shared loads on all {sms} SMs, {smem_meas['per_sm_per_clk']:.1f} B/clk/SM at "
                       f"{smem_meas['sm_mhz']:.0f} MHz",
        "peak_nominal": smem_nominal, "frac_nominal": smem_gbs / smem_nominal,
        "peak_nominal_source": f"{SMEM_BYTES_PER_CLK_SM} B/clk/SM x {sms} SMs x {sm_mhz:.0f} MHz",
        "kernel_ms": t_kern, "staging_ms": t_stage,
        "fp32": {"achieved": bp_tflops, "peak": fp32_peak_meas, "unit": "TFLOP/s",
                 "frac": bp_tflops / fp32_peak_meas, "work": f"{FLOPS_PER_UPDATE} FLOP per update",
                 "peak_source": "measured: risa_gb_measure_peak(RISA_GB_PEAK_FP32_FMA), "
                                f"{fma_meas['per_sm_per_clk']:.1f} FLOP/clk/SM at {fma_meas['sm_mhz']:.0f} MHz",
                 "peak_nominal": fp32_peak, "frac_nominal": bp_tflops / fp32_peak,
                 "peak_nominal_source": f"128 FMA lanes x 2 FLOP x {sms} SMs x {sm_mhz:.0f} MHz"},
    }
    out["bp"] = {"gupdates_per_s": updates / (t_bp / 1e3) / 1e9,
                 "gupdates_per_s_kernel": updates / (t_kern / 1e3) / 1e9,
                 "gupdates_per_s_full_square": B * N * N * Pp / (t_bp / 1e3) / 1e9,
                 "ms_per_launch": t_bp, "slices_per_launch": B, "variant": rg.Backprojection.variant_name(variant)}
    out["stages"] = {
        "attenuation_defects": {"ms": t_att, "gbs": att_bytes / (t_att / 1e3) / 1e9,
                                "frac_hbm": att_bytes / (t_att / 1e3) / 1e9 / hbm},
        "fan2para": {"ms": t_f2p, "gbs": f2p_bytes / (t_f2p / 1e3) / 1e9,
                     "frac_hbm": f2p_bytes / (t_f2p / 1e3) / 1e9 / hbm},
        "filter": {"ms": t_filt, "gbs": filt_bytes / (t_filt / 1e3) / 1e9,
                   "frac_hbm": filt_bytes / (t_filt / 1e3) / 1e9 / hbm,
                   "writes": "pair records, %d bins per angle and slice" % win_len if prefilled
                             else "filtered sinogram"},
        "backprojection": {"ms": t_bp},
        "defect_detect": {"ms": t_def, "gbs": B * fs * 2 / (t_def / 1e3) / 1e9},
        "hbm_peak_gbs": hbm, "batch": B,
    }

    # ---- the same job as two lanes: each chunk's backprojection beside the
    # next chunk's streaming stages (the headline runs them in sequence)
    fbp.set_lanes(2)
    g2 = fbp.graph_capture(raw, img, rg.PLANES_INTERLEAVED, n, stream)
    ms2 = timed(torch, stream, lambda: g2.replay(stream), 2)
    fbp.set_lanes(1)
    out["two_lanes"] = {"value": n / (ms2 / 1e3), "unit": "slices/s", "ms_per_step": ms2,
                        "graph_kernels": g2.kernel_count,
                        "how": "the headline's job captured with risa_gb_fbp_set_lanes(2), CUDA events"}
    del g2
    # the sum of the stages' isolated times over the job's chunks, against the
    # graph's step time: what a single persistent launch could save at most
    # without running stages concurrently
    chunks = n / B
    out["graph_overhead"] = {"sum_of_stage_ms_per_step": sum(es.values()) * chunks,
                             "chunks_per_step": chunks}

    # ---- plain per-stage path: one frame per launch, sync after every stage;
    # the backprojection variant autotuned for one slice per launch
    dfx = rg.Defects(g, p, max_batch=1)
    ws = torch.empty(dfx.workspace_bytes(1), dtype=torch.uint8, device=dev)
    raw1 = torch.empty((1, Pf, Df), dtype=torch.int16, device=dev)
    n_plain = min(64, n)
    bp1 = rg.Backprojection(g, p)
    bp1.reserve(1)
    bp1_variant = bp1.autotune(par_buf, img.data_ptr(), 1, stream)

    def plain():
        for f in range(n_plain):
            k = f % L
            raw1.copy_(raw[f:f + 1])
            dfx.enqueue(raw1, 1, ws, stream=stream)
            stream.synchronize()
            att.enqueue(raw1, fan_buf, k, 1, stream)
            stream.synchronize()
            f2p.enqueue(fan_buf, par_buf, k, 1, stream)
            stream.synchronize()
            filt.enqueue(par_buf, 1, stream)
            stream.synchronize()
            bp1.enqueue(par_buf, img[f:f + 1], 1, stream)
            stream.synchronize()

    with torch.cuda.stream(stream):
        plain()
        t0 = time.perf_counter()
        plain()
        t_plain = time.perf_counter() - t0
    plain_value = n_plain / t_plain
    out["plain"] = {"value": plain_value, "unit": "slices/s", "frames": n_plain,
                    "how": "this library's stage kernels, one frame per stage launch, stream sync after each "
                           "stage, device-resident input",
                    "bp_variant": rg.Backprojection.variant_name(bp1_variant)}
    try:
        out["plain_reference"] = measure_plain_reference(torch, rg, sc, raw, g, stream, min(32, n))
    except Exception as e:  # reported, never hides the headline line
        out["plain_reference"] = {"error": f"{type(e).__name__}: {e}"}
    out["bp"]["reference_kernel"] = out["plain_reference"].get("bp_gupdates_per_s")

    # ---- accuracy of the batched output against the FP64 oracle, and the CPU baseline
    cores = os.cpu_count() or 1
    n_cpu = min(n, max(4, cores))
    ref_imgs, sec, _ = oracle_fbp_sample(sc, n_cpu, cores)
    fbp.enqueue(raw[:B], img[:B], rg.PLANES_INTERLEAVED, B, stream)
    stream.synchronize()
    got = img[:n_cpu].cpu().numpy().astype(np.float64)
    d = got - ref_imgs
    out["accuracy"] = {
        "slices": n_cpu,
        "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref_imgs)),
        "max_rel": float(np.abs(d).max() / np.abs(ref_imgs).max()),
        "vs": "FP64 CPU oracle on the same inputs",
    }
    out["cpu_baseline"] = {"value": n_cpu / sec, "unit": "slices/s", "cores": cores, "kind": "port",
                           "sample": f"{n_cpu} slices of the workload, FP64 C oracle, {cores} threads"}

    # ---- the other workloads of the scope table, reported beside the headline
    for key, fn in (("precision", measure_precision), ("differentiation", measure_differentiation),
                    ("sweep", measure_sweep)):
        try:
            out[key] = fn(torch, rg, dev)
        except Exception as e:  # reported, never hides the headline line
            out[key] = {"error": f"{type(e).__name__}: {e}"}
    return out


def measure_plain_reference(torch, rg, sc, raw, g, stream, n_frames: int) -> dict:
    """The reference's own CUDA stages on the same workload: its stage sources
    compiled for sm_103a (oracle/ref_harness) and launched as its processor()
    loops launch them, one frame per stage launch with 16 x 16 blocks and a
    stream sync after each stage, device-resident raw frames:
      computeAttenuation (Attenuation.cu:158-161),
      setValue + interpolation (Fan2Para.cu:220-238; RISA-mode tables in the
        reference's layout, built by the oracle's pinned restatement of
        computeFan2ParaTransp),
      cuFFT R2C + applyFilter + C2R (Filter.cu:119-137; the reference filters
        rows of length Dp = 1024 without zero padding, this library pads to 2048),
      backProjectLinear (Backprojection.cu:187-189), mask (Masking.cu:134-135).
    Defect repair is left out: the reference runs it on the host
    (DetectorInterpolation.cu:113-139) and its pipeline does not wire it."""
    from oracle import ref_kernels as rk
    import oracle

    why = rk.unavailable()
    if why:
        return {"unavailable": why}
    w = dict(WORKLOAD, image_center_x=0.0, image_center_y=0.0)
    L, Pf, Df, N = w["n_planes"], w["n_fan_proj"], w["n_fan_det"], w["n_pixels"]
    Pp, Dp = w["n_par_proj"], w["n_par_det"]
    dev = raw.device
    torch.zeros(1, device=dev)  # the primary context is current for the driver API
    rk.lib()
    z = oracle.f2p_tables_risa(make_oracle_geom())
    f2p_in = rk.fan2para_inputs(w, z, 16)
    p_risa = rg.make_params(quirks=rg.QUIRKS_RISA, filter_type="sheppLogan", masking=True)
    ref_avg, dark_avg = rg.Attenuation(g, p_risa, sc.ref, 1, sc.dark, 1).tables()
    t_ref = torch.from_numpy(ref_avg).to(dev)
    t_dark = torch.from_numpy(dark_avg).to(dev)
    t_mask = torch.ones((Pf, Df), dtype=torch.float32, device=dev)
    n_h, h = rg.Filter(g, p_risa).response()
    assert n_h == Dp
    t_h = torch.from_numpy(np.ascontiguousarray(np.asarray(h, np.float32))).to(dev)
    sin_t, cos_t, norm, scale, center = rk.bp_setup(Pp, Dp, N, 0.0)
    rk.bp_constants(sin_t, cos_t, Pp, norm, scale, center)
    fan = torch.empty((Pf, Df), dtype=torch.float32, device=dev)
    par = torch.empty((2 * Pp, Dp), dtype=torch.float32, device=dev)
    freq = torch.empty((Pp, Dp // 2 + 1, 2), dtype=torch.float32, device=dev)
    img = torch.empty((N, N), dtype=torch.float32, device=dev)
    names = ("attenuation", "fan2para", "filter_cufft", "backprojection", "mask")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
    acc = dict.fromkeys(names, 0.0)

    def frame(f, timed):
        k = f % L
        steps = (lambda: rk.attenuation(raw[f], t_mask, fan, t_ref, t_dark, Df, Pf, k, 16),
                 lambda: (par.zero_(), rk.fan2para_run(k, fan, par, f2p_in)),
                 lambda: rk.filter_rows(par, freq, t_h, Dp, Pp, 16),
                 lambda: rk.backproject(False, par, img, N, Pp, Dp, 16),
                 lambda: rk.mask(img, 0.0, N))
        ev[0].record(stream)
        for i, step in enumerate(steps):
            step()
            ev[i + 1].record(stream)
            stream.synchronize()
        if timed:
            for i, nm in enumerate(names):
                acc[nm] += ev[i].elapsed_time(ev[i + 1])

    with torch.cuda.stream(stream):
        for f in range(2):
            frame(f, False)
        t0 = time.perf_counter()
        for f in range(n_frames):
            frame(f, True)
        wall = time.perf_counter() - t0
    ms = {k: v / n_frames for k, v in acc.items()}
    return {"value": n_frames / wall, "unit": "slices/s", "frames": n_frames,
            "kernel_ms_per_slice": ms, "bp_gupdates_per_s": N * N * Pp / (ms["backprojection"] / 1e3) / 1e9,
            "filter_length": Dp,
            "how": "the reference's own stage kernels (cubins built from its sources for sm_103a), one frame per "
                   "stage launch, 16x16 blocks, stream sync after each stage; RISA quirks; unpadded filter of "
                   f"length {Dp} (this library: {2 * Dp}); no defect repair (host-side in the reference)"}


def cuda_ms(torch, fn, reps=5):
    """Mean ms of fn() over reps launches after one warm-up, CUDA events on the current stream."""
    fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def err_pair(got, exp):
    d = np.asarray(got, np.float64) - exp
    return {"max_abs": float(np.abs(d).max()), "max_rel": float(np.abs(d).max() / np.abs(exp).max()),
            "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(exp))}


def measure_precision(torch, rg, dev):
    """Precision ablation: 64 slices of 1024 x 1024 parallel sinograms, pad 2048,
    Ram-Lak, filtered by the split-bf16 x 3 Toeplitz contraction on the tensor
    cores and by the FP32 FFT, then backprojected to 1024^2; errors against the
    FP64 oracle (filter outputs of 4 slices, images of 2 slices)."""
    from risa_gb300 import phantom
    import oracle

    S, Pp, Dp, N, pad = 64, 1024, 1024, 1024, 2048
    base, _ = phantom.parallel_sinograms(8, Pp, Dp, 200.0, seed=31)
    x = np.ascontiguousarray(np.concatenate([base] * (S // 8)))  # 8 distinct phantoms cycled
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    p = rg.make_params(filter_type="ramp", pad=pad)
    tz, tz16, ff = rg.Toeplitz(g, p), rg.Toeplitz(g, p), rg.Filter(g, p)
    tz16.set_precision(rg.SPLIT_F16X3)
    xs = torch.from_numpy(x).to(dev)
    t_fft, t_tz, t_tz16 = xs.clone(), xs.clone(), xs.clone()
    ws = torch.empty(tz.workspace_bytes(S), dtype=torch.uint8, device=dev)
    scratch = torch.empty_like(xs)
    ms_copy = cuda_ms(torch, lambda: scratch.copy_(xs))  # the refill each timed filter call includes
    ms_fft = cuda_ms(torch, lambda: (t_fft.copy_(xs), ff.enqueue(t_fft, S)))
    ms_tz = cuda_ms(torch, lambda: (t_tz.copy_(xs), tz.enqueue(t_tz, S, ws)))
    ms_tz16 = cuda_ms(torch, lambda: (t_tz16.copy_(xs), tz16.enqueue(t_tz16, S, ws)))
    tz.check()
    tz16.check()
    n_len, _ = ff.response()
    ho = oracle.design_filter(n_len, rg.FILTERS["ramp"], 1.0, oracle.QUIRK_NONE)
    exp_f = np.stack([oracle.filter_rows(x[b], n_len, ho) for b in range(4)])
    out = {"workload": f"{S} slices, {Pp} x {Dp} parallel, pad {pad}, Ram-Lak, backprojection to {N}^2"}
    bp = rg.Backprojection(g, rg.make_params())
    img = torch.empty((2, N, N), dtype=torch.float32, device=dev)
    og = ns_geom(Pp, Dp, N)
    exp_img = oracle.fbp_parallel(og, oracle.make_params(filter_type="ramp", pad=pad), x[:2])
    useful = 2.0 * S * Pp * Dp * Dp
    for name, t, ms in (("fft", t_fft, ms_fft - ms_copy), ("toeplitz_split_bf16x3", t_tz, ms_tz - ms_copy),
                        ("toeplitz_split_f16x3", t_tz16, ms_tz16 - ms_copy)):
        bp.enqueue(t[:2], img, 2)
        rec = {"ms_per_64_slices": ms, "filter": err_pair(t[:4].cpu().numpy(), exp_f),
               "image": err_pair(img.cpu().numpy(), exp_img)}
        if name.startswith("toeplitz"):
            rec["useful_tflops"] = useful / (ms / 1e3) / 1e12
            rec["executed_tflops"] = 3 * useful / (ms / 1e3) / 1e12
            kind = "fp16 (power-of-two scaled)" if name.endswith("_f16x3") else "bf16"
            rec["gemm"] = f"M = {S * Pp} rows, K = N = {Dp} (zero padding not computed), 3 {kind} products"
        out[name] = rec
    return out


def ns_geom(Pp, Dp, N, **over):
    from types import SimpleNamespace

    d = dict(n_planes=1, n_fan_det=432, n_fan_proj=500, n_par_proj=Pp, n_par_det=Dp, n_pixels=N,
             source_offset=0.0, detector_diameter=480.0, image_width=200.0, image_center_x=0.0,
             image_center_y=0.0, rotation_offset=0.0, source_diameter=[430.0], delta_x=[0.0],
             delta_z=[1417.0], source_angle=[360.0])
    d.update(over)
    return SimpleNamespace(**d)


def measure_differentiation(torch, rg, dev):
    """Differentiation: 16 slices of 720 x 768 -> 512^2 with 1024 filter taps.
    Forward = taps filter + backprojection; backward = backprojection adjoint,
    transposed filter and the taps gradient. Reports the timings and the
    dot-product test <A s, y> = <s, A^T y> (relative to the sum of |terms|)."""
    S, Pp, Dp, N, T = 16, 720, 768, 512, 1024
    g = rg.make_geometry(n_par_proj=Pp, n_par_det=Dp, n_pixels=N)
    p = rg.make_params()
    rng = np.random.default_rng(4)
    taps = rng.standard_normal(T).astype(np.float32) / T
    filt = rg.Filter(g, p, taps=taps)
    bp = rg.Backprojection(g, p)
    bp.reserve(S)
    bp.reserve_adjoint(S)
    s = torch.from_numpy(rng.standard_normal((S, Pp, Dp)).astype(np.float32)).to(dev)
    y = torch.from_numpy(rng.standard_normal((S, N, N)).astype(np.float32)).to(dev)
    fs, img = torch.empty_like(s), torch.empty((S, N, N), dtype=torch.float32, device=dev)
    gs, gsf = torch.empty_like(s), torch.empty_like(s)
    gt = torch.empty(T, dtype=torch.float32, device=dev)
    ws = torch.empty(filt.taps_grad_workspace_bytes(S), dtype=torch.uint8, device=dev)

    def forward():
        fs.copy_(s)
        filt.enqueue(fs, S)
        bp.enqueue(fs, img, S)

    def backward():
        bp.enqueue_adjoint(y, gsf, S)            # d/d(filtered sinogram)
        filt.taps_grad(s, gsf, gt, S, ws)        # d/d(taps)
        gs.copy_(gsf)
        filt.enqueue_adjoint(gs, S)              # d/d(sinogram)

    ms_f, ms_b = cuda_ms(torch, forward), cuda_ms(torch, backward)
    ms_parts = {"bp_adjoint": cuda_ms(torch, lambda: bp.enqueue_adjoint(y, gsf, S)),
                "taps_grad": cuda_ms(torch, lambda: filt.taps_grad(s, gsf, gt, S, ws)),
                "filter_adjoint": cuda_ms(torch, lambda: (gs.copy_(gsf), filt.enqueue_adjoint(gs, S)))}
    forward()
    backward()
    torch.cuda.synchronize()
    tl = img.double() * y.double()
    tr = s.double() * gs.double()
    dot = abs(float(tl.sum()) - float(tr.sum())) / max(float(tl.abs().sum()), float(tr.abs().sum()))
    return {"workload": f"{S} slices, {Pp} x {Dp} -> {N}^2, {T} filter taps", "ms_forward": ms_f,
            "ms_backward": ms_b, "ms_backward_parts": ms_parts, "adjoint_dot_rel": dot,
            "fd_check": "FP64 central differences on 32 taps in tests/test_gpu_autograd.py"}


def measure_sweep(torch, rg, dev):
    """Uneven sweep: 256 seeded instances (side log-uniform 128..1024, 180..1440
    angles, rays 1.25 x side, 0..2% defective columns, Ram-Lak or Hann) in one
    persistent launch; throughput, per-instance latency from device timestamps,
    and the error of the 4 smallest instances against the FP64 oracle."""
    from risa_gb300 import phantom
    import oracle

    inst = phantom.sweep_instances(256, seed=5)
    raws = [phantom.sweep_counts(d, 1000 + i) for i, d in enumerate(inst)]
    sw = rg.Sweep(inst)
    _, io, _, it = sw.layout()
    raw = torch.from_numpy(np.concatenate([r.ravel() for r in raws]).view(np.int16)).to(dev)
    img = torch.empty(it, dtype=torch.float32, device=dev)
    ms = cuda_ms(torch, lambda: sw.enqueue(raw, img))
    sw.check()
    graph = sw.graph_capture(raw, img, torch.cuda.Stream(device=dev))
    ms_graph = cuda_ms(torch, lambda: graph.replay(None))
    sw.check()
    first, done, launch = sw.times()
    span = (done - first) / 1e6
    comp = (done - launch) / 1e6
    upd = sum(d["n_pixels"] ** 2 * d["n_par_proj"] for d in inst)
    small = sorted(range(len(inst)), key=lambda i: inst[i]["n_pixels"] ** 2 * inst[i]["n_par_proj"])[:4]
    host = img.cpu().numpy()
    worst = 0.0
    for i in small:
        d = inst[i]
        n = d["n_pixels"]
        flags = np.zeros(d["n_par_det"] + 1, np.int32)
        flags[:-1] = d["defect_map"]
        rep = oracle.interpolate_defects(raws[i], flags, oracle.QUIRK_NONE)
        att = oracle.attenuation(rep, np.full(raws[i].shape, d["ref_level"], np.float32),
                                 np.full(d["n_par_det"], d["dark_level"], np.float32))
        exp = oracle.fbp_parallel(ns_geom(d["n_par_proj"], d["n_par_det"], n),
                                  oracle.make_params(filter_type=d["filter_type"], masking=True), att[None])[0]
        got = host[io[i]:io[i] + n * n].reshape(n, n)
        worst = max(worst, float(np.abs(got - exp).max() / np.abs(exp).max()))
    return {"workload": "256 instances: side log-uniform 128..1024, angles 180..1440, rays 1.25 x side "
                        "(multiple of 32), 0..2% defective columns, Ram-Lak or Hann, circular mask",
            "ms_per_launch": ms, "instances_per_s": 256 / (ms / 1e3), "gupdates_per_s": upd / (ms / 1e3) / 1e9,
            "ms_per_graph_replay": ms_graph, "grid": sw.grid(), "launches": 1,
            "instance_span_ms": {"p50": float(np.percentile(span, 50)), "p99": float(np.percentile(span, 99))},
            "completion_ms": {"p50": float(np.percentile(comp, 50)), "p99": float(np.percentile(comp, 99))},
            "max_rel_vs_fp64_4_smallest": worst}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.only:
        import torch

        import risa_gb300 as rg

        dev = torch.device("cuda", local_rank)
        torch.cuda.set_device(dev)
        fn = {"precision": measure_precision, "differentiation": measure_differentiation,
              "sweep": measure_sweep}[args.only]
        print(json.dumps({"workload": args.only, **fn(torch, rg, dev)}), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
