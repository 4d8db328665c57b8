"""Benchmark: 1080p MPTC encode throughput (frames/s) on GB300.

A step is one pass of the encoder hot path (stb DXT1 encode + index-block
search + unique palette) over the 120-frame 1920x1080 synthetic stream
(search area 8, error threshold 5, intra interval 16: 8 intra + 112 inter
frames). `value` times K steps with the frames already resident in HBM
(746 MB of input, larger than the 129 MB L2, so nothing stays cached between
steps), one mptc_encode_stream_device call per step (outputs in HBM; intra
frames on the call's second lane, concurrent with the inter frames before
them); `e2e` times the same stream through the C ABI's host-buffer stream
call, mptc_encode_stream_host (pinned host frames in, final blocks / motion
codes / unique palette out, the copies overlapping the encode).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

N>1 (under torchrun) runs one independent stream per GPU ("replicas": streams
shard across GPUs with no data exchange). `--impl reference` times the CPU
restatement of the reference encoder (the oracle port) on the host cores.
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
sys.path.insert(0, ROOT)

from mptc_gb300.encoder import intra_schedule  # noqa: E402

METRIC = "1080p encoded frames/s: learned-proposal vs exhaustive GPU search at ≤0.1 dB loss"
W, H, FRAMES, SA, THR, II = 1920, 1080, 120, 8, 5, 16
# Scalar ops per candidate evaluation (refit 16x(6 mul + 6 add for the
# pixel sums + 3 mul + 3 add for the weight sums), 2x2 solve, rounding and
# 5/6-bit snap, palette, 16-pixel squared error) and per stb block encode.
C_CAND, C_DXT = 600, 1500
# DRAM bytes (read + write) per launch of the search kernels on the 1080p
# stream, from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum);
# the summaries under profiles/ give the commands.
NCU_TRAFFIC = {"inter_search": 10_906_368 + 96_768, "intra_search_kernel": 9_365_248 + 382_464}


def algo_bytes(kernel: str, n: int) -> int:
    """Algorithmic HBM bytes of one launch: the RGB8 frame plus the per-block
    arrays the kernel must read (stb block, stb error, previous final block)
    and write (final block, motion code, completion flag)."""
    frame = W * H * 3
    if kernel == "dxt1_encode_kernel":
        return frame + n * (8 + 4)
    return frame + n * (8 + 4 + 8 + 8 + 2 + 4)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def max_over_ranks(x: float, dist, device) -> float:
    """The largest value of x over the ranks (the whole job's time): the
    replicas' timings are reduced once, after the timed region."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all ranks processed per second of the slowest rank."""
    return world * units_per_rank / seconds


# --------------------------------------------------------------------------
# CPU baseline: the oracle (CPU restatement of the reference hot path)
# --------------------------------------------------------------------------
def cpu_gop_sample(g: int, threads: int):
    """Times one sample of GOP g of the 1080p stream on the host cores with the
    oracle: its intra frame 16g and the inter frame 16g + 1 after it (which
    needs only the intra frame's final blocks). The stb encode is in both
    times. Returns (t_intra, t_inter, info)."""
    import oracle
    from mptc_gb300.synth import FHD1080
    frames = FHD1080.generate(II * g, 2)
    t0 = time.perf_counter()
    stb0 = oracle.dxt1_encode(frames[0])
    r0 = oracle.reencode(frames[0], stb0, None, SA, THR, threads, want_psnr=False)
    t1 = time.perf_counter()
    stb1 = oracle.dxt1_encode(frames[1])
    r1 = oracle.reencode(frames[1], stb1, r0.final, SA, THR, threads, want_psnr=False)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1, dict(intra_visited=r0.stats.intra_visited, inter_visited=r1.stats.inter_visited,
                                  inter_frame_intra_visited=r1.stats.intra_visited, prev=r0.final, stb1=stb1,
                                  frame1=frames[1])


def stream_rate(t_intra: float, t_inter: float) -> float:
    """Frames/s of the 120-frame stream (8 intra + 112 inter frames) at the
    given per-frame times."""
    n_intra = sum(intra_schedule(FRAMES, II))
    return FRAMES / (n_intra * t_intra + (FRAMES - n_intra) * t_inter)


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(threads: int):
    """The GPU arm's CPU baseline: GOPs 0 and 1 sampled (two intra and two
    inter frames), extrapolated to the stream's 8 intra + 112 inter mix."""
    ti, tp = [], []
    info = None
    for g in (0, 1):
        a, b, inf = cpu_gop_sample(g, threads)
        ti.append(a)
        tp.append(b)
        info = info or inf
    info["inter_distinct"] = window_distinct(info.pop("prev"), info.pop("stb1"), W // 4, H // 4, SA)
    info.pop("frame1")
    info.update(t_intra=statistics.mean(ti), t_inter=statistics.mean(tp))
    return stream_rate(statistics.mean(ti), statistics.mean(tp)), info


def window_distinct(prev_final: np.ndarray, stb: np.ndarray, bw: int, bh: int, sa: int) -> int:
    """Sum over blocks of the distinct index words, other than the block's own,
    among the in-bounds positions of its inter window: the candidate
    evaluations a search that evaluates each distinct word once performs."""
    from numpy.lib.stride_tricks import sliding_window_view
    prev = (prev_final >> np.uint64(32)).astype(np.int64).reshape(bh, bw)
    own = (stb >> np.uint64(32)).astype(np.int64).reshape(bh, bw)
    pad = np.full((bh + 2 * sa, bw + 2 * sa), -1, np.int64)
    pad[sa:sa + bh, sa:sa + bw] = prev
    win = sliding_window_view(pad, (2 * sa, 2 * sa))[:bh, :bw]
    total = 0
    for y0 in range(0, bh, 16):
        w = win[y0:y0 + 16].reshape(-1, 4 * sa * sa).copy()
        o = own[y0:y0 + 16].reshape(-1, 1)
        w[w == o] = -1
        w.sort(axis=1)
        d = (np.diff(w, axis=1) != 0).sum(axis=1) + 1 - (w[:, 0] == -1)
        total += int(d.sum())
    return total


def run_reference(args, rank: int) -> None:
    """The reference arm: the oracle (the reference hot path restated in C and
    pinned to the reference's outputs) on all host cores. Step k encodes a
    sample of GOP k mod 8 of the 1080p stream (its intra frame and the inter
    frame after it), so the timed steps spread over all eight GOPs; ms_per_step
    is the measured time of a step. `value` is the stream's frames/s at the
    measured mean intra and inter frame times (8 intra + 112 inter frames);
    the samples' own rate and a one-thread rate are reported beside it."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ti, tp, steps_s = [], [], []
    for k in range(args.warmup + args.steps):
        a, b, _ = cpu_gop_sample(k % (FRAMES // II), threads)
        if k >= args.warmup:
            ti.append(a)
            tp.append(b)
            steps_s.append(a + b)
    v = stream_rate(statistics.mean(ti), statistics.mean(tp))
    # one inter frame on one thread (the intra search is sequential anyway)
    _, _, inf = cpu_gop_sample(0, 1)
    import oracle
    t0 = time.perf_counter()
    oracle.reencode(inf["frame1"], oracle.dxt1_encode(inf["frame1"]), inf["prev"], SA, THR, 1, want_psnr=False)
    tp1 = time.perf_counter() - t0
    v1 = stream_rate(statistics.mean(ti), tp1)
    step_ms = 1000.0 * statistics.mean(steps_s)
    sample = (f"step k: GOP k mod 8 of the 1080p stream, its intra frame and the inter frame after it (frames "
              f"16g, 16g+1), timed on {threads} threads (inter search threaded, intra search sequential as in the "
              f"reference); value = the 120-frame stream's 8 intra + 112 inter frames at the measured mean times "
              f"({statistics.mean(ti):.3f} s intra, {statistics.mean(tp):.3f} s inter)")
    line = dict(impl="reference", metric=METRIC, value=round(v, 4), unit="frames/s", n_gpus=args.gpus,
                steps=args.steps, warmup=args.warmup, ms_per_step=round(step_ms, 3),
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="fp32+int32",
                data="synthetic", config=workload_config(),
                cpu_baseline=dict(value=round(v, 4), unit="frames/s", cores=threads, kind="port", sample=sample,
                                  cpu_model=cpu_model(), sample_fps=round(2000.0 / step_ms, 4),
                                  stream_fps_extrapolated=round(v, 4),
                                  single_thread=dict(value=round(v1, 4), unit="frames/s",
                                                     inter_frame_s=round(tp1, 3),
                                                     note="intra frames as measured (sequential), one inter "
                                                          "frame timed on one thread")),
                e2e=dict(value=round(v, 4), unit="frames/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def workload_config() -> dict:
    return {"workload": "1080p MPTC encode, 120-frame synthetic stream (moving squares over periodic "
                        "gradients, seeded, 1920x1080)",
            "width": W, "height": H, "frames_per_step": FRAMES, "search_area": SA,
            "err_threshold": THR, "intra_interval": II, "search": "exhaustive (bit-exact plain path)",
            "l2": "inputs larger than L2: 120 frames x 6.2 MB resident, each read once per step",
            "parallelism": "replicas (one stream per GPU)"}


# --------------------------------------------------------------------------
# Clock sampling during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200",
                                       "-i", str(gpu_index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict | None:
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def alu_peak_gops(torch) -> float:
    """Measured fp32 scalar-add throughput (the probe kernel in libmptc_gb300)."""
    import ctypes
    from mptc_gb300._lib import check, lib
    sink = torch.zeros(1, dtype=torch.int32, device="cuda")
    ops = ctypes.c_double(0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    stream = torch.cuda.current_stream()
    s = ctypes.c_void_p(stream.cuda_stream)
    best = 0.0
    for _ in range(3):
        check(lib().mptc_alu_probe(sms * 8, 2048, sink.data_ptr(), ctypes.byref(ops), s))
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        check(lib().mptc_alu_probe(sms * 8, 2048, sink.data_ptr(), ctypes.byref(ops), s))
        b.record(stream)
        b.synchronize()
        best = max(best, ops.value / (a.elapsed_time(b) * 1e-3) / 1e9)
    return best


def check_against_reference(fin_all, mot_all, uni_all, nu_all) -> dict | None:
    """Compares the last timed step's outputs, frame by frame, with the
    unmodified reference encoder's records of the same stream (SHA-256 of the
    final blocks, motion codes and unique palette of every frame). Raises if
    any frame differs: a bench number of a wrong encoder is not a number."""
    import hashlib
    path = os.path.join(ROOT, "tests", "golden", "configs.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        case = {c["name"]: c for c in json.load(f)["cases"]}.get("fhd1080_120f_sa8_thr5")
    if case is None or fin_all.shape[0] != case["count"]:
        return None

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    fin, mot, uni, nu = (t.cpu().numpy() for t in (fin_all, mot_all, uni_all, nu_all))
    bad = [k for k, g in enumerate(case["frames"])
           if (sha(fin[k]), sha(mot[k]), sha(uni[k, :nu[k]])) != (g["final"], g["motion"], g["unique"])]
    if bad:
        raise RuntimeError(f"bench outputs differ from the reference encoder's on frames {bad[:8]}")
    return {"frames_checked": len(case["frames"]), "bit_exact": True,
            "against": "reference encoder's per-frame SHA-256 of final blocks, motion codes and unique "
                       "palette (tests/golden/configs.json)"}


def run_gpu(args, rank: int, world: int, dist) -> None:
    import torch

    from mptc_gb300.encoder import Encoder
    from mptc_gb300.synth import FHD1080, StreamSpec

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    spec = StreamSpec(**{**FHD1080.__dict__, "seed": FHD1080.seed + rank})
    nf = args.frames
    t = time.time()
    frames_np = spec.generate(0, nf)
    log(f"[rank {rank}] generated {nf} frames in {time.time() - t:.1f}s")
    frames_dev = torch.from_numpy(frames_np).to(dev)
    enc = Encoder(W, H, SA, THR, II)
    n = enc.nblk
    sched = intra_schedule(nf, II)
    stream = torch.cuda.current_stream()

    # a step is one mptc_encode_stream_device call over the stream's frames:
    # outputs stay in HBM, intra frames run on the call's second lane
    fin_all = torch.empty((nf, n), dtype=torch.int64, device=dev)
    mot_all = torch.empty((nf, 2 * n), dtype=torch.uint8, device=dev)
    uni_all = torch.empty((nf, n), dtype=torch.int32, device=dev)
    nu_all = torch.empty(nf, dtype=torch.int32, device=dev)

    def step():
        enc.encode_stream_device(frames_dev, fin_all, mot_all, uni_all, nu_all, is_intra=sched, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    enc.kernel_times()  # clear
    enc.kernel_launches()  # clear
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = clk.stop()
    launches = enc.kernel_launches()
    elapsed_ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    # per-kernel CUDA-event times come from separate steps after the timed
    # region (events around every launch would add to the timed step)
    enc.set_kernel_timing(True)
    for _ in range(min(args.steps, 3)):
        step()
    torch.cuda.synchronize()
    enc.set_kernel_timing(False)
    ktimes = enc.kernel_times()
    value = whole_job_rate(nf * args.steps, world, elapsed_ms * 1e-3)
    st = enc.stats(stream)  # also raises on a device-side timeout
    parity = check_against_reference(fin_all, mot_all, uni_all, nu_all) if rank == 0 else None
    if args.quick:
        if rank == 0:
            print(json.dumps(dict(quick=True, frames=nf, value=value, kernels={
                k: {"launches": v[0], "total_ms": v[1]} for k, v in ktimes.items()})), flush=True)
        enc.close()
        return

    # ---- end to end through the C ABI's host-buffer call --------------------
    # one mptc_encode_stream_host call per step over the stream's frames in
    # pinned host memory: uploads and downloads overlap the encode
    pin_frames = torch.from_numpy(frames_np).pin_memory()
    fb = pin_frames.numpy()
    from mptc_gb300.encoder import StreamOutput
    out = StreamOutput(torch.empty((nf, n), dtype=torch.int64).pin_memory().numpy().view(np.uint64),
                       torch.empty((nf, 2 * n), dtype=torch.uint8).pin_memory().numpy(),
                       torch.empty((nf, n), dtype=torch.int32).pin_memory().numpy().view(np.uint32),
                       torch.empty(nf, dtype=torch.int32).pin_memory().numpy().view(np.uint32))
    e2e_enc = Encoder(W, H, SA, THR, II)

    def host_step():
        e2e_enc.encode_stream_host(fb, is_intra=sched, out=out)

    host_step()  # warm-up
    if dist is not None:
        dist.barrier()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e_value = whole_job_rate(nf * e2e_steps, world, e2e_s)
    h2d = nf * W * H * 3
    d2h = nf * (n * 8 + n * 2 + n * 4 + 4) + 4  # per frame: final, motion, palette, count; the run's status
    e2e_enc.close()

    # ---- roofline of the dominant kernel -------------------------------------
    # The step time is set by the first lane (stb encode, inter search, intra
    # pass, palette of every inter frame): the intra frames run concurrently
    # on the second lane. The dominant kernel is the first lane's largest; its
    # event times include the contention with the overlapping intra frames.
    dom = ("inter_search", ktimes["inter_search"]) if "inter_search" in ktimes else \
        max(ktimes.items(), key=lambda kv: kv[1][1])
    line = dict(metric=METRIC, value=round(value, 3), unit="frames/s", n_gpus=world, steps=args.steps,
                warmup=args.warmup, ms_per_step=round(elapsed_ms / args.steps, 3), higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="fp32+int32", data="synthetic",
                config=workload_config(), clocks=clocks,
                e2e=dict(value=round(e2e_value, 3), unit="frames/s", h2d_bytes_per_step=h2d,
                         d2h_bytes_per_step=d2h),
                gpu_launches=int(launches),
                kernels={k: {"calls": v[0], "total_ms": round(v[1], 3),
                             "avg_us": round(1000 * v[1] / max(1, v[0]), 2)} for k, v in ktimes.items()},
                last_frame={"n_inter": st.n_inter, "n_intra": st.n_intra, "n_unique": st.n_unique},
                parity=parity)
    if rank == 0:
        info = None
        if world == 1:
            threads = os.cpu_count() or 1
            cfps, info = cpu_sample(threads)
            line["cpu_baseline"] = dict(
                value=round(cfps, 4), unit="frames/s", cores=threads, kind="port", cpu_model=cpu_model(),
                sample="GOPs 0 and 1 of the 1080p stream (intra frames 0, 16 and inter frames 1, 17), "
                       "extrapolated to the 8 intra + 112 inter frames at the measured mean times "
                       f"({info['t_intra']:.3f} s, {info['t_inter']:.3f} s); inter search on {threads} threads, "
                       "intra search sequential")
        peak = alu_peak_gops(torch)
        name, (nl, tot) = dom
        avg_s = tot / nl * 1e-3
        units = None
        if info is not None:
            units = {"inter_search": info["inter_visited"],
                     "intra_search_kernel": info["intra_visited"],
                     "intra_sweep_kernel/inter_frame": info["inter_frame_intra_visited"],
                     "dxt1_encode_kernel": n}.get(name)
        if units is not None:
            per = C_DXT if name == "dxt1_encode_kernel" else C_CAND
            ref_units = units
            if name == "inter_search":
                # the kernel evaluates each distinct index word of a window once
                units = info["inter_distinct"]
            ach = units * per / avg_s / 1e9
            line["roofline"] = dict(bound="alu", achieved=round(ach, 1), peak=round(peak, 1), unit="Gop/s",
                                    frac=round(ach / peak, 4), kernel=name,
                                    units_per_launch=int(units), ops_per_unit=per,
                                    reference_units_per_launch=int(ref_units),
                                    reference_frac=round(ref_units * per / avg_s / 1e9 / peak, 4),
                                    traffic=NCU_TRAFFIC.get(name),
                                    hbm=dict(achieved_gbs=round(algo_bytes(name, n) / avg_s / 1e9, 2),
                                             peak_gbs=6782.1, bytes_per_launch=algo_bytes(name, n)),
                                    peak_note="measured fp32 add probe (libmptc_gb300 mptc_alu_probe), "
                                              "152 SMs x 128 lanes at the clock seen",
                                    timing_note="CUDA-event launch times of the same step, run after the timed region, where the "
                                                "intra frames of the second lane overlap the inter frames")
    if rank == 0 and world == 1 and not args.no_learned and nf == FRAMES:
        line["learned"] = learned_comparison(args, torch, dev, frames_dev, value, log)
    if rank == 0:
        print(json.dumps(line), flush=True)
    enc.close()


def run_batch(args, rank: int, world: int, dist) -> None:
    """S concurrent 1080p streams through the batched encoder's run call (see
    time_batch), plain exhaustive search."""
    import torch

    from mptc_gb300.synth import FHD1080, StreamSpec

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    S, nf = args.batch, args.frames
    frames_dev = torch.from_numpy(StreamSpec(**{**FHD1080.__dict__, "seed": FHD1080.seed + rank}).generate(0, nf)).to(dev)
    if dist is not None:
        dist.barrier()
    clk = ClockSampler(local)
    value, tuned = time_batch(torch, frames_dev, S, None, 0, args.steps, args.warmup)
    clocks = clk.stop()
    value = whole_job_rate(S * nf * args.steps, world, max_over_ranks(S * nf * args.steps / value, dist, dev))
    if rank == 0:
        cfg = workload_config()
        cfg.update({"workload": f"batched 1080p MPTC encode: {S} concurrent streams x {nf} frames",
                    "streams_per_gpu": S, "intra_phase": "stream k: 16k/S", "autotune": tuned})
        print(json.dumps(dict(metric=METRIC, value=round(value, 3), unit="frames/s", n_gpus=world,
                              steps=args.steps, warmup=args.warmup,
                              ms_per_step=round(1000.0 * S * nf * world / value, 3), higher_is_better=True,
                              scaling="weak", vs_baseline=None, dtype="fp32+int32", data="synthetic",
                              config=cfg, clocks=clocks)), flush=True)


def adaptive_code_bits(symbols: np.ndarray, alphabet: int) -> float:
    """Code length of an adaptive order-0 model whose counts start at 1:
    log2(A (A+1) ... (A+N-1)) - sum_s log2(n_s!), in closed form."""
    from math import lgamma, log
    n = np.bincount(np.asarray(symbols, np.int64), minlength=alphabet).astype(np.float64)
    N = float(n.sum())
    nats = lgamma(alphabet + N) - lgamma(alphabet) - float(sum(lgamma(c + 1.0) for c in n if c > 0))
    return nats / log(2.0)


def encode_stream_quality(torch, enc, frames_dev, sched, W_, H_):
    """Encodes a stream once (device API) and returns per-frame decoded SSE,
    motion-code + palette adaptive code length (bits) and stats."""
    import ctypes
    from mptc_gb300._lib import check, lib
    n = (W_ // 4) * (H_ // 4)
    dev = frames_dev.device
    fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
    stb = torch.empty(n, dtype=torch.int64, device=dev)
    mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
    uni = torch.empty(n, dtype=torch.int32, device=dev)
    nu = torch.zeros(1, dtype=torch.int32, device=dev)
    sse = torch.zeros(1, dtype=torch.int64, device=dev)
    out = dict(sse=[], bits=[], unique=[], fallback=0, inter=0)
    for f in range(frames_dev.shape[0]):
        prev = None if sched[f] else fin[(f - 1) % 2]
        enc.encode_frame_device(frames_dev[f], prev, stb, fin[f % 2], mot, uni, nu)
        check(lib().mptc_decoded_sse(frames_dev[f].data_ptr(), W_, H_, fin[f % 2].data_ptr(), sse.data_ptr(),
                                     ctypes.c_void_p(0)))
        st = enc.stats()
        out["sse"].append(int(sse.item()))
        m = mot.cpu().numpy()
        k = int(nu.item())
        pal = uni[:k].cpu().numpy().view(np.uint8)
        out["bits"].append(adaptive_code_bits(m.astype(np.int64), 256) + adaptive_code_bits(pal.astype(np.int64), 256))
        out["unique"].append(k)
        out["fallback"] += st.n_fallback
        out["inter"] += st.n_inter
    return out


def pad_to_tiles(torch, frames_dev):
    """Edge-replicates frames to multiples of 256 pixels, the sizes the MPTC
    stream's endpoint wavelet accepts (1920x1080 -> 2048x1280)."""
    n, h, w, _ = frames_dev.shape
    H2, W2 = -(-h // 256) * 256, -(-w // 256) * 256
    out = torch.empty((n, H2, W2, 3), dtype=torch.uint8, device=frames_dev.device)
    out[:, :h, :w] = frames_dev
    out[:, h:, :w] = frames_dev[:, h - 1:h, :]
    out[:, :, w:] = out[:, :, w - 1:w]
    return out


def stream_size(torch, enc, frames_dev, sched, ui):
    """Encodes the frames (device API), writes the MPTC stream (GPU endpoint
    transform + host arithmetic coder) and decodes it with the GPU decoder.
    Returns (stream bytes, every frame decoded bit-exactly)."""
    from mptc_gb300.decoder import Decoder, endpoint_coefficients
    from mptc_gb300.stream import StreamReader, StreamWriter
    nf, H_, W_, _ = frames_dev.shape
    n = (W_ // 4) * (H_ // 4)
    dev = frames_dev.device
    fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
    stb = torch.empty(n, dtype=torch.int64, device=dev)
    mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
    uni = torch.empty(n, dtype=torch.int32, device=dev)
    nu = torch.zeros(1, dtype=torch.int32, device=dev)
    coeff = torch.empty(6 * n, dtype=torch.uint8, device=dev)
    sw = StreamWriter(W_, H_, SA, ui, nf)
    finals = []
    for f in range(nf):
        prev = None if sched[f] else fin[(f - 1) % 2]
        enc.encode_frame_device(frames_dev[f], prev, stb, fin[f % 2], mot, uni, nu)
        endpoint_coefficients(W_, H_, fin[f % 2], coeff)
        k = int(nu.item())
        sw.add_frame_coefficients(coeff.cpu().numpy(), mot.cpu().numpy(), uni[:k].cpu().numpy().view(np.uint32))
        finals.append(fin[f % 2].cpu().numpy().view(np.uint64).copy())
    data = sw.finish()
    sw.close()
    rd = StreamReader(data)
    dec = Decoder(W_, H_, SA)
    exact = True
    for k, (m, c, u) in enumerate(rd):
        exact &= bool((dec.decode_frame(m, c, u).cpu().numpy().view(np.uint64) == finals[k]).all())
    dec.check()
    dec.close()
    rd.close()
    return len(data), exact


def psnr_db(sse_list, W_, H_):
    return float(np.mean([10.0 * np.log10(3.0 * 255.0 ** 2 / (s / (W_ * H_))) for s in sse_list]))


def time_stream_call(torch, enc, frames_dev, sched, steps, warmup):
    """Frames/s of mptc_encode_stream_device over the frames (outputs in HBM)."""
    nf = frames_dev.shape[0]
    n = enc.nblk
    dev = frames_dev.device
    fin = torch.empty((nf, n), dtype=torch.int64, device=dev)
    mot = torch.empty((nf, 2 * n), dtype=torch.uint8, device=dev)
    uni = torch.empty((nf, n), dtype=torch.int32, device=dev)
    nu = torch.empty(nf, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        enc.encode_stream_device(frames_dev, fin, mot, uni, nu, is_intra=sched, stream=s)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        enc.encode_stream_device(frames_dev, fin, mot, uni, nu, is_intra=sched, stream=s)
    e1.record(s)
    torch.cuda.synchronize()
    enc.stats(s)  # raises on a device-side timeout
    return nf * steps / (e0.elapsed_time(e1) * 1e-3)


def time_batch(torch, frames_dev, S, model, topk, steps, warmup):
    """S concurrent 1080p streams (stream k plays the 120-frame stream from
    frame offset 15k, its intra frames at phase 16k/S) through the batched
    encoder: the launch shapes are tuned on a mixed frame step, then each step
    is one mptc_batch_encode_run over every stream's 120 frames (outputs in
    HBM). Returns (frames/s of all streams together, the tuned shapes)."""
    from mptc_gb300.batch import BatchEncoder
    nf = frames_dev.shape[0]
    n = (W // 4) * (H // 4)
    dev = frames_dev.device
    b = BatchEncoder([(W, H)] * S, SA, THR, II)
    if model is not None:
        b.set_model(model, topk)
    offsets = [(15 * k) % nf for k in range(S)]
    phases = [(II * k) // S for k in range(S)]
    s = torch.cuda.current_stream()

    def flags(f):
        return [f == 0 or (f - phases[k]) % II == 0 for k in range(S)]
    for f in range(2):
        for k in range(S):
            b.upload(k, frames_dev[(f + offsets[k]) % nf], s)
        b.encode(flags(f), s)
    tuned = b.autotune(flags(2), s)
    runs = [torch.roll(frames_dev, -offsets[k], dims=0).contiguous() for k in range(S)]
    fins = [torch.empty((nf, n), dtype=torch.int64, device=dev) for _ in range(S)]
    mots = [torch.empty((nf, 2 * n), dtype=torch.uint8, device=dev) for _ in range(S)]
    unis = [torch.empty((nf, n), dtype=torch.int32, device=dev) for _ in range(S)]
    nus = [torch.empty(nf, dtype=torch.int32, device=dev) for _ in range(S)]
    run_flags = [[flags(f)[k] for f in range(nf)] for k in range(S)]

    def step():
        b.encode_run(runs, fins, mots, unis, nus, run_flags, s)
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    b.close()
    del runs, fins, mots, unis, nus
    return S * nf * steps / (e0.elapsed_time(e1) * 1e-3), tuned


def learned_comparison(args, torch, dev, frames_dev, plain_fps, log):
    """The learned proposal against the exhaustive search on the 1080p stream:
    trains on 200 separate seeded 1080p frames with the library's kernels, then
    measures the learned form single-stream and batched beside the plain form,
    the decoded PSNR and motion/palette code length of the same 120 frames, and
    the bytes of whole MPTC streams of the first 32 frames (edge-padded to
    256-pixel multiples, decoded back bit-exactly on the GPU)."""
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.synth import FHD1080_CALIB, FHD1080_TRAIN
    from mptc_gb300.training import choose_topk, train_proposal
    t0 = time.time()
    train_dev = torch.from_numpy(FHD1080_TRAIN.generate()).to(dev)
    gen_s = time.time() - t0
    model, losses, tinfo = train_proposal(torch, train_dev, SA, THR, II, steps=args.train_steps, batch=4096,
                                          cands=32, lr=1e-3, log=log)
    del train_dev
    torch.cuda.empty_cache()
    # K: given, or the fastest that stays within half the PSNR budget on
    # separate calibration frames, judged by the exhaustive search
    calib = torch.from_numpy(FHD1080_CALIB.generate()).to(dev)
    if getattr(args, "save_model", ""):
        model.save(args.save_model)
    K, k_table = choose_topk(torch, model, calib, SA, THR, II, ks=(args.topk,) if args.topk > 0 else (4, 8, 16),
                             log=log)
    del calib
    nf = frames_dev.shape[0]
    sched = intra_schedule(nf, II)
    plain_enc = Encoder(W, H, SA, THR, II)
    learned_enc = Encoder(W, H, SA, THR, II)
    learned_enc.set_model(model, K)
    qp = encode_stream_quality(torch, plain_enc, frames_dev, sched, W, H)
    ql = encode_stream_quality(torch, learned_enc, frames_dev, sched, W, H)
    ns, UI = min(nf, 32), 8
    padded = pad_to_tiles(torch, frames_dev[:ns])
    pw, ph = padded.shape[2], padded.shape[1]
    enc_p = Encoder(pw, ph, SA, THR, II)
    bytes_p, exact_p = stream_size(torch, enc_p, padded, sched, UI)
    enc_p.set_model(model, K)
    bytes_l, exact_l = stream_size(torch, enc_p, padded, sched, UI)
    enc_p.close()
    del padded
    steps, warm = max(1, min(args.steps, 3)), max(1, min(args.warmup, 2))
    learned_fps = time_stream_call(torch, learned_enc, frames_dev, sched, steps, warm)
    S = args.batch if args.batch > 0 else 8
    plain_b, tuned_p = time_batch(torch, frames_dev, S, None, K, steps, warm)
    learned_b, tuned_l = time_batch(torch, frames_dev, S, model, K, steps, warm)
    plain_enc.close()
    learned_enc.close()
    model.close()
    inter_blocks = sum(1 for f in sched if not f) * (W // 4) * (H // 4)
    psnr_p, psnr_l = psnr_db(qp["sse"], W, H), psnr_db(ql["sse"], W, H)
    bits_p, bits_l = sum(qp["bits"]), sum(ql["bits"])
    return {
        "method": f"top-{K} distinct window words scored by f(block).g(word) on the tensor cores, exact test of the "
                  "K with the reference's selection rule, exhaustive search of the blocks none passes",
        "topk": K, "topk_calibration": {str(k): {"psnr_loss_db": v[0], "ms_per_frame": v[1], "fallback": v[2]}
                                         for k, v in k_table.items()},
        "streams_batched": S,
        "plain_single_fps": round(plain_fps, 2), "learned_single_fps": round(learned_fps, 2),
        "plain_batched_fps": round(plain_b, 2), "learned_batched_fps": round(learned_b, 2),
        "speedup_learned_batched_vs_plain_single": round(learned_b / plain_fps, 3),
        "speedup_learned_vs_plain_single_stream": round(learned_fps / plain_fps, 3),
        "psnr_plain_db": round(psnr_p, 4), "psnr_learned_db": round(psnr_l, 4),
        "psnr_delta_db": round(psnr_l - psnr_p, 4),
        "motion_palette_bits_delta": round(bits_l / bits_p - 1.0, 5),
        "stream_frames": ns, "stream_padding": f"{W}x{H} edge-replicated to {pw}x{ph}",
        "stream_bytes_plain": bytes_p, "stream_bytes_learned": bytes_l,
        "stream_bytes_delta": round(bytes_l / bytes_p - 1.0, 5),
        "streams_decode_exactly": bool(exact_p and exact_l),
        "fallback_rate": round(ql["fallback"] / max(1, inter_blocks), 4),
        "gates": {"psnr_loss_le_0.1db": bool(psnr_p - psnr_l <= 0.1),
                  "bytes_increase_le_2pct": bool(bytes_l <= 1.02 * bytes_p)},
        "autotune": {"plain": tuned_p, "learned": tuned_l},
        "train": {**tinfo, "frames_generated_s": round(gen_s, 1), "loss_first": round(losses[0], 4),
                  "loss_last": round(float(np.mean(losses[-50:])), 4), "optimizer": "AdamW lr 1e-3 wd 1e-4"},
    }


def run_learned(args, rank: int, world: int, dist) -> None:
    """Learned proposal + batching as the headline value: the same measurements
    as the default run's `learned` object, printed as their own line."""
    import torch

    from mptc_gb300.encoder import Encoder
    from mptc_gb300.synth import FHD1080

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nf = args.frames
    frames_dev = torch.from_numpy(FHD1080.generate(0, nf)).to(dev)
    sched = intra_schedule(nf, II)
    if args.quick:
        # profiling: an untrained model of the same shapes, kernel times of the
        # learned stream call only (no training, quality or batch runs)
        from mptc_gb300.model import ProposalModel
        model = ProposalModel(seed=1)
        if args.model:
            model.load(args.model)
        enc = Encoder(W, H, SA, THR, II)
        enc.set_model(model, args.topk or 8)
        from mptc_gb300._lib import check, lib
        check(lib().mptc_ctx_set_learned_shape(enc.handle, args.score_rows), enc.handle)
        fps = time_stream_call(torch, enc, frames_dev, sched, max(1, args.steps), max(1, args.warmup))
        enc.set_kernel_timing(True)
        time_stream_call(torch, enc, frames_dev, sched, 1, 0)
        enc.set_kernel_timing(False)
        kt = enc.kernel_times()
        if rank == 0:
            print(json.dumps(dict(quick=True, learned=True, frames=nf, score_rows=args.score_rows, topk=args.topk or 8,
                                  value=round(fps, 2), kernels={
                k: {"launches": v[0], "total_ms": round(v[1], 3)} for k, v in kt.items()})), flush=True)
        enc.close()
        model.close()
        return
    enc = Encoder(W, H, SA, THR, II)
    clk = ClockSampler(local)
    plain_fps = time_stream_call(torch, enc, frames_dev, sched, max(1, min(args.steps, 3)), 2)
    enc.close()
    cmp_ = learned_comparison(args, torch, dev, frames_dev, plain_fps, log if rank == 0 else None)
    clocks = clk.stop()
    value = cmp_["learned_batched_fps"]
    if rank == 0:
        cfg = workload_config()
        cfg.update({"workload": f"learned proposal + batching on the 1080p stream ({cmp_['streams_batched']} "
                                f"streams x {nf} frames); top-K {cmp_['topk']}",
                    "search": cmp_["method"], "streams_per_gpu": cmp_["streams_batched"]})
        print(json.dumps(dict(metric=METRIC, value=round(value, 3), unit="frames/s", n_gpus=world, steps=args.steps,
                              warmup=args.warmup, ms_per_step=round(1000.0 * nf * cmp_["streams_batched"] / value, 3),
                              higher_is_better=True, scaling="weak", vs_baseline=None, dtype="bf16+fp32+int32",
                              data="synthetic", config=cfg, clocks=clocks, learned=cmp_)), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--frames", type=int, default=FRAMES,
                    help="frames per step (profiling runs use a short prefix of the stream)")
    ap.add_argument("--batch", type=int, default=0,
                    help="S > 0: S concurrent 1080p streams per GPU through the batched encoder")
    ap.add_argument("--learned", action="store_true",
                    help="learned proposal: train on 200 separate seeded frames, then time plain vs learned")
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--score-rows", type=int, default=8, choices=(4, 8),
                    help="--learned --quick: dictionary slice per stage of the window scoring (x16 words)")
    ap.add_argument("--no-learned", action="store_true",
                    help="default run without the learned-proposal comparison")
    ap.add_argument("--topk", type=int, default=0,
                    help="proposals per block (4, 8, 16); 0 = chosen on calibration frames")
    ap.add_argument("--save-model", default="",
                    help="--learned: write the trained model's weights to this file")
    ap.add_argument("--model", default="",
                    help="--learned --quick: weights to load (a file --save-model wrote) instead of an untrained model")
    ap.add_argument("--quick", action="store_true",
                    help="device-timed region only: no e2e pass, CPU baseline or ALU probe (profiling)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    if args.learned:
        run_learned(args, rank, world, dist)
    elif args.batch > 0:
        run_batch(args, rank, world, dist)
    else:
        run_gpu(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
