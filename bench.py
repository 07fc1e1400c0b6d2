#!/usr/bin/env python3
"""Benchmark: 1080p decoded frames/s of the GB300 reconstruction engine.

Workload (the reference's 1080p High configuration as seeded bitstreams):
S independent CAVLC streams of 1920x1088, 30 pictures each, GOP 15 IBBP,
8x8 transforms, P partitions down to 4x4, 4 reference pictures, explicit
weighted bi-prediction, MVs +-256 quarter samples with 5% past the picture
edges, QP 22..40, alpha/beta offsets +-6, written by the library's seeded
writer (include/h264r_writer.h; seeds 1000 + stream) and parsed by its front
end before the timed region.  Stream 0 is a case of
tests/golden/writer_streams.json, so its pictures are compared with the
reference decoder's own output of the same stream.

One step reconstructs every picture of every stream (30 * S frames): the
pictures of all streams that do not reference each other go into one
batched launch sequence (inter -> intra wavefront -> bS -> deblocking
wavefront), batches in decoding order.

  value     records resident in HBM, batched path, CUDA events on the
            engine's batch stream
  e2e       host records through h264r_submit_batch (pinned staging + H2D)
            and every decoded frame copied back to pinned host memory
  plain_fps one picture per launch sequence with a host sync after each
  tuning    launch shapes and graph replay chosen by the engine's autotuner
            (h264r_autotune_batch_device) per batch geometry mix, before
            the warm-up; kernel times for the roofline come from a separate
            pass with per-kernel CUDA events (graph replay off in it)
  cpu_baseline  the CPU oracle (a restatement of the reference's
            reconstruction) on a bounded sample, one host core
  --impl reference  that CPU implementation with every host core

Prints one JSON line (rank 0).
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
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "1080p decoded fps (bit-exact): batched/served vs plain GPU path; p99 frame ms"
WORKLOAD = "1080p_high"
FRAME_BYTES = 1920 * 1088 * 3 // 2
SEED_BASE = 1000  # configuration index 1 * 1000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--streams", type=int, default=32)
    ap.add_argument("--pictures", type=int, default=30)
    ap.add_argument("--pipelines", type=int, default=3, help="concurrent batch pipelines over disjoint stream sets")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline (quick runs)")
    ap.add_argument("--skip-configs", action="store_true", help="omit the mixed-size and CIF runs")
    ap.add_argument("--tune", default="auto", choices=["auto", "off"],
                    help="auto: autotune launch shapes and graph replay per batch mix; off: default shapes, no graphs")
    ap.add_argument("--tune-from", default="",
                    help="JSON file with the 'tuning' object of an earlier bench line: use those choices, no autotuning")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="length of the Poisson arrival window of the serving run (0: skip it)")
    ap.add_argument("--sweep-seconds", type=float, default=4.0,
                    help="arrival window of each point of the serving saturation sweep (0: skip it)")
    return ap.parse_args()


def gen_streams(n, pictures, seed0, workloads=None, overrides=None):
    """Records of n seeded streams (generated in parallel; the generator is C).
    workloads: per-stream workload names (default: the 1080p High one)."""
    import h264_video_decoder_demo_gb300 as h
    h.lib()
    out = [None] * n
    slots = [0] * n
    errors = []

    def work(i):
        try:
            name, over = (workloads[i] if workloads else WORKLOAD), dict(overrides or {})
            if isinstance(name, tuple):  # (workload, per-stream overrides)
                name, extra = name
                over.update(extra)
            g = h.synth(name, seed=seed0 + i, num_pictures=pictures, **over)
            out[i] = list(g)
            slots[i] = g.dpb_slots
            g.close()
        except Exception as exc:  # surfaced below
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(n)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return out, slots


def gen_written(n, seed0, name="1080p_high", pictures=None):
    """Records of n seeded bitstreams: each stream is written by the library's
    bitstream writer (the named configuration, seed seed0 + i) and parsed by
    its front end, in parallel threads (both are C; ctypes releases the
    GIL).  Returns (pictures per stream in decoding order with their
    dependency groups, DPB slots per stream)."""
    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300.engine import parse_stream
    h.lib()
    out = [None] * n
    slots = [0] * n
    errors = []
    over = {} if pictures is None else {"num_pictures": pictures}

    def work(i):
        try:
            data = h.write_stream(name, seed=seed0 + i, **over)
            out[i], slots[i] = parse_stream(data)
        except Exception as exc:  # surfaced below
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(n)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return out, slots


def reference_pictures(name, seed, pictures):
    """The reference decoder's md5 of every picture of a written stream, in
    decoding order (planes after deblocking; the last picture, which it
    outputs without deblocking, from its output frames), when the stream is
    a case of tests/golden/writer_streams.json; else None."""
    from h264_video_decoder_demo_gb300.engine import STREAMS
    with open(os.path.join(ROOT, "tests", "golden", "writer_streams.json")) as f:
        cases = json.load(f)["cases"]
    want = dict(STREAMS[name], seed=seed, num_pictures=pictures)
    for c in cases.values():
        if c["writer"] == want:
            md5s = [p["post_md5"] for p in c["pictures"]]
            last = {f["poc"]: f["yuv_md5"] for f in c["frames"]}
            return md5s, last
    return None


def oracle_sample(pics, slots, seconds, check=None):
    """Time the CPU oracle on pictures in decoding order (one thread) until
    `seconds` of work; optionally compare each picture with check(i)."""
    from oracle_cpu import OracleDPB
    p0 = pics[0]
    dpb = OracleDPB(p0.width_mbs, p0.height_mbs, slots)
    n, t0, exact = 0, time.perf_counter(), True
    for i, p in enumerate(pics):
        rc, _ = dpb.reconstruct(p)
        if rc != 0:
            raise RuntimeError("oracle error %d" % rc)
        n += 1
        if check is not None:
            exact = exact and check(i, dpb.planes(p.dst_slot))
        if time.perf_counter() - t0 > seconds:
            break
    return n, time.perf_counter() - t0, exact


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(f) > 3 + k and f[3 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# DRAM bytes (read + write) per MB of each timed kernel, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) over 40 launches of 8 streams
# of the 1080p High mix, 6 pictures each; scaled to a launch by the MBs it
# processes.  The boundary strengths (k_bs) run on
# a side stream beside k_inter and k_intra, so the deblocking stage timed
# after k_intra is the deblocking kernel alone.
DRAM_BYTES_PER_MB = {"k_inter": 494, "k_intra": 418, "k_deblock_frame": 669}
# Warp instructions per MB of k_inter on a batch of nine B pictures of this
# mix (ncu smsp__inst_executed per launch / MBs of the launch), for the
# issue-rate line of the roofline: B MBs are the costliest of the step, so the
# line is an upper bound.  Measured before the weighting rewrite, which took
# 3.1 % off the instructions of a six-picture batch.
K_INTER_WARP_INST_PER_MB = 1876
# The same for k_bs (a 1080p P picture) and the frame deblocking kernel (a
# 1080p picture, its wavefront waits included), from their ncu summaries.
K_BS_WARP_INST_PER_MB = 407
K_DEBLOCK_WARP_INST_PER_MB = 784


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.impl == "engine" else "gloo")
    return world, rank, local, dist


def run_reference(args, rank):
    """The CPU implementation of the path (the oracle port) on every host core,
    on the engine arm's workload: its written streams (seeds 1000 + i), each
    step a bounded sample of one picture per host thread, thread i decoding
    stream i in decoding order (I, P and B pictures in the workload's mix)."""
    if rank != 0:
        return None
    S = args.streams
    threads = max(1, min(os.cpu_count() or 1, S))
    pics, slots = gen_written(S, SEED_BASE, pictures=args.pictures)
    from oracle_cpu import OracleDPB
    dpbs = [None] * S
    cursor = [0] * S

    def step():
        def work(s):
            k = cursor[s] % len(pics[s])
            if k == 0:
                dpbs[s] = OracleDPB(pics[s][0].width_mbs, pics[s][0].height_mbs, slots[s])
            rc, _ = dpbs[s].reconstruct(pics[s][k])
            if rc != 0:
                raise RuntimeError("oracle error %d" % rc)
            cursor[s] += 1
        th = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
        for t in th:
            t.start()
        for t in th:
            t.join()

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    fps = threads * args.steps / dt
    sample = ("%d pictures per step, one per host thread: %d of the %d streams x %d pictures of %s, each "
              "in decoding order" % (threads, threads, S, args.pictures, WORKLOAD))
    return {
        "impl": "reference", "metric": METRIC, "value": round(fps, 3), "unit": "frames/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded 1080p High CAVLC bitstreams written by the library's writer, parsed by its "
                "front end; CPU restatement of the reference's reconstruction)",
        "config": {"workload": WORKLOAD, "streams_per_gpu": S, "pictures_per_stream": args.pictures,
                   "frames_per_step": S * args.pictures, "coded_size": "1920x1088", "gop": "15, IBBP", "refs": 4,
                   "weighted_prediction": "explicit", "parallelism": "%d host threads" % threads},
        "cpu_baseline": {"value": round(fps, 3), "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(fps, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_mixed(args, device, seed=4000):
    """Batched configuration: 32 independent streams, 12 CIF, 12 720p and 8
    1080p, 60 pictures each, I/P anchors with B pictures between them (the
    generator puts two B between anchors), the CIF configuration's value
    distributions (MVs +-64 quarter samples, QP 20..36, 10% intra),
    records resident in HBM; every step reconstructs all 1920 pictures, one
    fused launch per dependency group of each of three stream sets.  Reports
    frames/s and MB/s."""
    sizes = [(22, 18)] * 12 + [(80, 45)] * 12 + [(120, 68)] * 8
    kinds = [("cif_ippp", dict(width_mbs=w, height_mbs=hh)) for w, hh in sizes]
    out = run_batched(device, kinds, 60, seed, dict(gop_kind=1, gop_length=15), pipelines=3)
    out["config"] = ("32 streams (12 CIF, 12 720p, 8 1080p) x 60 pictures, IBBP, CIF-configuration distributions, "
                     "one launch per dependency group of each of 3 pipelines over disjoint stream sets (sizes "
                     "interleaved), records in HBM")
    return out


def run_interlaced(args, device, seed=3000):
    """Interlaced configuration: 1920x1088, 20 frames, half of them coded
    as a top and a bottom field picture (PAFF) and half as MBAFF frames (half
    the MB pairs field pairs, field references of either parity), GOP 12
    with B pictures, MVs +-128 quarter samples; 8 streams batched, records in
    HBM.  Frames/s counts a field pair as one frame."""
    out = run_batched(device, ["1080i_mbaff"] * 8, 20, seed, dict(paff_percent=50), pipelines=2)
    out["config"] = ("8 streams of 1080i x 20 frames: 50% PAFF field pairs, 50% MBAFF frames (50% field MB pairs), "
                     "one launch per dependency group of each of 2 pipelines over disjoint stream sets, records in HBM")
    return out


def run_batched(device, kinds, pictures, seed, overrides, pipelines=1):
    """Frames/s of streams of the given workloads, batched per dependency
    group across the streams of each of `pipelines` disjoint stream sets (the
    batches of one set run beside the others'), records resident in HBM (3
    timed steps)."""
    import numpy as np
    import torch

    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300 import records as R

    pics, slots = gen_streams(len(kinds), pictures, seed, workloads=kinds, overrides=overrides)
    dev = torch.device("cuda", device)
    ctx = h.Context(device, max_batch=256)
    streams = [h.Stream(ctx, p[0].width_mbs, p[0].height_mbs, sl) for p, sl in zip(pics, slots)]
    keep, cp = [], []
    for ps in pics:
        row = []
        for p in ps:
            c = p.to_c()
            for name in R.Picture._ARRAYS:
                a = np.ascontiguousarray(getattr(p, name)).view(np.uint8).reshape(-1)
                t = torch.from_numpy(a.copy()).to(dev) if a.size else torch.empty(1, dtype=torch.uint8, device=dev)
                keep.append(t)
                setattr(c, name, t.data_ptr())
            row.append(c)
        cp.append(row)
    ngroups = max(p.group for ps in pics for p in ps) + 1
    sets = [list(range(j, len(pics), pipelines)) for j in range(max(1, min(pipelines, len(pics))))]
    batches = []
    for g in range(ngroups):
        for idxs in sets:
            ss, cc = [], []
            for i in idxs:
                for k, p in enumerate(pics[i]):
                    if p.group == g:
                        ss.append(streams[i])
                        cc.append(cp[i][k])
            if ss:
                batches.append((ss, cc))
    cs = torch.cuda.ExternalStream(streams[0].cuda_stream(), device=dev)

    def step():
        for ss, cc in batches:
            rc = ctx.submit_batch_device(ss, cc)
            if rc != 0:
                raise RuntimeError("mixed batch: %d %s" % (rc, ctx.last_error()))

    for _ in range(2):
        step()
    ctx.sync()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nsteps = 3
    torch.cuda.synchronize()
    t0.record(cs)
    for _ in range(nsteps):
        step()
    for st in streams:  # every stream's work, seen from the first stream
        ev = torch.cuda.Event()
        ev.record(torch.cuda.ExternalStream(st.cuda_stream(), device=dev))
        cs.wait_event(ev)
    t1.record(cs)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / nsteps
    # a field picture (PAFF) is half a frame
    frames = sum(1.0 if p.structure == 0 else 0.5 for ps in pics for p in ps)
    mbs = sum(len(p.mbs) for ps in pics for p in ps)
    for st in streams:
        st.close()
    ctx.close()
    return {"fps": round(frames / (ms / 1000.0), 1), "mb_per_s": round(mbs / (ms / 1000.0), 1),
            "ms_per_step": round(ms, 3), "batches_per_step": len(batches)}


def run_plain_cif(device):
    """CIF 352x288, 8 pictures IPPP, Baseline CAVLC (the writer's cif_ippp
    stream, seed 1, whose output the reference's fixture pins), one picture
    per launch sequence with a host sync after each."""
    import h264_video_decoder_demo_gb300 as h
    pics, slots = gen_written(1, 1, name="cif_ippp")
    ctx = h.Context(device)
    s = h.Stream(ctx, 22, 18, slots[0])
    for p in pics[0]:
        s.submit(p)
        s.sync()
    t0 = time.perf_counter()
    n = 0
    for _ in range(20):
        for p in pics[0]:
            s.submit(p)
            s.sync()
            n += 1
    dt = time.perf_counter() - t0
    s.close()
    ctx.close()
    return {"fps": round(n / dt, 1), "config": "CIF IPPP 8 pictures, host records, one picture per launch, host sync"}


def run_bitstream(device, streams=12, repeats=24):
    """The drop-in path on real bitstreams: the two CAVLC cut streams of
    tests/golden (1080p, 4 and 6 pictures, each repeated `repeats` times as
    one stream) decoded by `streams` decoders at once (one host thread each:
    the front end parses, the engine reconstructs on the GPU, every output
    picture is copied back to pinned host memory and handed to the
    callback).  Also the front end alone on one core.  Frames/s."""
    import ctypes
    import threading

    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300 import records as R
    from h264_video_decoder_demo_gb300.engine import lib

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden")
    sources = []
    for name in ("gop121_cavlc_4pics", "heavyhand_cavlc_b4_6pics"):
        with open(os.path.join(here, name + ".h264"), "rb") as f:
            sources.append(f.read() * repeats)
    # the front end alone, one core
    data = sources[1]
    p = h.Parser()
    buf = (ctypes.c_uint8 * len(data)).from_buffer_copy(data)
    out = R.CParsed()
    t0 = time.perf_counter()
    lib().h264r_parser_feed(p.h, buf, len(data))
    lib().h264r_parser_end(p.h)
    n_parse = 0
    while lib().h264r_parser_next(p.h, ctypes.byref(out)) == 1:
        n_parse += 1
    parse_fps = n_parse / (time.perf_counter() - t0)
    p.close()
    # decoders in parallel
    ctx = h.Context(device)
    counts = [0] * streams
    errors = []

    def work(i):
        def on_frame(f, code):
            if f is not None:
                counts[i] += 1
            return 0
        d = h.Decoder(ctx, on_frame, copy_planes=False)
        try:
            d.push(sources[i % 2])
            d.flush()
        except Exception as e:  # reported in the result line
            errors.append(str(e))
        d.close()

    work(0)  # warm-up: buffers, first launches
    counts[0] = 0
    threads = [threading.Thread(target=work, args=(i,)) for i in range(streams)]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    dt = time.perf_counter() - t0
    ctx.close()
    frames = sum(counts)
    return {"fps": round(frames / dt, 1), "frames": frames, "streams": streams, "wall_s": round(dt, 3),
            "front_end_fps_one_core": round(parse_fps, 1), "errors": errors[:2],
            "config": "1080p CAVLC bitstreams (the bundled gop121 and HeavyHand B_frames_4 streams cut after 4 and 6 "
                      "pictures, each repeated %d times), %d decoders on their own host threads and engine streams, "
                      "parse + GPU reconstruction + every frame to pinned host memory" % (repeats, streams)}


SERVE_RES = [("cif", 22, 18, 0.3), ("720p", 80, 45, 0.4), ("1080p", 120, 68, 0.3)]
# coding modes of the serving configuration: CAVLC IP (CIF-configuration
# tools), CABAC IBP (1080p-configuration tools), MBAFF CAVLC (frame/field MB
# pairs, half of them field pairs; 720p is coded 46 MB rows high so that it
# has whole MB pairs)
SERVE_MODES = ("cavlc_ip", "cabac_ibp", "mbaff_cavlc")


def serving_pools(seed=5000):
    """Records of one 120-picture pool stream per resolution and coding mode."""
    import h264_video_decoder_demo_gb300 as h
    pools = {}
    errors = []

    def gen(job):
        res, wmb, hmb, kind = job
        base = ("cif_ippp", "1080p_high", "1080i_mbaff")[kind]
        over = dict(width_mbs=wmb, height_mbs=hmb, num_pictures=120)
        if kind == 0:
            over.update(gop_kind=0, num_refs=1)
        if kind == 2:
            over.update(height_mbs=hmb + (hmb & 1))
        try:
            g = h.synth(base, seed=seed + len(res) * 10 + kind, **over)
            pools[(res, kind)] = (list(g), g.dpb_slots)
            g.close()
        except Exception as exc:  # surfaced below
            errors.append(exc)

    threads = [threading.Thread(target=gen, args=((res, wmb, hmb, kind),))
               for res, wmb, hmb, _ in SERVE_RES for kind in range(len(SERVE_MODES))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return pools


def run_serving(args, device, pools, rate=40.0, seconds=60.0, seed=5000):
    """Serving: Poisson arrivals of streams at `rate` streams/s for `seconds`,
    resolution drawn from {CIF, 720p, 1080p} with p = {0.3, 0.4, 0.3}, length
    uniform in [8, 120] pictures, coding mode drawn from {CAVLC IP, CABAC IBP,
    MBAFF CAVLC}, DPBs device-resident and admitted by a 40 GB DPB budget.
    Each request replays the records of the pool stream of its size and mode
    (its own DPB, the records shared read-only).  Pictures are pushed as each
    stream's window of 4 allows and every decoded picture is copied to pinned
    host memory.  Returns aggregate frames/s and the per-picture latency from
    push to planes ready on the host."""
    import random

    import torch

    import h264_video_decoder_demo_gb300 as h

    rng = random.Random(seed)
    # the request schedule
    reqs, t = [], 0.0
    while True:
        t += rng.expovariate(rate)
        if t > seconds:
            break
        u, acc = rng.random(), 0.0
        for res, wmb, hmb, p in SERVE_RES:
            acc += p
            if u <= acc:
                break
        reqs.append((t, res, rng.randint(0, len(SERVE_MODES) - 1), rng.randint(8, 120)))
    window = 4
    pushers = 12  # producer threads, standing in for a parser thread per stream
    free_bufs = {}
    buf_mu = threading.Lock()

    def take_buf(nbytes):
        with buf_mu:
            lst = free_bufs.setdefault(nbytes, [])
            if lst:
                return lst.pop()
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()

    # C arguments of every pool picture, built once (a parser emits them)
    cpool = {key: [p.to_c() for p in pics] for key, (pics, _) in pools.items()}
    for (res, kind), (pics, _) in pools.items():  # pinned output buffers, allocated before the clock starts
        nbytes = pics[0].plane_bytes
        if nbytes not in free_bufs:
            free_bufs[nbytes] = [torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy() for _ in range(256)]
    ctx = h.Context(device, dpb_budget_bytes=40 << 30, max_batch=128)
    srv = h.Server(ctx, queue_depth=window)
    total = sum(r[3] for r in reqs)
    # One producer thread per group of streams, as a parser thread per stream
    # would push: it pushes a stream's next picture while the stream holds
    # fewer than `window` unfinished ones.  The main thread admits arrivals and
    # polls finished pictures.
    lock = threading.Lock()
    queues = [[] for _ in range(pushers)]  # new streams per producer
    pending = {}  # stream id -> pushed, not yet polled
    inflight = {}
    state = {"done": 0, "stop": False, "error": None}
    wake = threading.Event()

    def producer(j):
        active = []
        while not state["stop"]:
            with lock:
                active += queues[j]
                queues[j] = []
            did = False
            for e in active:
                sid, pics, cps, n = e[0], e[1], e[2], e[3]
                while e[4] < n and pending[sid] < window:
                    k = e[4]
                    p = pics[k]
                    buf = take_buf(p.plane_bytes)
                    with lock:
                        pending[sid] += 1
                        inflight[(sid, k)] = buf
                    rc = srv.push_c(sid, cps[k], p.group, k, buf.ctypes.data)
                    if rc != 0:
                        state["error"] = "server push: %d" % rc
                        state["stop"] = True
                        return
                    e[4] = k + 1
                    did = True
                if e[4] == n and not e[5]:
                    srv.end(sid)
                    e[5] = True
            active = [e for e in active if not e[5]]
            if not did:
                wake.wait(0.0005)
                wake.clear()

    threads = [threading.Thread(target=producer, args=(j,), daemon=True) for j in range(pushers)]
    for t in threads:
        t.start()
    t0 = time.perf_counter()
    nxt = 0
    done = 0
    try:
        while done < total and not state["stop"]:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and reqs[nxt][0] <= now:
                _, res, kind, n = reqs[nxt]
                pics, slots = pools[(res, kind)]
                sid = srv.open(pics[0].width_mbs, pics[0].height_mbs, slots)
                with lock:
                    pending[sid] = 0
                    queues[sid % pushers].append([sid, pics, cpool[(res, kind)], n, 0, False])
                nxt += 1
            got = srv.poll(max_items=1024, wait_ms=1)
            if got:
                with lock:
                    for sid, tag, status, _ in got:
                        if status != 0:
                            raise RuntimeError("serving: picture failed (%d)" % status)
                        pending[sid] -= 1
                        buf = inflight.pop((sid, tag))
                        with buf_mu:
                            free_bufs[buf.nbytes].append(buf)
                done += len(got)
                wake.set()
    finally:
        state["stop"] = True
        for t in threads:
            t.join()
    if state["error"]:
        raise RuntimeError(state["error"])
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    ctx.close()
    mbs = 0
    for _, res, kind, n in reqs:
        pics, _ = pools[(res, kind)]
        mbs += n * pics[0].width_mbs * pics[0].height_mbs
    return {
        "fps": round(total / wall, 1), "fps_1080p_equivalent": round(mbs / 8160.0 / wall, 1),
        "arrival_streams_per_s": rate, "pictures": total, "streams": len(reqs), "wall_s": round(wall, 3),
        "p50_frame_ms": round(st["p50_ms"], 3), "p99_frame_ms": round(st["p99_ms"], 3),
        "max_frame_ms": round(st["max_ms"], 3), "batches": st["batches"],
        "pictures_per_batch": round(st["batch_pictures"] / max(1, st["batches"]), 2),
        "waiting_peak": st["waiting_peak"], "dpb_peak_gb": round(st["dpb_bytes_peak"] / 1e9, 3),
        "config": "Poisson %g streams/s for %.1f s, CIF/720p/1080p p=0.3/0.4/0.3, 8..120 pictures, modes CAVLC IP / "
                  "CABAC IBP / MBAFF CAVLC (records of the modes' tools), 40 GB DPB budget, window 4 pictures per "
                  "stream pushed by 12 producer threads, outputs to pinned host memory" % (rate, seconds),
    }


def run_serving_sweep(args, device, pools, plain_fps):
    """Serving at rising arrival rates (short windows): the highest served
    throughput whose push-to-ready p99 stays under 33 ms."""
    points = []
    for rate in (80.0, 160.0, 240.0, 280.0, 320.0, 480.0):
        r = run_serving(args, device, pools, rate=rate, seconds=args.sweep_seconds, seed=6000 + int(rate))
        points.append({k: r[k] for k in ("arrival_streams_per_s", "fps", "fps_1080p_equivalent", "p50_frame_ms",
                                         "p99_frame_ms", "pictures", "wall_s")})
    ok = [p for p in points if p["p99_frame_ms"] < 33.0]
    best = max(ok, key=lambda p: p["fps_1080p_equivalent"]) if ok else None
    out = {"points": points, "window_s": args.sweep_seconds,
           "best_under_33ms": best}
    if best and plain_fps:
        out["best_1080p_equivalent_over_plain"] = round(best["fps_1080p_equivalent"] / plain_fps, 2)
    return out


def run_engine(args, world, rank, local, dist):
    import ctypes

    import numpy as np
    import torch

    import h264_video_decoder_demo_gb300 as h
    from h264_video_decoder_demo_gb300 import records as R

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    S = args.streams
    streams_pics, slots = gen_written(S, SEED_BASE + 100 * rank, pictures=args.pictures)
    ngroups = max(p.group for ps in streams_pics for p in ps) + 1
    # the records are uploaded and complete before any step: the strengths of
    # a batch are derived as soon as it is submitted (H264R_CFG_DEVICE_RECORDS_READY)
    ctx = h.Context(local, max_batch=4 * S, records_ready=True)
    streams = [h.Stream(ctx, 120, 68, slots[i]) for i in range(S)]

    # ---- records resident in HBM
    keep = []
    cpics = []  # per stream, per picture: CPicture with device pointers
    algo = np.zeros(4, np.int64)  # bytes per step: inter, intra, deblock, records
    rec_bytes = 0
    for i in range(S):
        row = []
        for p in streams_pics[i]:
            algo += np.array(h.engine.picture_bytes(p), np.int64)
            c = p.to_c()
            parts = []
            for name in R.Picture._ARRAYS:
                a = np.ascontiguousarray(getattr(p, name)).view(np.uint8).reshape(-1)
                t = torch.from_numpy(a.copy()).to(dev) if a.size else torch.empty(1, dtype=torch.uint8, device=dev)
                keep.append(t)
                setattr(c, name, t.data_ptr())
                rec_bytes += a.size
            row.append(c)
        cpics.append(row)
    # two pipelines over disjoint stream sets: the batches of one overlap
    # the other's (each batch runs on its first member's CUDA stream)
    npipe = max(1, min(args.pipelines, S))
    sets = [list(range(j, S, npipe)) for j in range(npipe)]
    batches = []  # (pipeline, streams, device pictures, host pictures)
    for g in range(ngroups):
        for j, idxs in enumerate(sets):
            ss, cc, hp = [], [], []
            for i in idxs:
                for k, p in enumerate(streams_pics[i]):
                    if p.group == g:
                        ss.append(streams[i])
                        cc.append(cpics[i][k])
                        hp.append(p)
            batches.append((j, ss, cc, hp))
    frames_per_step = S * args.pictures
    pipes = [torch.cuda.ExternalStream(streams[idxs[0]].cuda_stream(), device=dev) for idxs in sets]
    cs = pipes[0]

    # ---- autotuner: one batch per geometry mix (here: per pictures per
    # batch, all 1080p), and the one-picture mix of the plain path; run
    # before the warm-up, which re-decodes every picture in order
    tuning = {}
    kp = next(k for k, p in enumerate(streams_pics[0]) if p.group > 0)
    if args.tune_from:
        with open(args.tune_from) as f:
            kept = json.load(f)
        kept = kept.get("tuning", kept)
        for j, ss, cc, hp in batches:
            key = "batch_%d_pictures" % len(ss)
            if key in kept and key not in tuning:
                t = kept[key]
                ctx.set_mix_tuning(cc, t["inter_mbs_per_cta"], t["deblock_pairs_per_cta"], bool(t["graphs"]))
                tuning[key] = dict(t, source=args.tune_from)
        if "plain_1_picture" in kept:
            t = kept["plain_1_picture"]
            ctx.set_mix_tuning([cpics[0][kp]], t["inter_mbs_per_cta"], t["deblock_pairs_per_cta"], bool(t["graphs"]))
            tuning["plain_1_picture"] = dict(t, source=args.tune_from)
    elif args.tune == "auto":
        for j, ss, cc, hp in batches:
            key = "batch_%d_pictures" % len(ss)
            if key not in tuning and hp[0].group > 0:
                best, ms = ctx.autotune_batch_device(ss, cc, reps=5)
                tuning[key] = dict(best, ms_per_batch=round(ms, 3))
        best, ms = ctx.autotune_batch_device([streams[0]], [cpics[0][kp]], reps=10)
        tuning["plain_1_picture"] = dict(best, ms_per_batch=round(ms, 3))

    def step(evs=None):
        for bi, (j, ss, cc, _) in enumerate(batches):
            if evs is not None:
                evs[bi][0].record(pipes[j])
            rc = ctx.submit_batch_device(ss, cc)
            if rc != 0:
                raise RuntimeError("submit_batch_device: %d %s" % (rc, ctx.last_error()))
            if evs is not None:
                evs[bi][1].record(pipes[j])

    for _ in range(args.warmup):
        step()
    ctx.sync()

    # ---- timed region
    launches0 = ctx.kernel_launches()
    replays0 = ctx.graph_counts()[0]
    batch_evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in batches]
                 for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(cs)
        for q in pipes[1:]:
            q.wait_event(start)
        for k in range(args.steps):
            step(batch_evs[k])
        for q in pipes[1:]:
            ev = torch.cuda.Event()
            ev.record(q)
            cs.wait_event(ev)
        end.record(cs)
        torch.cuda.synchronize()
    ctx.sync()
    if dist:
        dist.barrier()
    elapsed_ms = start.elapsed_time(end)
    launches = ctx.kernel_launches() - launches0
    graph_replays = ctx.graph_counts()[0] - replays0
    # kernel times: a separate pass of the same steps, one launch sequence in
    # flight at a time (the device is synchronised after every batch, so no
    # other pipeline's kernels overlap), k_bs in line, CUDA events around each
    # kernel on the stream it runs on (launched directly, same shapes)
    kt_steps = 2
    ctx.set_timing(True)
    for _ in range(kt_steps):
        for j, ss, cc, _ in batches:
            rc = ctx.submit_batch_device(ss, cc)
            if rc != 0:
                raise RuntimeError("submit_batch_device: %d %s" % (rc, ctx.last_error()))
            torch.cuda.synchronize()
    ctx.sync()
    ktimes, nlaunch = ctx.kernel_timing()
    ctx.set_timing(False)
    if dist:
        t = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    lat = sorted(b[0].elapsed_time(b[1]) for stepev in batch_evs for b in stepev)
    value = world * frames_per_step * args.steps / (elapsed_ms / 1000.0)

    # ---- roofline of every kernel; the dominant one is the line's figure.
    # Algorithmic bytes per step (h264r_picture_bytes): k_inter reads records
    # + reference samples and writes 384 B per inter MB; k_intra 384 B per
    # intra MB + records; k_bs reads the MB records (32 B) and motion and
    # writes its 256-byte strength table per MB; the filter reads and writes
    # 768 B per deblocked MB and reads its 32-byte record and 256 B of
    # strengths.
    names = ["k_inter", "k_intra", "k_bs", "k_deblock_frame"]
    mbs_step = frames_per_step * 120 * 68
    motion_step = sum(len(p.motion) for ps in streams_pics for p in ps)
    bs_bytes = mbs_step * (32 + 256) + motion_step
    flt_bytes = algo[2] + mbs_step * 256
    kbytes = [float(algo[0]), float(algo[1]), float(bs_bytes), float(flt_bytes)]
    peak, peak_kind = peak_hbm()
    per_kernel = {}
    for k, nm in enumerate(names):
        ms = ktimes[k] / kt_steps
        gbs = kbytes[k] / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
        per_kernel[nm] = {"ms_per_step": round(ms, 3), "bytes_per_step": int(kbytes[k]),
                          "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    dom = int(np.argmax(ktimes))
    achieved = per_kernel[names[dom]]["achieved_gbs"]
    mbs_per_launch = mbs_step / len(batches)
    traffic = int(DRAM_BYTES_PER_MB[names[dom]] * mbs_per_launch) if names[dom] in DRAM_BYTES_PER_MB else None
    inter_mb_per_s = mbs_step / (ktimes[0] / kt_steps / 1000.0) if ktimes[0] > 0 else 0.0
    issue_peak = 152 * 4 * 2.07e9  # warp instructions/s: 152 SMs x 4 schedulers x 2.07 GHz
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "traffic_note": "ncu DRAM bytes per MB of this kernel on the same mix, scaled to the MBs of one launch",
                "algorithmic_bytes_per_launch": int(kbytes[dom] / len(batches)),
                "per_kernel": per_kernel,
                "k_inter_issue": {"warp_inst_per_mb": K_INTER_WARP_INST_PER_MB, "mb_per_s": round(inter_mb_per_s, 1),
                                  "frac_of_issue_peak": round(K_INTER_WARP_INST_PER_MB * inter_mb_per_s / issue_peak, 4)},
                # the issue rate of the other two MB-parallel and wavefront kernels, on the same
                # footing: warp instructions per MB x MBs per second of their serialised time
                "issue": {nm: {"warp_inst_per_mb": ipm,
                               "frac_of_issue_peak": round(ipm * (mbs_step / (ktimes[k] / kt_steps / 1000.0)) / issue_peak, 4)
                               if ktimes[k] > 0 else None}
                          for nm, k, ipm in (("k_bs", 2, K_BS_WARP_INST_PER_MB),
                                             ("k_deblock_frame", 3, K_DEBLOCK_WARP_INST_PER_MB))},
                "kernel_timing": "%d steps after the timed region, one launch sequence in flight at a time, "
                                 "k_bs in line, CUDA events per kernel" % kt_steps}

    extra = {}
    if rank == 0:
        # ---- plain path: one picture per launch sequence, host sync after each
        s0 = h.Stream(ctx, 120, 68, slots[0])
        for c in cpics[0][:3]:
            s0.submit_device(c)
            s0.sync()
        t0 = time.perf_counter()
        nplain = 0
        for rep in range(2):
            for c in cpics[0]:
                s0.submit_device(c)
                s0.sync()
                nplain += 1
        plain_fps = nplain / (time.perf_counter() - t0)
        # ---- bit-exactness of stream 0 against the CPU oracle (also the CPU baseline sample)
        s0.close()
        s1 = h.Stream(ctx, 120, 68, slots[0])
        gpu_frames = []
        for p in streams_pics[0]:
            s1.submit(p)
            gpu_frames.append(s1.output(p.dst_slot).copy())
        s1.close()
        ref = reference_pictures("1080p_high", SEED_BASE, args.pictures) if rank == 0 else None
        ref_exact = None
        if ref is not None:
            import hashlib
            md5s, last = ref
            got = [hashlib.md5(f.tobytes()).hexdigest() for f in gpu_frames]
            ref_exact = {"pictures": len(got), "equal": got[:len(md5s)] == md5s and len(got) == len(md5s) + 1,
                         "source": "the reference decoder's own planes for stream 0 (tests/golden/writer_streams.json)"}
        if args.skip_cpu:
            cpu = None
            exact = None
        else:
            n, dt, exact = oracle_sample(streams_pics[0], slots[0], 20.0,
                                         check=lambda i, planes: bool(np.array_equal(gpu_frames[i], planes)))
            cpu = {"value": round(n / dt, 3), "unit": "frames/s", "cores": 1, "kind": "port",
                   "sample": "%d pictures of stream 0 (%s, seed %d) in decoding order" % (n, WORKLOAD, SEED_BASE)}
        # ---- end to end: host records, pinned staging + H2D, every frame back to pinned host memory
        pinned = [[torch.empty(FRAME_BYTES, dtype=torch.uint8, pin_memory=True).numpy() for _ in range(3)] for _ in range(S)]
        e2e_steps = 6
        h2d = int(sum(p.record_bytes for ps in streams_pics for p in ps))
        sidx = {id(st): i for i, st in enumerate(streams)}

        # the C arguments of every batch and frame copy are built once, as a C
        # caller keeps the descriptors its parser emitted; every step still
        # validates, packs and uploads the records and copies every frame back
        prepared = []
        for j, ss, _, pp in batches:
            outs = []
            seen = {}
            for st, p in zip(ss, pp):
                k = seen.get(id(st), 0)
                seen[id(st)] = k + 1
                ysz = st.width_mbs * st.height_mbs * 256
                base = pinned[sidx[id(st)]][k % 3].ctypes.data
                outs.append((st.h, p.dst_slot, base, base + ysz, base + ysz + ysz // 4))
            prepared.append((ctx.prepare_batch(ss, pp), outs))
        L = h.engine.lib()

        host_s = [0.0, 0.0]  # time inside the submit calls, inside the copy-out calls

        def e2e_step():
            for prep, outs in prepared:
                t = time.perf_counter()
                ctx.submit_prepared(prep)
                u = time.perf_counter()
                for sh, slot, y, cb, cr in outs:
                    rc = L.h264r_output_async(sh, slot, y, cb, cr)
                    if rc != 0:
                        raise RuntimeError("output_async: %d %s" % (rc, ctx.last_error()))
                host_s[0] += u - t
                host_s[1] += time.perf_counter() - u

        def drain():  # every frame copy of every stream is on the host
            for st in streams:
                st.sync()

        # steps follow each other as a decoder's GOPs do: the host packs the
        # next step's first batches while the GPU finishes the last ones
        e2e_step()  # untimed: sizes the pinned staging of the launch ring
        drain()
        torch.cuda.synchronize()
        ctx.sync()
        host_s[0] = host_s[1] = 0.0
        hs0 = ctx.host_stats()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        drain()
        ctx.sync()
        e2e_dt = time.perf_counter() - t0
        hs1 = ctx.host_stats()
        e2e = {"value": round(frames_per_step * e2e_steps / e2e_dt, 2), "unit": "frames/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": frames_per_step * FRAME_BYTES,
               "ms_per_step": round(1000.0 * e2e_dt / e2e_steps, 3),
               # wall time the calling thread spent inside the calls (waits for a
               # free launch slot included)
               "submit_ms_per_step": round(1000.0 * host_s[0] / e2e_steps, 3),
               "copy_out_calls_ms_per_step": round(1000.0 * host_s[1] / e2e_steps, 3),
               # inside the submit calls: waiting for a free launch slot, validating
               # and packing the records on the host threads, upload and launch
               "submit_split_ms_per_step": {k: round(1000.0 * (hs1[i] - hs0[i]) / e2e_steps, 3)
                                            for i, k in enumerate(("wait_slot", "validate_pack", "upload_launch"))},
               "pack_threads": int(hs1[3])}
        extra = {"plain_fps": round(plain_fps, 2), "cpu_baseline": cpu, "e2e": e2e, "bit_exact_sample": exact,
                 "bit_exact_vs_reference": ref_exact}
        if args.serve_seconds > 0:
            pools = serving_pools()
            extra["serving"] = run_serving(args, local, pools, rate=40.0, seconds=args.serve_seconds)
            if args.sweep_seconds > 0:
                extra["serving_sweep"] = run_serving_sweep(args, local, pools, plain_fps)
        if not args.skip_configs:
            extra["batched_mixed"] = run_mixed(args, local)
            extra["interlaced_mbaff"] = run_interlaced(args, local)
            extra["plain_cif"] = run_plain_cif(local)
            extra["bitstream_decode"] = run_bitstream(local)

    for s in streams:
        s.close()
    ctx.close()
    if rank != 0:
        return None
    mbs = 120 * 68
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(elapsed_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded 1080p High CAVLC bitstreams with the 1080p configuration's tools and "
                "distributions, written by the library's writer and parsed by its front end before the timed region)",
        "config": {"workload": WORKLOAD, "streams_per_gpu": S, "pictures_per_stream": args.pictures,
                   "batches_per_step": len(batches), "frames_per_step": frames_per_step,
                   "coded_size": "1920x1088", "gop": "15, IBBP", "refs": 4, "weighted_prediction": "explicit",
                   "l2": "inputs larger than L2 (%.0f MB of records + %.0f MB of DPB per GPU)" %
                         (rec_bytes / 1e6, sum(slots) * FRAME_BYTES / 1e6),
                   "pipelines": npipe,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "mb_per_s": round(value * mbs, 1),
        "p50_batch_ms": round(statistics.median(lat), 3), "p99_batch_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
        "batch_latency_note": "device time of the batched launch sequence that reconstructs the frame",
        "roofline": roofline,
        "gpu_launches": int(launches),
        "graph_replays": int(graph_replays),
        "tuning": tuning if tuning else "default shapes (4 MBs per k_inter block, 8 row pairs per deblocking block), no graphs",
        "clocks": clk.summary(),
    }
    out.update(extra)
    if isinstance(out.get("serving"), dict):
        out["p50_frame_ms"] = out["serving"]["p50_frame_ms"]
        out["p99_frame_ms"] = out["serving"]["p99_frame_ms"]
        out["frame_latency_note"] = ("serving run: per picture, from h264r_server_push to its planes ready in pinned "
                                     "host memory")
    if out.get("plain_fps"):
        out["batched_over_plain"] = round(value / world / out["plain_fps"], 2)
    return out


def main():
    args = parse()
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        res = run_reference(args, rank)
    else:
        res = run_engine(args, world, rank, local, dist)
    if res is not None and rank == 0:
        print(json.dumps(res), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
