#!/usr/bin/env python
"""Benchmark of the iw_process_image() pixel pipeline on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload NAME]

One step = one pass of the pixel pipeline over one image of the workload
(default "precision": 4096x4096 RGBA16 -> 1000x1000 Mitchell, 8-bit output,
8x8 ordered dither; see imageworsener_gb300/workloads.py).  Rank 0 prints one
JSON line.

gb300 arm (default):
  value     output Mpix/s of the default (FP32 + guard band) form, input
            already resident in device memory: CUDA events on the library's
            stream around K back-to-back passes after W warm-up passes
            (iwg_process_image_timed).  The 134 MB input exceeds the 126 MB L2.
  e2e       the same metric through the unmodified C ABI with host buffers:
            iw_create_context .. iw_set_input_image .. iw_process_image ..
            iw_get_output_image per step, host->device upload of the input and
            device->host read of the output inside the timed region.
  plain_fp64  the reference's FP64 arithmetic on the GPU, same workload.
  roofline  dominant kernel (vertical pass): compulsory bytes (the input
            image) / its mean duration, against MEASURED_PEAKS.json hbm_gbs.
  cpu_baseline  the CPU oracle (a C restatement of the reference, built with
            the reference's flags) on one full image, one thread.
  Every output is checked against the reference's golden digest.

reference arm (--impl reference): the reference's CPU code on all host cores
  (the reference build when present, else the oracle port), one context per
  thread, each step = every thread processing one full image of the same
  workload (the reference cannot split an image); same "config" object as
  the gb300 arm.

Multi-GPU: the pipeline does not shard within an image; N ranks run N
independent replicas (weak scaling), value = all ranks' output pixels / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# the library's device lanes each want a hardware queue; this must be set
# before the process creates its CUDA context (torch does so first here)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from imageworsener_gb300 import workloads as W  # noqa: E402
from imageworsener_gb300.iwapi import IWLib, Image, run_job, _convert_arg, _libc  # noqa: E402

METRIC = "output Mpix/s FP32+batched vs FP64 plain on 1 GB300, bit-exact output; p99 latency"
WORKLOADS = {
    "precision": lambda: W.precision(),
    "small": lambda: W.small(),
    "downscale": lambda: W.downscale(),
    "downscale_fs4": lambda: W.downscale(fs4=True),
}


class Stats(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_device", C.c_double), ("ms_part", C.c_double * 4),
                ("flagged", C.c_longlong), ("form", C.c_int), ("kernels", C.c_int), ("zero_copy", C.c_int),
                ("flagged_exact", C.c_longlong), ("vertical_tensor", C.c_int), ("graph", C.c_int),
                ("fused", C.c_int), ("ms_phase", C.c_double * 6)]


_T0 = time.perf_counter()

# DRAM bytes (read + write) per launch of the vertical pass from one ncu
# capture of this workload (profiles/ holds the capture summaries).
ROOFLINE_TRAFFIC = {"precision": 184.2e6}


def progress(msg: str) -> None:
    """One line per bench phase on stderr (the JSON line stays alone on stdout)."""
    sys.stderr.write(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}\n")
    sys.stderr.flush()


def reduce_max(dist, values):
    """Max over ranks of each value (replicas: the job ends with its slowest rank)."""
    if dist is None:
        return list(values)
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_value(world: int, out_px: int, ms: float) -> float:
    """Whole-job output Mpix/s: every rank processes one image per step; the
    step takes the slowest rank's time."""
    return world * out_px / 1e6 / (ms / 1000.0)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows: list[list[str]] = []
        self.proc = None
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_ctx(lib: IWLib, job, extra_calls=()):
    """A context holding a copy of the job's input (the library owns it)."""
    ctx = lib.iw_create_context(None)
    n = job.bpr * job.height
    buf = _libc.malloc(n)
    C.memmove(buf, job.pixels, n)
    img = Image()
    img.imgtype, img.bit_depth, img.sampletype = job.imgtype, job.bit_depth, job.sampletype
    img.width, img.height, img.pixels, img.bpr = job.width, job.height, buf, job.bpr
    lib.iw_set_input_image(ctx, C.byref(img))
    for call in list(job.calls) + list(extra_calls):
        getattr(lib, call[0])(ctx, *[_convert_arg(a) for a in call[1:]])
    return ctx


def output_digest(lib: IWLib, ctx) -> str:
    from imageworsener_gb300.iwapi import Result
    out = Image()
    lib.iw_get_output_image(ctx, C.byref(out))
    pix = C.string_at(out.pixels, out.bpr * out.height)
    p = lib.iw_get_output_palette(ctx)
    pal = None
    if p:
        pal = [(p.contents.entry[i].r, p.contents.entry[i].g, p.contents.entry[i].b, p.contents.entry[i].a)
               for i in range(p.contents.num_entries)]
    r = Result(True, None, out.imgtype, out.bit_depth, out.sampletype, out.width, out.height, out.bpr, pix, pal,
               tuple(out.colorkey) if out.has_colorkey_trns else None,
               tuple(out.bkgdlabel.c) if out.has_bkgdlabel else None,
               tuple(out.maxcolorcode) if out.reduced_maxcolors else None)
    return r.digest()


def device_timed(lib: IWLib, job, warmup: int, steps: int, form: str, vertical: str = "auto", extra=()):
    lib.dll.iwg_process_image_timed.restype = C.c_int
    lib.dll.iwg_process_image_timed.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    ctx = make_ctx(lib, job, [("iw_set_option", b"gpu:precision", form.encode()),
                              ("iw_set_option", b"gpu:vertical", vertical.encode())] + list(extra))
    try:
        ok = lib.dll.iwg_process_image_timed(ctx, warmup, steps)
        if not ok:
            mb = C.create_string_buffer(256)
            raise RuntimeError(lib.iw_get_errormsg(ctx, mb, 256).decode())
        st = Stats()
        lib.dll.iwg_get_stats(ctx, C.byref(st))
        return st, output_digest(lib, ctx)
    finally:
        lib.iw_destroy_context(ctx)


def e2e_timed(lib: IWLib, job, warmup: int, steps: int, extra_calls=()):
    """Per step, wall clock: the C-ABI call sequence a caller makes with its
    image already in a malloc'd host buffer -- iw_create_context,
    iw_set_input_image (ownership passes to the library), the settings,
    iw_process_image (upload or zero-copy read, device passes, output in host
    memory, post-pass) and iw_get_output_image.  Buffers are filled before the
    timed region; contexts are destroyed after it."""
    lib.dll.iwg_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    n = job.bpr * job.height
    times, dig, zc, phases = [], None, {}, []
    for s in range(warmup + steps):
        buf = _libc.malloc(n)
        C.memmove(buf, job.pixels, n)
        img = Image()
        img.imgtype, img.bit_depth, img.sampletype = job.imgtype, job.bit_depth, job.sampletype
        img.width, img.height, img.pixels, img.bpr = job.width, job.height, buf, job.bpr
        t0 = time.perf_counter()
        ctx = lib.iw_create_context(None)
        lib.iw_set_input_image(ctx, C.byref(img))
        for call in list(job.calls) + list(extra_calls):
            getattr(lib, call[0])(ctx, *[_convert_arg(a) for a in call[1:]])
        ok = lib.iw_process_image(ctx)
        out = Image()
        lib.iw_get_output_image(ctx, C.byref(out))
        t1 = time.perf_counter()
        if not ok:
            raise RuntimeError("iw_process_image failed")
        st = Stats()
        lib.dll.iwg_get_stats(ctx, C.byref(st))
        if s == warmup + steps - 1:
            dig = output_digest(lib, ctx)
            zc = {"zero_copy": st.zero_copy, "device_ms": st.ms_device,
                  "kernel_ms": {"vertical": st.ms_part[0], "horizontal": st.ms_part[1], "fixup": st.ms_part[2]},
                  "host_ms_total": st.ms_total}
        lib.iw_destroy_context(ctx)
        if s >= warmup:
            times.append(t1 - t0)
            phases.append(list(st.ms_phase))
    if phases:
        med = [statistics.median(p[k] for p in phases) for k in range(6)]
        zc["phase_ms_median"] = {"plan": med[0], "h2d": med[1], "device": med[2], "d2h": med[3], "post_pass": med[4],
                                 "device_part_wall": med[5]}
        zc["h2d_GBps"] = n / 1e6 / med[1] if med[1] > 0 else None
        k = max(range(len(times)), key=lambda q: times[q])
        names = ("plan", "h2d", "device", "d2h", "post_pass", "device_part_wall")
        zc["slowest_step"] = {"ms": 1000.0 * times[k], "phase_ms": dict(zip(names, phases[k]))}
    return times, dig, zc


def cpu_oracle_sample(job, seconds_hint="one full image, one thread"):
    oracle_so = os.path.join(ROOT, "oracle", "_build", "liboracle_iw.so")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    lib = IWLib(oracle_so)
    t0 = time.perf_counter()
    res = run_job(lib, job)
    dt = time.perf_counter() - t0
    return dt, res.digest(), seconds_hint


def golden_digest(name):
    try:
        with open(os.path.join(ROOT, "tests", "golden", "workloads.json")) as f:
            return json.load(f)[name]["output_digest"]
    except Exception:
        return None


def workload_config(name: str, job, world: int) -> dict:
    """The "config" object of both arms' JSON lines: the workload by its
    sizes.  The two arms print the same object, so the driver sees one
    configuration; how each arm spreads it over its hardware (replicas on
    GPUs, contexts on host threads) is reported beside it."""
    return {"workload": name, "input": f"{job.width}x{job.height} x{len(job.pixels) // (job.width * job.height)}B/px",
            "output_px": W.out_pixels(job), "parallelism": f"replicas x{world}",
            "l2": "input (134 MB) larger than L2; passes back to back" if name == "precision" else "per workload"}


def run_reference_arm(args, rank, world):
    """The reference's CPU implementation on the full workload: every step,
    each of the host's threads runs one whole image through its own context
    (the reference cannot split one image), so a step produces threads x the
    workload's output pixels.  Under torchrun only rank 0 runs."""
    if rank != 0:
        return 0
    job = WORKLOADS[args.workload]()
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libimagew_ref.so")
    if os.path.exists(ref_so):
        lib, kind = IWLib(ref_so), "reference"
    else:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
        lib, kind = IWLib(os.path.join(ROOT, "oracle", "_build", "liboracle_iw.so")), "port"
    threads = os.cpu_count() or 1
    out_px = W.out_pixels(job)
    gold = golden_digest(args.workload)
    times, digests = [], []
    for s in range(args.warmup + args.steps):
        res = [None] * threads

        def one(k):
            res[k] = run_job(lib, job)

        ths = [threading.Thread(target=one, args=(k,)) for k in range(threads)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
        if s == 0:
            digests = [r.digest() for r in res]
    ms = 1000.0 * statistics.mean(times)
    value = threads * out_px / 1e6 / (ms / 1000.0)
    sample = (f"{threads} host threads, each one full {job.width}x{job.height} image of the workload "
              f"({out_px} output px) through its own context, per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, job, world),
        "threads": threads,
        "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "bit_exact": {"reference": all(d == gold for d in digests), "golden": gold is not None},
    }
    print(json.dumps(line), flush=True)
    return 0


def batch_leg(lib: IWLib, n_images: int, pool_size: int, cpu_threads: int, cpu_images: int,
              modes=("stage", "pull", "copy", "zero")):
    """The batched configuration: n_images contexts (image content drawn from a
    pool of pool_size generated images, sizes log-uniform 64..2048, gray/RGB/RGBA,
    8/16-bit, five filters, each fitted to a 256x256 box) through one
    iwg_process_batch call, timed end to end (planning, transfers, post-pass)."""
    pool = W.batch(pool_size, seed=4)
    jobs = [pool[k % pool_size] for k in range(n_images)]
    out_px = sum(W.out_pixels(j) for j in jobs)
    in_bytes = sum(len(j.pixels) for j in jobs)
    f = lib.dll.iwg_process_batch
    f.restype = C.c_int
    f.argtypes = [C.POINTER(C.c_void_p), C.c_int]

    def run(js, mode):
        ctxs = [make_ctx(lib, j, [("iw_set_option", b"gpu:upload", mode.encode())]) for j in js]
        arr = (C.c_void_p * len(ctxs))(*ctxs)
        t0 = time.perf_counter()
        ok = f(arr, len(ctxs))
        dt = time.perf_counter() - t0
        st = Stats()
        lib.dll.iwg_get_stats(C.c_void_p(ctxs[0]), C.byref(st))
        return ctxs, ok, dt, st

    def free(ctxs):
        for c in ctxs:
            lib.iw_destroy_context(c)

    ctxs, _, _, _ = run(jobs[:64], modes[0])     # warm-up: device tables, kernel modules
    free(ctxs)
    per_mode = {}
    phases = (C.c_double * 14)()
    lib.dll.iwg_batch_phase_ms.restype = C.c_int
    lib.dll.iwg_batch_phase_ms.argtypes = [C.POINTER(C.c_double), C.c_int]
    host_phase = None
    for mode in modes:
        lib.dll.iwg_batch_phase_ms(phases, 14)
        before = list(phases)
        ctxs, ok_m, wall_m, st_m = run(jobs, mode)
        lib.dll.iwg_batch_phase_ms(phases, 14)
        if host_phase is None:   # the first (default) mode's breakdown
            names = ("plan", "fast_batches", "plain_batches", "post_pass", "prepare", "upload", "launch_passes",
                     "launch_fixup", "wait_download", "rest", "of_which_tables", "of_which_attributes",
                     "of_which_d2h_wait", "of_which_d2h_copy")
            host_phase = {k: round(a - b, 3) for k, a, b in zip(names, phases, before)}
        dig_m = [output_digest(lib, ctxs[k]) for k in range(min(pool_size, n_images))]
        free(ctxs)
        per_mode[mode] = {"wall_ms": 1000 * wall_m, "e2e_mpix_s": out_px / 1e6 / wall_m, "device_ms": st_m.ms_device}
        if mode == modes[0]:
            ok, wall, st, digests = ok_m, wall_m, st_m, dig_m
    # the same images one by one through iw_process_image, for the batching gain and identity
    t0 = time.perf_counter()
    lone = []
    for j in pool:
        c = make_ctx(lib, j)
        lib.iw_process_image(c)
        lone.append(output_digest(lib, c))
        lib.iw_destroy_context(c)
    lone_dt = time.perf_counter() - t0
    pool_px = sum(W.out_pixels(j) for j in pool)
    res = {"images": n_images, "pool": pool_size, "ok": ok, "output_px": out_px, "input_bytes": in_bytes,
           "e2e_mpix_s": out_px / 1e6 / wall, "wall_ms": 1000 * wall,
           "device_ms": st.ms_device, "device_mpix_s": out_px / 1e6 / (st.ms_device / 1000.0) if st.ms_device else None,
           "last_chunk_ms": {"vertical": st.ms_part[0], "horizontal": st.ms_part[1], "fixup": st.ms_part[2]},
           "last_chunk_flagged": st.flagged, "last_chunk_left_to_fp64": st.flagged_exact,
           "lone_mpix_s": pool_px / 1e6 / lone_dt,
           "identical_to_lone": digests == lone[:len(digests)], "transfer": modes[0], "by_transfer_mode": per_mode,
           "host_phase_ms": host_phase}
    if cpu_images > 0:
        import concurrent.futures as cf
        oracle = IWLib(os.path.join(ROOT, "oracle", "_build", "liboracle_iw.so"))
        sample = pool[:cpu_images]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=cpu_threads) as ex:
            outs = list(ex.map(lambda j: run_job(oracle, j).digest(), sample))
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sum(W.out_pixels(j) for j in sample) / 1e6 / dt, "unit": "Mpix/s",
                               "cores": cpu_threads, "kind": "port",
                               "sample": f"{cpu_images} images of the pool, one context per thread",
                               "matches_gpu": outs == lone[:cpu_images]}
    return res


def serving_leg(lib: IWLib, rate: float, seconds: float, thumbs, ups):
    """The serving configuration: Poisson arrivals at 'rate' requests/s for
    'seconds'; 70 % thumbnails (the batched config's images), 30 % 2-4x
    upscales (4:3 inputs 160x120..1024x768, Catmull-Rom), 10 % of all with
    Floyd-Steinberg error diffusion; an 8 GiB device budget per batch.
    Latency = submit -> completion as the server measures it."""
    import queue
    from imageworsener_gb300.iwapi import Completion, ServerStats, server_api, CT_ALL, DITHER_ERRDIFF
    d = server_api(lib)
    sched = W.serving_schedule(rate, seconds)
    ed = [("iw_set_dither_type", CT_ALL, DITHER_ERRDIFF, 0)]
    srv = d.iwg_server_create(8 << 30, 0, 0)
    ready = queue.Queue(maxsize=512)
    lat = {}
    phases = {}
    out_px = {}
    stop = threading.Event()

    def producer():
        for k, (t, kind, errdiff) in enumerate(sched):
            job = thumbs[k % len(thumbs)] if kind == "thumb" else ups[k % len(ups)]
            ctx = make_ctx(lib, job, ed if errdiff else [])
            ready.put((k, t, ctx, W.out_pixels(job)))

    ctxs = {}

    def poller():
        buf = (Completion * 256)()
        while not stop.is_set() or len(lat) < len(sched):
            n = d.iwg_server_poll(srv, buf, 256, 50)
            for i in range(n):
                k = buf[i].tag
                lat[k] = (buf[i].latency_ms, buf[i].ok)
                phases[k] = (buf[i].planned_ms, buf[i].started_ms, buf[i].ran_ms, buf[i].latency_ms)
                lib.iw_destroy_context(ctxs.pop(k))
            if stop.is_set() and len(lat) >= len(sched):
                break

    pt = threading.Thread(target=producer, daemon=True)
    pt.start()
    po = threading.Thread(target=poller, daemon=True)
    po.start()
    t0 = time.perf_counter()
    late = 0
    for _ in range(len(sched)):
        k, t, ctx, px = ready.get(timeout=120)
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        elif now - t > 0.005:
            late += 1
        ctxs[k] = ctx
        out_px[k] = px
        d.iwg_server_submit(srv, ctx, k)
    t_sub = time.perf_counter() - t0
    stop.set()
    po.join(timeout=max(60.0, 6 * seconds))
    wall = time.perf_counter() - t0
    drained = len(lat) == len(sched)
    info = ServerStats()
    d.iwg_server_info(srv, C.byref(info))
    if drained:
        d.iwg_server_destroy(srv)   # (left running otherwise: the backlog did not drain in time)
    snap = dict(lat)   # a snapshot: the poller may still be collecting if the backlog did not drain
    ls = sorted(v[0] for v in snap.values())
    pct = lambda q: ls[min(len(ls) - 1, int(q * len(ls)))] if ls else None
    done_px = sum(out_px[k] for k in snap)

    ph = dict(phases)

    def cls(sel):
        keys = [k for k in snap if sel(sched[k])]
        v = sorted(snap[k][0] for k in keys)
        med = lambda xs: sorted(xs)[len(xs) // 2] if xs else None
        # median time in each stage: planning (submit -> planned), waiting for
        # the device, on the device, post-pass
        stages = {"plan": med([ph[k][0] for k in keys if k in ph]),
                  "wait": med([ph[k][1] - ph[k][0] for k in keys if k in ph]),
                  "device": med([ph[k][2] - ph[k][1] for k in keys if k in ph]),
                  "post": med([ph[k][3] - ph[k][2] for k in keys if k in ph])}
        return {"n": len(v), "p50_ms": v[len(v) // 2] if v else None,
                "p99_ms": v[min(len(v) - 1, int(0.99 * len(v)))] if v else None, "stage_p50_ms": stages}
    def windows(span=10.0):
        """Latency by arrival window: a backlog that grows shows as a rising p99."""
        out = []
        nwin = int(seconds // span + (1 if seconds % span else 0))
        for w in range(nwin):
            keys = [k for k in snap if w * span <= sched[k][0] < (w + 1) * span]
            v = sorted(snap[k][0] for k in keys)
            ed = sorted(snap[k][0] for k in keys if sched[k][2] and sched[k][1] == "up")
            q = lambda xs, f: xs[min(len(xs) - 1, int(f * len(xs)))] if xs else None
            out.append({"from_s": w * span, "n": len(v), "p50_ms": q(v, 0.5), "p99_ms": q(v, 0.99),
                        "errdiff_up_p50_ms": q(ed, 0.5), "errdiff_up_p99_ms": q(ed, 0.99)})
        return out
    last_submit = max((t for t, _, _ in sched), default=0.0)
    done_at = [sched[k][0] + snap[k][0] / 1000.0 for k in snap]
    return {"rate_req_s": rate, "seconds": seconds, "requests": len(sched), "completed": len(snap),
            "windows_10s": windows(), "drain_after_last_arrival_s": (max(done_at) - last_submit) if done_at else None,
            "failed": sum(1 for v in snap.values() if not v[1]),
            "errdiff_requests": sum(1 for x in sched if x[2]), "upscale_requests": sum(1 for x in sched if x[1] == "up"),
            "p50_ms": pct(0.50), "p90_ms": pct(0.90), "p99_ms": pct(0.99), "max_ms": ls[-1] if ls else None,
            "throughput_mpix_s": done_px / 1e6 / wall, "wall_s": wall, "submit_s": t_sub,
            "late_submits": late, "device_budget_gib": 8, "drained": drained,
            "by_class": {"thumb": cls(lambda x: x[1] == "thumb" and not x[2]), "up": cls(lambda x: x[1] == "up" and not x[2]),
                         "errdiff_thumb": cls(lambda x: x[1] == "thumb" and x[2]),
                         "errdiff_up": cls(lambda x: x[1] == "up" and x[2])},
            "lanes": {"batches": info.batches, "batched_requests": info.batched_requests,
                      "device_ms": info.device_ms, "scan_lane_batches": info.slow_batches,
                      "scan_lane_requests": info.slow_requests, "scan_lane_device_ms": info.slow_device_ms,
                      "batch_wall_ms": info.batch_wall_ms, "rest_wall_ms": info.rest_wall_ms, "plan_ms": info.plan_ms,
                      "batch_phase_ms": dict(zip(("prepare", "upload", "launch_passes", "launch_fixup", "wait_download",
                                                  "rest", "of_which_tables", "of_which_attributes",
                                                  "of_which_d2h_wait", "of_which_d2h_copy"),
                                                 list(info.batch_phase_ms)))}}


def fp_error_leg(lib: IWLib, job, name: str) -> dict:
    """Max / RMS error of the fp32 form's linear-light values against the
    fp64 form's (the reference's arithmetic), per configuration: the float
    intermediate after the vertical pass and the value each output sample is
    quantised from, with the flagged fraction and the count of samples
    beyond the fp32 form's own bound (0 expected).  The batched entry pools
    16 images of the batched configuration that the fp32 form takes."""
    from imageworsener_gb300.iwapi import fp_error
    out = {name: fp_error(lib, job)}
    for other in ("small", "downscale"):
        if other != name:
            out[other] = fp_error(lib, WORKLOADS[other]())
    agg = {"images": 0, "interm_max": 0.0, "final_max": 0.0, "bound_violations": 0, "samples": 0,
           "final_sq": 0.0, "flagged_px": 0.0, "px": 0}
    for j in W.batch(16, seed=4):
        st = fp_error(lib, j)
        if st.get("form") != 1 or "interm_max" not in st:
            continue
        agg["images"] += 1
        for k in ("interm_max", "final_max"):
            agg[k] = max(agg[k], st[k])
        agg["bound_violations"] += st["bound_violations"]
        agg["final_sq"] += st["final_rms"] ** 2 * st["samples"]
        agg["samples"] += st["samples"]
        px = W.out_pixels(j)
        agg["flagged_px"] += st["flagged_fraction"] * px
        agg["px"] += px
    out["batched_sample"] = {"images": agg["images"], "interm_max": agg["interm_max"], "final_max": agg["final_max"],
                             "final_rms": (agg["final_sq"] / agg["samples"]) ** 0.5 if agg["samples"] else None,
                             "bound_violations": agg["bound_violations"],
                             "flagged_fraction": agg["flagged_px"] / agg["px"] if agg["px"] else None}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="precision", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-images", type=int, default=4096, help="batched leg: contexts per call (0: skip)")
    ap.add_argument("--batch-pool", type=int, default=256, help="batched leg: distinct generated images")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serving leg: length of the arrival stream (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="serving leg: requests per second")
    ap.add_argument("--no-large", action="store_true", help="skip the large-downscale leg")
    ap.add_argument("--fuse", action="store_true",
                    help="device-timed leg with the fused vertical+horizontal pass (option gpu:fuse=on)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()

    if args.impl == "reference":
        return run_reference_arm(args, rank, world)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from imageworsener_gb300 import load
    lib = load()
    job = WORKLOADS[args.workload]()
    out_px = W.out_pixels(job)
    in_bytes = job.bpr * job.height
    out_bytes = W.out_pixels(job) * 4
    gold = golden_digest(args.workload)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    with ClockSampler(local) as clk:
        barrier()
        progress("device-timed fp32")
        st, dig_fast = device_timed(lib, job, args.warmup, args.steps, "fp32",
                                    extra=[("iw_set_option", b"gpu:fuse", b"on")] if args.fuse else ())
        barrier()
        progress("device-timed fp64")
        st64, dig_plain = device_timed(lib, job, 1, max(2, min(args.steps, 5)), "fp64")
        barrier()
        progress("end to end")
        e2e_times, dig_e2e, e2e_zc = e2e_timed(lib, job, max(3, args.warmup), max(3, min(args.steps, 20)))
        e2e_modes = {}
        for mode in ("zero", "stage", "copy", "pull"):
            progress(f"end to end, transfer {mode}")
            tm, dg, info = e2e_timed(lib, job, 2, 5, [("iw_set_option", b"gpu:upload", mode.encode())])
            e2e_modes[mode] = {"ms_per_step": 1000.0 * statistics.mean(tm), "bit_exact": dg == gold,
                               "device_ms": info.get("device_ms"), "phase_ms_median": info.get("phase_ms_median"),
                               "h2d_GBps": info.get("h2d_GBps")}
        barrier()
        batched = None
        if args.batch_images > 0:
            progress("batched configuration")
            batched = batch_leg(lib, args.batch_images, min(args.batch_pool, args.batch_images),
                                os.cpu_count() or 1, 0 if args.no_cpu_baseline else 64)
        large = {}
        # the large downscale also with its vertical pass on the CUDA cores
        # (the default puts windows this wide on the tensor cores)
        legs = (("small", "small", "auto"), ("downscale", "downscale", "auto"),
                ("downscale_cuda_vertical", "downscale", "cuda"), ("downscale_fs4", "downscale_fs4", "auto"))
        for label, name, vertical in (() if args.no_large else legs):
            progress(f"other configuration: {label}")
            ljob = WORKLOADS[name]()
            lst, ldig = device_timed(lib, ljob, 1, 3, "fp32", vertical)
            large[label] = {"ms": lst.ms_device, "mpix_s": W.out_pixels(ljob) / 1e6 / (lst.ms_device / 1000.0),
                            "input_gb_s": len(ljob.pixels) / 1e9 / (lst.ms_device / 1000.0), "form": lst.form,
                            "vertical_tensor": lst.vertical_tensor, "flagged": lst.flagged,
                            "left_to_fp64": lst.flagged_exact, "kernel_ms": list(lst.ms_part)[:3],
                            "bit_exact": ldig == golden_digest(name)}
        progress("fp error of the fp32 form against fp64, per configuration")
        fp_err = fp_error_leg(lib, job, args.workload)
        serving = None
        if args.serve_seconds > 0:
            progress("serving configuration")
            serving = serving_leg(lib, args.serve_rate, args.serve_seconds, W.batch(128, seed=4),
                                  W.upscale_pool(64))
        barrier()

    ms, e2e_ms, ms64 = reduce_max(dist, [st.ms_device, 1000.0 * statistics.mean(e2e_times), st64.ms_device])
    if rank != 0:
        dist.destroy_process_group() if dist else None
        return 0

    value = replica_value(world, out_px, ms)
    peak, peak_src = peaks()
    parts = list(st.ms_part)
    names = ["vertical pass (k_vbulk / k_vstream_px)", "horizontal pass + guarded quantisation (k_hpass_fast)",
             "re-evaluation of flagged pixels, double-float then FP64 (k_fix_stage)"]
    slowest = max(range(3), key=lambda k: parts[k])
    # The roofline is reported for the vertical pass: it moves the compulsory
    # bytes (the input image) and is the HBM-bound kernel of the pipeline.
    # The re-evaluation has no compulsory traffic (FP64 / latency bound).
    dom = 0
    # compulsory bytes of each launch group: vertical reads the input image;
    # horizontal writes the output image; the fix-up has no compulsory traffic.
    comp = [in_bytes, out_bytes, 0]
    achieved = comp[dom] / (parts[dom] / 1000.0) / 1e9 if parts[dom] > 0 else None
    cpu = None
    if not args.no_cpu_baseline:
        dt, dig_cpu, sample = cpu_oracle_sample(job)
        cpu = {"value": out_px / 1e6 / dt, "unit": "Mpix/s", "cores": 1, "kind": "port", "sample": sample,
               "seconds": dt, "matches_reference": dig_cpu == gold}
    line = {
        "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 (fp64 guard)", "data": "synthetic",
        "config": workload_config(args.workload, job, world),
        "e2e": {"value": world * out_px / 1e6 / (e2e_ms / 1000.0), "unit": "Mpix/s", "h2d_bytes_per_step": in_bytes,
                "d2h_bytes_per_step": out_bytes, "ms_per_step": e2e_ms, "p50_ms": 1000 * statistics.median(e2e_times),
                "host_buffers": "pageable (caller-malloc'd, as the libimagew ownership model requires)",
                "transfer": "zero-copy (GPU reads/writes host memory over NVLink-C2C)" if e2e_zc.get("zero_copy") else
                            "default: a copy kernel pulls the caller's pageable input over NVLink-C2C into device "
                            "memory; the output comes back by cudaMemcpyAsync",
                "step_ms": [round(1000 * t, 3) for t in e2e_times],
                "last_call": e2e_zc, "by_transfer_mode": e2e_modes},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": ROOFLINE_TRAFFIC.get(args.workload), "algorithmic_bytes_per_launch": comp[dom],
                     "pipeline_GBps": (in_bytes + out_bytes) / (ms / 1000.0) / 1e9,
                     "pipeline_frac": (in_bytes + out_bytes) / (ms / 1000.0) / 1e9 / peak,
                     "slowest_kernel": names[slowest], "slowest_share": parts[slowest] / sum(parts) if sum(parts) else None},
        "kernel_ms": {"vertical": parts[0], "horizontal": parts[1], "fixup": parts[2]},
        "flagged_pixels": st.flagged, "flagged_fraction": st.flagged / out_px,
        "flagged_left_to_fp64": st.flagged_exact,
        "plain_fp64": {"value": world * out_px / 1e6 / (ms64 / 1000.0), "ms_per_step": ms64,
                       "kernel_ms": {"vertical": st64.ms_part[0], "horizontal": st64.ms_part[1]}},
        "speedup_vs_plain": ms64 / ms,
        "bit_exact": {"fp32": dig_fast == gold, "fp64": dig_plain == gold, "e2e": dig_e2e == gold,
                      "golden": gold is not None},
        "batched": batched,
        "serving": serving,
        "fp_error": fp_err,
        "other_configs": large,
        "gpu_launches": st.kernels * args.steps,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
