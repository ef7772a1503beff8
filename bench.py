#!/usr/bin/env python
"""Headline benchmark: f32 compress + decompress throughput on one GB300.

A step is one compress of the workload field (device-resident input) followed by one decompress of
the archive it produced.  `value` is input bytes (4 N) per second of step time over all ranks, with
--inflight (default 4) steps in flight at once, each on its own stream with its own workspace,
archive and output, so that one step's host tree step and small kernels overlap another's kernels;
`serial` is the same K steps one after another on one stream, and `compress_gbs` /
`decompress_gbs`, the stage table and the roofline come from that serial pass.  `e2e` is the same round trip through the
host C-ABI entry points (the reference's Compress / Decompress interface) with pinned host buffers,
host<->device copies inside the timed region.

Workload (default): 512^3 f32 Gaussian random field with a k^-11/3 power spectrum, exponentiated to
a log-normal density spanning ~4 decades (NYX-like), r2r eb 1e-4, dict 1024 (radius 512), block 8.
The field (537 MB) and its codes (268 MB) are larger than L2 (129 MB), so no L2 flush is needed.

--impl reference times the reference's CPU algorithm (the C restatement in oracle/, OpenMP over all
host cores, serial Huffman as in the reference) on the same workload field, a whole field per step.

Multi-GPU: the path does not shard across GPUs in this build ("replicas only"); under torchrun each
rank compresses its own field of the same size (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "f32 compress/decompress GB/s on 1 GB300 (frac of HBM), batched vs plain, eb 1e-4"
WORKLOADS = {
    # name: (numpy shape (z, y, x), generator, eb, mode, dict, bs)
    "nyx512": ((512, 512, 512), "grf", 1e-4, "r2r", 1024, 8),
    "nyx256": ((256, 256, 256), "grf", 1e-4, "r2r", 1024, 8),
    "nyx512s": ((192, 512, 512), "grf", 1e-4, "r2r", 1024, 8),
    "cesm": ((1, 1800, 3600), "bump", 1e-4, "abs", 1024, 8),
    "adversarial": ((256, 384, 384), "adv", 1e-6, "abs", 1024, 8),
}
WORKLOAD_DESC = {
    "nyx512": "512^3 f32 GRF k^-11/3 log-normal (NYX-like), r2r eb 1e-4, dict 1024, block 8",
    "nyx256": "256^3 f32 GRF k^-11/3 log-normal, r2r eb 1e-4, dict 1024, block 8",
    "nyx512s": "512x512x192 slab of the NYX-like field (ncu captures: > L2, ~1.5 GB on device)",
    "cesm": "1800x3600 f32 sum of 64 Gaussian bumps (CESM-like), abs eb 1e-4, dict 1024, block 8",
    "adversarial": "256x384x384 f32 GRF + 5% Cauchy spikes + 8 steps, abs eb 1e-6, dict 1024, block 8",
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="nyx512")
    ap.add_argument("--inflight", type=int, default=4,
                    help="round trips in flight in the timed pass, each on its own stream (1: one stream)")
    ap.add_argument("--e2e-steps", type=int, default=40)
    ap.add_argument("--e2e-ops", type=int, default=3, help="host operations in flight in the e2e pipeline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-plain mixed field set")
    ap.add_argument("--batch-fields", type=int, default=1000)
    ap.add_argument("--no-serving", action="store_true", help="skip the request-server stream")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the 1e-3, CESM-like and adversarial single-field configurations")
    ap.add_argument("--no-lossless", action="store_true", help="skip the device gzip / inflate timing")
    ap.add_argument("--serving-seconds", type=float, default=8.0)
    ap.add_argument("--serving-long-minutes", type=float, default=0.0,
                    help="also run the configured 2000 req/s stream for this many minutes (the full-length run)")
    ap.add_argument("--no-stage-profile", action="store_true",
                    help="no per-stage CUDA events in the timed loop (no roofline / stages)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_field_torch(name, device="cuda", seed=0):
    from vecsz_gb300 import fields
    shape, gen, *_ = WORKLOADS[name]
    nz, ny, nx = shape
    if gen == "grf":
        return fields.grf_3d_torch(nz, ny, nx, seed=seed, device=device)
    if gen == "adv":
        return fields.adversarial_3d_torch(nz, ny, nx, seed=seed, device=device)
    return fields.bump_field_2d_torch(ny, nx, seed=seed, device=device)


def ref_dims(name):
    shape = WORKLOADS[name][0]
    if shape[0] == 1:
        return (shape[2], shape[1])
    return (shape[2], shape[1], shape[0])


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
        except Exception:
            pass
    return 6800.0, "fallback 6.8 TB/s"


class ClockSampler:
    """nvidia-smi samples (200 ms) during the run; summarised over the timed window."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.samples = []
        self.proc = None
        self.gpu = gpu_index
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        win = [s for t, s in self.samples if t0 - 0.3 <= t <= t1 + 0.3] or [s for _, s in self.samples[-5:]]
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(s[1]) for s in win if num(s[1]) is not None]
        mx = [num(s[2]) for s in win if num(s[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in win:
            for name, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(win),
                "power_w_max": max([num(s[3]) or 0 for s in win])}


def stage_profile(V):
    import ctypes as C
    L = V.lib()
    ms = (C.c_double * 32)()
    cnt = (C.c_int * 32)()
    names = (C.c_char_p * 32)()
    n = L.vsz_profile_read(C.cast(ms, C.c_void_p), C.cast(cnt, C.c_void_p), C.cast(names, C.c_void_p), 32)
    return {names[i].decode(): (ms[i], cnt[i]) for i in range(n) if cnt[i] > 0}


def algorithmic_bytes(stage, n, res, desc):
    """Bytes a stage must move per launch: reads + writes of its inputs and outputs (n elements,
    nch = 512-code chunks of the decode index, nseg = 128-wide row segments of the gather)."""
    nseg = desc["nseg128"]
    nch = (n + 511) // 512
    nout = res.n_outlier
    payload = (res.payload_bits + 7) // 8
    table = {
        "eb_setup": 4 * n,                                         # min/max pass (r2r)
        "dualquant": 4 * n + 2 * n + nseg + 4 * nout,              # field in; codes, counts, outliers out
        "huff_count": 2 * n + 2 * nch + 2 * nch + 8 * nch,         # codes in; chunk bits; their scan
        "huff_pack": 2 * n + 8 * nch + payload + 24 * nch,         # codes, offsets in; bitstream, edges out
        "outlier_gather": nseg + 8 * nout,
        "huff_decode": payload + 10 * nch + 2 * n + 4 * nch,       # bitstream, index in; codes, zero counts out
        "lorenzo_decompress": 2 * n + 4 * nout + 8 * nch + 4 * n,  # codes, outliers, ranks in; field out
    }
    return table.get(stage)


def max_over_ranks(ms: float, world: int, device: str) -> float:
    """The slowest rank's time; every rank calls it (one rank: unchanged)."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(bytes_per_rank_step: int, world: int, steps: int, total_ms: float) -> float:
    """Input bytes of all ranks and steps per second of the slowest rank's time (weak scaling)."""
    return world * steps * bytes_per_rank_step / (total_ms * 1e-3) / 1e9


def run_ours(args):
    import torch
    import torch.distributed as dist

    import vecsz_gb300 as V
    from vecsz_gb300 import _lib as L

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    shape, gen, eb, mode, dct, bs = WORKLOADS[args.workload]
    dims = ref_dims(args.workload)
    n = int(np.prod(shape))
    x = make_field_torch(args.workload, seed=1000 + rank)
    torch.cuda.synchronize()
    codec = V.DeviceCodec(dims, eb=eb, mode=mode, dict_size=dct, block_size=bs)
    stream = torch.cuda.Stream()
    out = torch.empty_like(x)
    with torch.cuda.stream(stream):
        codec.compress(x, stream)
    stream.synchronize()
    archive = codec.archive_bytes()
    res = codec.result_host()
    codec.prepare_decompress(archive)

    def step():
        codec.compress(x, stream)
        codec.decompress(codec.archive, out, stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    # correctness of what we time: deterministic archive, bounded error
    assert codec.archive_bytes() == archive, "archive not deterministic"
    assert codec.decompress_status() == 0
    ebf = codec._desc.eb_final
    err = (out.double() - x.double()).abs()
    bound = ebf + 2.0 * torch.abs(x.double()) * 2.0 ** -23
    verified = bool((err <= bound).all())

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.6)
    L.lib().vsz_profile_reset()
    L.lib().vsz_profile_enable(0 if args.no_stage_profile else 1)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.lib().vsz_launch_count()
    t_wall0 = time.time()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        codec.compress(x, stream)
        ev[i][1].record(stream)
        codec.decompress(codec.archive, out, stream)
        ev[i][2].record(stream)
    stop.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    serial_launches = L.lib().vsz_launch_count() - launches0
    if world > 1:
        dist.barrier()
    L.lib().vsz_profile_enable(0)
    serial_ms = max_over_ranks(start.elapsed_time(stop), world, "cuda")
    # The headline pass: the same K round trips with `inflight` of them in flight at once, each on
    # its own stream with its own workspace, archive and output (the same input field), so one
    # round trip's host tree step and small kernels overlap another's kernels.  Every round trip
    # does all its work; the outputs are checked against the serial pass's.
    total_ms, launches = serial_ms, serial_launches
    pipe = None
    if args.inflight > 1:
        codecs, streams, outs = [codec], [stream], [out]
        for _ in range(args.inflight - 1):
            c2 = V.DeviceCodec(dims, eb=eb, mode=mode, dict_size=dct, block_size=bs)
            s2 = torch.cuda.Stream()
            with torch.cuda.stream(s2):
                c2.compress(x, s2)
            s2.synchronize()
            c2.prepare_decompress(c2.archive_bytes())
            codecs.append(c2)
            streams.append(s2)
            outs.append(torch.empty_like(x))

        def run_pipelined(count):
            for i in range(count):
                j = i % args.inflight
                codecs[j].compress(x, streams[j])
                codecs[j].decompress(codecs[j].archive, outs[j], streams[j])

        run_pipelined(args.warmup)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = L.lib().vsz_launch_count()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for s2 in streams[1:]:
            s2.wait_event(p0)
        run_pipelined(args.steps)
        for s2 in streams[1:]:
            e2 = torch.cuda.Event()
            e2.record(s2)
            stream.wait_event(e2)
        p1.record(stream)
        torch.cuda.synchronize()
        launches = L.lib().vsz_launch_count() - launches0
        if world > 1:
            dist.barrier()
        total_ms = max_over_ranks(p0.elapsed_time(p1), world, "cuda")
        same = all(bool(torch.equal(o.view(torch.int32), out.view(torch.int32))) for o in outs[1:])
        same = same and all(c2.decompress_status() == 0 for c2 in codecs)
        pipe = {"inflight": args.inflight, "outputs_identical": same}
        del codecs, streams, outs, c2, s2
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    t_wall1 = time.time()
    time.sleep(0.3)
    clocks.stop()
    comp_ms = [a.elapsed_time(b) for a, b, _ in ev]
    dec_ms = [b.elapsed_time(c) for _, b, c in ev]
    prof = stage_profile(V)
    peak, peak_src = measured_peaks()
    nx_ = (dims[0] + 127) // 128
    nrows = n // dims[0]
    desc = {"nseg128": nrows * nx_, "nseg256": nrows * ((dims[0] + 255) // 256)}
    dominant = max(prof.items(), key=lambda kv: kv[1][0])[0] if prof else None
    roof = None
    if dominant:
        ms, cnt = prof[dominant]
        per_launch_ms = ms / max(cnt, 1)
        alg = algorithmic_bytes(dominant, n, res, desc)
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            try:
                traffic = json.load(open(tpath)).get(args.workload, {}).get(dominant)
            except Exception:
                traffic = None
        if alg:
            ach = alg / (per_launch_ms * 1e-3) / 1e9
            roof = {"bound": "hbm", "kernel": dominant, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(ach / peak, 4), "traffic": traffic, "algorithmic_bytes": int(alg),
                    "ms_per_launch": round(per_launch_ms, 5), "peak_source": peak_src}
    stages = {k: {"ms_per_launch": round(v[0] / max(v[1], 1), 5), "launches": v[1],
                  "gbs": (round(algorithmic_bytes(k, n, res, desc) / (v[0] / max(v[1], 1) * 1e-3) / 1e9, 1)
                          if algorithmic_bytes(k, n, res, desc) else None),
                  "share": round(v[0] / max(sum(w[0] for w in prof.values()), 1e-9), 4)}
              for k, v in prof.items()}
    bytes_in = 4 * n
    value = whole_job_gbs(bytes_in, world, args.steps, total_ms)
    serial = {"value": round(whole_job_gbs(bytes_in, world, args.steps, serial_ms), 2),
              "ms_per_step": round(serial_ms / args.steps, 4), "gpu_launches": int(serial_launches),
              "what": "the same K round trips one after another on one stream (stage timing and the roofline "
                      "come from this pass)"}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_DESC[args.workload], "dims_xyz": list(dims), "eb": eb, "mode": mode,
                   "dict_size": dct, "block_size": bs, "path": "plain (one field per launch sequence)",
                   "l2": "inputs larger than L2 (field 4N bytes > 129 MB), no flush",
                   "parallelism": f"replicas x{world}", "round_trips_in_flight": args.inflight},
        "serial": serial, "pipelined": pipe,
        "compress_gbs": round(bytes_in / (statistics.median(comp_ms) * 1e-3) / 1e9, 2),
        "decompress_gbs": round(bytes_in / (statistics.median(dec_ms) * 1e-3) / 1e9, 2),
        "compression_ratio": round(bytes_in / res.data_size, 3),
        "archive_bytes": int(res.data_size), "index_trailer_bytes": int(res.trailer_size),
        "n_outlier": int(res.n_outlier), "verified_error_bound": verified,
        "roofline": roof, "stages": stages,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(t_wall0, t_wall1),
    }
    if not args.no_lossless:
        line["lossless"] = run_device_gzip(V, codec.archive, int(res.data_size), stream)
    if not args.no_e2e:
        line["e2e"] = run_e2e(V, x, dims, eb, mode, dct, bs, args.e2e_steps, bytes_in, world, want=out,
                              nops=args.e2e_ops)
    if not args.no_other_configs and args.workload == "nyx512":
        line["other_configs"] = run_other_configs(V, x, dims, stream, lossless=not args.no_lossless)
    if not args.no_batch:
        line["batched"] = run_batch(V, args.batch_fields, 1000 + rank, reps=3)
    if not args.no_serving:
        line["serving"] = run_serving_all(V, args.serving_seconds, 7000 + rank,
                                          long_minutes=args.serving_long_minutes)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(x, dims, eb, mode, dct, bs, gpu_archive=archive[: int(res.data_size)],
                          gpu_out=out.view(-1).cpu().numpy())
        par = cb.pop("parity")
        line["cpu_baseline"] = cb
        if par is not None:
            line["parity"] = bool(par["archive_identical"] and par["reconstruction_identical"])
            line["parity_detail"] = par
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_device_gzip(V, d_archive, nbytes, stream, reps=5, host_sample=16 << 20):
    """The -L gzip pass on the device (vsz_deflate) over a packed block already in device memory:
    GB/s of input by CUDA events (median of `reps` after 2 warm-ups), the frame's size, a check
    that host zlib inflates it to the block, and host zlib level 3 (the reference's -L gzip pass,
    one core) timed on the block's first `host_sample` bytes."""
    import ctypes as C
    import zlib

    import torch
    from vecsz_gb300 import _lib as L
    from vecsz_gb300.api import _ptr
    lib = L.lib()
    ws, cap = C.c_size_t(0), C.c_size_t(0)
    L.check(lib.vsz_deflate_bounds(nbytes, C.byref(ws), C.byref(cap)))
    d_ws = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    d_out = torch.empty(cap.value, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(8, dtype=torch.int64, device="cuda")

    def once():
        L.check(lib.vsz_deflate(_ptr(d_archive), nbytes, _ptr(d_ws), ws.value, _ptr(d_out), cap.value, _ptr(d_res),
                                C.c_void_p(stream.cuda_stream)), "deflate")

    for _ in range(2):
        once()
    ms = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        once()
        b.record(stream)
        stream.synchronize()
        ms.append(a.elapsed_time(b))
    r = d_res.cpu().numpy()
    frame = d_out[: int(r[0])].cpu().numpy().tobytes()
    block = d_archive[:nbytes].cpu().numpy().tobytes()
    ok = int(r[1]) == 0 and zlib.decompress(frame) == block
    # the device inflate of the same frame from its chunk sizes
    nch = int(r[2])
    sizes = torch.zeros(max(1, nch), dtype=torch.int32, device="cuda")
    L.check(lib.vsz_deflate_chunk_sizes(_ptr(d_ws), nbytes, _ptr(sizes), C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    offs = (2 + torch.cumsum(sizes[:nch].long(), 0) - sizes[:nch].long()) if nch else torch.zeros(1, dtype=torch.long,
                                                                                                    device="cuda")
    iws = C.c_size_t(0)
    L.check(lib.vsz_inflate_bounds(nch, C.byref(iws)))
    d_iws = torch.empty(iws.value, dtype=torch.uint8, device="cuda")
    d_back = torch.empty(max(1, nbytes), dtype=torch.uint8, device="cuda")
    d_st = torch.zeros(1, dtype=torch.int32, device="cuda")
    adler = int.from_bytes(frame[-4:], "big")

    def inflate_once():
        L.check(lib.vsz_inflate(_ptr(d_out), int(r[0]), _ptr(offs), _ptr(sizes), nch, adler, _ptr(d_back), nbytes,
                                _ptr(d_iws), iws.value, _ptr(d_st), C.c_void_p(stream.cuda_stream)), "inflate")

    for _ in range(2):
        inflate_once()
    ims = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        inflate_once()
        b.record(stream)
        stream.synchronize()
        ims.append(a.elapsed_time(b))
    inflate_ok = int(d_st.item()) == 0 and bool(torch.equal(d_back[:nbytes], d_archive[:nbytes]))
    t0 = time.perf_counter()
    zlib.decompress(frame)
    t_host_inflate = time.perf_counter() - t0
    # the reference's default lossless pass: zstd level 3 through the host library, whole block
    zstd = None
    out_p, out_n = C.c_void_p(0), C.c_size_t(0)
    blk = np.frombuffer(block, np.uint8)
    t0 = time.perf_counter()
    st = lib.vsz_lossless_compress(L.LOSSLESS_ZSTD, blk.ctypes.data_as(C.c_void_p), blk.size, C.byref(out_p),
                                   C.byref(out_n))
    t_zstd = time.perf_counter() - t0
    if st == 0:
        lib.vsz_free_host(out_p)
        zstd = {"ratio": round(out_n.value / max(blk.size, 1), 4), "gbs": round(blk.size / t_zstd / 1e9, 4),
                "cores": 1, "bytes": int(out_n.value), "api": "vsz_lossless_compress (libzstd, level 3)"}
    sample = block[:host_sample]
    t0 = time.perf_counter()
    z3 = zlib.compress(sample, 3)
    t_host = time.perf_counter() - t0
    return {"api": "vsz_deflate (device, zlib stream)", "input_bytes": nbytes,
            "gbs": round(nbytes / (statistics.median(ms) * 1e-3) / 1e9, 2), "ms": round(statistics.median(ms), 4),
            "frame_bytes": int(r[0]), "frame_ratio": round(int(r[0]) / max(nbytes, 1), 4),
            "chunks": {"stored": int(r[3]), "fixed": int(r[4]), "dynamic": int(r[5])}, "verified_inflate": ok,
            "inflate": {"api": "vsz_inflate (device, from the deflate index)",
                        "gbs": round(nbytes / (statistics.median(ims) * 1e-3) / 1e9, 2),
                        "ms": round(statistics.median(ims), 4), "verified": inflate_ok,
                        "host_zlib_gbs": round(nbytes / t_host_inflate / 1e9, 4)},
            "host_zstd3": zstd if zstd is not None else {"unavailable": "no libzstd on this host"},
            "host_zlib3": {"sample_bytes": len(sample), "ratio": round(len(z3) / max(len(sample), 1), 4),
                           "gbs": round(len(sample) / t_host / 1e9, 4), "cores": 1, "bytes": len(z3)}}


def run_other_configs(V, x512, dims512, stream, reps=5, lossless=True):
    """The reference's other single-field configurations, timed like the headline one (device
    buffers, CUDA events on the stream, median of `reps` runs after 2 warm-ups): the 512^3
    NYX-like field at r2r eb 1e-3, the 1800x3600 CESM-like field (abs 1e-4) and the adversarial
    256x384x384 field (abs 1e-6); each with its compression ratio and error-bound check."""
    import torch

    def one(x, dims, eb, mode):
        codec = V.DeviceCodec(dims, eb=eb, mode=mode, dict_size=1024, block_size=8)
        out = torch.empty_like(x)
        with torch.cuda.stream(stream):
            codec.compress(x, stream)
        stream.synchronize()
        codec.prepare_decompress(codec.archive_bytes())
        res = codec.result_host()
        for _ in range(2):
            codec.compress(x, stream)
            codec.decompress(codec.archive, out, stream)
        cm, dm = [], []
        for _ in range(reps):
            a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            a.record(stream)
            codec.compress(x, stream)
            b.record(stream)
            codec.decompress(codec.archive, out, stream)
            c.record(stream)
            stream.synchronize()
            cm.append(a.elapsed_time(b))
            dm.append(b.elapsed_time(c))
        ebf = codec._desc.eb_final
        err = (out.double() - x.double()).abs()
        bound = ebf + 2.0 * torch.abs(x.double()) * 2.0 ** -23
        nbytes = 4 * x.numel()
        gz = run_device_gzip(V, codec.archive, int(res.data_size), stream) if lossless else None
        return {"dims_xyz": list(dims), "eb": eb, "mode": mode, "lossless": gz,
                "compress_gbs": round(nbytes / (statistics.median(cm) * 1e-3) / 1e9, 1),
                "decompress_gbs": round(nbytes / (statistics.median(dm) * 1e-3) / 1e9, 1),
                "compression_ratio": round(nbytes / res.data_size, 3), "n_outlier": int(res.n_outlier),
                "max_code_len": int(res.max_code_len), "verified_error_bound": bool((err <= bound).all()),
                "max_err_over_eb": round(float(err.max().item()) / ebf, 6)}

    outd = {"nyx512_r2r_1e-3": one(x512, dims512, 1e-3, "r2r")}
    xc = make_field_torch("cesm", seed=1)
    outd["cesm_1800x3600_abs_1e-4"] = one(xc.reshape(-1), ref_dims("cesm"), 1e-4, "abs")
    del xc
    xa = make_field_torch("adversarial", seed=1)
    outd["adversarial_256x384x384_abs_1e-6"] = one(xa.reshape(-1), ref_dims("adversarial"), 1e-6, "abs")
    outd["note"] = ("abs 1e-6 on the adversarial field and 2D fields whose width is not a multiple of 8 "
                    "reproduce the reference's own overshoot and dropped tail columns; strict mode "
                    "(VSZ_FLAG_STRICT_EB) bounds them")
    return outd


def run_batch(V, n_fields, seed, reps, sample_every=25):
    """Mixed field set (1D/2D/3D at 20/40/40 %, 16K-16M elements, r2r eb log-uniform 1e-5..1e-2,
    dict 1024, block 8): the batched path (vsz_batch_compress replayed from a CUDA graph) against
    the plain path (one vsz_compress launch sequence per field, host tree step, one stream)."""
    import ctypes as C
    import torch
    from vecsz_gb300 import fields
    from vecsz_gb300 import _lib as L
    from vecsz_gb300.api import _ptr, make_params
    specs = fields.batch_field_specs(n_fields, seed=seed)
    xs = [fields.batch_field_torch(sp) for sp in specs]
    fdefs = [{"x": x, "dims": sp["dims"], "eb": sp["eb"], "mode": "r2r", "dict_size": 1024, "block_size": 8}
             for x, sp in zip(xs, specs)]
    total = sum(4 * x.numel() for x in xs)
    torch.cuda.synchronize()
    b = V.BatchCompressor(fdefs)
    stream = torch.cuda.Stream()
    lib = L.lib()
    # plain path: its own workspace (the largest field's) and result records, the batch's archives
    ps, ds, caps, wsmax = [], [], [], 0
    for f in fdefs:
        p = make_params(f["eb"], "r2r", 1024, 8)
        d = L.dims_arg(f["dims"])
        ws, cap = C.c_size_t(0), C.c_size_t(0)
        L.check(lib.vsz_compress_bounds(C.byref(p), len(f["dims"]), d, C.byref(ws), C.byref(cap)), "bounds")
        ps.append(p)
        ds.append(d)
        caps.append(cap.value)
        wsmax = max(wsmax, ws.value)
    pws = torch.empty(wsmax, dtype=torch.uint8, device="cuda")
    pres = torch.zeros(8 * n_fields, dtype=torch.int64, device="cuda")
    sptr = C.c_void_p(stream.cuda_stream)
    args = [(C.byref(ps[i]), len(f["dims"]), ds[i], _ptr(f["x"]), _ptr(pws), C.c_size_t(wsmax), _ptr(b.archives[i]),
             C.c_size_t(caps[i]), C.c_void_p(pres.data_ptr() + 64 * i), sptr) for i, f in enumerate(fdefs)]

    def plain_pass():
        for a in args:
            lib.vsz_compress(*a)

    plain_pass()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plain_pass()
    e1.record(stream)
    stream.synchronize()
    plain_ms = e0.elapsed_time(e1)
    # the same plain path with the device tree builder (no host step), so that the batched path's
    # gain is not only the host tree step removed
    prev = lib.vsz_set_tree_builder(L.TREE_DEVICE)
    plain_pass()
    stream.synchronize()
    e0.record(stream)
    plain_pass()
    e1.record(stream)
    stream.synchronize()
    plain_dev_ms = e0.elapsed_time(e1)
    lib.vsz_set_tree_builder(prev)
    sample = list(range(0, n_fields, sample_every))
    want = {i: b.archives[i][: int(pres[8 * i]) + int(pres[8 * i + 1])].cpu().numpy().tobytes() for i in sample}
    want_res = pres.view(-1, 8)[:, [0, 2, 4, 5]].cpu().clone()
    # batched path: task sizes autotuned, eager once, then captured and replayed
    tuned = b.autotune(iterations=1, stream=stream)
    b.compress(stream)
    stream.synchronize()
    e0.record(stream)
    b.compress(stream)
    e1.record(stream)
    stream.synchronize()
    eager_ms = e0.elapsed_time(e1)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        b.compress(stream)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        with torch.cuda.stream(stream):
            g.replay()
    e1.record(stream)
    stream.synchronize()
    graph_ms = e0.elapsed_time(e1) / reps
    got_res = b.results.view(-1, 8)[:, [0, 2, 4, 5]].cpu()
    ok = bool(torch.equal(got_res, want_res)) and int(got_res[:, 3].abs().sum()) == 0
    ok = ok and all(b.archive_bytes(i) == want[i] for i in sample)
    out_bytes = int(b.results.view(-1, 8)[:, 0].sum())
    dec = run_batch_decompress(V, b, fdefs, stream, reps, sample)
    b.close()
    del xs, fdefs, b
    torch.cuda.empty_cache()
    return {"fields": n_fields, "input_bytes": total, "archive_bytes": out_bytes,
            "batched_gbs": round(total / (graph_ms * 1e-3) / 1e9, 2),
            "batched_eager_gbs": round(total / (eager_ms * 1e-3) / 1e9, 2),
            "plain_gbs": round(total / (plain_ms * 1e-3) / 1e9, 2),
            "plain_device_tree_gbs": round(total / (plain_dev_ms * 1e-3) / 1e9, 2),
            "batched_vs_plain": round(plain_ms / graph_ms, 3),
            "batched_vs_plain_device_tree": round(plain_dev_ms / graph_ms, 3),
            "batched_ms": round(graph_ms, 3), "plain_ms": round(plain_ms, 3),
            "plain_device_tree_ms": round(plain_dev_ms, 3), "decompress": dec,
            "task_sizes": {"dq_warp_units": tuned[0], "enc_chunks": tuned[1], "chosen_by": "vsz_batch_autotune"},
            "verified": ok, "check": f"per-field results identical to the plain path for all fields, archives "
                                     f"byte-identical for every {sample_every}th field",
            "workload": f"{n_fields} mixed fields: 1D/2D/3D 20/40/40 %, 16K-16M elements log-uniform, random "
                        f"aspect ratios, k^-11/3 or smooth-bump fields, r2r eb log-uniform 1e-5..1e-2, dict 1024, "
                        f"block 8 (seed {seed})",
            "plain_path": "vsz_compress per field on one stream (11 kernel launches each, the tree by the host thread)",
            "batched_path": "vsz_batch_compress captured in a CUDA graph (one launch per stage / kernel class, "
                            "device tree build, one CTA per field)"}


def run_batch_decompress(V, b, fdefs, stream, reps, sample):
    """The same field set's archives decompressed: the batched path (vsz_dbatch_decompress replayed
    from a CUDA graph) against the plain one (one vsz_decompress launch sequence per field, one
    stream).  Every field's output of both paths is compared bit for bit, and the error bound is
    checked on every `sample`-th field against its input."""
    import ctypes as C
    import torch
    from vecsz_gb300 import _lib as L
    from vecsz_gb300.api import _ptr
    lib = L.lib()
    n_fields = len(fdefs)
    descs = []
    for i in range(n_fields):
        r = b.result(i)
        head = b.archives[i][: r.data_size + r.trailer_size].cpu().numpy().tobytes()
        descs.append(V.parse_archive(head))
    total = sum(4 * f["x"].numel() for f in fdefs)
    # plain path: one workspace (the largest field's), its own outputs
    opts = L.DecompressOpts(1024, 8, 1, 0.0)
    wsmax = 0
    for d in descs:
        ws = C.c_size_t(0)
        L.check(lib.vsz_decompress_bounds(C.byref(d), C.byref(opts), C.byref(ws)), "decompress_bounds")
        wsmax = max(wsmax, ws.value)
    pws = torch.empty(wsmax, dtype=torch.uint8, device="cuda")
    pouts = [torch.empty_like(f["x"]) for f in fdefs]
    pst = torch.zeros(n_fields, dtype=torch.int32, device="cuda")
    sptr = C.c_void_p(stream.cuda_stream)
    args = [(C.byref(descs[i]), C.byref(opts), _ptr(b.archives[i]), _ptr(pws), C.c_size_t(wsmax), _ptr(pouts[i]),
             C.c_void_p(pst.data_ptr() + 4 * i), sptr) for i in range(n_fields)]

    def plain_pass():
        for a in args:
            lib.vsz_decompress(*a)

    plain_pass()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plain_pass()
    e1.record(stream)
    stream.synchronize()
    plain_ms = e0.elapsed_time(e1)
    db = V.BatchDecompressor(b.archives, descs=descs)
    db.decompress(stream)
    stream.synchronize()
    e0.record(stream)
    db.decompress(stream)
    e1.record(stream)
    stream.synchronize()
    eager_ms = e0.elapsed_time(e1)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        db.decompress(stream)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        with torch.cuda.stream(stream):
            g.replay()
    e1.record(stream)
    stream.synchronize()
    graph_ms = e0.elapsed_time(e1) / reps
    ok = int(pst.abs().sum()) == 0 and all(v == 0 for v in db.statuses())
    ok = ok and all(bool(torch.equal(db.outputs[i].view(torch.int32), pouts[i].view(torch.int32)))
                    for i in range(n_fields))
    bound_ok = True
    for i in sample:
        dims = fdefs[i]["dims"]
        if len(dims) == 2 and dims[0] % 8:
            continue  # the reference drops a 2D field's last d0 % 8 columns (its own quirk, reproduced)
        x = fdefs[i]["x"].double()
        ebf = float(descs[i].eb_final)
        err = (db.outputs[i].double() - x).abs()
        bound_ok = bound_ok and bool((err <= ebf + 2.0 * x.abs() * 2.0 ** -23).all())
    db.close()
    del db, pouts, pws
    return {"batched_gbs": round(total / (graph_ms * 1e-3) / 1e9, 2),
            "batched_eager_gbs": round(total / (eager_ms * 1e-3) / 1e9, 2),
            "plain_gbs": round(total / (plain_ms * 1e-3) / 1e9, 2),
            "batched_vs_plain": round(plain_ms / graph_ms, 3),
            "batched_ms": round(graph_ms, 3), "plain_ms": round(plain_ms, 3),
            "verified": bool(ok), "verified_error_bound": bool(bound_ok),
            "check": "every field's output identical between the batched and plain paths; the error bound on "
                     "every sampled field but 2D ones whose width is not a multiple of 8 (the reference zeroes "
                     "their last columns)",
            "plain_path": "vsz_decompress per field on one stream",
            "batched_path": "vsz_dbatch_decompress captured in a CUDA graph (one launch per stage / kernel class)"}


def serving_pool(V, seed, pool=48):
    """Distinct fields (and their archives, for decompress requests) standing in for the stream:
    sizes log-uniform in bytes from 2D 256^2 to 3D 512^3, r2r eb from {1e-2, 1e-3, 1e-4, 1e-5}."""
    import torch
    from vecsz_gb300 import fields
    rng = np.random.default_rng(seed)
    lo, hi = 256 * 256 * 4, 512 ** 3 * 4
    items = []
    for i in range(pool):
        nbytes = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        n = max(65536, int(nbytes // 4))
        nd = 2 if n <= (1 << 22) else 3
        dims = fields._factor(n, nd, rng)
        eb = float(rng.choice([1e-2, 1e-3, 1e-4, 1e-5]))
        x = fields.grf_torch(tuple(reversed(dims)), seed=seed * 1000 + i).reshape(-1)
        codec = V.DeviceCodec(dims, eb=eb, mode="r2r", dict_size=1024, block_size=8)
        codec.compress(x)
        a = codec.archive_bytes()
        arc = torch.from_numpy(np.frombuffer(a + bytes(64), np.uint8).copy()).cuda()
        items.append({"x": x, "dims": dims, "eb": eb, "bytes": 4 * x.numel(), "arc": arc, "desc": V.parse_archive(a)})
        del codec
    torch.cuda.synchronize()
    return items


def run_serving(V, seconds, rate, seed, budget_gb=120, slots=8, pool=48, items=None):
    """Poisson stream of compress (70 %) / decompress (30 %) requests through the request server,
    over a pool of fields (serving_pool)."""
    import threading
    import torch
    from vecsz_gb300.api import DecompressOpts
    rng = np.random.default_rng(seed + rate)
    if items is None:
        items = serving_pool(V, seed, pool)
    pool = len(items)
    opts = DecompressOpts(1024, 8, 1, 0.0)
    srv = V.Server(budget_bytes=int(budget_gb * (1 << 30)), slots=slots)
    n_req = int(seconds * rate)
    gaps = rng.exponential(1.0 / rate, n_req)
    kinds = rng.random(n_req) < 0.7
    picks = rng.integers(0, pool, n_req)
    tickets = [None] * n_req
    done = []
    errors = []

    def waiter():
        for i in range(n_req):
            while tickets[i] is None:
                time.sleep(1e-4)
            t, nb = tickets[i]
            c = srv.wait(t, timeout_s=300.0)
            if c.status != 0:
                errors.append(c.status)
            done.append((c.t_submit, c.t_done, nb))
            srv.release(t)

    wt = threading.Thread(target=waiter)
    wt.start()
    t0 = time.perf_counter()
    at = t0
    for i in range(n_req):
        at += gaps[i]
        while True:
            dt = at - time.perf_counter()
            if dt <= 0:
                break
            if dt > 2e-4:
                time.sleep(dt - 1.5e-4)
        it = items[picks[i]]
        if kinds[i]:
            t = srv.submit_compress(it["x"], it["dims"], it["eb"], "r2r", 1024, 8)
        else:
            t = srv.submit_decompress(it["arc"], it["desc"], opts)
        tickets[i] = (t, it["bytes"])
    t_sub = time.perf_counter() - t0
    wt.join()
    srv.close()
    lat = np.array([d - s for s, d, _ in done]) * 1e3
    t_first = min(s for s, _, _ in done)
    t_last = max(d for _, d, _ in done)
    total = sum(nb for _, _, nb in done)
    offered = sum(items[p]["bytes"] for p in picks) / max(t_sub, 1e-9)
    minutes = []
    if seconds >= 120:  # a long run: latency and throughput per minute of submissions (drift, leaks)
        sub = np.array([s for s, _, _ in done])
        nbs = np.array([nb for _, _, nb in done], dtype=np.float64)
        for m in range(int(seconds // 60)):
            sel = (sub >= t_first + 60 * m) & (sub < t_first + 60 * (m + 1))
            if sel.any():
                minutes.append({"minute": m, "requests": int(sel.sum()),
                                "p50_ms": round(float(np.percentile(lat[sel], 50)), 3),
                                "p99_ms": round(float(np.percentile(lat[sel], 99)), 3),
                                "max_ms": round(float(lat[sel].max()), 3),
                                "gbs": round(float(nbs[sel].sum()) / 60.0 / 1e9, 2)})
    extra = {"per_minute": minutes} if minutes else {}
    return {**extra, "requests": n_req, "compress": int(kinds.sum()), "decompress": int(n_req - kinds.sum()),
            "rate_req_s": rate, "arrival_seconds": round(t_sub, 3), "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3), "max_ms": round(float(lat.max()), 3),
            "sustained_gbs": round(total / (t_last - t_first) / 1e9, 2), "offered_gbs": round(offered / 1e9, 2),
            "errors": len(errors), "budget_gb": budget_gb, "slots": slots,
            "workload": f"Poisson {rate} req/s for {seconds} s, 70/30 compress/decompress, sizes log-uniform in "
                        f"bytes from 256^2 (2D) to 512^3 (3D) over a pool of {pool} fields, r2r eb in "
                        f"{{1e-2, 1e-3, 1e-4, 1e-5}}, dict 1024, block 8",
            "latency": "submit to completion (host clock), including queueing for slots and memory"}


def run_serving_all(V, seconds, seed, sweep_seconds=3.0, rates=(2000, 8000, 32000), long_minutes=0.0):
    """The configured stream (2000 req/s) and a rate sweep that drives the server past its capacity:
    where sustained GB/s falls below offered, the server is saturated; p50 / p99 are reported there."""
    import torch
    items = serving_pool(V, seed)
    main = run_serving(V, seconds, 2000, seed, items=items)
    sweep = [run_serving(V, sweep_seconds, r, seed, items=items) for r in rates]
    for s_ in sweep:
        s_.pop("workload", None)
        s_.pop("latency", None)
    sat = [s_ for s_ in sweep if s_["sustained_gbs"] < 0.9 * s_["offered_gbs"]]
    main["sweep"] = sweep
    main["capacity_gbs"] = max(s_["sustained_gbs"] for s_ in sweep)
    main["saturated_at_req_s"] = sat[0]["rate_req_s"] if sat else None
    if long_minutes > 0:
        main["long_run"] = run_serving(V, 60.0 * long_minutes, 2000, seed + 1, items=items)
    del items
    torch.cuda.empty_cache()
    return main


def run_e2e(V, x, dims, eb, mode, dct, bs, steps, bytes_in, world, want=None, nops=5):
    """Round trip through vsz_compress_host_into / vsz_decompress_host_into with pinned buffers;
    `want` (the device round trip's output) checks the host result bit for bit."""
    import ctypes as C

    import torch
    from vecsz_gb300 import _lib as L
    lib = L.lib()
    n = x.numel()
    h_in = torch.empty(n, dtype=torch.float32, pin_memory=True)
    h_in.copy_(x.view(-1).cpu())
    p = V.make_params(eb, mode, dct, bs)
    cap = C.c_size_t(0)
    L.check(lib.vsz_compress_host_bound(C.byref(p), len(dims), L.dims_arg(dims), C.byref(cap)))
    h_arch = torch.empty(cap.value, dtype=torch.uint8, pin_memory=True)
    h_out = torch.empty(n, dtype=torch.float32, pin_memory=True)
    opts = L.DecompressOpts(dct, bs, 1 if mode == "r2r" else 0, 0.0)
    ob, ds, ls, no, nn = (C.c_size_t(0) for _ in range(5))

    def one():
        L.check(lib.vsz_compress_host_into(C.byref(p), len(dims), L.dims_arg(dims), C.c_void_p(h_in.data_ptr()),
                                           C.c_void_p(h_arch.data_ptr()), cap.value, C.byref(ob), C.byref(ds),
                                           C.byref(ls), C.byref(no)), "compress_host")
        L.check(lib.vsz_decompress_host_into(C.c_void_p(h_arch.data_ptr()), ob.value, ds.value, ls.value,
                                             C.byref(opts), C.c_void_p(h_out.data_ptr()), n, C.byref(nn)),
                "decompress_host")

    one()
    one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    torch.cuda.synchronize()
    dt_sync = (time.perf_counter() - t0) / steps
    ok_sync = bool(torch.equal(h_out.view(-1), want.view(-1).cpu())) if want is not None else None

    # stream-ordered: three host ops in a software pipeline.  Step k+1's compress is enqueued
    # before step k's is waited for (its archive is parsed on the host), and step k's decompress
    # is then left in flight, so the input copy of one step runs while the kernels and the output
    # copy of the steps before it run, in both directions of the link at once
    ops = [V.api.HostOp() for _ in range(nops)]
    h_ins = [h_in] + [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(nops - 1)]
    for t in h_ins[1:]:
        t.copy_(h_in)
    h_archs = [h_arch] + [torch.empty(cap.value, dtype=torch.uint8, pin_memory=True) for _ in range(nops - 1)]
    h_outs = [h_out] + [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(nops - 1)]
    h_res = [torch.zeros(8, dtype=torch.int64, pin_memory=True) for _ in range(nops)]
    h_st = [torch.zeros(1, dtype=torch.int32, pin_memory=True) for _ in range(nops)]

    def start(k):
        i = k % nops
        ops[i].compress(p, dims, h_ins[i].data_ptr(), h_archs[i].data_ptr(), cap.value, h_res[i].data_ptr())

    def finish(k):
        i = k % nops
        ops[i].wait()  # only step k's compress is queued on this op at this point
        r = h_res[i].numpy()
        if int(r[5]) != 0:
            raise RuntimeError(f"host op compress status {int(r[5])}")
        ops[i].decompress(h_archs[i].data_ptr(), int(r[0] + r[1]), opts, h_outs[i].data_ptr(), n,
                          h_st[i].data_ptr())
        return int(r[0] + r[1])

    ahead = max(1, nops - 2)  # compresses enqueued ahead of the one waited for

    def run(count):
        for j in range(min(ahead, count)):
            start(j)
        for k in range(count):
            if k + ahead < count:
                start(k + ahead)
            last = finish(k)
        for op in ops:
            op.wait()
        return last

    run(nops)
    t0 = time.perf_counter()
    arch_bytes = run(steps)
    dt = (time.perf_counter() - t0) / steps
    ok = all(int(s.item()) == 0 for s in h_st)
    if want is not None:
        w = want.view(-1).cpu()
        ok = ok and all(bool(torch.equal(o.view(-1), w)) for o in h_outs)
    for op in ops:
        op.close()
    link = link_probe(h_ins[1 % nops], h_archs[1 % nops], h_outs[1 % nops], h_archs[2 % nops], arch_bytes, dt)
    return {"value": round(world * bytes_in / dt / 1e9, 2), "unit": "GB/s", "link": link,
            "h2d_bytes_per_step": int(4 * n + arch_bytes), "d2h_bytes_per_step": int(arch_bytes + 4 * n),
            "ms_per_step": round(dt * 1e3, 3), "steps": steps,
            "api": f"vsz_host_op_compress / vsz_host_op_decompress on pinned host buffers, {nops} ops in a "
                   "software pipeline (step k+1's compress and step k's decompress in flight together)", "ok": ok,
            "sync": {"value": round(world * bytes_in / dt_sync / 1e9, 2), "ms_per_step": round(dt_sync * 1e3, 3),
                     "api": "vsz_compress_host_into + vsz_decompress_host_into (one call at a time)", "ok": ok_sync}}


def link_probe(h_in, h_arch_in, h_out, h_arch_out, arch_bytes, step_s, reps=5):
    """The host link on this machine, with one step's traffic: host to device the input and an
    archive, device to host an archive and the output (plain stream copies between the pinned
    buffers the step uses).  `duplex_ms` moves both directions at once, the time below which no
    pipelined step can go; `e2e_frac` = that bound / the measured step."""
    import torch
    n_in = h_in.numel() * h_in.element_size()
    d_in = torch.empty(n_in, dtype=torch.uint8, device="cuda")
    d_ar = torch.empty(max(arch_bytes, 1), dtype=torch.uint8, device="cuda")
    d_out = torch.empty(n_in, dtype=torch.uint8, device="cuda")
    d_ar2 = torch.empty(max(arch_bytes, 1), dtype=torch.uint8, device="cuda")
    hi, ho = h_in.view(torch.uint8), h_out.view(torch.uint8)
    hai, hao = h_arch_in.view(torch.uint8)[:arch_bytes], h_arch_out.view(torch.uint8)[:arch_bytes]
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()

    def up():
        with torch.cuda.stream(s_up):
            d_in.copy_(hi, non_blocking=True)
            d_ar[:arch_bytes].copy_(hai, non_blocking=True)

    def down():
        with torch.cuda.stream(s_down):
            hao.copy_(d_ar2[:arch_bytes], non_blocking=True)
            ho.copy_(d_out, non_blocking=True)

    def timed(fns):
        ms = []
        for _ in range(reps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(s_up)
            s_down.wait_event(e0)
            for f in fns:
                f()
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record(s_down)
            s_up.wait_event(e1)
            e2 = torch.cuda.Event(enable_timing=True)
            e2.record(s_up)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e2))
        return float(np.median(ms))

    up_ms, down_ms, both_ms = timed([up]), timed([down]), timed([up, down])
    nb = n_in + arch_bytes
    del d_in, d_ar, d_out, d_ar2
    return {"h2d_gbs": round(nb / up_ms / 1e6, 1), "d2h_gbs": round(nb / down_ms / 1e6, 1),
            "duplex_ms": round(both_ms, 3), "duplex_gbs": round(2 * nb / both_ms / 1e6, 1),
            "e2e_frac": round(both_ms / (step_s * 1e3), 3),
            "what": "one step's copies (input + archive up, archive + output down) alone and both at once, "
                    "stream copies between the step's pinned buffers"}


def cpu_baseline(x, dims, eb, mode, dct, bs, max_bytes=None, gpu_archive=None, gpu_out=None):
    """The reference's algorithm on the host cores: C oracle, OpenMP dual-quant, serial Huffman.
    With the GPU's packed block and reconstruction of the same field, `parity` compares them with the
    oracle's byte for byte and bit for bit."""
    import oracle as O
    xh = x.view(-1).cpu().numpy()
    if max_bytes is not None and xh.nbytes > max_bytes:
        # bounded sample: leading z-slab of the same field
        plane = dims[0] * dims[1]
        nz = max(1, max_bytes // (4 * plane))
        xh = xh[: plane * nz]
        dims = (dims[0], dims[1], nz) if len(dims) == 3 else dims
    r2r = mode == "r2r"
    tc = np.zeros(4)
    td = np.zeros(3)
    t0 = time.perf_counter()
    archive, meta = O.compress(xh, dims, bs, dct, eb, r2r, timings=tc)
    t1 = time.perf_counter()
    recon = O.decompress(archive, bs, dct, O.value_range(xh) if r2r else 0.0, timings=td)
    t2 = time.perf_counter()
    nbytes = xh.nbytes
    parity = None
    if gpu_archive is not None and max_bytes is None:
        same_archive = gpu_archive == archive
        same_recon = gpu_out is not None and bool(np.array_equal(gpu_out.view(np.uint32), recon.view(np.uint32)))
        parity = {"archive_identical": same_archive, "reconstruction_identical": same_recon,
                  "what": "the GPU packed block of this field vs the oracle's, byte for byte; the GPU "
                          "reconstruction vs the oracle's, bit for bit"}
    return {"parity": parity, "value": round(nbytes / (t2 - t0) / 1e9, 4), "unit": "GB/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"one compress + decompress round trip of {nbytes / 1e6:.0f} MB of the same field "
                      f"(dims {list(dims)}) with the C oracle (OpenMP dual-quant, serial Huffman as the reference)",
            "compress_gbs": round(nbytes / (t1 - t0) / 1e9, 4), "decompress_gbs": round(nbytes / (t2 - t1) / 1e9, 4),
            "stage_s": {"value_range": round(tc[0], 4), "dualquant": round(tc[1], 4), "huffman_encode": round(tc[2], 4),
                        "outlier_gather": round(tc[3], 4), "huffman_decode": round(td[0], 4),
                        "outlier_scatter": round(td[1], 4), "reverse_dualquant": round(td[2], 4)},
            "why_port": "the reference itself is x86 AVX code (src/dualquant.hh:6) and does not build on this "
                        "aarch64 host; oracle/vsz_oracle.c restates it and is pinned to it"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle as O
    shape, gen, eb, mode, dct, bs = WORKLOADS[args.workload]
    dims = ref_dims(args.workload)
    try:
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        x = make_field_torch(args.workload, device=dev, seed=1000)
    except Exception:
        from vecsz_gb300 import fields
        nz, ny, nx = shape
        x = None
        xh = fields.grf_3d(nz, ny, nx, seed=1000) if gen == "grf" else fields.bump_field_2d(ny, nx, seed=1000)
    xh = x.view(-1).cpu().numpy() if x is not None else xh.ravel()
    # each step is the whole workload field (the same config as our arm): about 3.3 s per step for
    # the 512^3 field on 16 host cores, so 20 + 5 steps take under two minutes
    xs, sdims = xh, dims
    r2r = mode == "r2r"
    vr = O.value_range(xs) if r2r else 0.0

    def step():
        a, _ = O.compress(xs, sdims, bs, dct, eb, r2r)
        O.decompress(a, bs, dct, vr)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = xs.nbytes / dt / 1e9
    sample = (f"each step: one compress + decompress round trip of the whole {xs.nbytes / 1e6:.0f} MB workload "
              f"field (dims {list(sdims)}, its own value range for r2r)")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD_DESC[args.workload], "dims_xyz": list(sdims), "eb": eb, "mode": mode,
                       "dict_size": dct, "block_size": bs, "path": "reference CPU algorithm"},
            "cpu_baseline": {"value": round(value, 4), "unit": "GB/s", "cores": O.num_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference = oracle/vsz_oracle.c, the pinned C restatement of vecSZ's AVX2+OpenMP path; the "
                    "reference's own AVX sources (src/dualquant.hh:6) do not build on the aarch64 host"}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.steps < 1:
        raise SystemExit("--steps must be >= 1")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
