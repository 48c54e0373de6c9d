"""Benchmark of the GB300 histogram sort (one JSON line on rank 0).

Workload (default): 1e9 records of [('key','u8'),('val','i8')] (16 B, 16 GB),
key uniform uint64 from a seeded generator, val = index -- the large plain
sort on one GB300.  A step is one sort of the whole array, input resident in
HBM, output to a second buffer (the inputs are far larger than L2, so no L2
flush is needed between steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--method learned|plain|lsd] [--n N] [--dist uniform|sorted1pct|zipf]

`value` is the device-resident throughput (records/s); `e2e` is the same
metric through the public host API (mpsort.sort on pinned host arrays, host
to device and back inside the timed region).  The reference arm times the
CPU implementation of the same path on this machine's cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "mp-sort_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)

METRIC = "sorted records/s (1e9 x 16 B u64-keyed records)"
UNIT = "records/s"
DTYPE_DESC = [('key', 'u8'), ('val', 'i8')]

# Algorithmic bytes per record of the pipeline's kernels: each must read
# (and, for the last three, also write) every record once.  The pipeline as a
# whole needs two passes, each a read and a write of every record.
E = 16
STAGE_KERNELS = {  # stage_ms key -> (kernel, algorithmic bytes per record, ncu summary)
    "count": ("k_l1_count", E, "l1_count_16B.md"),
    "scatter": ("k_l1_scatter", 2 * E, "l1_scatter_16B.md"),
    "split": ("k_split", 2 * E, "split_16B.md"),
    "local": ("k_local_staged", 2 * E, "local_16B.md"),
}
PIPELINE_BYTES_PER_RECORD = 2 * 2 * E


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_bytes_per_record(summary):
    """DRAM bytes per record of a kernel from its committed ncu summary
    under profiles/ (its `bytes_per_record:` line: dram__bytes_read.sum +
    dram__bytes_write.sum of one launch over 5e7 records, divided by 5e7;
    the traffic grows in proportion to the records), or None."""
    path = os.path.join(REPO, "profiles", summary)
    try:
        for line in open(path):
            if line.strip().startswith("bytes_per_record:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region.

    The timed region begins only after nvidia-smi's first sample has arrived,
    so that its start-up (NVML initialisation,
    which competes with the sort's host thread for the driver) stays outside
    the timed region; `window(t0, t1)` then keeps the samples taken inside it."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 100

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []          # (arrival time, csv line)
        self.bounds = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def ready(self, timeout_s=15.0):
        """Wait (bounded) for the first sample: nvidia-smi is up."""
        t_end = time.monotonic() + timeout_s
        while self.proc and not self.lines and time.monotonic() < t_end:
            time.sleep(0.01)

    def window(self, t0, t1):
        self.bounds = (t0, t1)

    def _in_window(self):
        if self.bounds is None:
            return [ln for _, ln in self.lines]
        t0, t1 = self.bounds
        inside = [ln for ts, ln in self.lines if t0 <= ts <= t1]
        if inside:
            return inside
        # a region shorter than the period: the first sample after it
        after = [ln for ts, ln in self.lines if ts > t1]
        return after[:1]

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self._in_window():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms, device="cuda"):
    """The slowest rank's time (every rank gets it); ms itself on one rank."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import numpy
    import torch
    import mpsort
    from mpsort import device as dev
    import workloads as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dt = numpy.dtype(DTYPE_DESC)
    n = args.n
    rec = torch.empty((n, 2), dtype=torch.int64, device="cuda")
    rec[:, 0] = W.keys_2(torch, n, args.dist, 1234 + rank)
    rec[:, 1] = torch.arange(n, device="cuda")
    out = torch.empty_like(rec)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step():
        dev.sort(rec.data_ptr(), out.data_ptr(), n, dt, 'key', args.method, sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # parity of the last warm-up output.  val is the input index, so these
    # four properties pin the unique stable order record for record: every
    # output record is the input record its val names (key_payload), each
    # input record appears once (permutation), keys ascend (sorted) and
    # equal keys keep input order (stable)
    parity = W.device_parity(torch, rec, out, n)

    stats_steps = []
    with ClockSampler(local) as clk:
        clk.ready()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.monotonic()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
            stats_steps.append(mpsort.last_stats())
        e1.record(stream)
        torch.cuda.synchronize()
        clk.window(t0, time.monotonic())
        time.sleep(2 * ClockSampler.PERIOD_MS / 1e3)
    ms = max_over_ranks(e0.elapsed_time(e1))
    if world > 1:
        torch.distributed.barrier()
    ms_per_step = ms / args.steps
    value = world * n / (ms_per_step / 1e3)

    # the plain form on the same data, for the learned-vs-plain comparison
    plain_rps = None
    if args.method == "learned" and not args.no_compare:
        for _ in range(2):
            dev.sort(rec.data_ptr(), out.data_ptr(), n, dt, 'key', 'plain', sp)
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(max(1, args.steps // 2)):
            dev.sort(rec.data_ptr(), out.data_ptr(), n, dt, 'key', 'plain', sp)
        p1.record(stream)
        torch.cuda.synchronize()
        plain_rps = n / (p0.elapsed_time(p1) / max(1, args.steps // 2) / 1e3)

    # orientation: the library sort of the same records with torch (a stable
    # key sort, CUB's radix sort underneath, then the record gather by index)
    torch_rps = None
    if not args.no_compare and world == 1:
        def torch_step():
            k = rec[:, 0] ^ (-2**63)  # uint64 order as int64
            _, idx = torch.sort(k, stable=True)
            torch.index_select(rec, 0, idx, out=out)
        torch_step()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(max(1, args.steps // 2)):
            torch_step()
        t1.record(stream)
        torch.cuda.synchronize()
        torch_rps = n / (t0.elapsed_time(t1) / max(1, args.steps // 2) / 1e3)

    st = stats_steps[-1]
    stage_ms = {k: round(sum(s["stage_ms"][k] for s in stats_steps) / len(stats_steps), 4)
                for k in st["stage_ms"]}

    # e2e through the host API: pinned host arrays, H2D + sort + D2H per step
    e2e = None
    if not args.no_e2e:
        del out
        torch.cuda.empty_cache()
        hin = torch.empty((n, 2), dtype=torch.int64, pin_memory=True)
        hin.copy_(rec)
        del rec
        torch.cuda.empty_cache()
        hout = torch.empty_like(hin, pin_memory=True)
        a_in = hin.numpy().view(dt).reshape(n)
        a_out = hout.numpy().view(dt).reshape(n)
        mpsort.sort(a_in, 'key', out=a_out, method=args.method)  # warm-up (allocates staging)
        # the mean over the steps; each step's time is listed too, since the
        # host link of a shared machine now and then stalls for one copy
        steps_e2e = max(1, min(args.steps, 5))
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(steps_e2e):
            s0 = time.perf_counter()
            mpsort.sort(a_in, 'key', out=a_out, method=args.method)
            step_ms.append(round((time.perf_counter() - s0) * 1e3, 2))
        t1 = time.perf_counter()
        e2e = {"value": n / ((t1 - t0) / steps_e2e), "unit": UNIT,
               "h2d_bytes_per_step": n * dt.itemsize, "d2h_bytes_per_step": n * dt.itemsize,
               "steps": steps_e2e, "step_ms": step_ms,
               "median_records_per_s": n / (sorted(step_ms)[len(step_ms) // 2] / 1e3),
               "host_memory": "pinned"}
        # the same call on ordinary (pageable) numpy arrays, which is what
        # most callers of mpsort.sort pass: every copy then stages through
        # the driver's bounce buffers
        if not args.no_pageable:
            p_in = numpy.empty(n, dtype=dt)
            p_in[...] = a_in
            p_out = numpy.empty_like(p_in)
            del hin, hout, a_in, a_out
            mpsort.sort(p_in, 'key', out=p_out, method=args.method)
            pms = []
            for _ in range(max(1, min(args.steps, 2))):
                s0 = time.perf_counter()
                mpsort.sort(p_in, 'key', out=p_out, method=args.method)
                pms.append(round((time.perf_counter() - s0) * 1e3, 2))
            e2e["pageable"] = {"value": n / (sum(pms) / len(pms) / 1e3), "unit": UNIT, "step_ms": pms}
            del p_in, p_out
        mpsort._lib.lib().gbsort_release()

    peak, peak_kind = load_peaks()
    # the dominant kernel: the stage with the most device time per sort
    dom = max(STAGE_KERNELS, key=lambda k: stage_ms.get(k, 0.0))
    kname, alg_bpr, summary = STAGE_KERNELS[dom]
    dom_ms = stage_ms[dom]
    achieved = n * alg_bpr / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
    tpr = ncu_bytes_per_record(summary)
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None, "peak_kind": peak_kind,
                "traffic": tpr * n if tpr else None,
                "algorithmic_bytes_per_launch": n * alg_bpr,
                "per_stage_frac": {k: (n * STAGE_KERNELS[k][1] / (stage_ms[k] / 1e3) / 1e9 / peak
                                       if stage_ms.get(k) else None) for k in STAGE_KERNELS},
                "pipeline_frac": n * PIPELINE_BYTES_PER_RECORD / (ms_per_step / 1e3) / 1e9 / peak}

    launches = st.get("launches")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 keys, 16 B records",
        "data": "synthetic (seeded %s uint64 keys, val = index)" % args.dist,
        "config": {"workload": "1e9 x 16 B [('key','u8'),('val','i8')] sort by key, %s keys" % args.dist,
                   "n": n, "elsize": E, "method": args.method, "l2": "inputs (16 GB) larger than L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": launches * args.steps if launches else None,
        "learned_vs_plain": {"learned_records_per_s": value / world if args.method == "learned" else None,
                             "plain_records_per_s": plain_rps},
        "orientation": {"torch_sort_records_per_s": torch_rps,
                        "what": "torch.sort(keys, stable=True) + index_select of the records, same GPU"},
        "stage_ms": stage_ms,
        "sort_stats": {k: v for k, v in st.items() if k != "stage_ms"},
        "parity": parity,
        "clocks": clk.summary(),
    }
    if rank == 0:
        line["cpu_baseline"] = None if args.no_cpu else cpu_baseline(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(args, seconds=None):
    """The CPU port of mpsort_omp (oracle/oracle.c, OpenMP over all host
    cores) on a bounded sample of the same workload."""
    import numpy
    import oracle as O
    threads = os.cpu_count() or 1
    n = args.cpu_sample
    rng = numpy.random.default_rng(0)
    a = numpy.empty(n, dtype=DTYPE_DESC)
    if args.dist == "uniform":
        a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    else:
        a['key'] = numpy.arange(n, dtype=numpy.uint64)
    a['val'] = numpy.arange(n)
    kind = "reference" if O.ref_lib() is not None else "port"
    if kind == "reference":
        O.set_ref_threads(threads)
        t = O.time_ref_sort(a, 'key', 'omp', repeat=3)
    else:
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            O.oracle_mpsort(a, 'key', threads)
            ts.append(time.perf_counter() - t0)
        ts.sort()
        t = ts[1]
    return {"value": n / t, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "%d records of the same 16 B layout, median of 3 sorts" % n,
            "extrapolated_to_full_size": nlogn_extrapolation(n / t, n, args.n)}


def nlogn_extrapolation(rate, n_sample, n_full):
    """Records/s of a comparison sort at n_full, scaled from the rate
    measured at n_sample by n log n work (time per record grows as log n)."""
    import math
    if n_sample <= 1 or n_full <= n_sample:
        return {"records_per_s": rate, "n": n_sample, "how": "measured at this size"}
    return {"records_per_s": rate * math.log(n_sample) / math.log(n_full), "n": n_full,
            "how": "n log n scaling of the sample's rate (not measured)"}


def cpu_sort_seconds(a, orderby, repeat=3):
    """Median wall time of the CPU port of mpsort_omp (or the reference
    build, where present) sorting array a on all host cores."""
    import oracle as O
    threads = os.cpu_count() or 1
    if O.ref_lib() is not None:
        O.set_ref_threads(threads)
        return O.time_ref_sort(a, orderby, 'omp', repeat=repeat), "reference", threads
    ts = []
    for _ in range(repeat):
        t0 = time.perf_counter()
        O.oracle_mpsort(a, orderby, threads)
        ts.append(time.perf_counter() - t0)
    ts.sort()
    return ts[len(ts) // 2], "port", threads


def run_config(args):
    """One JSON line for configurations 1, 3, 4, 5 (parity checked by
    size-independent properties on the device)."""
    import numpy
    import torch
    import mpsort
    from mpsort import device as dev
    import workloads as W
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    st = torch.cuda.current_stream()
    sp = st.cuda_stream
    ev = lambda: torch.cuda.Event(enable_timing=True)
    res = {"config_id": args.config, "steps": args.steps, "warmup": args.warmup}

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(st)
        for _ in range(steps):
            fn()
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    if args.config == "1":
        import oracle as O
        arr = W.records_1(torch)
        din = torch.from_numpy(arr.view(numpy.uint8).copy()).cuda()
        dout = torch.empty_like(din)
        n = len(arr)
        for m in ("learned", "plain", "lsd", "auto"):
            ms = timed(lambda: dev.sort(din.data_ptr(), dout.data_ptr(), n, W.DT1, 'key', m, sp), args.steps)
            res[m + "_records_per_s"] = n / (ms / 1e3)
        got = dout.cpu().numpy().view(W.DT1)
        ref = O.ref_sort(arr, 'key', 'omp')
        exp = ref if ref is not None else O.numpy_sorted(arr, 'key')
        res.update(value=res["auto_records_per_s"], n=n, value_method="auto (the call a user makes)",
                   parity={"equals_reference" if ref is not None else "equals_stable_sort": got.tobytes() == exp.tobytes()})
        if not args.no_cpu:
            t, kind, cores = cpu_sort_seconds(arr, 'key')
            res["cpu_baseline"] = {"value": n / t, "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": "the whole workload, median of 3 sorts"}
    elif args.config == "3":
        buf, dt, offs = W.segments_3(torch)
        out = torch.empty_like(buf)
        n = int(offs[-1])
        # the segment autotuner picks level 2 and the threshold for sorting a
        # segment on its own; the batch is then one graph-captured plan
        tuned = dev.autotune_segments(offs, dt, 'key', buf.data_ptr())
        plan = dev.Plan(0, dt, 'key', segments=offs)

        def plan_step():
            plan.sort(buf.data_ptr(), out.data_ptr(), sp)
            plan.wait()
        ms = timed(plan_step, args.steps)
        stats = mpsort.last_stats()
        ms_call = timed(lambda: dev.sort_segments(buf.data_ptr(), out.data_ptr(), offs, dt, 'key', 'auto', sp),
                        args.steps)

        def per_array():
            for i in range(len(offs) - 1):
                a, b = int(offs[i]), int(offs[i + 1])
                dev.sort(buf.data_ptr() + a * 8, out.data_ptr() + a * 8, b - a, dt, 'key', 'plain', sp)
        ms_loop = timed(per_array, 1)
        out.zero_()
        plan_step()
        plan.close()
        torch.cuda.synchronize()
        seg_start = torch.zeros(n, dtype=torch.bool, device="cuda")
        seg_start[torch.from_numpy(offs[:-1].astype(numpy.int64)).cuda().clamp_(max=n - 1)] = True
        parity = W.device_parity(torch, buf.view(torch.int32).view(-1, 2), out.view(torch.int32).view(-1, 2), n,
                               key_col=0, ident_col=1, segment_start=seg_start, signed=True)
        if not args.no_cpu:
            host = buf.cpu().numpy().view(dt)
            k = int(numpy.searchsorted(offs, 2_000_000))
            k = max(1, min(k, len(offs) - 1))
            t = 0.0
            for i in range(k):
                a, b = int(offs[i]), int(offs[i + 1])
                if b > a:
                    t += cpu_sort_seconds(host[a:b].copy(), 'key', repeat=1)[0]
            kind, cores = cpu_sort_seconds(host[:16].copy(), 'key', repeat=1)[1:]
            res["cpu_baseline"] = {"value": int(offs[k]) / t, "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": "the first %d arrays (%d records), one CPU sort per array" % (k, int(offs[k]))}
        res.update(value=n / (ms / 1e3), n=n, nseg=len(offs) - 1, ms_per_step=ms, graph=True,
                   graph_kernel_launches=stats["launches"], level2_engine=bool(stats["engine"]),
                   segments_sorted_alone=stats["sample"], tuned_entry=tuned,
                   synchronous_call_records_per_s=n / (ms_call / 1e3),
                   per_array_loop_records_per_s=n / (ms_loop / 1e3), per_array_loop_ms=ms_loop,
                   parity=parity, sort_stats=stats)
    elif args.config == "4":
        n = args.n if args.n != 10**9 else 5 * 10**8
        buf, dt = W.particles_4(torch, n)
        out = torch.empty_like(buf)
        for m in ("learned", "plain"):
            ms = timed(lambda: dev.sort(buf.data_ptr(), out.data_ptr(), n, dt, 'key', m, sp), args.steps)
            stl = mpsort.last_stats()
            res[m] = {"records_per_s": n / (ms / 1e3), "ms": ms, "stage_ms": stl["stage_ms"],
                      "bucket_imbalance": stl["max_bucket"] / (n / stl["nbuckets"]),
                      "resplits": stl["resplits"], "splits": stl["splits"],
                      "window_misses": stl["window_misses"], "widest_window": stl["widest_window"],
                      "bigbin_passes": stl["bigbin_passes"],
                      "parity": W.device_parity(torch, buf.view(torch.int64).view(-1, 5),
                                              out.view(torch.int64).view(-1, 5), n, key_col=4, ident_col=3)}
        res.update(value=res["learned"]["records_per_s"], n=n,
                   parity={k: res["learned"]["parity"][k] and res["plain"]["parity"][k]
                           for k in res["learned"]["parity"]})
        if not args.no_cpu:
            m = min(n, 2_000_000)
            sample = buf[:m * dt.itemsize].cpu().numpy().view(dt).copy()
            t, kind, cores = cpu_sort_seconds(sample, 'key')
            res["cpu_baseline"] = {"value": m / t, "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": "the first %d records of the workload, median of 3 sorts" % m}
    elif args.config == "5":
        buf, dt, na, nb, common = W.snapshots_5(torch)
        out = torch.empty_like(buf)
        offs = numpy.array([0, na, na + nb], dtype=numpy.uint64)
        pa = torch.empty(min(na, nb), dtype=torch.int64, device="cuda")
        pb = torch.empty_like(pa)
        npairs = torch.zeros(1, dtype=torch.int64, device="cuda")

        def step():
            dev.sort_segments(buf.data_ptr(), out.data_ptr(), offs, dt, 'id', 'auto', sp)
            dev.merge_join(out.data_ptr(), na, out.data_ptr() + na * 16, nb, dt, 'id', pa.data_ptr(),
                           pb.data_ptr(), npairs.data_ptr(), sp)
        ms = timed(step, args.steps)
        k = int(npairs.item())
        ids = out.view(torch.int64).view(-1, 2)[:, 0]
        ida, idb = ids[:na], ids[na:]
        ok_pairs = k == common and bool((ida[pa[:k]] == idb[pb[:k]]).all().item()) and \
            bool((pa[1:k] > pa[:k - 1]).all().item())
        ok_sorted = bool((ida[1:] > ida[:-1]).all().item()) and bool((idb[1:] > idb[:-1]).all().item())
        res.update(value=(na + nb) / (ms / 1e3), n=na + nb, ms_per_step=ms, pairs=k, expected_pairs=common,
                   parity={"pairs": ok_pairs, "sorted_unique": ok_sorted})
        if not args.no_cpu:
            m = 1_000_000
            host = buf.cpu().numpy().view(dt)
            sa, sb = host[:m].copy(), host[na:na + m].copy()
            ta, kind, cores = cpu_sort_seconds(sa, 'id', repeat=1)
            tb = cpu_sort_seconds(sb, 'id', repeat=1)[0]
            import oracle as O
            ssa, ssb = O.numpy_sorted(sa, 'id'), O.numpy_sorted(sb, 'id')
            t0 = time.perf_counter()
            numpy.intersect1d(ssa['id'], ssb['id'], assume_unique=True, return_indices=True)
            tj = time.perf_counter() - t0
            res["cpu_baseline"] = {"value": 2 * m / (ta + tb + tj), "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": "1e6 records of each snapshot: two CPU sorts + numpy.intersect1d"}
    line = {"metric": "sorted records/s, configuration " + args.config, "unit": UNIT, "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic (workloads.py, seeded)"}
    line.update(res)
    print(json.dumps(line), flush=True)


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy
    import oracle as O
    threads = os.cpu_count() or 1
    n = args.cpu_sample
    rng = numpy.random.default_rng(0)
    a = numpy.empty(n, dtype=DTYPE_DESC)
    a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    a['val'] = numpy.arange(n)
    kind = "reference" if O.ref_lib() is not None else "port"
    O.set_ref_threads(threads) if kind == "reference" else None

    def one():
        t0 = time.perf_counter()
        if kind == "reference":
            O.ref_sort(a, 'key', 'omp')
        else:
            O.oracle_mpsort(a, 'key', threads)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        one()
    t = sum(one() for _ in range(args.steps))
    ms_per_step = t / args.steps * 1e3
    value = n / (ms_per_step / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 keys, 16 B records",
        "data": "synthetic (seeded uniform uint64 keys, val = index)",
        "config": {"workload": "1e9 x 16 B [('key','u8'),('val','i8')] sort by key, uniform keys",
                   "n": args.n, "elsize": E, "parallelism": "CPU threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "each step sorts %d records of the workload's layout" % n,
                         "extrapolated_to_full_size": nlogn_extrapolation(value, n, args.n)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--method", choices=["learned", "plain", "lsd"], default="learned")
    ap.add_argument("--n", type=int, default=10**9)
    ap.add_argument("--dist", choices=["uniform", "sorted1pct", "zipf"], default="uniform")
    ap.add_argument("--cpu-sample", type=int, default=20_000_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-pageable", action="store_true", help="skip the e2e figure on pageable host arrays")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--config", choices=["1", "2a", "2b", "2c", "3", "4", "5"], default="2a",
                    help="workload; 2a/2b/2c give the contract's bench line (2b = --dist sorted1pct, "
                         "2c = --dist zipf), the others a JSON line of their own")
    args = ap.parse_args()
    if args.config in ("2b", "2c"):
        args.dist = {"2b": "sorted1pct", "2c": "zipf"}[args.config]
    if args.impl == "reference":
        run_reference(args)
    elif args.config in ("2a", "2b", "2c"):
        run_ours(args)
    else:
        run_config(args)


if __name__ == "__main__":
    main()
