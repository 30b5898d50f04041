"""Benchmark: exact 2^24 x 2^24-limb multiplication on GB300.

One step is one product of two 2^24-limb operands (uniform seeded 64-bit
limbs, the balanced-sweep configuration the headline metric is quoted on):
transform length 2^25, three 63-bit primes.  The metric is output limbs per
second, (na + nb) / seconds per product, summed over ranks.

  value   device-resident operands, hg_mul_device on the torch stream, timed
          with CUDA events (operands 256 MiB + workspace 1.6 GB: larger than
          L2, so no explicit flush).
  e2e     the same product through the host C-ABI entry point hg_mul from
          pinned host buffers, host->device and device->host copies inside
          the timed region (wall clock around synchronous calls).
  roofline  the kernel class with the most device time, its algorithmic
          bytes over its event-timed duration, against the measured HBM copy
          bandwidth.
  cpu_baseline  the oracle (a C restatement of the reference's algorithm,
          per-modulus threads like its with-parallel-work) timed on this
          host on one full product.
  sweep   a*b and a^2 at 2^18 .. 2^26 limbs per operand.
  batched 4096 uneven pairs (log-uniform 2^6 .. 2^14 limbs): an autotuned
          batch replayed from a CUDA graph against one call per product.
  expt    9^(9^9) with device-resident powers.
  mpd_pi  Chudnovsky pi/10 through the device-resident multiply service at
          2^22, 2^24, 2^26 bits, and the reference-exact mpd-pi at 10^4 bits
          against the CPU oracle.

`--impl reference` times that CPU restatement instead (the reference itself
is Common Lisp and cannot run here).  With --gpus N under torchrun each rank
runs an independent replica; value is the sum over ranks.
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
sys.path.insert(0, ROOT)

METRIC = "64-bit limbs multiplied/s at 2^24"
UNIT = "limbs/s"
LOG_SIZE = 24


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _pipes(kernel_class: str):
    """Pipe utilisation of a kernel class from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 8 and parts[0] == "pipe_pct" and parts[1] == kernel_class:
                    return {parts[2] + "_pct": float(parts[3]), parts[4] + "_pct": float(parts[5]),
                            parts[6] + "_pct": float(parts[7]), "source": "profiles/ntt_contig_mul_2e22.md (ncu)"}
    except (OSError, ValueError):
        pass
    return None


def _traffic(kernel_class: str):
    """Per-launch DRAM bytes of a kernel class from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and parts[0] == "dram_bytes_per_launch" and parts[1] == kernel_class:
                    return float(parts[2])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def rank_seeds(rank: int) -> tuple[int, int]:
    """SplitMix64 seeds of a rank's two operands: each replica multiplies its own."""
    return 1 + 1000 * rank, 2 + 1000 * rank


def max_over_ranks(x: float, dist, device: str) -> float:
    """The slowest rank's time (the job's time); x itself without a process group."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(ws: int, units_per_rank_step: int, steps: int, seconds: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return ws * units_per_rank_step * steps / seconds


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _cpu_info():
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return os.cpu_count() or 1, model


def cpu_product_rate(log_size: int, threads: int) -> tuple[float, float]:
    """One product of two 2^log_size-limb operands on the oracle; (limbs/s, s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    from hypergeometrica_gb300 import workloads as W

    n = 1 << log_size
    x, y = W.limbs(1, n), W.limbs(2, n)
    O.set_threads(threads)
    t = time.perf_counter()
    O.mpz_mul_ntt(x, y)
    dt = time.perf_counter() - t
    return 2 * n / dt, dt


def gmp_baseline(x, y, gpu_out) -> dict:
    """GMP's mpz_mul on the same operands (one thread): its rate, and whether
    its product equals the GPU's limb for limb."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gmp

    if not gmp.available():
        return {"unavailable": "libgmp not found on this host"}
    timer = []
    ref = gmp.mul(x, y, timer)
    return {"value": len(ref) / timer[0], "unit": UNIT, "cores": 1, "seconds": timer[0],
            "matches_gpu": bool(np.array_equal(ref, gpu_out))}


def run_reference(args) -> None:
    """The reference arm: the oracle port (the reference's algorithm with its
    per-modulus task structure, src/ntt-multiply.lisp:174-254 under
    with-parallel-work) timed on this host's cores on the bench's own
    workload, one full 2^24 x 2^24-limb product per timed step.  Warm-up
    steps run one 2^20 x 2^20 product each (they only page the code and the
    thread pool in).  Beside the per-modulus-threaded line, one full product
    runs single-threaded."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    cores, model = _cpu_info()
    threads = min(6, cores)  # 2k forward tasks of with-parallel-work (k = 3 primes)
    full = 1 << LOG_SIZE
    for _ in range(args.warmup):
        cpu_product_rate(20, threads)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_product_rate(LOG_SIZE, threads)
        times.append(dt)
    total = sum(times)
    value = 2 * full * args.steps / total
    rate1, dt1 = cpu_product_rate(LOG_SIZE, 1)
    sample = f"one {full}x{full}-limb product per timed step (warm-up steps: one 2^20 x 2^20 product each)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (SplitMix64 seeds 1, 2)",
        "config": {"workload": f"mul {full}x{full} limbs, transform 2^{LOG_SIZE + 1}, 3 primes",
                   "dist": "uniform", "parallelism": "replicas"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "cpu": model, "host_cores": cores,
                         "single_thread": {"value": rate1, "unit": UNIT, "cores": 1,
                                           "sample": f"one {full}x{full}-limb product ({dt1:.1f} s)"}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _residue_ok(out_u64, x_u64, y_u64) -> bool:
    """out == x*y modulo the prime 2^31 - 1 (an O(n) sanity check)."""
    import numpy as np

    q = 2147483647
    base = (1 << 64) % q

    def full(a):
        n = len(a)
        blk = 4096
        lo = np.empty(blk, dtype=np.uint64)
        v = 1
        for i in range(blk):
            lo[i] = v
            v = v * base % q
        nb = (n + blk - 1) // blk
        hi = np.empty(nb, dtype=np.uint64)
        w = 1
        for i in range(nb):
            hi[i] = w
            w = w * v % q
        pw = np.tile(lo, nb)[:n] * np.repeat(hi, blk)[:n] % np.uint64(q)
        return int(((a % np.uint64(q)) * pw % np.uint64(q)).sum(dtype=np.uint64) % np.uint64(q))

    return full(out_u64) == full(x_u64) * full(y_u64) % q


BATCH_PAIRS = 4096


def run_batched(stream, steps: int) -> dict:
    """4096 independent pairs, sizes log-uniform in [2^6, 2^14] limbs per
    operand (seeds 41, 42), uniform limbs: the binary-splitting-leaf workload.
    Times an autotuned batch replayed from a CUDA graph against one
    hg_mul_device call per product on the same stream; both must agree on
    every product."""
    import numpy as np
    import torch

    from hypergeometrica_gb300 import _lib
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import workloads as W

    sx = W.log_uniform_sizes(41, BATCH_PAIRS, 6, 14)
    sy = W.log_uniform_sizes(42, BATCH_PAIRS, 6, 14)
    host = np.concatenate([W.limbs(100_000 + k, int(sx[k]) + int(sy[k])) for k in range(BATCH_PAIRS)])
    ops = torch.from_numpy(host.view(np.int64)).cuda()
    nout = int((sx + sy).sum())
    out_pp = torch.zeros(nout, dtype=torch.int64, device="cuda")
    out_b = torch.full((nout,), -1, dtype=torch.int64, device="cuda")
    pp, items = [], []
    o = 0
    for k in range(BATCH_PAIRS):
        nx, ny = int(sx[k]), int(sy[k])
        x, y = ops[o: o + nx], ops[o + nx: o + nx + ny]
        pp.append((x, y, out_pp[o: o + nx + ny]))
        items.append((x, y, out_b[o: o + nx + ny]))
        o += nx + ny

    def per_product():
        for x, y, out in pp:
            D.mul(x, y, out, stream=stream)

    per_product()
    D.sync(stream)
    t0 = time.perf_counter()
    b = D.Batch(items, autotune=True)
    tune_s = time.perf_counter() - t0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.run(s)
    s.synchronize()
    _lib.profile_read()
    b.run(stream)
    D.sync(stream)
    launches_batch = sum(v["launches"] for v in _lib.profile_read().values())
    per_product()
    D.sync(stream)
    launches_pp = sum(v["launches"] for v in _lib.profile_read().values())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.run(s)
    out_b.fill_(-1)
    g.replay()
    torch.cuda.synchronize()
    D.sync(stream)
    correct = bool(torch.equal(out_b, out_pp))
    schedule, sched_launches = b.schedule()
    # Both schedules with the tuned pass splits, each captured in a graph.
    per_sched = {}
    for name in ("persistent", "per_pass"):
        bs = D.Batch(items, autotune=False, schedule=name)
        gs = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gs, stream=s):
            bs.run(s)
        out_b.fill_(-1)
        gs.replay()
        torch.cuda.synchronize()
        D.sync(stream)
        per_sched[name] = {"graph": gs, "batch": bs, "launches": bs.schedule()[1],
                           "correct": bool(torch.equal(out_b, out_pp))}
        correct = correct and per_sched[name]["correct"]

    def timed(fn, reps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    with torch.cuda.stream(stream):
        ms_graph = timed(g.replay, max(3, steps))
        for name, v in per_sched.items():
            v["ms"] = timed(v["graph"].replay, max(3, steps))
    ms_pp = timed(per_product, max(2, min(steps, 5)))
    D.sync(stream)

    # The same pairs through the device-resident service: four client threads
    # submit 256 pairs at a time; products join batches as slots free up.
    import threading

    svc_stats, svc_ok = {}, True
    with D.Service(workspace_bytes=4 << 30, slots=2, max_batch=4096) as svc:
        svc.submit(items)  # warm
        svc.wait_all()
        out_b.fill_(-1)
        torch.cuda.synchronize()
        svc.stats(reset=True)
        chunks = [items[i: i + 256] for i in range(0, len(items), 256)]
        t0 = time.perf_counter()
        threads = [threading.Thread(target=lambda c=chunks[k::4]: [svc.submit(x) for x in c]) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        svc.wait_all()
        wall = time.perf_counter() - t0
        st = svc.stats()
        svc_ok = bool(torch.equal(out_b, out_pp))
        svc_stats = {"products_per_s": BATCH_PAIRS / wall, "wall_ms": 1000 * wall, "p50_us": st["p50_us"],
                     "p99_us": st["p99_us"], "batches": st["batches"], "slots": st["slots"],
                     "clients": 4, "chunk": 256, "correct": svc_ok}
    return {
        "metric": "products/s, 4096 uneven pairs", "unit": "products/s",
        "workload": f"{BATCH_PAIRS} pairs, operand sizes log-uniform in [2^6, 2^14] limbs (seeds 41, 42), "
                    f"{nout} output limbs",
        "graph": BATCH_PAIRS / (ms_graph / 1000.0), "per_product": BATCH_PAIRS / (ms_pp / 1000.0),
        "speedup": ms_pp / ms_graph, "ms_graph": ms_graph, "ms_per_product_path": ms_pp,
        "gpu_launches_graph": launches_batch, "gpu_launches_per_product_path": launches_pp,
        "schedule": schedule, "schedule_launches": sched_launches,
        "schedules": {name: {"ms_graph": v["ms"], "launches": v["launches"], "correct": v["correct"]}
                      for name, v in per_sched.items()},
        "autotune_s": tune_s, "service": svc_stats, "correct": correct and svc_ok,
    }


SWEEP_LOG_SIZES = (18, 20, 22, 24, 26)
UNBALANCED = ((24, 16), (25, 20), (20, 6))
DISTS = ("uniform", "ones", "sparse")


class ExactChecks:
    """GMP's exact products of the sweep's operands, computed on host threads
    while the GPU is timed (ctypes releases the interpreter lock inside
    mpz_mul; four cores stay free for the launching thread).  check() compares
    a GPU result limb for limb; where libgmp is missing it falls back to the
    residue modulo 2^31 - 1 and says so."""

    def __init__(self, jobs):
        import concurrent.futures as cf

        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import gmp

        self.gmp = gmp if gmp.available() else None
        self.futs = {}
        self.ex = None
        if self.gmp:
            self.ex = cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), (os.cpu_count() or 5) - 4)))
            for key, (kind, xs, ys) in sorted(jobs.items(), key=lambda kv: -kv[1][1][1] * (kv[1][2] or kv[1][1])[1]):
                self.futs[key] = self.ex.submit(self._product, kind, xs, ys)

    def _product(self, kind, xs, ys):
        from hypergeometrica_gb300 import workloads as W

        x = W.limbs(*xs)
        return self.gmp.sqr(x) if kind == "sqr" else self.gmp.mul(x, W.limbs(*ys))

    def check(self, key, got, x, y) -> tuple[bool, str]:
        import numpy as np

        if key in self.futs:
            want = self.futs[key].result()
            return bool(len(got) >= len(want) and np.array_equal(got[: len(want)], want)
                        and not got[len(want):].any()), "gmp limb-exact"
        return _residue_ok(got, x, y), "residue mod 2^31-1"

    def close(self):
        if self.ex:
            self.ex.shutdown(wait=True, cancel_futures=True)


def run_sweep(stream, peak_gbs: float) -> dict:
    """The balanced single-product sweep: a x b and a^2 with |a| = |b| = 2^18 ..
    2^26 limbs (uniform limbs, seeds 11, 12), device-resident, CUDA events.
    Each line: ms per product, output limbs/s, and the minimum-pass HBM
    bytes (16 (na + nb) + 192 N for a product, 24 n + 96 N for a square) over
    the time as a fraction of the measured copy bandwidth."""
    import numpy as np
    import torch

    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import workloads as W

    jobs = {}
    for k in SWEEP_LOG_SIZES:
        jobs[("mul", k)] = ("mul", (11, 1 << k, "uniform"), (12, 1 << k, "uniform"))
        jobs[("sqr", k)] = ("sqr", (11, 1 << k, "uniform"), None)
    for ka, kb in UNBALANCED:
        for dist in DISTS:
            jobs[("unb", ka, kb, dist)] = ("mul", (13, 1 << ka, dist), (14, 1 << kb, dist))
    exact = ExactChecks(jobs)
    out = {"workload": "a*b and a^2, |a| = |b| = 2^k limbs, uniform", "unit": "limbs/s", "lines": []}
    for k in SWEEP_LOG_SIZES:
        n = 1 << k
        a = torch.from_numpy(W.limbs(11, n).view(np.int64)).cuda()
        b = torch.from_numpy(W.limbs(12, n).view(np.int64)).cuda()
        o = torch.empty(2 * n, dtype=torch.int64, device="cuda")
        N = 1 << (k + 1)
        reps = max(2, min(20, (1 << 26) // n))
        for kind in ("mul", "sqr"):
            f = (lambda: D.mul(a, b, o, stream=stream)) if kind == "mul" else (lambda: D.sqr(a, o, stream=stream))
            for _ in range(2):
                f()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            for _ in range(reps):
                f()
            ev1.record(stream)
            torch.cuda.synchronize()
            ms = ev0.elapsed_time(ev1) / reps
            D.sync(stream)
            x = W.limbs(11, n)
            ok, how = exact.check((kind, k), o.cpu().numpy().view(np.uint64), x,
                                  x if kind == "sqr" else W.limbs(12, n))
            algo = (16 * 2 * n + 192 * N) if kind == "mul" else (24 * n + 96 * N)
            out["lines"].append({"log_size": k, "kind": kind, "ms": ms, "limbs_per_s": 2 * n / (ms / 1000.0),
                                 "hbm_frac": algo / (ms / 1000.0) / 1e9 / peak_gbs, "correct": ok, "check": how})
        del a, b, o
        torch.cuda.empty_cache()
    # Unbalanced and edge-value products: 2^24 x 2^16, 2^25 x 2^20, 2^20 x 2^6
    # limbs, uniform, all-ones (the longest carry chains) and 1%-nonzero limbs,
    # through the NTT product (hg_mul_device, mpz-*/ntt semantics): as the
    # library runs them (in chunks against one spectrum of the short operand)
    # and as the reference's one transform of the least power of two >= nx + ny
    # points (chunking switched off); both results must agree.
    from hypergeometrica_gb300 import _lib

    out["unbalanced"] = []
    for ka, kb in UNBALANCED:
        na, nb = 1 << ka, 1 << kb
        for dist in DISTS:
            xh, yh = W.limbs(13, na, dist), W.limbs(14, nb, dist)
            a = torch.from_numpy(xh.view(np.int64)).cuda()
            b = torch.from_numpy(yh.view(np.int64)).cuda()
            o = torch.empty(na + nb, dtype=torch.int64, device="cuda")
            o1 = torch.empty_like(o)
            reps = max(2, min(10, (1 << 26) // na))

            def timed(dst):
                for _ in range(2):
                    D.mul(a, b, dst, stream=stream)
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                ev0.record(stream)
                for _ in range(reps):
                    D.mul(a, b, dst, stream=stream)
                ev1.record(stream)
                torch.cuda.synchronize()
                D.sync(stream)
                return ev0.elapsed_time(ev1) / reps

            ms = timed(o)
            _lib.set_chunking(False)
            try:
                ms1 = timed(o1)
            finally:
                _lib.set_chunking(True)
            ok, how = exact.check(("unb", ka, kb, dist), o.cpu().numpy().view(np.uint64), xh, yh)
            ok = ok and bool(torch.equal(o, o1))
            out["unbalanced"].append({"log_sizes": [ka, kb], "dist": dist, "ms": ms,
                                      "limbs_per_s": (na + nb) / (ms / 1000.0),
                                      "chunk_plan": _lib.chunk_plan(na, nb), "ms_one_transform": ms1,
                                      "correct": ok, "check": how + "; chunked equals one transform"})
            del a, b, o, o1
        torch.cuda.empty_cache()
    exact.close()
    out["correct"] = all(line["correct"] for line in out["lines"] + out["unbalanced"])
    return out


MPD_BITS = (1 << 22, 1 << 24, 1 << 26)
MPD_EXACT_BITS = 10000


def run_mpd_pi(cpu: bool) -> dict:
    """Chudnovsky pi/10 through the device-resident multiply service.

    At 2^22, 2^24 and 2^26 bits: binary splitting (partials in HBM, every
    product through the service) and Newton steps kept at working precision
    (the reference never truncates, so its own result at these sizes would
    need terabytes; this variant is labelled and is not its mantissa).  The
    largest run's partials are checked modulo a prime against the oracle's
    closed forms.  At 10^4 bits the untruncated, reference-identical mpd_pi
    runs on the GPU and on the CPU oracle; the two must be bit-identical."""
    import torch

    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import mpd as G
    from hypergeometrica_gb300 import series as S

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    out = {"metric": "mpd-pi wall time", "unit": "s", "runs": []}
    with D.Service(workspace_bytes=2 << 30, slots=2) as svc:
        G.mpd_pi_truncated(1 << 12, service=svc)  # warm the kernels and the service
        for bits in MPD_BITS:
            svc.stats(reset=True)
            t = {}
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            G.mpd_pi_truncated(bits, service=svc, timings=t)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            st = svc.stats()
            out["runs"].append({
                "bits": bits, "variant": "truncated Newton (not the reference's untruncated mantissa)",
                "wall_s": wall, **t,
                "service": {k: st[k] for k in ("completed", "batches", "p50_us", "p99_us", "mean_us",
                                               "products_per_s", "peak_batch_products")}})
        import series_oracle as SO

        bits = MPD_BITS[-1]
        n = S.chudnovsky_terms(bits)
        part = S.binary_split(S.make_chudnovsky_series(), 0, n, service=svc)
        m = (1 << 61) - 1
        got = tuple(x.to_int() % m for x in (part.p, part.q, part.b, part.r))
        out["partials_check"] = {"bits": bits, "terms": n, "modulus": "2^61-1",
                                 "match": got == SO.residues(SO.chudnovsky_series(), 0, n, m)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = G.mpd_pi(MPD_EXACT_BITS)
    torch.cuda.synchronize()
    exact = {"bits": MPD_EXACT_BITS, "variant": "untruncated, the reference's mpd-pi",
             "gpu_s": time.perf_counter() - t0, "mantissa_limbs": x.mantissa.size}
    if cpu:
        import mpd_oracle as MO

        t0 = time.perf_counter()
        ref = MO.mpd_pi(MPD_EXACT_BITS)
        exact["cpu_oracle_s"] = time.perf_counter() - t0
        exact["bit_identical"] = x.to_pair() == (ref.m, ref.e)
    out["exact"] = exact
    out["correct"] = out["partials_check"]["match"] and exact.get("bit_identical", True)
    return out


def run_expt() -> dict:
    """9^(9^9) by mpz-expt with every partial power in device memory (the
    x^x^x workload of the reference's published runs).  The bit length is the
    log's known answer; the published time is the reference's own run
    (logs/24apr21-999-ram.txt:205-226, SBCL with intrinsics and threads)."""
    import torch

    from hypergeometrica_gb300 import series as S

    S.mpz_expt_device(9, 9**5)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = S.mpz_expt_device(9, 9**9)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    top = int(x.t[x.size - 1].item()) & (2**64 - 1)
    bits = 64 * (x.size - 1) + top.bit_length()
    return {"workload": "9^(9^9) (mpz-expt: 28 squarings + 13 products by 9, largest 2^25-point)", "wall_s": wall,
            "bits": bits, "correct": bits == 1228093895,
            "reference_published_s": 136.233, "reference_published_note": "logs/24apr21-999-ram.txt, other hardware"}


# Thread instructions per radix-2 butterfly of the middle kernel (ncu,
# profiles/ntt_contig_mul_2e22.md): the fewest any pass of the product spends.
INSTR_PER_BUTTERFLY = 29.2


def _int_roofline(N: int, ms_per_product: float, sm_mhz) -> dict:
    """The product's radix-2 butterflies (3 primes x 3 transforms x N/2 log2 N)
    per second against two ceilings: hg_butterfly_peak, a memory-free network
    of the same modular butterflies over every SM measured now, and the
    issue-rate floor, every SM sub-partition issuing one warp instruction
    per clock at the clock sampled under load, with the middle kernel's
    29.2 thread instructions per butterfly."""
    import ctypes

    import torch

    from hypergeometrica_gb300 import _lib

    pk = ctypes.c_double()
    _lib.check(_lib.load().hg_butterfly_peak(ctypes.byref(pk)))
    bf = 3 * 3 * (N // 2) * (N.bit_length() - 1)
    achieved = bf / (ms_per_product / 1000.0)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_mhz or 2070.0
    issue = sms * 4 * mhz * 1e6 * 32 / INSTR_PER_BUTTERFLY
    return {"bound": "int-pipe", "butterflies_per_product": bf, "achieved": achieved, "peak": pk.value,
            "unit": "butterflies/s", "frac": achieved / pk.value,
            "peak_source": "hg_butterfly_peak (register-only network of the same butterflies)",
            "issue_floor": {"peak": issue, "frac": achieved / issue, "sms": sms, "sm_mhz": mhz,
                            "thread_instructions_per_butterfly": INSTR_PER_BUTTERFLY,
                            "source": "one warp instruction per clock per SM sub-partition (4 per SM)"}}


def host_link(nbytes: int = 256 << 20) -> dict:
    """Where the pinned buffers sit and what the host link moves: the NUMA
    nodes of this host, the GPU's node (sysfs), and plain pinned-memory copy
    rates host->device and device->host (torch copies, CUDA events)."""
    import glob

    import torch

    info = {"numa_nodes": len(glob.glob("/sys/devices/system/node/node[0-9]*"))}
    node = None
    for d in glob.glob("/sys/bus/pci/devices/*"):
        try:
            if open(os.path.join(d, "vendor")).read().strip() == "0x10de" and \
                    open(os.path.join(d, "class")).read().startswith("0x030"):
                node = int(open(os.path.join(d, "numa_node")).read())
                break
        except OSError:
            continue
    info["gpu_numa_node"] = node
    try:
        info["process_mems_allowed"] = [ln.split(":", 1)[1].strip() for ln in open("/proc/self/status")
                                        if ln.startswith("Mems_allowed_list")][0]
    except (OSError, IndexError):
        pass
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")

    def rate(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return 5 * nbytes / (e0.elapsed_time(e1) / 1000.0) / 1e9

    info["h2d_gbs"] = rate(lambda: d.copy_(h, non_blocking=True))
    info["d2h_gbs"] = rate(lambda: h.copy_(d, non_blocking=True))
    info["copy_bytes"] = nbytes
    return info


def run_ours(args) -> None:
    import numpy as np
    import torch

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    from hypergeometrica_gb300 import build as B

    if rank == 0 or ws == 1:
        B.build()
    if dist:
        dist.barrier()
    import hypergeometrica_gb300 as H
    from hypergeometrica_gb300 import _lib
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import workloads as W

    H.init(local)
    na = nb = 1 << args.log_size
    sx, sy = rank_seeds(rank)
    x = W.limbs(sx, na)
    y = W.limbs(sy, nb)
    tx = torch.from_numpy(x.view(np.int64)).cuda()
    ty = torch.from_numpy(y.view(np.int64)).cuda()
    out = torch.empty(na + nb, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        D.mul(tx, ty, out, stream=stream)

    for _ in range(args.warmup):
        step()
    D.sync(stream)
    ok = _residue_ok(out.cpu().numpy().view(np.uint64), x, y)

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    _lib.profile_read()  # reset counters
    _lib.profile_enable(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    _lib.profile_enable(False)
    prof = _lib.profile_read()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    D.sync(stream)

    # End to end through the host entry point, pinned host buffers.
    hx = torch.from_numpy(x.view(np.int64)).pin_memory()
    hy = torch.from_numpy(y.view(np.int64)).pin_memory()
    hout = torch.empty(na + nb, dtype=torch.int64).pin_memory()
    lib = _lib.load()
    rc = lib.hg_mul(hx.data_ptr(), na, hy.data_ptr(), nb, hout.data_ptr(), na + nb)  # warm the staging buffers
    _lib.check(rc)
    e2e_steps = max(3, min(args.steps, 20))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _lib.check(lib.hg_mul(hx.data_ptr(), na, hy.data_ptr(), nb, hout.data_ptr(), na + nb))
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    ok = ok and bool(np.array_equal(hout.numpy().view(np.uint64), out.cpu().numpy().view(np.uint64)))
    # The same products through hg_mul_host_pipeline: one call for all the
    # steps; each step's operands still go up and its result comes down, but
    # product k's download overlaps product k + 1's upload and transforms.
    hout2 = torch.empty(na + nb, dtype=torch.int64).pin_memory()
    outs = [hout, hout2]
    H.mul_host_pipeline([(hx, hy, outs[k % 2]) for k in range(2)])  # warm the second lane's buffers
    # Best of two calls: an occasional host-side stall of some tens of
    # milliseconds (seen on either API, outside the library) would otherwise
    # decide the number.
    pipe_runs = []
    for _ in range(2):
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        H.mul_host_pipeline([(hx, hy, outs[k % 2]) for k in range(e2e_steps)])
        pipe_runs.append(max_over_ranks(time.perf_counter() - t0, dist, "cuda"))
    pipe_s = min(pipe_runs)
    clocks = sampler.stop()
    want = out.cpu().numpy().view(np.uint64)
    ok = ok and all(bool(np.array_equal(o.numpy().view(np.uint64), want)) for o in outs)
    link = host_link()

    n_out = na + nb
    value = job_rate(ws, n_out, args.steps, ms / 1000.0)
    e2e_value = job_rate(ws, n_out, e2e_steps, pipe_s)
    e2e_single = job_rate(ws, n_out, e2e_steps, e2e_s)
    launches = sum(v["launches"] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k]["ms"])
    peak, peak_kind = _peaks()
    d = prof[dom]
    achieved = (d["bytes"] / d["launches"]) / (d["ms"] / d["launches"] / 1000.0) / 1e9 if d["ms"] > 0 else 0.0
    N = 1 << (args.log_size + 1)
    b_mul = 16 * n_out + 192 * N  # minimum-pass algorithmic bytes of one product
    prod_gbs = b_mul / (ms / args.steps / 1000.0) / 1e9
    traffic = _traffic(dom)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic (SplitMix64 limbs, seeds 1, 2 per rank)",
        "config": {"workload": f"mul {na}x{nb} limbs, transform 2^{args.log_size + 1}, 3 primes",
                   "dist": "uniform", "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "operands and workspace larger than L2; no flush"},
        "correct": ok,
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * (na + nb),
                "d2h_bytes_per_step": 8 * n_out,
                "api": "hg_mul_host_pipeline (host pointers, pinned; one call for all steps, each step's upload "
                       "and download inside it, overlapping the neighbouring steps' work)",
                "steps": e2e_steps, "ms_per_step": 1000 * pipe_s / e2e_steps,
                "timing": "best of two calls of `steps` products each",
                "ms_per_step_runs": [1000 * t / e2e_steps for t in pipe_runs],
                "single_call": {"value": e2e_single, "unit": UNIT, "api": "hg_mul (one synchronous call per step)",
                                "ms_per_step": 1000 * e2e_s / e2e_steps},
                "host_link": link},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "bytes_per_launch": d["bytes"] / max(1, d["launches"]),
                     "launches": d["launches"], "ms_per_launch": d["ms"] / max(1, d["launches"]),
                     "pipes": _pipes(dom)},
        "roofline_product": {"algorithmic_bytes": b_mul, "achieved": prod_gbs, "frac": prod_gbs / peak,
                             "unit": "GB/s", "formula": "16(na+nb) + 192 N"},
        "roofline_int": _int_roofline(N, ms / args.steps, clocks["sm_mhz"]),
        "kernels": {k: {"launches": v["launches"], "ms": v["ms"]} for k, v in prof.items() if v["launches"]},
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"],
                   "samples": clocks["samples"]},
    }
    if not args.no_sweep and ws == 1:
        line["sweep"] = run_sweep(stream, peak)
        line["correct"] = line["correct"] and line["sweep"]["correct"]
    if not args.no_batched:
        line["batched"] = run_batched(stream, args.steps)
        line["correct"] = line["correct"] and line["batched"]["correct"]
    if not args.no_mpd and ws == 1:
        line["expt"] = run_expt()
        line["correct"] = line["correct"] and line["expt"]["correct"]
    if not args.no_mpd and ws == 1:
        line["mpd_pi"] = run_mpd_pi(cpu=not args.no_cpu_baseline)
        line["correct"] = line["correct"] and line["mpd_pi"]["correct"]
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cores, model = _cpu_info()
        threads = min(6, cores)
        rate, dt = cpu_product_rate(args.log_size, threads)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"one {na}x{nb}-limb product ({dt:.1f} s)", "cpu": model,
                                "host_cores": cores,
                                "gmp": gmp_baseline(x, y, hout.numpy().view(np.uint64))}
        line["correct"] = line["correct"] and line["cpu_baseline"]["gmp"].get("matches_gpu", True)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--log-size", type=int, default=LOG_SIZE, help="log2 limbs per operand (default 24)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 4096-pair batched-products measurement")
    ap.add_argument("--no-mpd", action="store_true", help="skip the mpd-pi measurement")
    ap.add_argument("--no-sweep", action="store_true", help="skip the 2^18..2^26 balanced-product sweep")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
